"""Builds libmflops_gb300.so in-tree for sm_103a (GB300).

Each translation unit of ``csrc/`` is compiled by nvcc in parallel, then
linked into ``lib/libmflops_gb300.so`` (CUDA runtime linked statically, no
libcuda link dependency: the driver entry point for tensor maps is fetched at
run time).  Usage: ``python build.py`` or ``build.build()``.
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(HERE, "_build")
LIBNAME = "libmflops_gb300.so"
SOURCES = ["mf_common.cu", "mf_der.cu", "mf_solver.cu", "mf_tc.cu", "mf_setup.cpp",
           "mf_md.cu", "mf_filter.cu", "mf_les.cu", "mf_mlp.cu", "mf_flow.cu",
           "mf_stats.cu", "mf_navier.cu"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _flags():
    # host code: no floating-point contraction, so set-up arithmetic (the
    # double-double eigen refinement above all) is the same on x86 and Arm
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3,-ffp-contract=off",
                   "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def lib_path():
    return os.path.join(LIBDIR, LIBNAME)


def _compile(src, verbose=False):
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJDIR, src + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= _newest_input(path):
        return obj
    lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
    cmd = [_nvcc()] + _flags() + lang + ["-c", path, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, res.stdout, res.stderr))
    return obj


def _newest_input(path):
    newest = os.path.getmtime(path)
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                newest = max(newest, os.path.getmtime(os.path.join(d, f)))
    newest = max(newest, os.path.getmtime(os.path.abspath(__file__)))
    return newest


def build(verbose=False):
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    out = lib_path()
    if not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(o) for o in objs):
        cuda_lib = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64")
        cmd = ([_nvcc()] + ARCH + ["-shared", "-o", out] + objs +
               ["-cudart", "static", "-L" + cuda_lib, "-lcusolver", "-lcublas",
                "-Xlinker", "-rpath", "-Xlinker", cuda_lib])
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (res.stdout, res.stderr))
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
