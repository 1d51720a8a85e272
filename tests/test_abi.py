"""The C-ABI library loads without a GPU and exports every symbol declared
in include/mflops_gb300.h; handle creation fails cleanly without a device."""
import ctypes
import os
import re

import numpy as np

from conftest import ROOT


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "mflops_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(mf_\w+)\s*\(", txt, re.M)))


def test_exports_all_declared(mf):
    lib = ctypes.CDLL(mf.lib_path())
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binds_all_declared(mf):
    assert set(declared_symbols()) <= set(mf.exported_symbols())


def test_no_device_is_reported_cleanly(mf):
    import torch
    if torch.cuda.is_available():
        return
    assert mf.device_available() is False
    try:
        mf.DerivativesCoefficients(np.linspace(0, 1, 11), solve=False, so=6)
    except mf.MflopsError as e:
        assert e.code in (mf.MF_ERR_CUDA, mf.MF_ERR_ALLOC)
    else:
        raise AssertionError("handle creation must fail loudly without a GPU")


def test_argument_errors_need_no_device(mf):
    """Entry points reject bad arguments with MF_ERR_ARG before touching the
    device (null handles, right-hand-side counts outside 1..4, unknown modes)."""
    lib = ctypes.CDLL(mf.lib_path())
    P = ctypes.c_void_p
    PP = ctypes.POINTER(ctypes.c_void_p)
    lib.mf_md_solve_many.argtypes = [P, ctypes.c_int, PP, PP, PP, PP, PP, P]
    lib.mf_md_solve.argtypes = [P, PP, PP, PP, PP, PP, P]
    lib.mf_md_set_precision.argtypes = [P, ctypes.c_int, ctypes.c_int]
    lib.mf_md_set_interface_solve.argtypes = [P, ctypes.c_int]
    lib.mf_solver3d_set_residual.argtypes = [P, ctypes.c_int]
    arr = (ctypes.c_void_p * 8)()
    for nrhs in (0, 1, 3, 5):
        assert lib.mf_md_solve_many(None, nrhs, arr, arr, arr, arr, arr, None) == mf.MF_ERR_ARG
    assert lib.mf_md_solve(None, arr, arr, arr, arr, arr, None) == mf.MF_ERR_ARG
    assert lib.mf_md_set_precision(None, mf.MF_PREC_3XTF32, 1) == mf.MF_ERR_ARG
    assert lib.mf_md_set_interface_solve(None, mf.MD_IFACE_INVERSE) == mf.MF_ERR_ARG
    assert lib.mf_md_set_interface_solve(None, mf.MD_IFACE_TRIANGULAR_INVERSE) == mf.MF_ERR_ARG
    assert lib.mf_md_set_interface_solve(None, mf.MD_IFACE_TRIANGULAR_INVERSE_FP64) == mf.MF_ERR_ARG
    lib.mf_md_interface_form.argtypes = [P, P]
    assert lib.mf_md_interface_form(None, None) == mf.MF_ERR_ARG
    lib.mf_md_interface_solve.argtypes = [P, ctypes.c_int, P, P, P]
    for nrhs in (0, 1, 5):
        assert lib.mf_md_interface_solve(None, nrhs, None, None, None) == mf.MF_ERR_ARG
    for mode in (mf.MF_RESID_FF, mf.MF_RESID_FP64, mf.MF_RESID_FP64_LINE):
        assert lib.mf_solver3d_set_residual(None, mode) == mf.MF_ERR_ARG
