"""Extended-precision yardstick for the solver (test infrastructure only).

``exact_solve`` returns the solution of the discrete Poisson/Helmholtz
problem that ``solve_3d`` (src/class_solver/class_solver_3d.f90:83-299)
approximates, correct to FP64 rounding: the oracle's FP64 solve, one
correction solve with the residual computed in double-double by
``exact_dd.c`` (the interior operator of solver_matrix_init, :468-521, with
the boundary fold of :104-175), and the corrected interior written back
through the oracle's boundary insertion (:250-297).

Why it exists: two FP64 matrix-diagonalisation solves built on different,
equally correct eigen-decompositions differ by their rounding.  On a 257^3
grid that rounding is ~5e-12 of the solution: the smallest eigenvalues of
``inv(lhs) @ rhs`` (the ones a Poisson solution weights most) carry a
relative error of order eps * lambda_max / lambda_min.  Comparing each
implementation with this solution measures each one's own error, so their
distance from each other can be attributed.

The C part is compiled on first use with gcc (``build()``); the library
lives under ``oracle/_build/``.
"""
import ctypes
import os
import subprocess

import numpy as np

from . import solver as S

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "exact_dd.c")
_OUT = os.path.join(_HERE, "_build", "libexact_dd.so")
_lib = None


def build():
    """Compile exact_dd.c (gcc, OpenMP, no fused multiply-adds other than the
    explicit ``fma`` calls) unless the library is newer than the source."""
    os.makedirs(os.path.dirname(_OUT), exist_ok=True)
    if os.path.exists(_OUT) and os.path.getmtime(_OUT) >= os.path.getmtime(_SRC):
        return _OUT
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=c11",
           _SRC, "-o", _OUT, "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("gcc failed for exact_dd.c:\n%s%s" % (res.stdout, res.stderr))
    return _OUT


def _load():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        dp = ctypes.POINTER(ctypes.c_double)
        _lib.mfo_residual_dd.argtypes = ([ctypes.c_int] * 3 + [dp, dp, ctypes.c_double] + [dp] * 11)
        _lib.mfo_residual_dd.restype = ctypes.c_int
    return _lib


def _ptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def residual_dd(sc, g, u, sigma, bcx=None, bcy=None, bcz=None):
    """(hi, lo) of g - sigma*u - (Lx + Ly + Lz) u on the interior, boundary
    data included; every array Fortran-ordered (n1, n2, n3)."""
    lib = _load()
    g = np.asfortranarray(g, dtype=np.float64)
    u = np.asfortranarray(u, dtype=np.float64)
    n1, n2, n3 = g.shape
    hi = np.zeros((n1, n2, n3), order="F")
    lo = np.zeros((n1, n2, n3), order="F")
    tabs = []
    for ax in (sc.cx, sc.cy, sc.cz):
        tabs += [np.asfortranarray(ax.ddl), np.asfortranarray(ax.ddr)]
    bcs = [None if b is None else np.asfortranarray(b, dtype=np.float64) for b in (bcx, bcy, bcz)]
    rc = lib.mfo_residual_dd(n1, n2, n3, _ptr(g), _ptr(u), float(sigma), *[_ptr(t) for t in tabs],
                             *[_ptr(b) for b in bcs], _ptr(hi), _ptr(lo))
    if rc != 0:
        raise RuntimeError("mfo_residual_dd failed (%d)" % rc)
    return hi, lo


def exact_solve(sc, rhs, sigma, solf, bcx, bcy, bcz, steps=1):
    """solve_3d's result corrected to the exactly rounded discrete solution.

    Operators with a null eigenvalue at sigma = 0 are not supported (the
    correction would be defined only up to the null mode)."""
    n1, n2, n3 = rhs.shape
    zero = (np.zeros((n2, n3, 2), order="F"), np.zeros((n1, n3, 2), order="F"),
            np.zeros((n1, n2, 2), order="F"))
    blank = np.zeros((n1 + 2, n2 + 2, n3 + 2), order="F")
    u = np.asfortranarray(S.solve_3d(sc, rhs, sigma, blank, bcx, bcy, bcz)[1:-1, 1:-1, 1:-1])
    for _ in range(steps):
        hi, lo = residual_dd(sc, rhs, u, sigma, bcx, bcy, bcz)
        e = S.solve_3d(sc, hi + lo, sigma, blank, *zero)[1:-1, 1:-1, 1:-1]
        u = np.asfortranarray(u + e)
    return S.insert_bc(sc, u, solf, bcx, bcy, bcz)
