"""The extended-precision yardstick of the solver (oracle/exact.py), and what
it shows about two FP64 implementations of the reference's
matrix-diagonalisation solve (CPU only: the library's host set-up is called
through the C ABI without a device, the 3-D transforms are NumPy's).

* residual_dd is the oracle's interior operator (oracle.solver.residual)
  evaluated exactly: on a random iterate the two agree to FP64 rounding,
  and on exact_solve's result it vanishes to ~1e-16 of the right-hand side.
* On the 257^3 Poisson workload (x, z uniform, y tanh(2.0), seeded k^-5/3
  right-hand side) the oracle's own solve -- LAPACK dgeev tables, as the
  reference's solver_matrix_init (class_solver_3d.f90:468-566) -- is
  ~5e-12 from the exact discrete solution: its smallest eigenvalues carry a
  relative error of eps*lambda_max/lambda_min.  The library's tables
  (own QR plus a double-double refinement of the decomposition) applied
  by the same NumPy products stay within 1e-12 of it.  So the two solvers'
  distance at that size measures the oracle's rounding, not the library's.
"""
import numpy as np
import pytest

from oracle import exact as E
from oracle import solver as S

from helpers import bc_arrays, field, grids, max_rel, rel_l2


def _with_library_tables(mf, sc, gs, bct):
    for ax, g, b in zip((sc.cx, sc.cy, sc.cz), gs, (bct[0:2], bct[2:4], bct[4:6])):
        t = mf.solver_axis_setup(g, b, 6)
        ax.eigen = np.array(t["eigen"])
        ax.vect = np.array(t["vect"])
        ax.inv_vect = np.array(t["inv_vect"])
        ax.inv_lhs = np.array(t["inv_lhs"])
    return sc


@pytest.mark.parametrize("bct,sigma", [((1,) * 6, 0.0), ((2, 2, 1, 1, 2, 1), -30.0)])
def test_residual_dd_matches_fp64_operator(bct, sigma):
    gs = grids(15, 13, 17)
    n1, n2, n3 = 13, 11, 15
    sc = S.Solver3D(*gs, bct, 6)
    g = field((n1, n2, n3), 1)
    u = field((n1, n2, n3), 2)
    bcx, bcy, bcz = bc_arrays(n1, n2, n3, 3)
    hi, lo = E.residual_dd(sc, g, u, sigma, bcx, bcy, bcz)
    want = S.residual(sc, g, u, sigma, bcx, bcy, bcz)
    assert max_rel(hi + lo, want) < 1e-12
    assert np.all(np.abs(lo) <= 1.2e-16 * np.abs(hi))


@pytest.mark.parametrize("bct,sigma", [((1,) * 6, 0.0), ((1, 2, 2, 1, 1, 2), -1e3)])
def test_exact_solve_has_no_residual(bct, sigma):
    gs = grids(21, 19, 17)
    n1, n2, n3 = 19, 17, 15
    sc = S.Solver3D(*gs, bct, 6)
    rhs = field((n1, n2, n3), 4)
    bcx, bcy, bcz = bc_arrays(n1, n2, n3, 5)
    solf = np.zeros((n1 + 2, n2 + 2, n3 + 2), order="F")
    ex = E.exact_solve(sc, rhs, sigma, solf, bcx, bcy, bcz)
    # a rounded solution keeps a residual of order eps*|A||u|; what shows
    # that it is the exactly rounded one is that a second correction with
    # the exact residual no longer moves it
    ex2 = E.exact_solve(sc, rhs, sigma, solf, bcx, bcy, bcz, steps=2)
    assert rel_l2(ex2, ex) < 2e-16
    plain = S.solve_3d(sc, rhs, sigma, solf, bcx, bcy, bcz)
    assert rel_l2(plain[1:-1, 1:-1, 1:-1], ex[1:-1, 1:-1, 1:-1]) < 1e-12


def test_257_oracle_rounding_vs_library_tables(mf):
    import bench
    gs, rhs, bcs = bench.workload(257)
    bct = (1,) * 6
    sc = S.Solver3D(*gs, bct, 6)
    solf = np.zeros((257, 257, 257), order="F")
    ex = E.exact_solve(sc, rhs, 0.0, solf, *bcs)[1:-1, 1:-1, 1:-1]
    oracle = S.solve_3d(sc, rhs, 0.0, solf, *bcs)[1:-1, 1:-1, 1:-1]
    lib = S.solve_3d(_with_library_tables(mf, S.Solver3D(*gs, bct, 6), gs, bct), rhs, 0.0, solf,
                     *bcs)[1:-1, 1:-1, 1:-1]
    e_oracle = rel_l2(oracle, ex)
    e_lib = rel_l2(lib, ex)
    print("257^3: oracle (LAPACK tables) vs exact %.2e, library tables vs exact %.2e" % (e_oracle, e_lib))
    assert e_lib < 1e-12
    assert e_oracle > 2e-12          # the reference method's own FP64 rounding at this size
    assert e_lib < 0.25 * e_oracle
