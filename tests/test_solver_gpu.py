"""GPU plain FP64 matrix-diagonalisation solver (solve_3d / solver_3d)
against the FP64 oracle, through the C ABI.

Tolerance: max |gpu - oracle| <= 1e-12 * max |oracle| over the interior and
the six faces (edges/corners of solf are not written by either).  The two
sides use independent eigen-decompositions (the library's own QR solver,
the oracle LAPACK dgeev); the solve is invariant to the eigenvector basis,
so the comparison measures rounding only."""
import numpy as np
import pytest

from oracle import solver as S

from helpers import bc_arrays, field, grids, max_rel, solf_mask

pytestmark = pytest.mark.gpu


def run_case(mf, nall, bct, sigma, kind="tanh", seed=4, oracle_eigen=False):
    gx, gy, gz = grids(*nall, kind=kind)
    n1, n2, n3 = (v - 2 for v in nall)
    sc_ref = S.Solver3D(gx, gy, gz, bct, 6)
    sc = mf.SolverCoeffs3D(gx, gy, gz, bct, 6)
    if oracle_eigen:
        for a, ax in enumerate((sc_ref.cx, sc_ref.cy, sc_ref.cz)):
            sc.set_eigen(a, ax.eigen, ax.vect, ax.inv_vect)
    rhs = field((n1, n2, n3), seed)
    bcx, bcy, bcz = bc_arrays(n1, n2, n3, seed + 1)
    solf0 = field((n1 + 2, n2 + 2, n3 + 2), seed + 2)
    ref = S.solve_3d(sc_ref, rhs, sigma, solf0, bcx, bcy, bcz)
    got = sc.solve_3d(mf.to_device(rhs), sigma, mf.to_device(solf0), mf.to_device(bcx),
                      mf.to_device(bcy), mf.to_device(bcz))
    got = mf.to_host(got)
    m = solf_mask(n1, n2, n3)
    err = max_rel(got, ref, m)
    # edges and corners keep their input values
    assert np.array_equal(got[~m], solf0[~m])
    return err


BCTS = [(1, 1, 1, 1, 1, 1), (2, 2, 2, 2, 2, 2), (1, 2, 2, 1, 1, 2), (3, 1, 1, 3, 2, 1)]


@pytest.mark.parametrize("bct", BCTS)
@pytest.mark.parametrize("sigma", [0.0, -1e3, 2.0])
def test_solve_3d_kernels_same_eigenbasis(mf, gpu, bct, sigma):
    """GPU arithmetic vs oracle with the oracle's LAPACK eigen tables loaded:
    isolates the kernels from the choice of eigenvector basis."""
    if all(b == 2 for b in bct) and sigma == 0.0:
        pytest.skip("pure Neumann Poisson is covered by test_null_mode")
    assert run_case(mf, (19, 17, 23), bct, sigma, oracle_eigen=True) < 1e-12


@pytest.mark.parametrize("bct", BCTS)
@pytest.mark.parametrize("sigma", [0.0, -1e3, 2.0])
def test_solve_3d_own_eigensolver(mf, gpu, bct, sigma):
    """End to end with the library's own eigen-decomposition.  A bct = 3 face
    next to a Dirichlet face gives the 1D operator an exact null eigenvalue and
    its face values come from a 7-point extrapolation on the stretched grid;
    two correct FP64 decompositions (LAPACK vs the library's QR) then differ
    by ~4e-11 in solf, so those cases use 1e-10."""
    if all(b == 2 for b in bct) and sigma == 0.0:
        pytest.skip("pure Neumann Poisson is covered by test_null_mode")
    tol = 1e-10 if 3 in bct else 1e-12
    assert run_case(mf, (19, 17, 23), bct, sigma) < tol


@pytest.mark.parametrize("nall", [(65, 65, 65), (33, 47, 21), (9, 9, 9)])
def test_solve_3d_sizes(mf, gpu, nall):
    assert run_case(mf, nall, (1, 1, 1, 1, 1, 1), -1e3) < 1e-12


def test_null_mode(mf, gpu):
    # all-Neumann Poisson: the reference zeroes the null mode (class_solver_3d.f90:207-209)
    assert run_case(mf, (17, 17, 17), (2, 2, 2, 2, 2, 2), 0.0, kind="uniform") < 1e-10


def test_polynomial_kat_on_gpu(mf, gpu):
    """test_solver_3d recipe: GPU error vs exact equals the oracle's error."""
    from test_oracle_kat import poly_kat  # noqa: F401  (oracle error for comparison)
    from oracle import mesh
    n = 33
    gx, gy, gz = mesh.arcsin_grid(n), mesh.arcsin_grid(n), mesh.arcsin_grid(n, -0.25, 0.25)
    X, Y, Z = np.meshgrid(gx, gy, gz, indexing="ij")
    p, sigma = 9, 2.0
    uex = X ** p + Y ** p + X * Y
    g = np.asfortranarray((p - 1) * p * X ** (p - 2) + (p - 1) * p * Y ** (p - 2) + sigma * uex)
    bcx = np.asfortranarray(np.stack([uex[0, 1:-1, 1:-1], uex[-1, 1:-1, 1:-1]], -1))
    bcy = np.asfortranarray(np.stack([uex[1:-1, 0, 1:-1], uex[1:-1, -1, 1:-1]], -1))
    bcz = np.asfortranarray(np.stack([uex[1:-1, 1:-1, 0], uex[1:-1, 1:-1, -1]], -1))
    sc = mf.solver_coeffs_init_3d(gx, gy, gz, n, n, n, (1,) * 6, 6)
    u = mf.solver_3d(sc, g, np.zeros_like(g), bcx, bcy, bcz, sigma)  # host arrays
    m = solf_mask(n - 2, n - 2, n - 2)
    err = np.linalg.norm((u - uex)[m]) / np.linalg.norm(uex[m])
    assert abs(err - poly_kat(n)) < 1e-3 * err
    assert err < 1e-7


def test_shape_mismatch_is_an_error(mf, gpu):
    gx, gy, gz = grids(11, 11, 11)
    sc = mf.SolverCoeffs3D(gx, gy, gz, (1,) * 6, 6)
    bad = mf.to_device(np.zeros((10, 9, 9), order="F"))
    ok = mf.to_device(np.zeros((9, 9, 2), order="F"))
    with pytest.raises(mf.MflopsError) as e:
        sc.solve_3d(bad, 0.0, mf.to_device(np.zeros((11, 11, 11), order="F")), ok, ok, ok)
    assert e.value.code == mf.MF_ERR_ARG


def test_residual_matches_oracle(mf, gpu):
    nall = (21, 19, 17)
    gx, gy, gz = grids(*nall)
    n1, n2, n3 = (v - 2 for v in nall)
    bct = (1, 2, 1, 1, 2, 1)
    sc = mf.SolverCoeffs3D(gx, gy, gz, bct, 6)
    ref = S.Solver3D(gx, gy, gz, bct, 6)
    g = field((n1, n2, n3), 1)
    u = field((n1, n2, n3), 2)
    bcx, bcy, bcz = bc_arrays(n1, n2, n3, 3)
    want = S.residual(ref, g, u, -7.0, bcx, bcy, bcz)
    r = mf.empty_device((n1, n2, n3))
    sc.residual(mf.to_device(g), mf.to_device(u), -7.0, mf.to_device(bcx), mf.to_device(bcy),
                mf.to_device(bcz), r)
    assert max_rel(mf.to_host(r), want) < 1e-12
