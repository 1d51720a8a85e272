"""Host (CPU) set-up of the C ABI against the oracle: compact coefficients,
quasi-penta LU, solver matrices and the eigen-decomposition.  No GPU."""
import numpy as np
import pytest

from oracle import derivatives as D
from oracle import mesh
from oracle import solver as S

from helpers import max_rel


@pytest.mark.parametrize("so", [2, 4, 6, 8])
@pytest.mark.parametrize("der", [1, 2])
@pytest.mark.parametrize("kind", ["uniform", "tanh", "arcsin"])
def test_der_line_coeffs(mf, so, der, kind):
    n = 23
    g = {"uniform": mesh.uniform_grid(n), "tanh": mesh.tanh_grid(n, 2.0),
         "arcsin": mesh.arcsin_grid(n)}[kind]
    dl, dr = mf.der_line_coeffs(g, der, so)
    odl, odr = D.der_coeffs_global(g, der, so)
    # so=8 rows come from a 9x9 Taylor (Vandermonde-like) system whose
    # condition number on stretched grids reaches ~1e6-1e7: two partial-pivot
    # solvers (here, or two LAPACK builds of the reference) agree only to
    # ~cond*eps there.  so <= 6 systems agree to a few ulps.
    tol = 1e-12 if so <= 6 else 1e-9
    assert max_rel(dl, odl) < tol
    assert max_rel(dr, odr) < tol
    assert max_rel(mf.pentalu(dl), D.pentalu(odl)) < tol


@pytest.mark.parametrize("cl", [1, 2, 3])
def test_der_coeffs_generic_row(mf, cl):
    h0 = np.array([0.0, -0.01, -0.025, -0.04, -0.06, -0.085, -0.11])
    if cl == 3:
        h0 = np.array([0.02, 0.009, 0.0, -0.011, -0.023, 0.0, 0.0])
    ci, ce = mf.der_coeffs_generic(h0, cl, 1, 6)
    oci, oce = D.der_coeffs_generic(h0, cl, 1, 6)
    assert max_rel(ci, oci) < 1e-12 and max_rel(ce, oce) < 1e-12


@pytest.mark.parametrize("bct", [(1, 1), (2, 2), (1, 2), (3, 1), (2, 3)])
@pytest.mark.parametrize("so", [4, 6, 8])
def test_solver_axis_setup(mf, bct, so):
    g = mesh.tanh_grid(29, 1.5)
    try:
        ax = S.SolverAxis(g, bct, so)
    except S.EigenError:
        # the reference stops on complex eigenvalues (class_solver_3d.f90:537-540);
        # the library must refuse the same operator with MF_ERR_COMPLEX_EIG
        with pytest.raises(mf.MflopsError) as e:
            mf.solver_axis_setup(g, bct, so)
        assert e.value.code == mf.MF_ERR_COMPLEX_EIG
        return
    out = mf.solver_axis_setup(g, bct, so)
    tol = 1e-12 if so <= 6 else 1e-9  # so=8: ill-conditioned Taylor systems, see above
    assert max_rel(out["ddl"], ax.ddl) < tol
    assert max_rel(out["ddr"], ax.ddr) < tol
    assert max_rel(out["inv_lhs"], ax.inv_lhs) < max(tol, 1e-10)
    assert max_rel(out["neum"], ax.neum) < tol
    # eigenvalues: same set (order may differ)
    assert max_rel(np.sort(out["eigen"]), np.sort(ax.eigen)) < 1e-10
    # V diag(w) V^-1 reproduces inv_lhs * rhs
    lhs, rhs = S.lhs_rhs_matrices(ax.ddl, ax.ddr)
    T = np.linalg.solve(lhs, rhs)
    Tr = out["vect"] @ np.diag(out["eigen"]) @ out["inv_vect"]
    assert max_rel(Tr, T) < 1e-10
    assert max_rel(out["vect"] @ out["inv_vect"], np.eye(g.size - 2)) < 1e-11


def test_solver_axis_setup_large(mf):
    g = mesh.tanh_grid(257, 2.0)
    out = mf.solver_axis_setup(g, (1, 1), 6)
    ax = S.SolverAxis(g, (1, 1), 6)
    assert max_rel(np.sort(out["eigen"]), np.sort(ax.eigen)) < 1e-9
    lhs, rhs = S.lhs_rhs_matrices(ax.ddl, ax.ddr)
    T = np.linalg.solve(lhs, rhs)
    Tr = out["vect"] @ np.diag(out["eigen"]) @ out["inv_vect"]
    assert max_rel(Tr, T) < 1e-9


def test_setup_errors(mf):
    with pytest.raises(mf.MflopsError) as e:
        mf.solver_axis_setup(np.linspace(0, 1, 6), (1, 1), 6)
    assert e.value.code == mf.MF_ERR_ARG
    with pytest.raises(mf.MflopsError) as e:
        mf.solver_axis_setup(np.linspace(0, 1, 20), (1, 7), 6)
    assert e.value.code == mf.MF_ERR_ARG
    g = np.linspace(0, 1, 20)
    g[5] = g[4]  # coincident nodes -> singular Taylor system
    with pytest.raises(mf.MflopsError):
        mf.solver_axis_setup(g, (1, 1), 6)
