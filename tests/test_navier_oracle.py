"""CPU checks of the Navier-Stokes time-step oracle and of the step's host
logic (no GPU).

Known answer: the reference's exact solution (class_navier_3D.f90:927-1041) is
steady, and with one mode its sources are exact, so the incremental scheme
(pt = 2) started on it stays on it up to the spatial error; the flow-rate term
(:1140-1164) starts at debit = 1 for a mean-free u and then follows
g -= (mean(extrapol(u)) - debit) fac(1).
"""
import ctypes

import numpy as np
import pytest

from oracle import mesh
from oracle import navier as N


def start_on_exact(nav, nmodes=1):
    X, Y, Z = nav.points()
    for s in range(N.NT):
        nav.u[s] = N.sol(X, Y, Z, 0.0, "u", nav.rey, nmodes)
        nav.v[s] = N.sol(X, Y, Z, 0.0, "v", nav.rey, nmodes)
        nav.p[s] = N.sol(X, Y, Z, 0.0, "p", nav.rey, nmodes)
        nav.phi[s] = nav.p[s].copy()


def test_incremental_scheme_keeps_the_exact_solution():
    g = mesh.tanh_grid(21, 1.0)
    nav = N.Navier(g, g, g, ts=1e-2, rey=10.0, pt=2, flow_rate=False, nmodes=1)
    start_on_exact(nav)
    for _ in range(5):
        d = nav.advance(diagnostics=True)
    assert d["vel"][1] < 1e-6 and d["pres"][1] < 1e-6 and d["div"] < 1e-6


def test_exact_solution_is_divergence_free_and_mode_sum_is_not_exact():
    g = mesh.uniform_grid(33)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    h = 1e-6
    for nm in (1, 5):
        dudx = (N.sol(X + h, Y, Z, 0, "u", 1.0, nm) - N.sol(X - h, Y, Z, 0, "u", 1.0, nm)) / (2 * h)
        dvdy = (N.sol(X, Y + h, Z, 0, "v", 1.0, nm) - N.sol(X, Y - h, Z, 0, "v", 1.0, nm)) / (2 * h)
        assert np.abs(dudx + dvdy).max() < 1e-6
    # steady momentum residual of the sources: exact for one mode only
    def residual(nm, rey=1.0):
        u = lambda x, y: N.sol(x, y, 0 * x, 0, "u", rey, nm)
        v = lambda x, y: N.sol(x, y, 0 * x, 0, "v", rey, nm)
        p = lambda x, y: N.sol(x, y, 0 * x, 0, "p", rey, nm)
        x, y = X[:, :, 0], Y[:, :, 0]
        d = lambda f, a: ((f(x + h, y) - f(x - h, y)) if a == 0 else (f(x, y + h) - f(x, y - h))) / (2 * h)
        lap = lambda f: (f(x + h, y) + f(x - h, y) + f(x, y + h) + f(x, y - h) - 4 * f(x, y)) / h ** 2
        r = u(x, y) * d(u, 0) + v(x, y) * d(u, 1) + d(p, 0) - lap(u) / rey - N.sol(x, y, 0 * x, 0, "rhsu", rey, nm)
        return np.abs(r).max()
    assert residual(1) < 1e-3
    assert residual(5) > 1e-1


def test_flow_rate_term_follows_the_reference_update():
    g = mesh.tanh_grid(13, 1.0)
    nav = N.Navier(g, g, g, ts=0.1, rey=5.0, nmodes=5)
    start_on_exact(nav, 5)
    nav.advance()
    assert nav.debit == 1.0
    reft = nav.integrale(np.ones((13, 13, 13)))
    g1 = nav.g
    mean = nav.integrale(nav.extrapol(nav.u, "v")) / reft
    nav.advance()
    assert nav.g == pytest.approx(g1 - (mean - 1.0) * nav.fac[0], rel=1e-12)


def test_quadrature_weights_skip_edges():
    g = mesh.tanh_grid(9, 1.0)
    W = N.quad_weights(g, g, g)
    assert W[0, 0, 4] == 0 and W[0, 4, 0] == 0 and W[0, 0, 0] == 0
    assert W[0, 4, 4] > 0 and W[4, 4, 4] > 0


def test_navier_create_rejects_bad_parameters(mf):
    g = mesh.uniform_grid(17)
    for kw in ({"pt": 5}, {"tou": 4}, {"nlt": 5}, {"ts": 0.0}, {"reynolds": -1.0}, {"precision": 9}):
        with pytest.raises(mf.MflopsError) as e:
            mf.NavierStokes3D(g, g, g, **kw)
        assert e.value.code == mf.MF_ERR_ARG, kw
    with pytest.raises(mf.MflopsError):
        mf.NavierStokes3D(g[:8], g, g)
    prm = mf.NavierParams()
    assert mf._lib.mf_navier_defaults(ctypes.byref(prm)) == 0
    assert (prm.nlt, prm.pt, prm.tou, prm.top, prm.so_solver, prm.so_der, prm.nmodes) == (2, 1, 2, 2, 6, 6, 5)
    assert prm.ts == 1.0 and prm.reynolds == 1.0 and prm.flow_rate == 1
    assert prm.les_type == 0 and prm.les_c == 0.0
    with pytest.raises(mf.MflopsError):
        mf.NavierStokes3D(g, g, g, les_type=4)


@pytest.mark.parametrize("pt", [3, 4])
def test_velocity_correction_schemes_keep_the_exact_solution(pt):
    """Pressure types 3 (rot-rot Neumann data) and 4 (increments of the
    right-hand side) started on the one-mode exact solution stay on it; type 4
    needs the previous step's right-hand side, set here from the solution."""
    from oracle.les import zero_edges
    g = mesh.tanh_grid(21, 1.0)
    nav = N.Navier(g, g, g, ts=1e-2, rey=10.0, pt=pt, flow_rate=False, nmodes=1)
    start_on_exact(nav)
    if pt == 4:
        levels = {"u": nav.u, "v": nav.v, "w": nav.w}
        for c in "uvw":
            nav.rhs[c][0] = zero_edges(nav.forcing(c) - nav.nonlinear(levels[c]))
    for _ in range(5):
        d = nav.advance(diagnostics=True)
    assert d["vel"][1] < 2e-6 and d["pres"][1] < 2e-6 and d["div"] < 2e-6
