"""Committed golden fixtures (tests/golden/golden_small.npz, written by
tests/golden/make_golden.py from seeded inputs and the oracle).

CPU: the oracle still reproduces every fixture (1e-13 relative for the
direct computations; 1e-12 where a LAPACK eigen-decomposition or a dense
solve sits in between).  GPU, through the C ABI: the CUDA path against the
fixtures at the parity bars of the other tests (derivatives, filter, LES
1e-12; plain solver 1e-12; multidomain 1e-11; learned-coefficient gradient
2e-4 of its largest component, FP32 kernel)."""
import os

import numpy as np
import pytest

from oracle import derivatives as D
from oracle import filter as F
from oracle import les as L
from oracle import md as OMD
from oracle import mlp as OM
from oracle import solver as S

from helpers import max_rel, solf_mask

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def gold():
    with np.load(os.path.join(HERE, "golden", "golden_small.npz")) as z:
        return {k: z[k] for k in z.files}


def F_(a):
    return np.asfortranarray(a)


DER_OPS = {(0, 1): D.derx, (1, 1): D.dery, (2, 1): D.derz,
           (0, 2): D.dderx, (1, 2): D.ddery, (2, 2): D.dderz}


def der_keys():
    return [(so, sv, ax, od) for so in (4, 6) for sv in (0, 1) for (ax, od) in DER_OPS]


def solver_case(gold, c):
    p = "solver/%d/" % c
    grids = [gold[p + "grid%d" % a] for a in range(3)]
    bcs = [F_(gold[p + "bc%d" % a]) for a in range(3)]
    return (grids, tuple(int(v) for v in gold[p + "bct"]), float(gold[p + "sigma"]),
            F_(gold[p + "rhs"]), F_(gold[p + "solf0"]), bcs, gold[p + "solf"])


def md_case(gold):
    gx = [gold["md/sub0/gx"], gold["md/sub1/gx"]]
    gy, gz = [gold["md/gy"]], [gold["md/gz"]]
    subs = [(0, 0, 0), (1, 0, 0)]
    g = {c: F_(gold["md/sub%d/g" % c[0]]) for c in subs}
    bc = {c: [F_(gold["md/sub%d/bc%d" % (c[0], a)]) for a in range(3)] for c in subs}
    u = {c: gold["md/sub%d/u" % c[0]] for c in subs}
    return gx, gy, gz, subs, g, bc, u, float(gold["md/sigma"]), gold["md/lambda"]


# ---------------------------------------------------------------------------
# CPU: the oracle reproduces its committed outputs
# ---------------------------------------------------------------------------

def test_oracle_reproduces_derivative_fixtures(gold):
    f = gold["der/f"]
    grids = [gold["der/grid%d" % a] for a in range(3)]
    for so, sv, ax, od in der_keys():
        got = DER_OPS[(ax, od)](D.DerCoeffs(grids[ax], so, bool(sv)), f)
        assert max_rel(got, gold["der/so%d/solver%d/axis%d/order%d" % (so, sv, ax, od)]) < 1e-13


@pytest.mark.parametrize("c", range(4))
def test_oracle_reproduces_solver_fixtures(gold, c):
    grids, bct, sigma, rhs, solf0, bcs, want = solver_case(gold, c)
    got = S.solve_3d(S.Solver3D(*grids, bct, 6), rhs, sigma, solf0, *bcs)
    assert max_rel(got, want) < 1e-12


def test_oracle_reproduces_filter_fixtures(gold):
    xi, xn, xo, wi, k = (gold["filter/" + s] for s in ("xi", "xn", "xo", "wi", "k"))
    f = gold["filter/f"]
    for a in range(f.shape[1]):
        for b in range(f.shape[2]):
            yo, ypo = F.lsq_univariate_spline(xi, f[:, a, b], wi, xn, xo, int(k))
            assert max_rel(yo, gold["filter/yo"][:, a, b]) < 1e-13
            assert max_rel(ypo, gold["filter/ypo"][:, a, b]) < 1e-13
    yo = F.interp_period(gold["period/xi"], gold["period/yi"], gold["period/xo"])[0]
    assert max_rel(yo, gold["period/yo"]) < 1e-13


def test_oracle_reproduces_md_fixture(gold):
    gx, gy, gz, subs, g, bc, u, sigma, lam = md_case(gold)
    ref = OMD.MultiDomain((2, 1, 1), (0, 0, 0), gx, gy, gz, (1,) * 6)
    ref.influence_matrix(sigma, 0)
    want, lam2 = ref.solve(g, bc, sigma)
    assert max_rel(lam2, lam) < 1e-12
    for c in subs:
        assert max_rel(want[c], u[c]) < 1e-12


def test_oracle_reproduces_les_and_mlp_fixtures(gold):
    grids = [gold["les/grid%d" % a] for a in range(3)]
    du = [[gold["les/du%d%d" % (i, j)] for j in range(3)] for i in range(3)]
    for t in (1, 2, 3):
        assert max_rel(L.les_nu(du, *grids, t, 0.17), gold["les/nu%d" % t]) < 1e-13
    loss, g = OM.loss_and_grad(gold["mlp/params"], gold["mlp/X"], gold["mlp/base"], gold["mlp/target"],
                               np.zeros(6), np.ones(6), 0.02, 1000.0)
    assert abs(loss - float(gold["mlp/loss"])) <= 1e-13 * abs(loss)
    assert max_rel(g, gold["mlp/grad"]) < 1e-12


# ---------------------------------------------------------------------------
# GPU: the CUDA path against the fixtures
# ---------------------------------------------------------------------------

@pytest.mark.gpu
def test_gpu_derivatives_match_fixtures(mf, gpu, gold):
    f = mf.to_device(gold["der/f"])
    grids = [gold["der/grid%d" % a] for a in range(3)]
    for so, sv, ax, od in der_keys():
        dc = mf.DerivativesCoefficients(grids[ax], solve=bool(sv), so=so)
        got = mf.to_host(dc.apply(ax, od, f))
        assert max_rel(got, gold["der/so%d/solver%d/axis%d/order%d" % (so, sv, ax, od)]) < 1e-12, (so, sv, ax, od)


@pytest.mark.gpu
@pytest.mark.parametrize("c", range(4))
def test_gpu_solver_matches_fixtures(mf, gpu, gold, c):
    grids, bct, sigma, rhs, solf0, bcs, want = solver_case(gold, c)
    sc = mf.SolverCoeffs3D(*grids, bct, 6)
    got = mf.to_host(sc.solve_3d(mf.to_device(rhs), sigma, mf.to_device(solf0),
                                 *[mf.to_device(b) for b in bcs]))
    m = solf_mask(*rhs.shape)
    assert max_rel(got, want, m) < 1e-12


@pytest.mark.gpu
def test_gpu_filter_matches_fixtures(mf, gpu, gold):
    xi, xn, xo, wi, k = (gold["filter/" + s] for s in ("xi", "xn", "xo", "wi", "k"))
    flt = mf.SplineFilter(xi, xo, xn=xn, wi=wi, k=int(k))
    f = mf.to_device(gold["filter/f"])
    assert max_rel(mf.to_host(flt.apply(f, 0)), gold["filter/yo"]) < 1e-12
    assert max_rel(mf.to_host(flt.apply(f, 0, deriv=True)), gold["filter/ypo"]) < 1e-12
    yo = mf.interp_period(gold["period/xi"], gold["period/yi"], gold["period/xo"])
    assert max_rel(yo, gold["period/yo"]) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("iface", [0, 1])
def test_gpu_md_matches_fixture(mf, gpu, gold, iface):
    gx, gy, gz, subs, g, bc, u, sigma, lam = md_case(gold)
    dev = mf.MultiDomain((2, 1, 1), (0, 0, 0), gx, gy, gz, (1,) * 6)
    dev.set_interface_solve(iface)
    dev.influence_matrix_set(sigma, 0)
    gd = {c: mf.to_device(g[c]) for c in subs}
    ud = {c: mf.empty_device(g[c].shape) for c in subs}
    bd = {c: [mf.to_device(b) for b in bc[c]] for c in subs}
    dev.solve(gd, ud, bd)
    assert max_rel(dev.interface(), lam) < 1e-11
    for c in subs:
        got = mf.to_host(ud[c])
        assert max_rel(got[1:-1, 1:-1, 1:-1], u[c][1:-1, 1:-1, 1:-1]) < 1e-11


@pytest.mark.gpu
def test_gpu_les_and_mlp_match_fixtures(mf, gpu, gold):
    import torch
    grids = [gold["les/grid%d" % a] for a in range(3)]
    les = mf.LesModel(*grids)
    ddu = [[mf.to_device(gold["les/du%d%d" % (i, j)]) for j in range(3)] for i in range(3)]
    for t in (1, 2, 3):
        tol = 1e-10 if t == 3 else 1e-12
        assert max_rel(mf.to_host(les.nu(ddu, t, 0.17)), gold["les/nu%d" % t]) < tol
    m = mf.Mlp(0)
    m.set_params(gold["mlp/params"].astype(np.float32))
    inf = np.full(6, np.inf, np.float32)
    m.set_scaling(np.zeros(6), np.ones(6), -inf, inf, 0.02, 1000.0)
    t32 = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float32, device="cuda")
    loss, g = m.train_step(t32(gold["mlp/X"]), t32(gold["mlp/base"]), t32(gold["mlp/target"]), lr=0.0,
                           want_grad=True, want_loss=True)
    assert abs(loss - float(gold["mlp/loss"])) <= 1e-4 * abs(float(gold["mlp/loss"]))
    assert np.max(np.abs(g - gold["mlp/grad"])) <= 2e-4 * np.max(np.abs(gold["mlp/grad"]))
