"""Writes tests/golden/golden_small.npz: seeded inputs and the oracle's
outputs for small cases of every row of the path (test infrastructure).

The reference ships no stored vectors and cannot be built here, so these
fixtures come from the oracle restatement (itself pinned to the reference's
known-answer recipes in tests/test_oracle_kat.py).  They freeze the oracle's
outputs: tests/test_golden.py checks that the oracle still reproduces them
(CPU) and that the CUDA path matches them (GPU), so a change to either side
shows up against a fixed file.  Inputs are stored beside the outputs.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import derivatives as D  # noqa: E402
from oracle import filter as F  # noqa: E402
from oracle import les as L  # noqa: E402
from oracle import md as OMD  # noqa: E402
from oracle import mesh  # noqa: E402
from oracle import mlp as OM  # noqa: E402
from oracle import solver as S  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden_small.npz")


def rand(rng, shape, lo=-1.0, hi=1.0):
    return np.asfortranarray(rng.uniform(lo, hi, size=shape))


def derivative_cases(out, rng):
    shape = (12, 10, 9)
    grids = [mesh.tanh_grid(n, 1.5) for n in shape]
    f = rand(rng, shape)
    out["der/f"] = f
    for a, g in enumerate(grids):
        out["der/grid%d" % a] = g
    ops = {(0, 1): D.derx, (1, 1): D.dery, (2, 1): D.derz,
           (0, 2): D.dderx, (1, 2): D.ddery, (2, 2): D.dderz}
    for so in (4, 6):
        for solver in (False, True):
            dcs = [D.DerCoeffs(g, so, solver) for g in grids]
            for (axis, order), fn in ops.items():
                out["der/so%d/solver%d/axis%d/order%d" % (so, solver, axis, order)] = fn(dcs[axis], f)


SOLVER_CASES = [((13, 11, 9), (1, 1, 1, 1, 1, 1), 0.0), ((13, 11, 9), (1, 1, 1, 1, 1, 1), -1e3),
                ((11, 12, 10), (1, 2, 2, 1, 1, 2), 2.0), ((10, 10, 10), (2, 2, 2, 2, 2, 2), -5.0)]


def solver_cases(out, rng):
    for c, (nall, bct, sigma) in enumerate(SOLVER_CASES):
        grids = [mesh.tanh_grid(n, 1.5) for n in nall]
        n1, n2, n3 = (v - 2 for v in nall)
        rhs = rand(rng, (n1, n2, n3))
        bcs = [rand(rng, (n2, n3, 2)), rand(rng, (n1, n3, 2)), rand(rng, (n1, n2, 2))]
        solf0 = rand(rng, (n1 + 2, n2 + 2, n3 + 2))
        sc = S.Solver3D(*grids, bct, 6)
        ref = S.solve_3d(sc, rhs, sigma, solf0, *bcs)
        p = "solver/%d/" % c
        for a in range(3):
            out[p + "grid%d" % a] = grids[a]
            out[p + "bc%d" % a] = bcs[a]
        out[p + "bct"] = np.array(bct)
        out[p + "sigma"] = np.array(sigma)
        out[p + "rhs"] = rhs
        out[p + "solf0"] = solf0
        out[p + "solf"] = ref


def filter_cases(out, rng):
    ni, no, nn, k = 48, 13, 9, 3
    xi = mesh.tanh_grid(ni, 1.5)
    xn = mesh.tanh_grid(nn, 1.0)
    xo = mesh.tanh_grid(no, 1.5)
    wi = np.ones(ni)
    f = rand(rng, (ni, 4, 3))
    yo = np.zeros((no, 4, 3), order="F")
    ypo = np.zeros((no, 4, 3), order="F")
    for a in range(4):
        for b in range(3):
            yo[:, a, b], ypo[:, a, b] = F.lsq_univariate_spline(xi, f[:, a, b], wi, xn, xo, k)
    out.update({"filter/xi": xi, "filter/xn": xn, "filter/xo": xo, "filter/wi": wi,
                "filter/k": np.array(k), "filter/f": f, "filter/yo": yo, "filter/ypo": ypo})
    xp = np.linspace(0, 2.0, 40)
    yp = np.sin(np.pi * xp) + 0.3 * rng.uniform(-1, 1, xp.size)
    xos = mesh.tanh_grid(17, 0.8, 0, 2.0)
    out.update({"period/xi": xp, "period/yi": yp, "period/xo": xos,
                "period/yo": F.interp_period(xp, yp, xos)[0]})


def md_case(out, rng):
    nd, periods, bct, sigma = (2, 1, 1), (0, 0, 0), (1,) * 6, -3.0
    gx = [mesh.tanh_grid(9, 1.0, 0.0, 0.5), mesh.tanh_grid(11, 1.0, 0.5, 1.0)]
    gy = [mesh.tanh_grid(9, 1.0)]
    gz = [mesh.tanh_grid(9, 1.0)]
    ref = OMD.MultiDomain(nd, periods, gx, gy, gz, bct)
    ref.influence_matrix(sigma, 0)
    g, bc = {}, {}
    for i in range(2):
        c = (i, 0, 0)
        nx, ny, nz = gx[i].size, gy[0].size, gz[0].size
        g[c] = rand(rng, (nx, ny, nz))
        bc[c] = [rand(rng, (ny - 2, nz - 2, 2)), rand(rng, (nx - 2, nz - 2, 2)),
                 rand(rng, (nx - 2, ny - 2, 2))]
    want, lam = ref.solve(g, bc, sigma)
    for i in range(2):
        c = (i, 0, 0)
        p = "md/sub%d/" % i
        out[p + "gx"] = gx[i]
        out[p + "g"] = g[c]
        out[p + "u"] = want[c]
        for a in range(3):
            out[p + "bc%d" % a] = bc[c][a]
    out["md/gy"] = gy[0]
    out["md/gz"] = gz[0]
    out["md/sigma"] = np.array(sigma)
    out["md/lambda"] = lam


def les_cases(out, rng):
    shape = (10, 9, 8)
    grids = [mesh.tanh_grid(n, 1.5) for n in shape]
    du = [[rand(rng, shape) for _ in range(3)] for _ in range(3)]
    for a in range(3):
        out["les/grid%d" % a] = grids[a]
    for i in range(3):
        for j in range(3):
            out["les/du%d%d" % (i, j)] = du[i][j]
    for t in (1, 2, 3):
        out["les/nu%d" % t] = L.les_nu(du, *grids, t, 0.17)


def mlp_case(out, rng):
    p = np.zeros(OM.N_PARAMS)
    p[OM.W1:OM.B1] = rng.uniform(-1, 1, OM.B1 - OM.W1)
    p[OM.W2:OM.B2] = rng.uniform(-0.3, 0.3, OM.B2 - OM.W2)
    p[OM.W3:OM.B3] = rng.uniform(-0.3, 0.3, OM.B3 - OM.W3)
    p[OM.B1:OM.W2] = rng.uniform(-0.3, 0.3, OM.W2 - OM.B1)
    p[OM.B3] = 1.0
    p = p.astype(np.float32).astype(np.float64)
    X = rng.uniform(-1, 1, (300, 6)).astype(np.float32).astype(np.float64)
    b = rng.uniform(0.1, 1, 300).astype(np.float32).astype(np.float64)
    t = (0.02 * b * (1 + X[:, 0])).astype(np.float32).astype(np.float64)
    mean = np.zeros(6)
    istd = np.ones(6)
    loss, g = OM.loss_and_grad(p, X, b, t, mean, istd, 0.02, 1000.0)
    out.update({"mlp/params": p, "mlp/X": X, "mlp/base": b, "mlp/target": t,
                "mlp/loss": np.array(loss), "mlp/grad": g})


def main():
    rng = np.random.default_rng(20261203)
    out = {}
    derivative_cases(out, rng)
    solver_cases(out, rng)
    filter_cases(out, rng)
    md_case(out, rng)
    les_cases(out, rng)
    mlp_case(out, rng)
    np.savez_compressed(OUT, **out)
    print("wrote %s: %d arrays, %d bytes" % (OUT, len(out), os.path.getsize(OUT)))


if __name__ == "__main__":
    main()
