"""GPU solves at the two single-domain solver workloads as they are named,
against the FP64 oracle and against the exactly rounded discrete solution
(oracle/exact.py: the oracle's solve corrected once with a double-double
residual of the interior operator).

Bars:
* plain FP64 GPU solve vs the exact solution: rel-L2 and max-rel <= 1e-12
  over the interior;
* plain FP64 GPU solve with the oracle's LAPACK eigen tables loaded
  (mf_solver3d_set_eigen) vs the oracle: <= 1e-12 -- the kernels' rounding
  alone;
* plain FP64 GPU solve vs the oracle, library tables: <= 1e-12 at 65^3.
  At 257^3 the oracle itself is ~5e-12 from the exact solution (its
  smallest eigenvalues from dgeev carry eps*lambda_max/lambda_min), so there
  the bar is the oracle's own distance from the exact solution plus 1e-12;
* 3xTF32 + one refinement at 257^3: rel-L2 <= 1e-10 vs the oracle and vs
  the exact solution;
* derivatives of the 65^3 workload: max-rel <= 1e-12 vs the oracle.

The 257^3 workload is bench.py's: x, z uniform, y tanh(2.0), Dirichlet,
sigma = 0, seeded k^-5/3 right-hand side.  The 65^3 workload: tanh(1.5) on
every axis of [0,1]^3, 6th-order scheme, Dirichlet; right-hand side = the
compact-scheme Laplacian of sin(pi x) sin(pi y) sin(pi z) plus U(-1e-3, 1e-3)
noise (seed 1), boundary values those of the sine product; a Poisson solve
and a Helmholtz solve with coefficient 1e3 (sigma = -1e3); and d/dx, d/dy,
d/dz, d2/dx2 of a U(-1, 1) field (seed 2).
"""
import numpy as np
import pytest

from oracle import derivatives as D
from oracle import exact as E
from oracle import mesh
from oracle import solver as S

from helpers import max_rel, rel_l2

pytestmark = pytest.mark.gpu

INT = (slice(1, -1),) * 3


def _gpu_solve(mf, sc, rhs, sigma, solf, bcs, **kw):
    dev = [mf.to_device(a) for a in (rhs, solf) + tuple(bcs)]
    return mf.to_host(sc.solve_3d(dev[0], sigma, dev[1], *dev[2:], **kw))


@pytest.fixture(scope="module")
def w257():
    import bench
    gs, rhs, bcs = bench.workload(257)
    sc = S.Solver3D(*gs, (1,) * 6, 6)
    solf = np.zeros((257, 257, 257), order="F")
    oracle = S.solve_3d(sc, rhs, 0.0, solf, *bcs)
    exact = E.exact_solve(sc, rhs, 0.0, solf, *bcs)
    return {"grids": gs, "rhs": rhs, "bcs": bcs, "sc": sc, "solf": solf, "oracle": oracle,
            "exact": exact, "oracle_vs_exact": rel_l2(oracle[INT], exact[INT])}


def test_plain_257_vs_exact_and_oracle(mf, gpu, w257):
    sc = mf.SolverCoeffs3D(*w257["grids"], (1,) * 6, 6)
    got = _gpu_solve(mf, sc, w257["rhs"], 0.0, w257["solf"], w257["bcs"])
    e_exact = rel_l2(got[INT], w257["exact"][INT])
    m_exact = max_rel(got[INT], w257["exact"][INT])
    e_oracle = rel_l2(got[INT], w257["oracle"][INT])
    print("257^3 plain FP64: vs exact %.2e (max-rel %.2e), vs oracle %.2e; oracle vs exact %.2e"
          % (e_exact, m_exact, e_oracle, w257["oracle_vs_exact"]))
    assert e_exact < 1e-12 and m_exact < 1e-12
    assert e_oracle < w257["oracle_vs_exact"] + 1e-12
    assert e_exact < w257["oracle_vs_exact"]


def test_plain_257_with_oracle_tables(mf, gpu, w257):
    sc = mf.SolverCoeffs3D(*w257["grids"], (1,) * 6, 6)
    for a, ax in enumerate((w257["sc"].cx, w257["sc"].cy, w257["sc"].cz)):
        sc.set_eigen(a, ax.eigen, ax.vect, ax.inv_vect)
    got = _gpu_solve(mf, sc, w257["rhs"], 0.0, w257["solf"], w257["bcs"])
    e = rel_l2(got[INT], w257["oracle"][INT])
    m = max_rel(got[INT], w257["oracle"][INT])
    print("257^3 plain FP64, oracle tables: vs oracle %.2e (max-rel %.2e)" % (e, m))
    assert e < 1e-12 and m < 1e-12


def test_mixed_257_vs_oracle_and_exact(mf, gpu, w257):
    sc = mf.SolverCoeffs3D(*w257["grids"], (1,) * 6, 6)
    got = _gpu_solve(mf, sc, w257["rhs"], 0.0, w257["solf"], w257["bcs"],
                     precision=mf.MF_PREC_3XTF32, refine=1)
    e_oracle = rel_l2(got[INT], w257["oracle"][INT])
    e_exact = rel_l2(got[INT], w257["exact"][INT])
    print("257^3 3xTF32 + 1 refinement: vs oracle %.2e, vs exact %.2e" % (e_oracle, e_exact))
    assert e_oracle < 1e-10 and e_exact < 1e-10


@pytest.fixture(scope="module")
def w65():
    g = mesh.tanh_grid(65, 1.5)
    x = np.sin(np.pi * g)
    f = np.asfortranarray(x[:, None, None] * x[None, :, None] * x[None, None, :])
    dc = D.DerCoeffs(g, 6)
    lap = D.dderx(dc, f) + D.ddery(dc, f) + D.dderz(dc, f)
    rhs = np.asfortranarray(lap[INT] + np.random.default_rng(1).uniform(-1e-3, 1e-3, (63, 63, 63)))
    bcs = (np.asfortranarray(np.stack([f[0, 1:-1, 1:-1], f[-1, 1:-1, 1:-1]], axis=-1)),
           np.asfortranarray(np.stack([f[1:-1, 0, 1:-1], f[1:-1, -1, 1:-1]], axis=-1)),
           np.asfortranarray(np.stack([f[1:-1, 1:-1, 0], f[1:-1, 1:-1, -1]], axis=-1)))
    return {"g": g, "rhs": rhs, "bcs": bcs, "sc": S.Solver3D(g, g, g, (1,) * 6, 6)}


@pytest.mark.parametrize("sigma", [0.0, -1e3])
def test_config_65_solves(mf, gpu, w65, sigma):
    g = w65["g"]
    solf = np.zeros((65, 65, 65), order="F")
    oracle = S.solve_3d(w65["sc"], w65["rhs"], sigma, solf, *w65["bcs"])
    exact = E.exact_solve(w65["sc"], w65["rhs"], sigma, solf, *w65["bcs"])
    sc = mf.SolverCoeffs3D(g, g, g, (1,) * 6, 6)
    got = _gpu_solve(mf, sc, w65["rhs"], sigma, solf, w65["bcs"])
    m_or = max_rel(got[INT], oracle[INT])
    m_ex = max_rel(got[INT], exact[INT])
    print("65^3 sigma=%g: vs oracle %.2e, vs exact %.2e (oracle vs exact %.2e)"
          % (sigma, m_or, m_ex, max_rel(oracle[INT], exact[INT])))
    assert m_or < 1e-12 and m_ex < 1e-12


@pytest.mark.parametrize("axis,order", [(0, 1), (1, 1), (2, 1), (0, 2)])
def test_config_65_derivatives(mf, gpu, w65, axis, order):
    g = w65["g"]
    f = np.asfortranarray(np.random.default_rng(2).uniform(-1, 1, (65, 65, 65)))
    ref = [[D.derx, D.dery, D.derz], [D.dderx, D.ddery, D.dderz]][order - 1][axis](D.DerCoeffs(g, 6), f)
    fn = [[mf.derx, mf.dery, mf.derz], [mf.dderx, mf.ddery, mf.dderz]][order - 1][axis]
    got = mf.to_host(fn(mf.DerivativesCoefficients(g, so=6), mf.to_device(f)))
    assert max_rel(got, ref) < 1e-12
