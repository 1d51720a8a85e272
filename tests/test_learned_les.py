"""Learned LES coefficient (no reference counterpart; the plain models of
navier_LES, class_navier_3D.f90:1225-1455, are its fallback and baseline).

CPU: the oracle's backward pass against central finite differences (FP64),
its features' invariance under rotations and scaling of the gradient, and
Adam's first step against its closed form.  GPU, through the C ABI: the
fused gradient kernel against the oracle (FP32 kernel vs FP64 oracle:
max |g - g_ref| <= 2e-4 max |g_ref|, loss within 1e-4), Adam steps, the
prediction kernel (1e-5), features (5e-6 absolute: FP32 arithmetic on values
bounded by sqrt(3)) and SGS target (1e-5 relative) against the oracle, and
the fused viscosity kernel: network points within 2e-5 of the oracle,
fallback points bit-identical to the plain Smagorinsky kernel."""
import numpy as np
import pytest

from oracle import les as L
from oracle import mlp as O

from helpers import field, grids, max_rel


def random_params(seed, scale=1.0):
    rng = np.random.default_rng(seed)
    p = np.zeros(O.N_PARAMS)
    p[O.W1:O.B1] = rng.uniform(-1, 1, O.B1 - O.W1)
    p[O.B1:O.W2] = rng.uniform(-0.3, 0.3, O.W2 - O.B1)
    p[O.W2:O.B2] = rng.uniform(-0.3, 0.3, O.B2 - O.W2)
    p[O.B2:O.W3] = rng.uniform(-0.1, 0.1, O.W3 - O.B2)
    p[O.W3:O.B3] = rng.uniform(-0.3, 0.3, O.B3 - O.W3)
    p[O.B3] = 1.0
    return (p * scale).astype(np.float32).astype(np.float64)


def random_batch(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.uniform(-1, 1, (n, 6)).astype(np.float32).astype(np.float64)
    base = rng.uniform(0.1, 1.0, n).astype(np.float32).astype(np.float64)
    target = (0.02 * base * (1 + X[:, 0]) + 0.002 * rng.standard_normal(n)).astype(np.float32)
    return X, base, target.astype(np.float64)


SCALE = dict(mean=np.array([0.1, -0.2, 0.0, 0.05, 0.0, 0.1], np.float32),
             istd=np.array([1.5, 2.0, 1.0, 3.0, 1.0, 2.5], np.float32),
             cscale=0.02, loss_scale=1000.0)


def oracle_args():
    return (SCALE["mean"].astype(np.float64), SCALE["istd"].astype(np.float64), SCALE["cscale"],
            SCALE["loss_scale"])


def test_oracle_gradient_matches_finite_differences():
    p = random_params(1)
    X, b, t = random_batch(64, 2)
    args = (X, b, t) + oracle_args()
    _, g = O.loss_and_grad(p, *args)
    rng = np.random.default_rng(3)
    for q in list(rng.choice(O.N_PARAMS, 40, replace=False)) + [O.B3, O.W1, O.W2 + 5]:
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[q] += h
        pm[q] -= h
        fd = (O.loss_and_grad(pp, *args)[0] - O.loss_and_grad(pm, *args)[0]) / (2 * h)
        assert abs(fd - g[q]) <= 1e-6 * max(1.0, abs(g[q])), (q, fd, g[q])


def test_oracle_features_invariant():
    rng = np.random.default_rng(5)
    g = rng.standard_normal((50, 3, 3))
    f, ok = O.features(g)
    assert ok.all() and np.all(np.abs(f[:, :5]) <= 1.0 + 1e-12)
    assert np.all(np.abs(f[:, 5]) <= np.sqrt(3.0) + 1e-12)
    q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    fr, _ = O.features(q @ g @ q.T)
    fs, _ = O.features(7.5 * g)
    assert np.max(np.abs(fr - f)) < 1e-12 and np.max(np.abs(fs - f)) < 1e-12
    f0, ok0 = O.features(np.zeros((2, 3, 3)))
    assert not ok0.any() and np.all(f0 == 0)


def test_oracle_adam_closed_form():
    # the first Adam step moves every parameter by lr * sign(g) (up to eps)
    p = np.array([1.0, -2.0, 3.0])
    g = np.array([0.5, -4.0, 1e-3])
    p1, _, _ = O.adam(p, g, np.zeros(3), np.zeros(3), 1, 0.01)
    assert np.allclose(p1, p - 0.01 * np.sign(g), atol=1e-7)


# ---------------------------------------------------------------------------
# GPU: kernels against the oracle
# ---------------------------------------------------------------------------

def make_mlp(mf, p, lo=None, hi=None):
    m = mf.Mlp(0)
    m.set_params(p.astype(np.float32))
    lo = np.full(6, -np.inf, np.float32) if lo is None else lo
    hi = np.full(6, np.inf, np.float32) if hi is None else hi
    m.set_scaling(SCALE["mean"], SCALE["istd"], lo, hi, SCALE["cscale"], SCALE["loss_scale"])
    return m


def dev32(torch, a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float32, device="cuda")


@pytest.mark.gpu
@pytest.mark.parametrize("n,use_idx", [(1000, False), (4096, True), (77, False)])
def test_gradient_kernel_matches_oracle(mf, gpu, n, use_idx):
    import torch
    p = random_params(7)
    X, b, t = random_batch(6000, 8)
    idx = np.random.default_rng(9).choice(6000, n, replace=False).astype(np.int32) if use_idx \
        else np.arange(n, dtype=np.int32)
    m = make_mlp(mf, p)
    loss, g = m.train_step(dev32(torch, X), dev32(torch, b), dev32(torch, t),
                           idx=torch.tensor(idx, device="cuda") if use_idx else None, n=n, lr=0.0,
                           want_grad=True, want_loss=True)
    lref, gref = O.loss_and_grad(p, X[idx], b[idx], t[idx], *oracle_args())
    assert abs(loss - lref) <= 1e-4 * abs(lref)
    assert np.max(np.abs(g - gref)) <= 2e-4 * np.max(np.abs(gref))
    # lr = 0 leaves the parameters untouched
    assert np.array_equal(m.params(), p.astype(np.float32))


@pytest.mark.gpu
def test_adam_steps_match_oracle(mf, gpu):
    import torch
    p = random_params(11)
    X, b, t = random_batch(2048, 12)
    m = make_mlp(mf, p)
    Xd, bd, td = dev32(torch, X), dev32(torch, b), dev32(torch, t)
    pr, mm, vv = p.copy(), np.zeros_like(p), np.zeros_like(p)
    stable = np.ones(O.N_PARAMS, bool)
    for step in range(1, 4):
        m.train_step(Xd, bd, td, lr=1e-3)
        _, g = O.loss_and_grad(pr, X, b, t, *oracle_args())
        # Adam moves a parameter by about lr * sign(g) early on: where |g| is
        # within FP32 rounding of zero the two signs may differ, so those
        # parameters are left out of the close comparison
        stable &= np.abs(g) > 1e-4 * np.max(np.abs(g))
        pr, mm, vv = O.adam(pr, g, mm, vv, step, 1e-3)
    got = m.params().astype(np.float64)
    assert stable.mean() > 0.8
    assert np.max(np.abs(got - pr)[stable]) < 2e-5
    assert np.max(np.abs(got - pr)) <= 3 * 2e-3 + 1e-6
    assert np.max(np.abs(got - p)) > 1e-3


@pytest.mark.gpu
def test_predict_matches_oracle(mf, gpu):
    import torch
    p = random_params(13)
    X, _, _ = random_batch(5000, 14)
    m = make_mlp(mf, p)
    c = m.predict(dev32(torch, X)).cpu().numpy().astype(np.float64)
    y, _ = O.forward(p, O.standardise(X, SCALE["mean"], SCALE["istd"]))
    assert max_rel(c, SCALE["cscale"] * y) < 1e-5


def gradient_fields(shape, seed):
    return [[field(shape, seed + 3 * i + j) for j in range(3)] for i in range(3)]


def flat_to_field(a, shape, comps=None):
    """x-fastest flat device array -> NumPy (nx, ny, nz[, comps])."""
    a = a.cpu().numpy()
    if comps is None:
        return a.reshape(shape[::-1]).T
    return a.reshape(shape[2], shape[1], shape[0], comps).transpose(2, 1, 0, 3)


@pytest.mark.gpu
def test_features_and_target_match_oracle(mf, gpu):
    shape = (20, 17, 13)
    gx, gy, gz = grids(*shape, kind="tanh")
    du = gradient_fields(shape, 30)
    les = mf.LesModel(gx, gy, gz)
    ddu = [[mf.to_device(du[i][j]) for j in range(3)] for i in range(3)]
    X, b = les.features(ddu)
    X, b = flat_to_field(X, shape, 6), flat_to_field(b, shape)
    g = O.grad_tensor(du)
    f, _ = O.features(g)
    edge = L.zero_edges(np.ones(shape)) == 0
    f[edge] = 0.0
    bref = np.where(edge, 0.0, np.sqrt(2 * O.strain_ss(g)) * O.delta2(gx, gy, gz))
    assert np.max(np.abs(X - f)) < 5e-6
    assert max_rel(b, bref) < 1e-6
    ub = [field(shape, 50 + q) for q in range(3)]
    uu = [field(shape, 60 + q) for q in range(6)]
    t = les.sgs_target([mf.to_device(a) for a in ub], [mf.to_device(a) for a in uu], ddu)
    assert max_rel(flat_to_field(t, shape), O.sgs_target(ub, uu, du)) < 1e-5


@pytest.mark.gpu
def test_nu_mlp_matches_oracle_with_fallback(mf, gpu):
    shape = (24, 19, 16)
    gx, gy, gz = grids(*shape, kind="tanh")
    du = gradient_fields(shape, 70)
    p = random_params(17, scale=0.5)
    f, _ = O.features(O.grad_tensor(du))
    # training range: the central part of each feature's spread, so that a
    # good share of the points falls back; each limit lies midway between two
    # neighbouring feature values, far from both next to FP32 rounding
    fs = np.sort(f.reshape(-1, 6), axis=0)
    q0, q1 = int(0.05 * len(fs)), int(0.95 * len(fs))
    lo = (0.5 * (fs[q0] + fs[q0 + 1])).astype(np.float32)
    hi = (0.5 * (fs[q1] + fs[q1 + 1])).astype(np.float32)
    m = make_mlp(mf, p, lo, hi)
    les = mf.LesModel(gx, gy, gz)
    ddu = [[mf.to_device(du[i][j]) for j in range(3)] for i in range(3)]
    nu, nfb = les.nu_mlp(m, 0.031, ddu, count=True)
    nu = mf.to_host(nu)
    ref, fb = O.nu_mlp(p, du, gx, gy, gz, SCALE["mean"], SCALE["istd"], lo, hi, SCALE["cscale"], 0.031)
    assert nfb == int(fb.sum()) and 0 < nfb < fb.size
    plain = mf.to_host(les.nu(ddu, 1, 0.031))
    assert np.array_equal(nu[fb], plain[fb])
    net = ~fb
    assert np.max(np.abs(nu[net] - ref[net])) <= 2e-5 * np.max(np.abs(ref[net]))


# ---------------------------------------------------------------------------
# GPU: training data and what the trained network gains
# ---------------------------------------------------------------------------

@pytest.mark.gpu
def test_box_flow_projection_and_decay(mf, gpu):
    from mflops_gb300 import learn
    fl = learn.BoxFlow(49, 5e-3, seed=3, k0=15.0)
    assert fl.divergence_norm() < 1e-10          # projected initial condition
    ke0, _ = fl.stats()
    fl.run(60, every=20)
    ke1, skew = fl.stats()
    assert 0.2 * ke0 < ke1 < ke0                  # decays, stays bounded
    assert fl.divergence_norm() < 0.05
    assert skew < 0.0                             # forward cascade: negative skewness


@pytest.mark.gpu
def test_learned_coefficient_beats_best_constant(mf, gpu):
    """A-priori gain on a held-out flow: fine 97^3 runs (nu = 2e-3) filtered
    to a 25^3 LES grid; the network is trained on seed 1 and evaluated on
    seed 2 against the best constant Smagorinsky coefficient fitted on the
    same training data.  Measured: MSE ratio 0.85, correlation 0.48 vs 0.28."""
    import torch
    from mflops_gb300 import learn

    def pairs(seed):
        fl = learn.BoxFlow(97, 2e-3, seed=seed, k0=30.0)
        pm = learn.PairMaker(fl.grid, 25, margin=3)
        parts = []
        fl.run(400, every=50, callback=lambda f, it: parts.append(pm.pairs(f.u)) if it >= 300 else None)
        return [torch.cat([p[q] for p in parts]) for q in range(3)]

    train, held = pairs(1), pairs(2)
    m = mf.Mlp(0)
    s, hist = learn.fit(m, *train, steps=2000, batch=8192, lr=2e-3, log_every=1000)
    assert s["c0"] > 0.0                          # forward cascade in the data
    assert hist[-1][1] < hist[0][1]
    ev = learn.evaluate(m, s, *held)
    assert ev["mse_const"] < ev["mse_zero"]
    assert ev["mse_mlp"] < 0.92 * ev["mse_const"], ev
    assert ev["corr_mlp"] > ev["corr_const"] + 0.1, ev


@pytest.mark.gpu
def test_learned_closure_a_posteriori(mf, gpu):
    """A-posteriori judgement inside the time step: the network is trained on
    a fine 97^3 box flow (nu = 5e-3, seed 1) filtered to a 33^3 LES grid;
    from the filtered held-out flow (seed 2) the LES runs of mf_navier_step
    -- no model, Smagorinsky with the best constant coefficient, and the
    learned coefficient (les_type 4) -- are compared with the filtered fine
    run at four times.  Without a model the run diverges; the network keeps
    the run stable like the plain model and its energy spectrum is closer to
    the filtered fine run's (measured: mean spectrum error 0.051 against
    0.085, mean-profile error 0.028 against 0.030)."""
    import torch
    from mflops_gb300 import learn
    fl = learn.BoxFlow(97, 5e-3, seed=1, k0=8.0)
    pm = learn.PairMaker(fl.grid, 33, margin=3)
    parts = []
    fl.run(400, every=50, callback=lambda f, it: parts.append(pm.pairs(f.u)) if it >= 300 else None)
    train = [torch.cat([p[q] for p in parts]) for q in range(3)]
    net = mf.Mlp(0)
    s, _ = learn.fit(net, *train, steps=2000, batch=8192, lr=2e-3)
    held = learn.BoxFlow(97, 5e-3, seed=2, k0=8.0)
    held.run(300, every=50)
    res = learn.APosteriori(held, pm, net, s).run(200 * held.cfl_dt(0.3), checkpoints=4, cfl=0.1)
    print({m: (res[m]["profile_error_mean"], res[m]["spectrum_error_mean"]) for m in (0, 1, 4)})
    smag, learned = res[1], res[4]
    for r in (smag, learned):
        assert np.isfinite(r["profile_error_mean"]) and np.isfinite(r["spectrum_error_mean"])
    assert learned["spectrum_error_mean"] < smag["spectrum_error_mean"]
    assert learned["profile_error_mean"] < 1.2 * smag["profile_error_mean"]
    nomodel = res[0]["spectrum_error_mean"]
    assert not np.isfinite(nomodel) or nomodel > learned["spectrum_error_mean"]
