"""Navier-Stokes time step on the GPU (mf_navier_*) against the oracle's
restatement of navier3d.f90 / class_navier_3D.f90: every field of every time
level and the driver's diagnostics after each of six steps (more than one
rotation of the nt = 4 slots, so the cached nonlinear terms are exercised),
for the reference's defaults, other scheme options and the three LES models;
the mixed-precision solves; a CUDA-graph capture of four steps replayed
bit-identically."""
import numpy as np
import pytest

from oracle import mesh
from oracle import navier as N

pytestmark = pytest.mark.gpu

VARS = ("u", "v", "w", "p", "phi")


def grids():
    return mesh.tanh_grid(17, 1.0), mesh.tanh_grid(15, 1.5), mesh.uniform_grid(13)


def initial_levels(nav, seed, nmodes):
    """Exact solution plus a seeded perturbation, different in every slot."""
    rng = np.random.default_rng(seed)
    X, Y, Z = nav.points()
    shape = X.shape
    for s in range(N.NT):
        nav.u[s] = N.sol(X, Y, Z, 0.0, "u", nav.rey, nmodes) + 0.05 * rng.standard_normal(shape)
        nav.v[s] = N.sol(X, Y, Z, 0.0, "v", nav.rey, nmodes) + 0.05 * rng.standard_normal(shape)
        nav.w[s] = 0.05 * rng.standard_normal(shape)
        nav.p[s] = N.sol(X, Y, Z, 0.0, "p", nav.rey, nmodes) + 0.05 * rng.standard_normal(shape)
        nav.phi[s] = nav.p[s] + 0.01 * rng.standard_normal(shape)


def make_pair(mf, seed=3, **kw):
    gx, gy, gz = grids()
    okw = {k: kw[k] for k in ("nlt", "pt", "tou", "top", "flow_rate", "nmodes", "les_type", "les_c", "nsubite")
           if k in kw}
    ora = N.Navier(gx, gy, gz, ts=kw["ts"], rey=kw["reynolds"], **okw)
    initial_levels(ora, seed, okw.get("nmodes", N.NMODES))
    gpu = mf.NavierStokes3D(gx, gy, gz, **kw)
    for lev in range(N.NT):
        for var in VARS:
            gpu.set_field(var, lev, mf.to_device(getattr(ora, var)[ora.it[lev]]))
    return ora, gpu


def max_rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def compare(mf, ora, gpu, tol):
    worst = 0.0
    for lev in range(N.NT):
        for var in VARS:
            got = mf.to_host(gpu.field(var, lev))
            ref = getattr(ora, var)[ora.it[lev]]
            err = max_rel(got, ref)
            assert err < tol, (var, lev, err)
            worst = max(worst, err)
    return worst


CASES = {
    "defaults": dict(ts=1e-2, reynolds=50.0),
    "pt2_bdf3_advective": dict(ts=5e-3, reynolds=20.0, pt=2, tou=3, top=3, nlt=1, flow_rate=0),
    "pt1_euler_no_advection": dict(ts=2e-2, reynolds=5.0, pt=1, tou=1, top=1, nlt=0, nmodes=1),
    "pt3_rotrot": dict(ts=1e-2, reynolds=50.0, pt=3, top=3),
    "pt4_bdf3": dict(ts=5e-3, reynolds=50.0, pt=4, tou=3, nlt=1),
    "pt2_subiterations": dict(ts=1e-2, reynolds=50.0, pt=2, nsubite=3),
    "pt4_subiterations": dict(ts=1e-2, reynolds=50.0, pt=4, nsubite=3, les_type=1, les_c=0.1),
    # LES cases: parameters for which the explicit LES term stays stable on
    # these coarse noisy fields (a blowing-up run amplifies rounding)
    "les_smagorinsky": dict(ts=2e-3, reynolds=100.0, les_type=1, les_c=0.17),
    "les_wale_pt2": dict(ts=5e-3, reynolds=500.0, pt=2, les_type=2, les_c=0.5),
    "les_sigma": dict(ts=1e-2, reynolds=100.0, les_type=3, les_c=0.5),
}


@pytest.mark.parametrize("name", list(CASES))
def test_steps_match_the_oracle(mf, gpu, name):
    kw = CASES[name]
    ora, nav = make_pair(mf, **kw)
    # the sigma model's acos amplifies rounding near coincident singular
    # values (1e-10 bound on the viscosity itself, tests/test_les.py)
    tol = 1e-9 if kw.get("les_type") == 3 else 1e-10
    for step in range(6):
        d_ref = ora.advance(diagnostics=True)
        d = nav.step(diagnostics=True)
        worst = compare(mf, ora, nav, tol)
        assert d["div"] == pytest.approx(d_ref["div"], rel=10 * tol)
        for key, pos in (("vel", 0), ("pres", 0)):
            assert d[key + "_err"] == pytest.approx(d_ref[key][pos], rel=10 * tol), (step, key)
        assert d["vel_acc"] == pytest.approx(d_ref["vel"][2], rel=10 * tol)
        assert d["pres_acc"] == pytest.approx(d_ref["pres"][2], rel=10 * tol)
        assert d["kinetic"] == pytest.approx(d_ref["kinetic"], rel=10 * tol)
        assert d["station_p"] == pytest.approx(d_ref["station_p"][0], rel=10 * tol)
        assert d["station_v"] == pytest.approx(d_ref["station_v"][0], rel=10 * tol)
    st = nav.state()
    assert st["time"] == pytest.approx(ora.time, rel=1e-15)
    if kw.get("flow_rate", 1):
        assert st["debit"] == pytest.approx(ora.debit, rel=1e-12)
        assert st["g"] == pytest.approx(ora.g, rel=1e-9)
    print("%s: worst field max-rel %.2e after 6 steps" % (name, worst))


def test_learned_les_steps_match_the_oracle(mf, gpu):
    """les_type 4: the eddy viscosity from a (seeded, untrained) network of
    the learned coefficient inside the step, against the oracle step with the
    FP64 network.  The GPU network runs in FP32 with a 3xTF32 hidden layer
    (coefficient ~1e-6 relative), so the fields agree to about that (1e-6;
    the pressure, through the projection, is the most sensitive: 1.3e-7
    measured after four steps); the training range is unbounded here, so no
    point sits on the fallback boundary (the fallback itself is covered by
    tests/test_learned_les.py)."""
    kw = dict(ts=2e-3, reynolds=100.0, les_type=4, les_c=0.17)
    ora, nav = make_pair(mf, **kw)
    net = mf.Mlp(7)
    inf = np.full(6, np.inf, np.float32)
    mean = np.array([0.3, 0.0, 0.0, 0.1, 0.0, 0.0])
    istd = np.array([3.0, 5.0, 5.0, 3.0, 5.0, 5.0])
    net.set_scaling(mean, istd, -inf, inf, 0.03, 1.0)
    nav.set_les_network(net)
    ora.les_network = dict(params=net.params().astype(np.float64), mean=mean.astype(np.float32).astype(np.float64),
                           istd=istd.astype(np.float32).astype(np.float64), lo=-np.inf, hi=np.inf,
                           cscale=float(np.float32(0.03)))
    for _ in range(4):
        ora.advance()
        nav.step()
    worst = compare(mf, ora, nav, 1e-6)
    print("learned LES: worst field max-rel %.2e after 4 steps" % worst)
    # the LES term is active: the learned viscosity differs from zero
    assert float(np.abs(ora.les_nu).max()) > 0.0
    bare = mf.NavierStokes3D(*grids(), **kw)
    with pytest.raises(mf.MflopsError):
        bare.step()


@pytest.mark.parametrize("prec_name,refine", [("MF_PREC_3XTF32", 1), ("MF_PREC_SPLIT_BF16", 2)])
def test_mixed_precision_solves(mf, gpu, prec_name, refine):
    kw = dict(CASES["defaults"], precision=getattr(mf, prec_name), refine=refine)
    ora, nav = make_pair(mf, **kw)
    for _ in range(6):
        ora.advance()
        nav.step()
    worst = compare(mf, ora, nav, 1e-8)
    print("%s + %d refinements: worst field max-rel %.2e after 6 steps" % (prec_name, refine, worst))


def test_four_step_graph_replays_like_eager_steps(mf, gpu):
    import torch
    kw = CASES["defaults"]
    _, eager = make_pair(mf, **kw)
    _, graphed = make_pair(mf, **kw)
    for _ in range(8):
        eager.step()
    for _ in range(4):
        graphed.step()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side, capture_error_mode="relaxed"):
            for _ in range(4):
                graphed.step()
    torch.cuda.current_stream().wait_stream(side)
    g.replay()
    torch.cuda.synchronize()
    for lev in range(N.NT):
        for var in VARS:
            assert torch.equal(graphed.field(var, lev), eager.field(var, lev)), (var, lev)
    assert graphed.state() == eager.state()


def test_repeat_runs_are_bit_identical(mf, gpu):
    """Fresh instances (new solver handles, first mixed solves on the forked
    streams) started from the same state give bit-identical steps: the
    handles' set-up work is ordered before their first use on any stream."""
    import torch
    kw = dict(CASES["defaults"], precision=mf.MF_PREC_SPLIT_BF16, refine=2)
    runs = []
    for _ in range(3):
        _, nav = make_pair(mf, **kw)
        for _ in range(3):
            nav.step()
        torch.cuda.synchronize()
        runs.append([nav.field(var, lev) for lev in range(N.NT) for var in VARS])
        nav.close()
    for other in runs[1:]:
        for a, b in zip(runs[0], other):
            assert torch.equal(a, b)


def test_subiterations_stop_on_the_convergence_test(mf, gpu):
    """pt 3 started on the one-mode exact solution converges within the
    sub-iteration cap; the GPU stops after the same number of sub-iterations
    as the oracle and gives the same fields."""
    from test_navier_oracle import start_on_exact
    gx, gy, gz = grids()
    kw = dict(ts=1e-2, reynolds=10.0, pt=3, flow_rate=0, nmodes=1, nsubite=12)
    ora = N.Navier(gx, gy, gz, ts=kw["ts"], rey=kw["reynolds"], pt=3, flow_rate=False, nmodes=1, nsubite=12)
    start_on_exact(ora)
    nav = mf.NavierStokes3D(gx, gy, gz, **kw)
    for lev in range(N.NT):
        for var in VARS:
            nav.set_field(var, lev, mf.to_device(getattr(ora, var)[ora.it[lev]]))
    counts = []
    for _ in range(3):
        ora.advance()
        nav.step()
        assert nav.subiterations() == ora.subiterations
        counts.append(ora.subiterations)
    assert max(counts) < 12
    # w is zero in the exact solution (rounding noise only): errors against
    # the scale of the velocity, O(1)
    for lev in range(N.NT):
        for var in VARS:
            ref = getattr(ora, var)[ora.it[lev]]
            err = np.abs(mf.to_host(nav.field(var, lev)) - ref).max()
            assert err < 1e-10 * max(1.0, np.abs(ref).max()), (var, lev, err)


def test_checkpoint_resumes_bit_identically(mf, gpu, tmp_path):
    """Save after some steps, continue; a fresh instance loaded from the file
    continues to the same fields, time and flow-rate state (pt 4: the
    right-hand-side history is part of the state).  Another grid and a
    truncated file are refused."""
    import torch
    kw = dict(ts=1e-2, reynolds=50.0, pt=4, tou=3)
    _, a = make_pair(mf, **kw)
    for _ in range(5):
        a.step()
    path = tmp_path / "ns.chk"
    a.save(path)
    for _ in range(6):
        a.step()
    gx, gy, gz = grids()
    b = mf.NavierStokes3D(gx, gy, gz, **kw)
    b.load(path)
    for _ in range(6):
        b.step()
    for lev in range(N.NT):
        for var in VARS:
            assert torch.equal(a.field(var, lev), b.field(var, lev)), (var, lev)
    assert a.state() == b.state()
    other = mf.NavierStokes3D(gx, gy, mesh.uniform_grid(15), **kw)
    with pytest.raises(mf.MflopsError):
        other.load(path)
    # a refused file leaves the running state as it was: truncated inside the
    # field data (after the header and several fields) or with extra bytes
    data = path.read_bytes()
    before = {(var, lev): b.field(var, lev).clone() for lev in range(N.NT) for var in VARS}
    state = b.state()
    (tmp_path / "cut.chk").write_bytes(data[: len(data) // 2])
    (tmp_path / "long.chk").write_bytes(data + b"\0" * 8)
    for bad in ("cut.chk", "long.chk"):
        with pytest.raises(mf.MflopsError):
            b.load(tmp_path / bad)
        for (var, lev), t in before.items():
            assert torch.equal(b.field(var, lev), t), (bad, var, lev)
        assert b.state() == state


MD_GRIDS = {
    "2x1x1": ((2, 1, 1), (0, 0, 0), [mesh.tanh_grid(11, 1.0, 0.0, 0.5), mesh.tanh_grid(13, 1.0, 0.5, 1.0)],
              [mesh.tanh_grid(13, 1.0)], [mesh.uniform_grid(11)]),
    "periodic_xz": ((1, 1, 1), (1, 0, 1), [mesh.uniform_grid(17, 0.0, 2.0)], [mesh.tanh_grid(13, 1.0)],
                    [mesh.uniform_grid(11, 0.0, 2.0)]),
    "2x1x2_periodic_x": ((2, 1, 2), (1, 0, 0), [mesh.uniform_grid(11, 0.0, 1.0), mesh.uniform_grid(11, 1.0, 2.0)],
                         [mesh.tanh_grid(12, 1.0)], [mesh.tanh_grid(10, 1.0, 0.0, 0.5), mesh.tanh_grid(11, 1.0, 0.5, 1.0)]),
}
MD_CASES = {
    "2x1x1_defaults": ("2x1x1", dict(ts=1e-2, reynolds=50.0)),
    "periodic_xz_pt2": ("periodic_xz", dict(ts=1e-2, reynolds=50.0, pt=2)),
    # the channel rows' settings: reference defaults (pt 1, flow-rate term),
    # no manufactured sources, Re 180, ts 1e-3
    "periodic_xz_channel": ("periodic_xz", dict(ts=1e-3, reynolds=180.0, nmodes=0)),
    "2x1x2_periodic_x_pt3_les_sub": ("2x1x2_periodic_x", dict(ts=1e-2, reynolds=100.0, pt=3, les_type=1,
                                                               les_c=0.1, nsubite=2)),
}


def make_md_pair(mf, grid_key, kw, seed=5):
    nd, periods, gx, gy, gz = MD_GRIDS[grid_key]
    okw = {k: kw[k] for k in ("nlt", "pt", "tou", "top", "flow_rate", "nmodes", "les_type", "les_c", "nsubite")
           if k in kw}
    ora = N.NavierMD(nd, periods, gx, gy, gz, kw["ts"], kw["reynolds"], **okw)
    for q, c in enumerate(ora.subs):
        initial_levels(ora.dom[c], seed + q, okw.get("nmodes", N.NMODES))
    nav = mf.NavierStokes3D(gx, gy, gz, nd=nd, periods=periods, **kw)
    for s, c in enumerate(ora.subs):
        d = ora.dom[c]
        for lev in range(N.NT):
            for var in VARS:
                nav.set_field(var, lev, mf.to_device(getattr(d, var)[d.it[lev]]), sub=s)
    return ora, nav


@pytest.mark.parametrize("name", list(MD_CASES))
def test_multidomain_steps_match_the_oracle(mf, gpu, name):
    """The multidomain branch (influence-matrix solves, sums over all
    subdomains) against the oracle's restatement on every field of every
    subdomain and level, with the driver's diagnostics, after four steps."""
    grid_key, kw = MD_CASES[name]
    ora, nav = make_md_pair(mf, grid_key, kw)
    worst = 0.0
    for step in range(4):
        d_ref = ora.advance(diagnostics=True)
        d = nav.step(diagnostics=True)
        for s, c in enumerate(ora.subs):
            dom = ora.dom[c]
            for lev in range(N.NT):
                for var in VARS:
                    err = max_rel(mf.to_host(nav.field(var, lev, sub=s)), getattr(dom, var)[dom.it[lev]])
                    assert err < 1e-9, (step, s, var, lev, err)
                    worst = max(worst, err)
        assert d["div"] == pytest.approx(d_ref["div"], rel=1e-8)
        assert d["vel_err"] == pytest.approx(d_ref["vel"][0], rel=1e-8)
        assert d["pres_err"] == pytest.approx(d_ref["pres"][0], rel=1e-8)
        assert d["kinetic"] == pytest.approx(d_ref["kinetic"], rel=1e-8)
    if kw.get("nsubite", 1) > 1:
        assert nav.subiterations() == ora.subiterations
    print("%s: worst field max-rel %.2e after 4 steps" % (name, worst))


def test_multidomain_mixed_subdomain_solves(mf, gpu):
    """The multidomain branch with 3xTF32 subdomain solves (FP64 influence
    matrices, the explicit interface inverse) against the FP64 oracle."""
    grid_key, kw = MD_CASES["periodic_xz_pt2"]
    kw = dict(kw, precision=mf.MF_PREC_3XTF32, refine=1, md_interface=mf.MD_IFACE_INVERSE)
    ora, nav = make_md_pair(mf, grid_key, kw)
    for _ in range(4):
        ora.advance()
        nav.step()
    for s, c in enumerate(ora.subs):
        dom = ora.dom[c]
        for lev in range(N.NT):
            for var in VARS:
                err = max_rel(mf.to_host(nav.field(var, lev, sub=s)), getattr(dom, var)[dom.it[lev]])
                assert err < 1e-8, (s, var, lev, err)
