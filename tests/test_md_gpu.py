"""Influence-matrix multidomain solve on the GPU (multidomain_solve,
class_field.f90:1295-1388) against the FP64 oracle, through the C ABI.
Tolerance: max |gpu - oracle| <= 1e-11 * max |oracle| per subdomain field
(the interface solve adds an LU on top of the 1e-12 subdomain solves).
The three interface-solve forms are checked: the inverse formed at set-up
(the default for small systems), the inverted LU factors (the default for
large ones) and the triangular solves on the LU factors."""
import numpy as np
import pytest

from oracle import md as omd
from oracle import mesh

from helpers import max_rel

pytestmark = pytest.mark.gpu


def slabs(nd, nodes, lo=0.0, hi=1.0, alpha=1.0):
    edges = np.linspace(lo, hi, nd + 1)
    if isinstance(nodes, int):
        nodes = [nodes] * nd
    return [mesh.tanh_grid(nodes[s], alpha, edges[s], edges[s + 1]) for s in range(nd)]


def exact(X, Y, Z):
    return np.sin(1.3 * X + 0.2) * np.cos(0.7 * Y - 0.1) * np.exp(0.5 * Z)


def problem(grids, subs, sigma, bct):
    gx, gy, gz = grids
    g, bc, ex = {}, {}, {}
    for c in subs:
        X, Y, Z = np.meshgrid(gx[c[0]], gy[c[1]], gz[c[2]], indexing="ij")
        ue = exact(X, Y, Z)
        ex[c] = ue
        lap = (-1.3 ** 2 - 0.7 ** 2 + 0.25) * ue
        g[c] = np.asfortranarray(lap + sigma * ue)
        dx = 1.3 * np.cos(1.3 * X + 0.2) * np.cos(0.7 * Y - 0.1) * np.exp(0.5 * Z)
        dy = -0.7 * np.sin(1.3 * X + 0.2) * np.sin(0.7 * Y - 0.1) * np.exp(0.5 * Z)
        dz = 0.5 * ue
        fv = []
        for l, d in enumerate((dx, dy, dz)):
            sides = []
            for m in range(2):
                sl = [slice(1, -1)] * 3
                sl[l] = 0 if m == 0 else -1
                src = ue if bct[2 * l + m] == 1 else d
                sides.append(src[tuple(sl)])
            fv.append(np.asfortranarray(np.stack(sides, -1)))
        bc[c] = fv
    return g, bc, ex


def run(mf, nd, periods, nodes, sigma, bct=(1,) * 6, null=0, iface=0, precision=None):
    grids = tuple(slabs(nd[l], nodes[l]) for l in range(3))
    ref = omd.MultiDomain(nd, periods, *grids, bct)
    ref.influence_matrix(sigma, null)
    dev = mf.MultiDomain(nd, periods, *grids, bct)
    dev.set_interface_solve(iface)
    if precision is not None:
        dev.set_precision(*precision)
    dev.influence_matrix_set(sigma, null)
    subs = dev.subdomains()
    g, bc, ex = problem(grids, subs, sigma, bct)
    want, lam_ref = ref.solve(g, bc, sigma)
    gd = {c: mf.to_device(g[c]) for c in subs}
    ud = {c: mf.empty_device(g[c].shape) for c in subs}
    bd = {c: [mf.to_device(b) for b in bc[c]] for c in subs}
    dev.solve(gd, ud, bd)
    lam = dev.interface()
    errs = [max_rel(mf.to_host(ud[c])[1:-1, 1:-1, 1:-1], want[c][1:-1, 1:-1, 1:-1]) for c in subs]
    return max(errs), max_rel(lam, lam_ref), want, ex


@pytest.mark.parametrize("nd,periods", [((2, 1, 1), (0, 0, 0)), ((2, 2, 1), (0, 0, 0)),
                                        ((2, 2, 2), (0, 0, 0)), ((2, 1, 1), (1, 0, 0)),
                                        ((1, 2, 1), (0, 1, 0))])
def test_md_matches_oracle(mf, gpu, nd, periods):
    err, lerr, want, ex = run(mf, nd, periods, (11, 11, 11), -3.0)
    assert err < 1e-11 and lerr < 1e-11, (err, lerr)


def test_md_uneven_slabs(mf, gpu):
    err, lerr, _, _ = run(mf, (2, 2, 1), (0, 0, 0), ([11, 15], [13, 9], [11]), -1e3)
    assert err < 1e-11 and lerr < 1e-11


def test_md_known_answer(mf, gpu):
    # manufactured smooth solution: the coupled solution is as accurate as
    # a single-domain solve of the same resolution
    err, lerr, want, ex = run(mf, (2, 2, 1), (0, 0, 0), (13, 13, 13), -3.0)
    assert err < 1e-11
    assert max(np.max(np.abs((want[c] - ex[c])[1:-1, 1:-1, 1:-1])) for c in want) < 1e-7


@pytest.mark.parametrize("null", [1, 2])
def test_md_pure_neumann_null_space(mf, gpu, null):
    # all physical faces Neumann, sigma = 0: the interface system is singular;
    # the reference pins row 0 (null=2) or works with a constant null space (null=1)
    err, lerr, _, _ = run(mf, (2, 1, 1), (0, 0, 0), (11, 11, 11), 0.0, bct=(2,) * 6, null=null)
    assert err < 1e-10 and lerr < 1e-10, (err, lerr)


@pytest.mark.parametrize("iface", ["MD_IFACE_LU", "MD_IFACE_TRIANGULAR_INVERSE",
                                   "MD_IFACE_TRIANGULAR_INVERSE_FP64"])
@pytest.mark.parametrize("nd,periods", [((2, 2, 2), (0, 0, 0)), ((2, 1, 1), (1, 0, 0))])
def test_md_triangular_interface_solve(mf, gpu, nd, periods, iface):
    err, lerr, _, _ = run(mf, nd, periods, (11, 11, 11), -3.0, iface=getattr(mf, iface))
    assert err < 1e-11 and lerr < 1e-11, (err, lerr)


@pytest.mark.parametrize("iface", ["MD_IFACE_LU", "MD_IFACE_TRIANGULAR_INVERSE",
                                   "MD_IFACE_TRIANGULAR_INVERSE_FP64"])
@pytest.mark.parametrize("null", [1, 2])
def test_md_null_space_triangular_interface_solve(mf, gpu, null, iface):
    err, lerr, _, _ = run(mf, (2, 1, 1), (0, 0, 0), (11, 11, 11), 0.0, bct=(2,) * 6, null=null,
                          iface=getattr(mf, iface))
    assert err < 1e-10 and lerr < 1e-10, (err, lerr)


def test_md_interface_forms_agree(mf, gpu):
    # the same problem through both forms: both match the oracle, and the
    # interface values agree to rounding
    a = run(mf, (2, 2, 1), (0, 0, 0), ([11, 15], [13, 9], [11]), -1e3, iface=mf.MD_IFACE_AUTO)
    b = run(mf, (2, 2, 1), (0, 0, 0), ([11, 15], [13, 9], [11]), -1e3, iface=mf.MD_IFACE_LU)
    assert a[0] < 1e-11 and b[0] < 1e-11
    assert a[1] < 1e-11 and b[1] < 1e-11


@pytest.mark.parametrize("nd,periods", [((2, 2, 1), (0, 0, 0)), ((2, 1, 1), (1, 0, 0))])
def test_md_mixed_subdomain_solves_forced_inverse(mf, gpu, nd, periods):
    """Subdomain solves with 3xTF32 transforms + two FP64 refinement steps and
    the interface through the explicit inverse (forced) against the FP64
    oracle: the influence matrix stays FP64, the subdomain fields carry the
    refined solves' accuracy."""
    err, lerr, _, _ = run(mf, nd, periods, (11, 11, 11), -3.0, iface=mf.MD_IFACE_INVERSE,
                          precision=(mf.MF_PREC_3XTF32, 2))
    assert err < 1e-10 and lerr < 1e-10, (err, lerr)


@pytest.mark.parametrize("iface", ["MD_IFACE_INVERSE", "MD_IFACE_LU", "MD_IFACE_TRIANGULAR_INVERSE",
                                   "MD_IFACE_TRIANGULAR_INVERSE_FP64"])
def test_md_solve_many_equals_single_solves(mf, gpu, iface):
    """Three right-hand sides in one mf_md_solve_many call (subdomain work per
    right-hand side in turn, the interface systems together) give the three
    single solves bit for bit."""
    nd, periods, nodes, sigma = (2, 2, 1), (0, 0, 0), (11, 11, 11), -3.0
    grids = tuple(slabs(nd[l], nodes[l]) for l in range(3))
    bct = (1,) * 6
    dev = mf.MultiDomain(nd, periods, *grids, bct)
    dev.set_interface_solve(getattr(mf, iface))
    dev.influence_matrix_set(sigma, 0)
    subs = dev.subdomains()
    gs, bcs, singles, many = [], [], [], []
    for r in range(3):
        g, bc, _ = problem(grids, subs, sigma, bct)
        rng = np.random.default_rng(40 + r)
        g = {c: g[c] * (1.0 + r) + 0.1 * rng.standard_normal(g[c].shape) for c in subs}
        gs.append({c: mf.to_device(np.asfortranarray(g[c])) for c in subs})
        bcs.append({c: [mf.to_device(b * (1.0 - 0.3 * r)) for b in bc[c]] for c in subs})
        u1 = {c: mf.empty_device(g[c].shape) for c in subs}
        dev.solve(gs[r], u1, bcs[r])
        singles.append({c: mf.to_host(u1[c]) for c in subs})
        many.append({c: mf.empty_device(g[c].shape) for c in subs})
    dev.solve_many(gs, many, bcs)
    for r in range(3):
        for c in subs:
            assert np.array_equal(mf.to_host(many[r][c]), singles[r][c]), (r, c)


def test_factor_cache_round_trip(mf, gpu, tmp_path):
    """The factor written for one (grids, sigma, null mode) reloads into a
    fresh handle and solves identically; a factor of another sigma or a
    damaged file is refused; the cached entry point builds once and then
    loads."""
    import torch
    nd = (2, 1, 1)
    grids = [[mesh.tanh_grid(11, 1.0, 0.0, 0.5), mesh.tanh_grid(13, 1.0, 0.5, 1.0)],
             [mesh.tanh_grid(12, 1.0)], [mesh.tanh_grid(10, 1.0)]]
    make = lambda: mf.MultiDomain(nd, (0, 0, 0), grids[0], grids[1], grids[2], (1,) * 6, 6)
    a = make()
    a.set_interface_solve(mf.MD_IFACE_LU)
    a.influence_matrix_set(-3.0, 0)
    key = a.factor_key(-3.0, 0)
    assert len(key) == 16 and key != a.factor_key(-4.0, 0) and key != a.factor_key(-3.0, 1)
    path = tmp_path / (key + ".mffac")
    a.save_factor(path)
    b = make()
    b.set_interface_solve(mf.MD_IFACE_LU)
    b.load_factor(-3.0, 0, path)
    rng = np.random.default_rng(9)
    g, ua, ub, bc = {}, {}, {}, {}
    for c in a.subdomains():
        sh = a.shape(*c)
        g[c] = mf.to_device(rng.standard_normal(sh))
        ua[c], ub[c] = mf.empty_device(sh), mf.empty_device(sh)
        bc[c] = tuple(mf.to_device(rng.standard_normal(s)) for s in
                      ((sh[1] - 2, sh[2] - 2, 2), (sh[0] - 2, sh[2] - 2, 2), (sh[0] - 2, sh[1] - 2, 2)))
    a.solve(g, ua, bc)
    b.solve(g, ub, bc)
    torch.cuda.synchronize()
    for c in a.subdomains():
        assert torch.equal(ua[c], ub[c])
    with pytest.raises(mf.MflopsError):
        b.load_factor(-4.0, 0, path)
    data = path.read_bytes()
    (tmp_path / "cut.mffac").write_bytes(data[: len(data) - 16])
    with pytest.raises(mf.MflopsError):
        b.load_factor(-3.0, 0, tmp_path / "cut.mffac")
    cache = tmp_path / "cache"
    cache.mkdir()
    c1 = make()
    c1.influence_matrix_set(-3.0, 0, cache_dir=cache)
    assert (cache / (key + ".mffac")).exists()
    c2 = make()
    c2.influence_matrix_set(-3.0, 0, cache_dir=cache)
    uc = {c: mf.empty_device(a.shape(*c)) for c in a.subdomains()}
    c2.solve(g, uc, bc)
    ud = {c: mf.empty_device(a.shape(*c)) for c in a.subdomains()}
    c1.solve(g, ud, bc)
    torch.cuda.synchronize()
    for c in a.subdomains():
        assert torch.equal(uc[c], ud[c])


@pytest.mark.parametrize("nd,periods,bct,sigma,null", [
    ((2, 1, 1), (0, 0, 0), (1,) * 6, -3.0, 0),
    ((2, 2, 1), (0, 0, 0), (1, 2, 1, 2, 1, 2), -1e3, 0),
    ((2, 1, 2), (0, 0, 0), (2,) * 6, 0.0, 1),
    ((1, 1, 1), (1, 0, 1), (2,) * 6, 0.0, 1),
    ((2, 2, 2), (1, 0, 0), (1,) * 6, -10.0, 0),
])
def test_eigen_assembly_matches_solve_assembly(mf, gpu, nd, periods, bct, sigma, null):
    """Influence matrices formed in the solvers' eigenbasis (default) and by
    batched Dirac-column solves give the same subdomain solutions."""
    import torch
    sizes = [[11, 13], [12, 10], [10, 12]]
    lo_hi = [(0.0, 0.5), (0.5, 1.0)]
    grids = [[mesh.tanh_grid(sizes[l][q], 1.0, *lo_hi[q]) if nd[l] == 2 else mesh.uniform_grid(sizes[l][q], 0.0, 1.0)
              for q in range(nd[l])] for l in range(3)]
    out = []
    for mode in (mf.MD_ASSEMBLY_EIGEN, mf.MD_ASSEMBLY_SOLVES):
        md = mf.MultiDomain(nd, periods, grids[0], grids[1], grids[2], bct, 6)
        md.set_assembly(mode)
        md.influence_matrix_set(sigma, null)
        rng = np.random.default_rng(21)
        g, u, bc = {}, {}, {}
        for c in md.subdomains():
            sh = md.shape(*c)
            g[c] = mf.to_device(rng.standard_normal(sh))
            u[c] = mf.empty_device(sh)
            bc[c] = tuple(mf.to_device(rng.standard_normal(s)) for s in
                          ((sh[1] - 2, sh[2] - 2, 2), (sh[0] - 2, sh[2] - 2, 2), (sh[0] - 2, sh[1] - 2, 2)))
        md.solve(g, u, bc)
        torch.cuda.synchronize()
        out.append({c: mf.to_host(u[c]) for c in md.subdomains()})
        md.close()
    for c in out[0]:
        a, b = out[0][c][1:-1, 1:-1, 1:-1], out[1][c][1:-1, 1:-1, 1:-1]
        if null:  # the null-space solution is defined up to a constant
            a, b = a - a.mean(), b - b.mean()
        assert max_rel(a, b) < 1e-11, (c, max_rel(a, b))


def _random_solve(mf, dev, seed):
    import torch
    gen = torch.Generator("cuda").manual_seed(seed)
    g, u, bc = {}, {}, {}
    for c in dev.subdomains():
        sh = dev.shape(*c)
        g[c] = torch.randn(tuple(reversed(sh)), dtype=torch.float64, device="cuda",
                           generator=gen).permute(2, 1, 0)
        u[c] = mf.empty_device(sh)
        bc[c] = (mf.empty_device((sh[1] - 2, sh[2] - 2, 2)), mf.empty_device((sh[0] - 2, sh[2] - 2, 2)),
                 mf.empty_device((sh[0] - 2, sh[1] - 2, 2)))
        for b in bc[c]:
            b.zero_()
    return g, u, bc


@pytest.mark.parametrize("sigma,bct,null", [(-1e3, (1,) * 6, 0), (0.0, (2,) * 6, 1)])
def test_persistent_triangular_solves(mf, gpu, sigma, bct, null):
    """The persistent triangular solves (one cooperative launch per triangle)
    against the block-step form on an interface system large enough that
    every CTA owns several 64-row blocks (2 x 2 x 2 slabs of 41 nodes,
    18,252 unknowns): same interface values and fields to 1e-11, for one and
    for three right-hand sides, velocity-like and pressure-like (null space)
    operators; the device status stays clean."""
    import torch
    grids = tuple(slabs(2, 41) for _ in range(3))
    dev = mf.MultiDomain((2, 2, 2), (0, 0, 0), *grids, bct)
    dev.set_interface_solve(mf.MD_IFACE_LU)
    dev.influence_matrix_set(sigma, null)
    assert dev.ninf() > 152 * 64
    g, u, bc = _random_solve(mf, dev, 11)
    lam = {}
    fields = {}
    for form in (mf.MD_TRI_STEPS, mf.MD_TRI_PERSISTENT):
        dev.set_triangular_form(form)
        dev.solve(g, u, bc)
        dev.device_status()
        lam[form] = dev.interface()
        fields[form] = {c: u[c].clone() for c in u}
    assert max_rel(lam[mf.MD_TRI_PERSISTENT], lam[mf.MD_TRI_STEPS]) < 1e-11
    for c in u:
        a, b = fields[mf.MD_TRI_PERSISTENT][c], fields[mf.MD_TRI_STEPS][c]
        assert float((a - b).abs().max() / b.abs().max()) < 1e-11
    # several right-hand sides in one call (K = 3 in the persistent kernel)
    sets = [_random_solve(mf, dev, 20 + q) for q in range(3)]
    outs = {}
    for form in (mf.MD_TRI_STEPS, mf.MD_TRI_PERSISTENT):
        dev.set_triangular_form(form)
        dev.solve_many([s[0] for s in sets], [s[1] for s in sets], [s[2] for s in sets])
        dev.device_status()
        outs[form] = [{c: s[1][c].clone() for c in s[1]} for s in sets]
    for q in range(3):
        for c in sets[q][1]:
            a, b = outs[mf.MD_TRI_PERSISTENT][q][c], outs[mf.MD_TRI_STEPS][q][c]
            assert float((a - b).abs().max() / b.abs().max()) < 1e-11
    torch.cuda.synchronize()


@pytest.mark.parametrize("sigma,bct,null", [(-1e3, (1,) * 6, 0), (0.0, (2,) * 6, 1)])
def test_inverted_factors_large_system(mf, gpu, sigma, bct, null):
    """Above 12,000 unknowns the default interface form is the inverted LU
    factors (trtri at set-up, two row-parallel double-float products per
    solve): on the 18,252-unknown system of 2 x 2 x 2 slabs of 41 nodes it
    gives the triangular solves' interface values and fields to 1e-11, for
    one and for three right-hand sides, velocity-like and pressure-like
    operators."""
    import torch
    grids = tuple(slabs(2, 41) for _ in range(3))
    dev = mf.MultiDomain((2, 2, 2), (0, 0, 0), *grids, bct)
    dev.influence_matrix_set(sigma, null)
    assert dev.ninf() > 12000
    assert dev.interface_form() == mf.MD_IFACE_TRIANGULAR_INVERSE
    g, u, bc = _random_solve(mf, dev, 11)
    lam, fields = {}, {}
    for form in (mf.MD_IFACE_AUTO, mf.MD_IFACE_LU):
        dev.set_interface_solve(form)
        dev.solve(g, u, bc)
        lam[form] = dev.interface()
        fields[form] = {c: u[c].clone() for c in u}
    assert dev.interface_form() == mf.MD_IFACE_LU
    assert max_rel(lam[mf.MD_IFACE_AUTO], lam[mf.MD_IFACE_LU]) < 1e-11
    for c in u:
        a, b = fields[mf.MD_IFACE_AUTO][c], fields[mf.MD_IFACE_LU][c]
        assert float((a - b).abs().max() / b.abs().max()) < 1e-11
    sets = [_random_solve(mf, dev, 20 + q) for q in range(3)]
    outs = {}
    for form in (mf.MD_IFACE_AUTO, mf.MD_IFACE_LU):
        dev.set_interface_solve(form)
        dev.solve_many([s[0] for s in sets], [s[1] for s in sets], [s[2] for s in sets])
        outs[form] = [{c: s[1][c].clone() for c in s[1]} for s in sets]
    for q in range(3):
        for c in sets[q][1]:
            a, b = outs[mf.MD_IFACE_AUTO][q][c], outs[mf.MD_IFACE_LU][q][c]
            assert float((a - b).abs().max() / b.abs().max()) < 1e-11
    dev.device_status()
    torch.cuda.synchronize()


@pytest.mark.parametrize("null", [0, 1, 2])
@pytest.mark.parametrize("iface", ["MD_IFACE_INVERSE", "MD_IFACE_LU", "MD_IFACE_TRIANGULAR_INVERSE",
                                   "MD_IFACE_TRIANGULAR_INVERSE_FP64"])
def test_interface_solve_matches_oracle(mf, gpu, iface, null):
    """md_solve alone (mf_md_interface_solve): the interface system of a
    2 x 2 x 1 decomposition for one and for three random right-hand sides,
    in each form, against the oracle's dense solve of its own influence
    matrix (with the same null-space handling) to 1e-10."""
    import torch
    nd, periods = (2, 2, 1), (0, 0, 0)
    bct = (2,) * 6 if null else (1,) * 6
    sigma = 0.0 if null else -3.0
    grids = tuple(slabs(nd[l], 11) for l in range(3))
    ref = omd.MultiDomain(nd, periods, *grids, bct)
    ref.influence_matrix(sigma, null)
    dev = mf.MultiDomain(nd, periods, *grids, bct)
    dev.set_interface_solve(getattr(mf, iface))
    dev.influence_matrix_set(sigma, null)
    assert dev.interface_form() == getattr(mf, iface)
    rng = np.random.default_rng(5 + null)
    rhs = rng.standard_normal((3, dev.ninf()))
    want = np.stack([ref.interface_solve(r) for r in rhs])
    one = dev.interface_solve(torch.from_numpy(rhs[0].copy()).cuda())
    three = dev.interface_solve(torch.from_numpy(rhs).cuda())
    assert max_rel(one.cpu().numpy(), want[0]) < 1e-10
    for q in range(3):
        assert max_rel(three[q].cpu().numpy(), want[q]) < 1e-10, q
