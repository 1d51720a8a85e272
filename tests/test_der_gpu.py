"""GPU compact derivatives (class_derivatives + class_field pencil drivers)
against the FP64 oracle, through the C ABI.  Tolerance: max |gpu - oracle|
<= 1e-12 * max |oracle| (so <= 6); so = 8 uses 1e-9 (ill-conditioned
Taylor systems, see test_setup_host.py)."""
import numpy as np
import pytest

from oracle import derivatives as D
from oracle import mesh

from helpers import field, max_rel

pytestmark = pytest.mark.gpu

FUNCS = {(0, 1): D.derx, (1, 1): D.dery, (2, 1): D.derz,
         (0, 2): D.dderx, (1, 2): D.ddery, (2, 2): D.dderz}


def tol(so):
    return 1e-12 if so <= 6 else 1e-9


@pytest.mark.parametrize("so", [4, 6, 8])
@pytest.mark.parametrize("solver", [False, True])
@pytest.mark.parametrize("shape", [(17, 13, 11), (33, 29, 9), (65, 65, 65), (150, 9, 11), (200, 11, 9)])
def test_field_derivatives(mf, gpu, so, solver, shape):
    # x lines: staged through shared memory up to nx = 191 (nx = 150), one
    # thread per line above (nx = 200)
    f = field(shape, seed=2)
    fd = mf.to_device(f)
    for axis in range(3):
        g = mesh.tanh_grid(shape[axis], 1.5)
        dc_ref = D.DerCoeffs(g, so, solver)
        dc = mf.DerivativesCoefficients(g, solve=solver, so=so)
        assert dc.dertype() == solver
        for order in (1, 2):
            ref = FUNCS[(axis, order)](dc_ref, f)
            got = mf.to_host(dc.apply(axis, order, fd))
            assert max_rel(got, ref) < tol(so), (axis, order)


def test_reference_named_drivers_and_host_arrays(mf, gpu):
    nx, ny, nz = 21, 18, 15
    f = field((nx, ny, nz), seed=7)
    gx, gy, gz = mesh.arcsin_grid(nx), mesh.arcsin_grid(ny), mesh.arcsin_grid(nz, -0.25, 0.25)
    dcs = [mf.der_coeffs_init(g, g.size, False, 6) for g in (gx, gy, gz)]
    refs = [D.DerCoeffs(g, 6) for g in (gx, gy, gz)]
    pairs = [(mf.derx, D.derx, 0), (mf.dery, D.dery, 1), (mf.derz, D.derz, 2),
             (mf.dderx, D.dderx, 0), (mf.ddery, D.ddery, 1), (mf.dderz, D.dderz, 2)]
    for fn, ofn, a in pairs:
        host = fn(dcs[a], f)                     # host NumPy path (staged)
        dev = mf.to_host(fn(dcs[a], mf.to_device(f)))
        ref = ofn(refs[a], f)
        assert max_rel(host, ref) < 1e-12
        assert np.array_equal(host, dev)


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("variant", [False, True])
def test_pencil_forms(mf, gpu, order, variant):
    n, count = 41, 37
    g = mesh.tanh_grid(n, 2.0)
    dc = mf.DerivativesCoefficients(g, solve=True, so=6)
    ref = D.DerCoeffs(g, 6, True)
    x = field((n, count), seed=11)
    got = mf.to_host(dc.lines(order, mf.to_device(x), solver_variant=variant))
    fn = {(1, False): ref.der, (2, False): ref.dder, (1, True): ref.der_s, (2, True): ref.dder_s}
    want = fn[(order, variant)](x)
    assert max_rel(got, want) < 1e-12


def test_large_pencils_and_in_place(mf, gpu):
    # x pencils long enough to use the strided fallback, and an in-place call
    shape = (900, 5, 4)
    g = mesh.tanh_grid(900, 1.0)
    f = field(shape, seed=3)
    dc = mf.DerivativesCoefficients(g, so=6)
    ref = D.derx(D.DerCoeffs(g, 6), f)
    assert max_rel(mf.to_host(mf.derx(dc, mf.to_device(f))), ref) < 1e-12
    gy = mesh.tanh_grid(5, 0.0) if False else None
    shape2 = (12, 40, 9)
    f2 = field(shape2, seed=4)
    g2 = mesh.tanh_grid(40, 1.5)
    dc2 = mf.DerivativesCoefficients(g2, so=6)
    t = mf.to_device(f2)
    mf.dery(dc2, t, out=t)
    assert max_rel(mf.to_host(t), D.dery(D.DerCoeffs(g2, 6), f2)) < 1e-12


def test_shape_errors(mf, gpu):
    dc = mf.DerivativesCoefficients(np.linspace(0, 1, 11), so=6)
    with pytest.raises(mf.MflopsError) as e:
        dc.apply(0, 1, mf.to_device(np.zeros((12, 3, 3), order="F")))
    assert e.value.code == mf.MF_ERR_ARG
    # the GPU is still usable afterwards
    out = dc.apply(0, 1, mf.to_device(np.ones((11, 3, 3), order="F")))
    assert np.max(np.abs(mf.to_host(out))) < 1e-9


def test_der_apply_many_equals_separate_sweeps(mf, gpu):
    """Nine sweeps of mixed axes, orders and fields in one launch give the
    results of nine mf_der_apply calls, for plain and solver-type coefficients."""
    import torch
    from oracle import mesh
    shape = (19, 14, 17)
    for solver in (False, True):
        dcs = [mf.DerivativesCoefficients(g, solve=solver, so=6)
               for g in (mesh.tanh_grid(shape[0], 1.0), mesh.tanh_grid(shape[1], 1.5), mesh.uniform_grid(shape[2]))]
        rng = np.random.default_rng(7)
        fs = [mf.to_device(rng.standard_normal(shape)) for _ in range(3)]
        jobs = [(dcs[a], a, 1 + (q % 2), fs[q % 3], mf.empty_device(shape)) for q, a in
                enumerate((0, 1, 2, 0, 1, 2, 2, 1, 0))]
        mf.der_apply_many(jobs)
        for dc, a, order, f, out in jobs:
            assert torch.equal(out, dc.apply(a, order, f)), (solver, a, order)
