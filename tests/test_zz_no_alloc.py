"""The allocation-free solve entry point (mf_solve_3d_noalloc) against the
regular plain FP64 entry point, through the C ABI.

The entry point exists for callers that cannot let a library call
cudaMalloc (applications whose pool allocator owns and budgets all device
memory; host loops that cannot afford cudaMalloc's implicit device
synchronisation); its work arrays live in a fixed file-scope device array of
2 x 262144 doubles shared by all calls.
This file is collected last so that a failure here comes after every other
test has run; it also passes alone in a fresh process.
Tolerance: the two entry points run the same kernels on the same data, so
they must agree to 1e-12 relative (the plain-path tolerance of the suite)."""
import numpy as np
import pytest

from helpers import bc_arrays, field, grids, max_rel, solf_mask

pytestmark = pytest.mark.gpu


def test_noalloc_matches_regular_entry_point_twice(mf, gpu):
    nall = (33, 29, 35)
    gx, gy, gz = grids(*nall)
    n1, n2, n3 = (v - 2 for v in nall)
    sc = mf.SolverCoeffs3D(gx, gy, gz, (1, 2, 1, 1, 2, 1), 6)
    m = solf_mask(n1, n2, n3)
    # two calls in a row with different data: the shared scratch keeps the
    # previous call's contents, which must not leak into the next result
    for seed, sigma in ((11, -1e3), (23, 0.0)):
        rhs = mf.to_device(field((n1, n2, n3), seed))
        bcs = [mf.to_device(b) for b in bc_arrays(n1, n2, n3, seed + 1)]
        solf0 = field((n1 + 2, n2 + 2, n3 + 2), seed + 2)
        want = sc.solve_3d(rhs, sigma, mf.to_device(solf0), *bcs)
        got = sc.solve_3d_noalloc(rhs, sigma, mf.to_device(solf0), *bcs)
        gpu.cuda.synchronize()
        w, g = mf.to_host(want), mf.to_host(got)
        assert max_rel(g, w, m) < 1e-12
        assert np.array_equal(g[~m], solf0[~m])


def test_noalloc_at_the_size_limit(mf, gpu):
    # 64^3 = 262144 interior points: both work arrays filled to their last
    # entry; two calls with different data and sigma
    nall = (66, 66, 66)
    gx, gy, gz = grids(*nall)
    n = 64
    sc = mf.SolverCoeffs3D(gx, gy, gz, (2, 1, 1, 1, 1, 2), 6)
    m = solf_mask(n, n, n)
    for seed, sigma in ((31, -20.0), (41, 0.0)):
        rhs = mf.to_device(field((n, n, n), seed))
        bcs = [mf.to_device(b) for b in bc_arrays(n, n, n, seed + 1)]
        solf0 = field((n + 2, n + 2, n + 2), seed + 2)
        want = sc.solve_3d(rhs, sigma, mf.to_device(solf0), *bcs)
        got = sc.solve_3d_noalloc(rhs, sigma, mf.to_device(solf0), *bcs)
        gpu.cuda.synchronize()
        assert max_rel(mf.to_host(got), mf.to_host(want), m) < 1e-12


def test_noalloc_rejects_sizes_and_host_data(mf, gpu):
    gx, gy, gz = grids(67, 67, 67)
    sc = mf.SolverCoeffs3D(gx, gy, gz, (1,) * 6, 6)
    n = 65
    rhs = mf.empty_device((n, n, n))
    bcs = [mf.empty_device((n, n, 2)) for _ in range(3)]
    with pytest.raises(mf.MflopsError) as e:
        sc.solve_3d_noalloc(rhs, 0.0, mf.empty_device((n + 2,) * 3), *bcs)
    assert e.value.code == mf.MF_ERR_UNSUPPORTED
    g2 = grids(17, 17, 17)
    sc2 = mf.SolverCoeffs3D(*g2, (1,) * 6, 6)
    host = np.zeros((15, 15, 15), order="F")
    with pytest.raises(mf.MflopsError) as e:
        sc2.solve_3d_noalloc(host, 0.0, np.zeros((17, 17, 17), order="F"),
                             *[np.zeros((15, 15, 2), order="F")] * 3)
    assert e.value.code == mf.MF_ERR_ARG
