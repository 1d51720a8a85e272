"""Batched plain solves (mf_solve_3d_batch): B problems of one operator in
one pass of launches give exactly the results of B separate mf_solve_3d
calls (same per-problem arithmetic), with per-problem or shared (stride 0)
right-hand sides and boundary arrays; argument errors are reported."""
import numpy as np
import pytest

from helpers import bc_arrays, field, grids

pytestmark = pytest.mark.gpu


def stack(mf, arrays):
    """(..., B) device tensor, x fastest and the batch index slowest."""
    return mf.to_device(np.stack(arrays, axis=-1))


@pytest.mark.parametrize("shared", [False, True])
def test_batch_equals_single_solves(mf, gpu, shared):
    import torch
    nall = (19, 14, 17)
    gx, gy, gz = grids(*nall, kind="tanh")
    sc = mf.SolverCoeffs3D(gx, gy, gz, (1, 2, 1, 1, 2, 1), 6)
    n1, n2, n3 = (v - 2 for v in nall)
    B = 7
    rhs = [field((n1, n2, n3), 40 + b) for b in range(B)]
    bcs = [bc_arrays(n1, n2, n3, 60 + b) for b in range(B)]
    if shared:
        rhs_d = mf.to_device(rhs[0])
        bc_d = [mf.to_device(bcs[0][a]) for a in range(3)]
    else:
        rhs_d = stack(mf, rhs)
        bc_d = [stack(mf, [bcs[b][a] for b in range(B)]) for a in range(3)]
    out = mf.empty_device(tuple(v for v in nall) + (B,))
    sc.solve_3d_batch(rhs_d, -7.0, out, *bc_d)
    torch.cuda.synchronize()
    for b in range(B):
        r = rhs[0] if shared else rhs[b]
        bc = bcs[0] if shared else bcs[b]
        one = mf.empty_device(nall)
        sc.solve_3d(mf.to_device(r), -7.0, one, *[mf.to_device(x) for x in bc])
        assert torch.equal(out[..., b], one), b


def test_batch_argument_errors(mf, gpu):
    nall = (12, 12, 12)
    g = grids(*nall, kind="uniform")
    sc = mf.SolverCoeffs3D(*g, (1,) * 6, 6)
    n = 10
    rhs = mf.empty_device((n, n, n))
    bc = [mf.empty_device((n, n, 2)) for _ in range(3)]
    out = mf.empty_device((12, 12, 12, 3))
    import ctypes
    # overlapping outputs
    rc = mf._lib.mf_solve_3d_batch(sc._h, 3, ctypes.c_void_p(rhs.data_ptr()), 0, 0.0,
                                   ctypes.c_void_p(out.data_ptr()), 5, *[v for b in bc for v in
                                                                          (ctypes.c_void_p(b.data_ptr()), 0)],
                                   n, n, n, None)
    assert rc == mf.MF_ERR_ARG
    # host arrays are refused
    host = np.zeros((12, 12, 12, 3), order="F")
    rc = mf._lib.mf_solve_3d_batch(sc._h, 3, ctypes.c_void_p(rhs.data_ptr()), 0, 0.0,
                                   ctypes.c_void_p(host.ctypes.data), 12 ** 3,
                                   *[v for b in bc for v in (ctypes.c_void_p(b.data_ptr()), 0)], n, n, n, None)
    assert rc == mf.MF_ERR_ARG
