"""The two plans of the 3xTF32 tensor-core transform (mf_tc_tf32_plan_set)
through full mixed solves: 64-column slices with the matrix resident in
shared memory, and 128-column slices with the matrix streamed through the
TMA ring (axes padded to a multiple of 128).  Every output sums the same
products in the same accumulators and the epilogue adds them in the same
order, so the two plans must agree bit for bit; the refined solve is held to
rel-L2 <= 1e-10 against the plain FP64 GPU solve.  With the tuner on, the
plan is measured per shape and the results stay identical."""
import numpy as np
import pytest

from oracle import mesh

from helpers import bc_arrays, field, rel_l2

pytestmark = pytest.mark.gpu

SHAPES = [
    (130, 130, 130),   # every axis padded to 128: both plans
    (66, 258, 130),    # 64 (narrow only), 256 and 128
    (201, 97, 140),    # 256, 128 and 192 (narrow only for z)
]


def _solve(mf, nall, precision, seed=7):
    gx, gy, gz = mesh.uniform_grid(nall[0]), mesh.tanh_grid(nall[1], 2.0), mesh.tanh_grid(nall[2], 1.0)
    n = [v - 2 for v in nall]
    sc = mf.SolverCoeffs3D(gx, gy, gz, (1,) * 6, 6)
    rhs = mf.to_device(field(tuple(n), seed))
    bcs = [mf.to_device(b) for b in bc_arrays(*n, seed + 1)]
    solf = mf.empty_device(tuple(nall))
    if precision is None:
        sc.solve_3d(rhs, 0.0, solf, *bcs)
    else:
        sc.solve_3d(rhs, 0.0, solf, *bcs, precision=precision, refine=1)
    return solf


@pytest.mark.parametrize("nall", SHAPES)
def test_tf32_plans_identical(mf, gpu, nall):
    import torch
    ref = _solve(mf, nall, None)
    outs = {}
    try:
        for plan in (1, 2):
            mf.tc_tf32_plan(plan)
            outs[plan] = _solve(mf, nall, mf.MF_PREC_3XTF32)
    finally:
        mf.tc_tf32_plan(0)
    torch.cuda.synchronize()
    assert torch.equal(outs[1], outs[2])
    inner = (slice(1, -1),) * 3
    err = rel_l2(mf.to_host(outs[2])[inner], mf.to_host(ref)[inner])
    assert err < 1e-10, err


def test_tuner_picks_a_plan_per_shape(mf, gpu):
    import torch
    mf.tune(mode=0, clear=True)
    nall = SHAPES[1]
    base = _solve(mf, nall, mf.MF_PREC_3XTF32)
    try:
        mf.tune(mode=1)
        tuned = _solve(mf, nall, mf.MF_PREC_3XTF32)
        torch.cuda.synchronize()
        entries = mf.tune()[1]
    finally:
        mf.tune(mode=0, clear=True)
    assert torch.equal(base, tuned)
    assert entries >= 2  # at least the y (256) and z (128) transform shapes
