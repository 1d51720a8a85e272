"""Split-BF16 and 3xTF32 tensor-core transforms + FP64 iterative refinement
against the FP64 oracle.  Tolerance: relative L2 error <= 1e-10 after
refinement; the unrefined split-precision error is reported alongside."""
import numpy as np
import pytest

from oracle import solver as S
from oracle import mesh

from helpers import bc_arrays, field, grids, rel_l2, solf_mask

pytestmark = pytest.mark.gpu


def mixed_case(mf, nall, bct, sigma, refine, kind="tanh", seed=5, prec=None):
    prec = mf.MF_PREC_SPLIT_BF16 if prec is None else prec
    gx, gy, gz = grids(*nall, kind=kind)
    n1, n2, n3 = (v - 2 for v in nall)
    sc_ref = S.Solver3D(gx, gy, gz, bct, 6)
    sc = mf.SolverCoeffs3D(gx, gy, gz, bct, 6)
    rhs = field((n1, n2, n3), seed)
    bcx, bcy, bcz = bc_arrays(n1, n2, n3, seed + 1)
    solf0 = np.zeros((n1 + 2, n2 + 2, n3 + 2), order="F")
    ref = S.solve_3d(sc_ref, rhs, sigma, solf0, bcx, bcy, bcz)
    got = sc.solve_3d(mf.to_device(rhs), sigma, mf.to_device(solf0), mf.to_device(bcx),
                      mf.to_device(bcy), mf.to_device(bcz), precision=prec, refine=refine)
    m = solf_mask(n1, n2, n3)
    return rel_l2(mf.to_host(got)[m], ref[m])


def test_mixed_unrefined_is_split_precision_accurate(mf, gpu):
    err = mixed_case(mf, (66, 66, 66), (1,) * 6, -1e3, refine=0)
    print("split-bf16 unrefined rel L2 error: %.3e" % err)
    assert err < 1e-3


@pytest.mark.parametrize("sigma", [0.0, -1e3])
def test_mixed_refined_reaches_1e10(mf, gpu, sigma):
    err = mixed_case(mf, (66, 66, 66), (1,) * 6, sigma, refine=3)
    print("split-bf16 + 3 refinements rel L2 error: %.3e" % err)
    assert err < 1e-10


def test_mixed_uneven_and_neumann(mf, gpu):
    err = mixed_case(mf, (50, 66, 98), (1, 2, 1, 1, 2, 1), -1e6 * 1e-3, refine=3)
    assert err < 1e-10


def test_mixed_slice_shapes(mf, gpu):
    # padded sizes 192 (two 96-column slices), 64 and 128 on the three axes
    err = mixed_case(mf, (150, 34, 98), (1,) * 6, -1e6, refine=3)
    assert err < 1e-10


def test_mixed_matches_fp64_gpu_at_257(mf, gpu):
    """Headline shape: 257^3 Poisson, tanh(2.0) in y; refined split-BF16
    solution vs the plain FP64 GPU solution."""
    import torch
    from oracle import mesh
    n = 255
    gx, gy = mesh.uniform_grid(257), mesh.tanh_grid(257, 2.0)
    sc = mf.SolverCoeffs3D(gx, gy, gx, (1,) * 6, 6)
    rhs = torch.randn((n, n, n), dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(5)).permute(2, 1, 0)
    bc = [mf.empty_device((n, n, 2)) for _ in range(3)]
    plain = mf.empty_device((257, 257, 257))
    mixed = mf.empty_device((257, 257, 257))
    sc.solve_3d(rhs, 0.0, plain, *bc)
    sc.solve_3d(rhs, 0.0, mixed, *bc, precision=mf.MF_PREC_SPLIT_BF16, refine=2)
    sc.device_status()
    err = (torch.linalg.vector_norm(mixed - plain) / torch.linalg.vector_norm(plain)).item()
    print("257^3 split-bf16 + 2 refinements vs FP64 GPU: %.3e" % err)
    assert err < 1e-10


def test_tf32_unrefined_is_more_accurate(mf, gpu):
    err_bf = mixed_case(mf, (66, 66, 66), (1,) * 6, -1e3, refine=0)
    err = mixed_case(mf, (66, 66, 66), (1,) * 6, -1e3, refine=0, prec=mf.MF_PREC_3XTF32)
    print("3xtf32 unrefined rel L2 error: %.3e (split-bf16 %.3e)" % (err, err_bf))
    assert err < 1e-5 and err < err_bf


@pytest.mark.parametrize("sigma", [0.0, -1e3])
def test_tf32_one_refinement_reaches_1e10(mf, gpu, sigma):
    err = mixed_case(mf, (66, 66, 66), (1,) * 6, sigma, refine=1, prec=mf.MF_PREC_3XTF32)
    print("3xtf32 + 1 refinement rel L2 error: %.3e" % err)
    assert err < 1e-10


def test_tf32_slice_shapes_and_neumann(mf, gpu):
    # padded sizes 192 (three 64-column slices), 64 and 128 (one slice)
    err = mixed_case(mf, (150, 34, 98), (1, 2, 1, 1, 2, 1), -1e6, refine=2,
                     prec=mf.MF_PREC_3XTF32)
    assert err < 1e-10


def test_tf32_matches_fp64_gpu_at_257(mf, gpu):
    import torch
    from oracle import mesh
    n = 255
    gx, gy = mesh.uniform_grid(257), mesh.tanh_grid(257, 2.0)
    sc = mf.SolverCoeffs3D(gx, gy, gx, (1,) * 6, 6)
    rhs = torch.randn((n, n, n), dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(5)).permute(2, 1, 0)
    bc = [mf.empty_device((n, n, 2)) for _ in range(3)]
    plain = mf.empty_device((257, 257, 257))
    mixed = mf.empty_device((257, 257, 257))
    sc.solve_3d(rhs, 0.0, plain, *bc)
    errs = []
    for refine in (0, 1, 2):
        sc.solve_3d(rhs, 0.0, mixed, *bc, precision=mf.MF_PREC_3XTF32, refine=refine)
        sc.device_status()
        errs.append((torch.linalg.vector_norm(mixed - plain) / torch.linalg.vector_norm(plain)).item())
    print("257^3 3xtf32 vs FP64 GPU, refine 0/1/2: %.3e %.3e %.3e" % tuple(errs))
    assert errs[2] < 1e-10


@pytest.mark.parametrize("prec_name,refine", [("MF_PREC_3XTF32", 1), ("MF_PREC_SPLIT_BF16", 2)])
def test_residual_arithmetic_modes_agree(mf, gpu, prec_name, refine):
    """Double-FP32 and FP64 sweeps of the refinement residual give solutions
    within 1e-10 of the FP64 oracle and within 1e-11 of each other."""
    nall = (66, 50, 82)
    gx, gy, gz = grids(*nall, kind="tanh")
    n1, n2, n3 = (v - 2 for v in nall)
    bct = (1, 2, 1, 1, 2, 1)
    sc_ref = S.Solver3D(gx, gy, gz, bct, 6)
    sc = mf.SolverCoeffs3D(gx, gy, gz, bct, 6)
    rhs = field((n1, n2, n3), 9)
    bcx, bcy, bcz = bc_arrays(n1, n2, n3, 10)
    solf0 = np.zeros((n1 + 2, n2 + 2, n3 + 2), order="F")
    ref = S.solve_3d(sc_ref, rhs, -30.0, solf0, bcx, bcy, bcz)
    m = solf_mask(n1, n2, n3)
    got = {}
    for mode in (mf.MF_RESID_FF, mf.MF_RESID_FP64, mf.MF_RESID_FP64_LINE):
        sc.set_residual(mode)
        out = sc.solve_3d(mf.to_device(rhs), -30.0, mf.to_device(solf0), mf.to_device(bcx),
                          mf.to_device(bcy), mf.to_device(bcz), precision=getattr(mf, prec_name),
                          refine=refine)
        got[mode] = mf.to_host(out)[m]
        assert rel_l2(got[mode], ref[m]) < 1e-10
    assert rel_l2(got[mf.MF_RESID_FF], got[mf.MF_RESID_FP64]) < 1e-11
    assert rel_l2(got[mf.MF_RESID_FP64_LINE], got[mf.MF_RESID_FP64]) < 1e-11


@pytest.mark.parametrize("nall,bct,kind", [((10, 11, 12), (1,) * 6, "tanh"),
                                           ((11, 10, 13), (2, 1, 1, 2, 2, 2), "tanh"),
                                           ((35, 36, 34), (1, 2, 2, 1, 1, 1), "uniform"),
                                           ((130, 67, 41), (1,) * 6, "tanh")])
def test_two_sided_residual_matches_line_residual(mf, gpu, nall, bct, kind):
    """The residual with two lanes per line (top and bottom elimination meeting
    at the twist row; odd and even axis lengths, the shortest axes the
    moment form accepts, Neumann ends, inhomogeneous boundary data) gives the
    one-thread-per-line solution to the refined solves' accuracy (the two
    residual evaluations round differently), and both refine to the FP64
    oracle."""
    gx, gy, gz = grids(*nall, kind=kind)
    n1, n2, n3 = (v - 2 for v in nall)
    sc_ref = S.Solver3D(gx, gy, gz, bct, 6)
    sc = mf.SolverCoeffs3D(gx, gy, gz, bct, 6)
    rhs = field((n1, n2, n3), 21)
    bcx, bcy, bcz = bc_arrays(n1, n2, n3, 22)
    solf0 = np.zeros((n1 + 2, n2 + 2, n3 + 2), order="F")
    sigma = -7.0
    ref = S.solve_3d(sc_ref, rhs, sigma, solf0, bcx, bcy, bcz)
    m = solf_mask(n1, n2, n3)
    got = {}
    for mode in (mf.MF_RESID_FP64, mf.MF_RESID_FP64_LINE):
        sc.set_residual(mode)
        out = sc.solve_3d(mf.to_device(rhs), sigma, mf.to_device(solf0), mf.to_device(bcx),
                          mf.to_device(bcy), mf.to_device(bcz), precision=mf.MF_PREC_3XTF32, refine=2)
        sc.device_status()
        got[mode] = mf.to_host(out)[m]
        assert rel_l2(got[mode], ref[m]) < 1e-10, (mode, rel_l2(got[mode], ref[m]))
    assert rel_l2(got[mf.MF_RESID_FP64], got[mf.MF_RESID_FP64_LINE]) < 1e-11



def test_mixed_rejects_axes_longer_than_256(mf, gpu):
    # 259 nodes: 257 interior points, above the transforms' 256-point tiles;
    # the plain path accepts the same problem
    g = mesh.uniform_grid(259)
    g2 = mesh.uniform_grid(9)
    sc = mf.SolverCoeffs3D(g, g2, g2, (1,) * 6, 6)
    rhs = mf.to_device(np.zeros((257, 7, 7), order="F"))
    bc = [mf.to_device(np.zeros(s, order="F")) for s in ((7, 7, 2), (257, 7, 2), (257, 7, 2))]
    solf = mf.empty_device((259, 9, 9))
    with pytest.raises(RuntimeError, match="256"):
        sc.solve_3d(rhs, 0.0, solf, *bc, precision=mf.MF_PREC_3XTF32, refine=1)
    sc.solve_3d(rhs, 0.0, solf, *bc)


@pytest.mark.parametrize("prec_name,refine", [("MF_PREC_FP64", -1), ("MF_PREC_3XTF32", 1)])
def test_many_problems_equal_single_calls(mf, gpu, prec_name, refine):
    """mf_solve_3d_mixed_many (uploads/downloads overlapping the solves) gives
    each problem exactly the result of a single call, host arrays in and out,
    and of the same call on device arrays; the host paths upload only the
    edges of the solution array, which come back as they were.  Two calls in
    a row: the second replays every slot's graph."""
    nall = (34, 30, 26)
    gx, gy, gz = grids(*nall, kind="tanh")
    sc = mf.SolverCoeffs3D(gx, gy, gz, (1, 2, 1, 1, 2, 1), 6)
    n1, n2, n3 = (v - 2 for v in nall)
    prec = getattr(mf, prec_name)
    B = 8  # mixed: problem 0 eager, 1-3 capture each staging slot's graph, 4-7 replay them
    rhs = [field((n1, n2, n3), 80 + b) for b in range(B)]
    bcs = [bc_arrays(n1, n2, n3, 90 + b) for b in range(B)]
    solf0 = [field(nall, 100 + b) for b in range(B)]  # edges and corners are kept
    outs = [np.asfortranarray(s.copy()) for s in solf0]
    for _ in range(2):
        outs = [np.asfortranarray(s.copy()) for s in solf0]
        sc.solve_3d_many(rhs, -4.0, outs, [b[0] for b in bcs], [b[1] for b in bcs], [b[2] for b in bcs],
                         precision=prec, refine=refine)
    edge = np.zeros(nall, dtype=bool)
    for a in range(3):
        for c in range(a + 1, 3):
            for ia in (0, -1):
                for ic in (0, -1):
                    sl = [slice(None)] * 3
                    sl[a], sl[c] = ia, ic
                    edge[tuple(sl)] = True
    for b in range(B):
        one = np.asfortranarray(solf0[b].copy())
        sc.solve_3d(rhs[b], -4.0, one, *bcs[b], precision=prec, refine=refine)
        assert np.array_equal(outs[b], one), b
        dev = mf.to_device(solf0[b])
        sc.solve_3d(mf.to_device(rhs[b]), -4.0, dev, *[mf.to_device(x) for x in bcs[b]], precision=prec,
                    refine=refine)
        assert np.array_equal(mf.to_host(dev), one), b
        assert np.array_equal(one[edge], solf0[b][edge]), b


def test_many_after_new_eigen_tables(mf, gpu):
    """New eigen tables (mf_solver3d_set_eigen) between two
    mf_solve_3d_mixed_many calls: the staging slots' graphs of the first call
    are not replayed by the second.  All-Neumann operator at sigma = -10,
    first with the oracle's tables (closed: one null eigenvalue per axis, so
    FP64 residual passes), then with axis 0's null eigenvalue moved to 1e-3
    (no longer closed: the residual passes store the operand directly); the
    second call's problems must equal single eager calls with those tables."""
    nall = (26, 22, 18)
    gx, gy, gz = grids(*nall, kind="tanh")
    n1, n2, n3 = (v - 2 for v in nall)
    bct = (2,) * 6
    sc_ref = S.Solver3D(gx, gy, gz, bct, 6)
    sc = mf.SolverCoeffs3D(gx, gy, gz, bct, 6)
    axes = (sc_ref.cx, sc_ref.cy, sc_ref.cz)
    for a, ax in enumerate(axes):
        sc.set_eigen(a, ax.eigen, ax.vect, ax.inv_vect)
    prec, sigma, B = mf.MF_PREC_3XTF32, -10.0, 5
    rhs = [field((n1, n2, n3), 140 + b) for b in range(B)]
    bcs = [bc_arrays(n1, n2, n3, 150 + b) for b in range(B)]
    solf0 = [field(nall, 160 + b) for b in range(B)]

    def many():
        outs = [np.asfortranarray(x.copy()) for x in solf0]
        sc.solve_3d_many(rhs, sigma, outs, [b[0] for b in bcs], [b[1] for b in bcs], [b[2] for b in bcs],
                         precision=prec, refine=1)
        return outs

    first = many()  # problems 1-3 capture the slots' graphs, 4 replays one
    e0 = np.array(axes[0].eigen, dtype=np.float64)
    k = int(np.argmin(np.abs(e0)))
    assert abs(e0[k]) < 1e-8
    e0[k] = 1e-3
    sc.set_eigen(0, e0, axes[0].vect, axes[0].inv_vect)
    second = many()
    for b in range(B):
        one = np.asfortranarray(solf0[b].copy())
        sc.solve_3d(rhs[b], sigma, one, *bcs[b], precision=prec, refine=1)
        assert np.array_equal(second[b], one), b
    assert not np.array_equal(first[0], second[0])


@pytest.mark.parametrize("prec_name,refine", [("MF_PREC_3XTF32", 1), ("MF_PREC_3XTF32", 2),
                                              ("MF_PREC_SPLIT_BF16", 2), ("MF_PREC_SPLIT_BF16", 3)])
@pytest.mark.parametrize("sigma", [0.0, -10.0])
def test_mixed_pure_neumann_pressure(mf, gpu, prec_name, refine, sigma):
    """All-Neumann operator (closed: a null mode at sigma = 0, the pressure
    equation; a near-null one at sigma = -10).  Its refinement residuals are
    formed in FP64, and at sigma = 0 the right-hand side's component along
    the null mode, which no iterate removes, is projected out of each one, so
    the refinement keeps converging.  The mean-free part and the whole field
    (at sigma = 0 the null mode's coefficient is zero in both) against the
    FP64 oracle."""
    nall = (42, 38, 34)
    gx, gy, gz = grids(*nall, kind="tanh")
    n1, n2, n3 = (v - 2 for v in nall)
    bct = (2,) * 6
    sc_ref = S.Solver3D(gx, gy, gz, bct, 6)
    sc = mf.SolverCoeffs3D(gx, gy, gz, bct, 6)
    rhs = field((n1, n2, n3), 31)
    rhs = np.asfortranarray(rhs - rhs.mean())
    bcx, bcy, bcz = (np.zeros_like(b) for b in bc_arrays(n1, n2, n3, 32))
    solf0 = np.zeros((n1 + 2, n2 + 2, n3 + 2), order="F")
    ref = S.solve_3d(sc_ref, rhs, sigma, solf0, bcx, bcy, bcz)
    got = mf.to_host(sc.solve_3d(mf.to_device(rhs), sigma, mf.to_device(solf0), mf.to_device(bcx),
                                 mf.to_device(bcy), mf.to_device(bcz), precision=getattr(mf, prec_name),
                                 refine=refine))
    r, g = ref[1:-1, 1:-1, 1:-1], got[1:-1, 1:-1, 1:-1]
    err, full = rel_l2(g - g.mean(), r - r.mean()), rel_l2(g, r)
    print("all-Neumann sigma %g %s refine %d: mean-free %.3e whole %.3e" % (sigma, prec_name, refine, err, full))
    assert err < 1e-10 and full < 1e-10


def test_error_after_staging_pinned_arrays(mf, gpu):
    """A solve refused after the caller's (pinned) host arrays were staged
    -- an unknown precision, checked by the solve itself -- returns its
    error only after the queued copies are done; the handle then solves
    normally, single and pipelined, with the same arrays."""
    import torch
    nall = (22, 20, 18)
    gx, gy, gz = grids(*nall, kind="tanh")
    n1, n2, n3 = (v - 2 for v in nall)
    sc = mf.SolverCoeffs3D(gx, gy, gz, (1,) * 6, 6)

    def pinned(a):
        t = torch.empty(a.size, dtype=torch.float64, pin_memory=True).numpy().reshape(a.shape, order="F")
        t[...] = a
        return t

    rhs = pinned(field((n1, n2, n3), 170))
    bcs = [pinned(b) for b in bc_arrays(n1, n2, n3, 171)]
    solf0 = field(nall, 172)
    out = pinned(solf0)
    with pytest.raises(mf.MflopsError) as e:
        sc.solve_3d(rhs, -2.0, out, *bcs, precision=99, refine=1)
    assert e.value.code == mf.MF_ERR_UNSUPPORTED
    with pytest.raises(mf.MflopsError):
        sc.solve_3d_many([rhs, rhs], -2.0, [out, out], [bcs[0]] * 2, [bcs[1]] * 2, [bcs[2]] * 2,
                         precision=99, refine=1)
    assert np.array_equal(out, solf0)  # nothing was written back
    sc.solve_3d(rhs, -2.0, out, *bcs, precision=mf.MF_PREC_3XTF32, refine=1)
    ref = np.asfortranarray(solf0.copy())
    mf.SolverCoeffs3D(gx, gy, gz, (1,) * 6, 6).solve_3d(np.array(rhs), -2.0, ref, *[np.array(b) for b in bcs],
                                                         precision=mf.MF_PREC_3XTF32, refine=1)
    assert np.array_equal(out, ref)
