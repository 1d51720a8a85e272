"""CUDA-graph capture of the device-pointer entry points.

With device pointers the solve, derivative and LES calls neither
synchronise the host nor allocate once their work buffers exist (a first
call before capture creates them), so a whole step can be captured into one
CUDA graph and replayed.  Checked here: a plain FP64 solve, a mixed 3xTF32
solve with one refinement, and one step made of the LES viscosity from the
velocity (nine derivative sweeps + model), three Helmholtz solves and a
Poisson solve, each replayed from a graph and compared with the same calls
made eagerly (identical kernels and inputs, so the results are bit-identical).
"""
import numpy as np
import pytest

from oracle import mesh

from helpers import bc_arrays, field

pytestmark = pytest.mark.gpu


def capture(torch, fn, warm=1):
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s, capture_error_mode="relaxed"):
            fn()
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    return g


@pytest.mark.parametrize("precision,refine", [(0, -1), (2, 1)])
def test_solve_replays_from_a_graph(mf, gpu, precision, refine):
    import torch
    n = 33
    g = mesh.tanh_grid(n, 1.5)
    sc = mf.SolverCoeffs3D(g, g, g, (1,) * 6, 6)
    m = n - 2
    rhs = mf.to_device(field((m, m, m), 3))
    bcs = [mf.to_device(b) for b in bc_arrays(m, m, m, 4)]
    eager = mf.empty_device((n, n, n))
    sc.solve_3d(rhs, -2.0, eager, *bcs, precision=precision, refine=refine)
    torch.cuda.synchronize()
    out = mf.empty_device((n, n, n))
    graph = capture(torch, lambda: sc.solve_3d(rhs, -2.0, out, *bcs, precision=precision, refine=refine))
    out.zero_()
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(out, eager)
    # new right-hand side in the captured buffer: the replay follows it
    rhs.copy_(mf.to_device(field((m, m, m), 5)))
    sc.solve_3d(rhs, -2.0, eager, *bcs, precision=precision, refine=refine)
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(out, eager)


def test_les_and_five_solves_step_replays_from_a_graph(mf, gpu):
    import torch
    n = 33
    g = mesh.tanh_grid(n, 1.5)
    m = n - 2
    dc = mf.DerivativesCoefficients(g, so=6)
    les = mf.LesModel(g, g, g)
    vel = [mf.to_device(field((n, n, n), 10 + q)) for q in range(3)]
    sc_u = mf.SolverCoeffs3D(g, g, g, (1,) * 6, 6)
    sc_p = mf.SolverCoeffs3D(g, g, g, (2,) * 6, 6)
    rhs = [mf.to_device(field((m, m, m), 20 + q)) for q in range(4)]
    bcs = [mf.to_device(b) for b in bc_arrays(m, m, m, 30)]
    zbc = [torch.zeros_like(b) for b in bcs]

    def step(outs, nu):
        les.nu_velocity(dc, dc, dc, *vel, 1, 0.17, out=nu)
        for q in range(3):
            sc_u.solve_3d(rhs[q], -1e3, outs[q], *bcs, precision=2, refine=1)
        sc_p.solve_3d(rhs[3], -1e-3, outs[3], *zbc)
        # pressure at sigma = 0 through the mixed path: FP64 refinement
        # residuals, null-mode projection and removal
        sc_p.solve_3d(rhs[3], 0.0, outs[4], *zbc, precision=mf.MF_PREC_3XTF32, refine=2)

    eager = [mf.empty_device((n, n, n)) for _ in range(5)]
    nu_e = mf.empty_device((n, n, n))
    step(eager, nu_e)
    torch.cuda.synchronize()
    outs = [mf.empty_device((n, n, n)) for _ in range(5)]
    nu = mf.empty_device((n, n, n))
    graph = capture(torch, lambda: step(outs, nu))
    for o in outs + [nu]:
        o.zero_()
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(nu, nu_e)
    for a, b in zip(outs, eager):
        assert torch.equal(a, b)


def test_multidomain_solve_replays_from_a_graph(mf, gpu):
    import torch
    nd = (2, 2, 1)
    grids = [[mesh.tanh_grid(11, 1.0, 0.0, 0.5), mesh.tanh_grid(13, 1.0, 0.5, 1.0)],
             [mesh.tanh_grid(12, 1.0, 0.0, 0.5), mesh.tanh_grid(10, 1.0, 0.5, 1.0)],
             [mesh.tanh_grid(11, 1.0)]]
    md = mf.MultiDomain(nd, (0, 0, 0), *grids, (1,) * 6)
    md.influence_matrix_set(-5.0)
    subs = md.subdomains()
    g = {c: mf.to_device(field(md.shape(*c), 50 + i)) for i, c in enumerate(subs)}
    bc = {}
    for i, c in enumerate(subs):
        nx, ny, nz = md.shape(*c)
        bc[c] = [mf.to_device(b) for b in bc_arrays(nx - 2, ny - 2, nz - 2, 70 + i)]
    eager = {c: mf.empty_device(md.shape(*c)) for c in subs}
    md.solve(g, eager, bc)
    torch.cuda.synchronize()
    out = {c: mf.empty_device(md.shape(*c)) for c in subs}
    graph = capture(torch, lambda: md.solve(g, out, bc))
    for c in subs:
        out[c].zero_()
    graph.replay()
    torch.cuda.synchronize()
    for c in subs:
        assert torch.equal(out[c], eager[c])
