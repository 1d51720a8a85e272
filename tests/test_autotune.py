"""Launch-shape autotuner (mf_tune_*): CPU checks of the decision cache and
its text file; GPU checks that measured decisions are cached per shape and
that tuned calls give results identical to the heuristic ones (the
candidate launch shapes differ only in speed)."""
import numpy as np
import pytest

from oracle import mesh

from helpers import bc_arrays, field


def test_tune_cache_file_round_trip(mf, tmp_path):
    mf.tune(clear=True)
    path = tmp_path / "tune.txt"
    path.write_text("# decisions\n0 3969 63 63 1 1\n1 129 16641 1 0 0\n")
    mode, n = mf.tune(load=path)
    assert n == 2
    out = tmp_path / "out.txt"
    mf.tune(save=out)
    lines = [l for l in out.read_text().splitlines() if not l.startswith("#")]
    assert sorted(lines) == sorted(["0 3969 63 63 1 1", "1 129 16641 1 0 0"])
    mf.tune(clear=True)
    assert mf.tune()[1] == 0
    with pytest.raises(RuntimeError):
        mf.tune(mode=2)


@pytest.mark.gpu
def test_tuned_launches_match_heuristic_ones(mf, gpu, tmp_path):
    import torch
    mf.tune(mode=0, clear=True)
    results = {}
    for mode in (0, 1):
        mf.tune(mode=mode)
        outs = []
        for n in (33, 65):
            g = mesh.tanh_grid(n, 1.5)
            sc = mf.SolverCoeffs3D(g, g, g, (1,) * 6, 6)
            m = n - 2
            solf = mf.empty_device((n, n, n))
            sc.solve_3d(mf.to_device(field((m, m, m), 3)), -2.0, solf,
                        *[mf.to_device(b) for b in bc_arrays(m, m, m, 4)])
            outs.append(solf)
        gx = mesh.tanh_grid(129, 1.5)
        dc = mf.DerivativesCoefficients(gx, so=6)
        f = mf.to_device(field((129, 40, 9), 5))
        outs.append(dc.apply(0, 1, f))
        torch.cuda.synchronize()
        results[mode] = outs
    n_tuned = mf.tune()[1]
    assert n_tuned >= 3  # transform shapes of both sizes and the x sweep
    for a, b in zip(results[0], results[1]):
        assert torch.equal(a, b)
    path = tmp_path / "tune.txt"
    mf.tune(save=path)
    mf.tune(mode=0, clear=True)
    assert mf.tune(load=path)[1] == n_tuned
    mf.tune(mode=0, clear=True)
