"""Channel-flow statistics (post_prod.f90:40-238): the oracle's restatement
checked on a laminar profile with a known friction velocity and for the
symmetries it imposes (CPU); the GPU plane reductions against the oracle on
seeded turbulent-like snapshots (max |gpu - oracle| <= 1e-11 of each
profile's magnitude, u_tau to 1e-12)."""
import numpy as np
import pytest

from oracle import mesh
from oracle import stats as ST

from helpers import max_rel


def channel(nx, ny, nz, nt, seed, re=180.0):
    gx, gy, gz = mesh.uniform_grid(nx, 0.0, 4.0), mesh.tanh_grid(ny, 1.5), mesh.uniform_grid(nz, 0.0, 2.0)
    rng = np.random.default_rng(seed)
    Y = np.broadcast_to(gy[None, :, None], (nx, ny, nz))
    prof = 1.5 * (1.0 - (2.0 * Y - 1.0) ** 2)
    us, vs, ws, ps = [], [], [], []
    for _ in range(nt):
        wall = np.sin(np.pi * Y)
        us.append(np.asfortranarray(prof + 0.1 * wall * rng.standard_normal((nx, ny, nz))))
        vs.append(np.asfortranarray(0.05 * wall * rng.standard_normal((nx, ny, nz))))
        ws.append(np.asfortranarray(0.05 * wall * rng.standard_normal((nx, ny, nz))))
        ps.append(np.asfortranarray(0.02 * rng.standard_normal((nx, ny, nz))))
    return (us, vs, ws, ps), (gx, gy, gz), re


def test_oracle_laminar_profile():
    # u = 1.5 (1 - (2y - 1)^2): du/dy(0) = 6, u_tau = sqrt(6 / Re); no fluctuations
    nx, ny, nz = 6, 41, 5
    gx, gy, gz = mesh.uniform_grid(nx), mesh.tanh_grid(ny, 1.2), mesh.uniform_grid(nz)
    Y = np.broadcast_to(gy[None, :, None], (nx, ny, nz))
    u = np.asfortranarray(1.5 * (1.0 - (2.0 * Y - 1.0) ** 2))
    z = np.zeros((nx, ny, nz))
    out = ST.channel_stats([u], [z], [z], [z], gx, gy, gz, re=100.0)
    assert abs(out["utau"] - np.sqrt(6.0 / 100.0)) < 1e-9
    assert np.max(np.abs(out["moyu"] * out["utau"] - u[0, :, 0])) < 1e-12
    assert np.max(np.abs(out["rmsu"])) < 1e-10


def test_oracle_symmetries():
    f, g, re = channel(8, 21, 6, 2, 3)
    out = ST.channel_stats(*f, *g, re)
    for k in ("moyu", "moyw", "moyp", "rmsu", "rmsv", "rmsw", "rmsp", "rmsuw"):
        assert np.allclose(out[k], out[k][::-1], rtol=0, atol=1e-14)
    # odd profiles: the centre plane of an odd ny is left as computed
    # (the reference symmetrises j = 1..ny/2 only)
    c = 21 // 2
    for k in ("moyv", "rmsuv", "rmsvw"):
        odd = out[k] + out[k][::-1]
        odd[c] = 0.0
        assert np.max(np.abs(odd)) < 1e-14


@pytest.mark.gpu
@pytest.mark.parametrize("shape,nt", [((20, 33, 12), 3), ((9, 18, 7), 1)])
def test_gpu_stats_match_oracle(mf, gpu, shape, nt):
    f, g, re = channel(*shape, nt, 11)
    ref = ST.channel_stats(*f, *g, re)
    dev = [[mf.to_device(x) for x in comp] for comp in f]
    got = mf.channel_stats(*dev, *g, re)
    assert abs(got["utau"] - ref["utau"]) <= 1e-12 * ref["utau"]
    for k, v in ref.items():
        if k == "utau":
            continue
        assert max_rel(got[k], v) < 1e-11, k
