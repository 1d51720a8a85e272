"""1D grids of class_mesh (mf_grid1d, mf_grid_spacing, mf_mesh_grid_init)
against the oracle's restatement (oracle/mesh.py) -- host only, no GPU.

The formulas are evaluated in the same operation order on both sides; the
transcendental functions (tanh, cos, asin) come from different libraries
(the C library here, NumPy's loops in the oracle), so the bar is 2 ulp of
the interval length rather than bit equality (measured: identical or 1 ulp).
"""
import numpy as np
import pytest

from oracle import mesh


def _ulps(a, b, scale):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / (np.finfo(float).eps * scale))


@pytest.mark.parametrize("n,alpha", [(65, 1.5), (257, 2.0), (97, 0.0), (9, 3.0)])
def test_tanh_grid(mf, n, alpha):
    got = mf.grid1d(mf.MF_GRID_TANH, n, 0.0, 1.0, alpha)
    assert _ulps(got, mesh.tanh_grid(n, alpha), 1.0) <= 2
    assert got[0] == 0.0 and abs(got[-1] - 1.0) <= 2e-16
    assert np.all(np.diff(got) > 0)


@pytest.mark.parametrize("n,xa,xb", [(65, -0.5, 0.5), (129, -0.25, 0.25), (33, 0.0, 2.0)])
def test_arcsin_grid(mf, n, xa, xb):
    got = mf.grid1d(mf.MF_GRID_ARCSIN, n, xa, xb, 33.3)
    assert _ulps(got, mesh.arcsin_grid(n, xa, xb, 33.3), xb - xa) <= 2


def test_uniform_grid(mf):
    got = mf.grid1d(mf.MF_GRID_UNIFORM, 128, 0.0, 2 * np.pi)
    assert np.array_equal(got, mesh.uniform_grid(128, 0.0, 2 * np.pi))


@pytest.mark.parametrize("choice,coord,nd,xa,xb", [("x", 0, 1, -0.5, 0.5), ("y", 1, 2, 0.0, 0.5),
                                                   ("z", 0, 2, -0.25, 0.0), ("z", 2, 3, 0.25 / 3, 0.25)])
def test_mesh_grid_init_subdomains(mf, choice, coord, nd, xa, xb):
    """mesh_grid_init's interval per direction and its slab per subdomain
    (class_mesh.f90:137-170), the arcsin grid on the slab and dgrid1d."""
    g, d = mf.mesh_grid_init(choice, 49, coord, nd)
    assert _ulps(g, mesh.arcsin_grid(49, xa, xb, 33.3), 1.0) <= 4
    want_d = np.empty(49)
    want_d[0] = g[1] - g[0]
    want_d[-1] = g[-1] - g[-2]
    want_d[1:-1] = (g[2:] - g[:-2]) * 0.5
    assert np.array_equal(d, want_d)


def test_mesh_arguments(mf):
    with pytest.raises(mf.MflopsError) as e:
        mf.mesh_grid_init("w", 33)
    assert e.value.code == mf.MF_ERR_ARG
    with pytest.raises(mf.MflopsError) as e:
        mf.mesh_grid_init("x", 33, 2, 2)
    assert e.value.code == mf.MF_ERR_ARG
    with pytest.raises(mf.MflopsError):
        mf.grid1d(mf.MF_GRID_ARCSIN, 2, 0.0, 1.0, 33.3)
