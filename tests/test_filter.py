"""Least-squares B-spline filter (class_filter.f90:104-347).

CPU: the oracle restatement of FITPACK's fixed-knot fits is pinned against
SciPy's FITPACK (the same Dierckx library the reference vendors), and the
library's host operators against the oracle.  GPU: batched application
along each axis of a 3D field and the reference-signature pencil forms.
Tolerance: max |a - b| <= 1e-12 * max |b|."""
import numpy as np
import pytest

from oracle import filter as F
from oracle import mesh

from helpers import max_rel


def lsq_case(ni=97, nn=25, no=49, k=3, seed=0):
    rng = np.random.default_rng(seed)
    xi = mesh.tanh_grid(ni, 1.5)
    wi = 0.5 + rng.random(ni)
    xn = mesh.tanh_grid(nn, 1.0)
    xo = mesh.tanh_grid(no, 0.7)
    return xi, wi, xn, xo, k


@pytest.mark.parametrize("k", [3, 5])
def test_oracle_lsq_matches_scipy_fitpack(k):
    si = pytest.importorskip("scipy.interpolate")
    xi, wi, xn, xo, _ = lsq_case(k=k)
    yi = np.sin(6 * xi) + 0.1 * np.random.default_rng(1).normal(size=xi.size)
    yo, ypo = F.lsq_univariate_spline(xi, yi, wi, xn, xo, k)
    s = si.LSQUnivariateSpline(xi, yi, xn[1:-1], w=wi, k=k)
    assert max_rel(yo, s(xo)) < 1e-13
    assert max_rel(ypo, s.derivative()(xo)) < 1e-13


def test_oracle_periodic_matches_scipy_fitpack():
    si = pytest.importorskip("scipy.interpolate")
    ni = 96
    xi = np.linspace(0, 2 * np.pi, ni)
    yi = np.sin(3 * xi) + 0.3 * np.cos(7 * xi)
    yi[-1] = yi[0]
    xos = mesh.tanh_grid(40, 1.2, 0, 2 * np.pi)
    yos, _, _, _ = F.interp_period(xi, yi, xos)
    nn = ni - 6
    xn = (xi[-1] - xi[0]) * np.arange(nn) / (nn - 1)
    tck = si.splrep(xi, yi, k=5, task=-1, t=xn[1:-1], per=1)
    assert max_rel(yos, si.splev(xos, tck)) < 1e-13


@pytest.mark.parametrize("k", [1, 3, 5])
def test_lsq_operator_matches_oracle(mf, k):
    xi, wi, xn, xo, _ = lsq_case(k=k)
    P, Pd = mf.filter_lsq_matrix(xi, wi, xn, xo, k)
    rng = np.random.default_rng(3)
    for _ in range(3):
        yi = rng.normal(size=xi.size)
        yo, ypo = F.lsq_univariate_spline(xi, yi, wi, xn, xo, k)
        assert max_rel(P @ yi, yo) < 1e-12
        assert max_rel(Pd @ yi, ypo) < 1e-12


def test_periodic_operator_matches_oracle(mf):
    ni = 64
    xi = np.linspace(0, 1.0, ni)
    xos = mesh.tanh_grid(33, 1.0)
    P, Pd = mf.filter_period_matrix(xi, xos)
    rng = np.random.default_rng(4)
    yi = rng.normal(size=ni)
    yos, ypos, _, _ = F.interp_period(xi, yi, xos)
    assert max_rel(P @ yi, yos) < 1e-12
    assert max_rel(Pd @ yi, ypos) < 1e-12


def test_filter_errors(mf):
    xi = np.linspace(0, 1, 20)
    with pytest.raises(mf.MflopsError) as e:
        mf.filter_lsq_matrix(xi[::-1].copy(), None, np.linspace(0, 1, 5), xi, 3)
    assert e.value.code == mf.MF_ERR_ARG
    with pytest.raises(mf.MflopsError):
        mf.filter_period_matrix(np.linspace(0, 1, 8), xi)


@pytest.mark.gpu
@pytest.mark.parametrize("axis,k", [(0, 3), (1, 3), (2, 3), (0, 1), (2, 2), (0, 4), (1, 5)])
def test_filter_apply_along_axes(mf, gpu, axis, k):
    # fine field 3 axes, filtered along one axis onto a coarse grid (the
    # banded kernel is instantiated per spline degree)
    shape = [21, 19, 17]
    ni, no, nn = 65, 33, 17
    shape[axis] = ni
    xi = mesh.tanh_grid(ni, 1.5)
    xn = mesh.tanh_grid(nn, 1.0)
    xo = mesh.tanh_grid(no, 1.5)
    wi = np.ones(ni)
    f = np.asfortranarray(np.random.default_rng(5).normal(size=shape))
    flt = mf.SplineFilter(xi, xo, xn=xn, wi=wi, k=k)
    got = mf.to_host(flt.apply(mf.to_device(f), axis))
    gotd = mf.to_host(flt.apply(mf.to_device(f), axis, deriv=True))
    g = np.moveaxis(f, axis, 0)
    want = np.zeros((no,) + g.shape[1:])
    wantd = np.zeros_like(want)
    for a in range(g.shape[1]):
        for b in range(g.shape[2]):
            want[:, a, b], wantd[:, a, b] = F.lsq_univariate_spline(xi, g[:, a, b], wi, xn, xo, k)
    assert max_rel(got, np.moveaxis(want, 0, axis)) < 1e-12
    assert max_rel(gotd, np.moveaxis(wantd, 0, axis)) < 1e-12


@pytest.mark.gpu
def test_filter_pencil_forms(mf, gpu):
    xi, wi, xn, xo, k = lsq_case(k=5)
    yi = np.cos(4 * xi)
    yo, ypo = mf.lsq_univariate_spline(xi, yi, wi, xn, xo, k)
    ryo, rypo = F.lsq_univariate_spline(xi, yi, wi, xn, xo, k)
    assert max_rel(yo, ryo) < 1e-12 and max_rel(ypo, rypo) < 1e-12
    ni = 80
    xp = np.linspace(0, 2.0, ni)
    yp = np.sin(np.pi * xp) + 0.2 * np.cos(5 * np.pi * xp)
    xos = mesh.tanh_grid(31, 0.8, 0, 2.0)
    ref, _, _, _ = F.interp_period(xp, yp, xos)
    assert max_rel(mf.interp_period(xp, yp, xos), ref) < 1e-12
