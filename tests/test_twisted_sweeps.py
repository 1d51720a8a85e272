"""CPU check of the algebra of the two-lane refinement residual (no GPU).

The residual's sweeps solve T y = S with T = L U, L unit lower bidiagonal
(sub-diagonal ft), U unit upper bidiagonal (super-diagonal dt):
x_i = S_i - ft_i x_{i-1}, y_i = x_i - dt_i y_{i+1}.  The two-lane form keeps
those sweeps on rows 0..m and runs the U L elimination of the same T from the
bottom on rows n-1..m+1 (pivots q_i, gt_i = T_{i,i+1}/q_i, et_i = T_{i,i-1}/q_i,
right-hand side S_i/q_i), then joins the halves at the twist:
y_m = tw (x_m - dt_m z_{m+1}), y_{m+1} = tw (z_{m+1} - et_{m+1} x_m),
tw = 1 / (1 - dt_m et_{m+1}).  This restates the table construction of the
solver's set-up and the kernel's arithmetic in NumPy and checks them against
the one-sided sweeps and a dense solve.
"""
import numpy as np
import pytest


def one_sided(ft, dt, S):
    n = len(S)
    x = np.empty(n)
    x[0] = S[0]
    for i in range(1, n):
        x[i] = S[i] - ft[i] * x[i - 1]
    y = np.empty(n)
    y[-1] = x[-1]
    for i in range(n - 2, -1, -1):
        y[i] = x[i] - dt[i] * y[i + 1]
    return y


def bottom_table(ft, dt):
    """Mirrored bottom table: entry k = row n-1-k with (scale 1/q, gt, et)."""
    n = len(ft)
    m = (n - 1) // 2
    tdiag = lambda i: 1.0 + (ft[i] * dt[i - 1] if i > 0 else 0.0)
    q = np.ones(n)
    q[n - 1] = tdiag(n - 1)
    for i in range(n - 2, m, -1):
        q[i] = tdiag(i) - dt[i] * ft[i + 1] / q[i + 1]
    cb = n - 1 - m
    scale, gt, et = np.empty(cb), np.empty(cb), np.empty(cb)
    for k in range(cb):
        i = n - 1 - k
        scale[k] = 1.0 / q[i]
        gt[k] = dt[i] / q[i]
        et[k] = ft[i] / q[i]
    tw = 1.0 / (1.0 - dt[m] * et[cb - 1])
    return m, scale, gt, et, tw


def two_sided(ft, dt, S):
    n = len(S)
    m, scale, gt, et, tw = bottom_table(ft, dt)
    cb = n - 1 - m
    # top lane: rows 0..m
    x = np.empty(m + 1)
    x[0] = S[0]
    for i in range(1, m + 1):
        x[i] = S[i] - ft[i] * x[i - 1]
    # bottom lane, mirrored: entry k = row n-1-k
    z = np.empty(cb)
    z[0] = S[n - 1] * scale[0]
    for k in range(1, cb):
        z[k] = S[n - 1 - k] * scale[k] - gt[k] * z[k - 1]
    # the twist: each lane combines its last value with its partner's
    y = np.empty(n)
    y[m] = tw * (x[m] - dt[m] * z[cb - 1])
    y[m + 1] = tw * (z[cb - 1] - et[cb - 1] * x[m])
    for i in range(m - 1, -1, -1):
        y[i] = x[i] - dt[i] * y[i + 1]
    for k in range(cb - 2, -1, -1):
        y[n - 1 - k] = z[k] - et[k] * y[n - 2 - k]
    return y


@pytest.mark.parametrize("n", [8, 9, 10, 17, 64, 127, 255, 256])
def test_two_sided_sweeps_equal_one_sided(n):
    rng = np.random.default_rng(n)
    # factors of a diagonally dominant operator, as the compact scheme's
    ft = rng.uniform(-0.45, 0.45, n)
    dt = rng.uniform(-0.45, 0.45, n)
    ft[0] = 0.0
    dt[-1] = 0.0
    S = rng.standard_normal(n) * 1e3
    y1 = one_sided(ft, dt, S)
    y2 = two_sided(ft, dt, S)
    T = np.eye(n) + np.diag(ft[1:], -1) + np.diag(dt[:-1], 1)
    T[np.arange(1, n), np.arange(1, n)] += ft[1:] * dt[:-1]
    y3 = np.linalg.solve(T, S)
    scale = np.abs(y3).max()
    assert np.abs(y1 - y3).max() < 1e-12 * scale
    assert np.abs(y2 - y3).max() < 1e-12 * scale
    assert np.abs(y2 - y1).max() < 1e-12 * scale


def test_halves_cover_the_line():
    for n in range(8, 300):
        m = (n - 1) // 2
        top, bottom = m + 1, n - 1 - m
        assert top + bottom == n and 0 <= top - bottom <= 1 and bottom >= 4
