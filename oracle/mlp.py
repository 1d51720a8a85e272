"""Oracle of the learned LES coefficient (test infrastructure only).

No reference counterpart: the reference has only the plain models of
navier_LES (src/class_navier/class_navier_3D.f90:1225-1455), whose
Smagorinsky form nu = C Delta^2 sqrt(2 S:S) the network refines with a
pointwise C(x).  Everything here is FP64 NumPy, restating the library's
definitions so its FP32 kernels can be checked:

* ``features``       six invariants of g = grad(u) (S:S/G2, tr S^3/G2^1.5,
                     tr W^2 S/G2^1.5, tr W^2 S^2/G2^2, det g/G2^1.5, tr g/G2^0.5)
* ``forward``/``loss_and_grad``  6-64-64-1 ReLU network, loss
                     L = s/n sum (cscale net(x) b - nu)^2, backward pass by hand
* ``adam``           Adam (Kingma & Ba 2015) with bias correction
* ``sgs_target``     nu = -tau^d : S / (2 S:S), tau_ij = F(u_i u_j) - F(u_i) F(u_j)
* ``nu_mlp``         network coefficient inside the training range, plain
                     Smagorinsky outside, zero on the edge lines
"""
import numpy as np

from oracle import les as L

N_IN, N_H = 6, 64
W1, B1 = 0, N_H * N_IN
W2 = B1 + N_H
B2 = W2 + N_H * N_H
W3 = B2 + N_H
B3 = W3 + N_H
N_PARAMS = B3 + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[W1:B1].reshape(N_H, N_IN), p[B1:W2], p[W2:B2].reshape(N_H, N_H), p[B2:W3], p[W3:B3], p[B3])


def grad_tensor(du):
    """(..., 3, 3) array from du[i][j] = d u_i / d x_j."""
    return np.stack([np.stack([du[i][j] for j in range(3)], -1) for i in range(3)], -2)


def features(g):
    """g: (..., 3, 3) -> (features (..., 6), valid (...))."""
    g = np.asarray(g, dtype=np.float64)
    g2 = np.einsum('...ij,...ij', g, g)
    valid = (g2 > 1e-30) & (g2 < 1e30)
    g2s = np.where(valid, g2, 1.0)
    S = 0.5 * (g + np.swapaxes(g, -1, -2))
    W = 0.5 * (g - np.swapaxes(g, -1, -2))
    S2, W2 = S @ S, W @ W
    r = np.sqrt(g2s)
    f = np.stack([np.einsum('...ij,...ij', S, S) / g2s,
                  np.einsum('...ii', S2 @ S) / (g2s * r),
                  np.einsum('...ii', W2 @ S) / (g2s * r),
                  np.einsum('...ii', W2 @ S2) / (g2s * g2s),
                  np.linalg.det(g) / (g2s * r),
                  np.einsum('...ii', g) / r], -1)
    return np.where(valid[..., None], f, 0.0), valid


def strain_ss(g):
    ss = np.zeros(g.shape[:-2])
    for a in range(3):
        ss = ss + g[..., a, a] ** 2
        for b in range(a + 1, 3):
            ss = ss + 0.5 * (g[..., a, b] + g[..., b, a]) ** 2
    return ss


def delta2(gx, gy, gz):
    dx, dy, dz = L.spacing(gx), L.spacing(gy), L.spacing(gz)
    return (dx[:, None, None] ** 2 + dy[None, :, None] ** 2 + dz[None, None, :] ** 2) / 3.0


def forward(p, x):
    """x: (n, 6) standardised inputs -> (y (n,), cache)."""
    w1, b1, w2, b2, w3, b3 = unpack(p)
    a1 = x @ w1.T + b1
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ w2.T + b2
    h2 = np.maximum(a2, 0.0)
    return h2 @ w3 + b3, (x, a1, h1, a2, h2)


def standardise(X, mean, istd):
    return (np.asarray(X, dtype=np.float64) - mean) * istd


def loss_and_grad(p, X, base, target, mean, istd, cscale, loss_scale):
    """Loss and gradient over all rows of X (raw features)."""
    w1, b1, w2, b2, w3, b3 = unpack(p)
    x = standardise(X, mean, istd)
    y, (x, a1, h1, a2, h2) = forward(p, x)
    n = len(y)
    r = cscale * y * base - target
    loss = loss_scale / n * np.sum(r * r)
    dy = 2.0 * r * base * cscale * loss_scale / n
    g = np.zeros(N_PARAMS)
    g[W3:B3] = h2.T @ dy
    g[B3] = dy.sum()
    da2 = (dy[:, None] * w3[None, :]) * (a2 > 0)
    g[W2:B2] = (da2.T @ h1).ravel()
    g[B2:W3] = da2.sum(0)
    da1 = (da2 @ w2) * (a1 > 0)
    g[W1:B1] = (da1.T @ x).ravel()
    g[B1:W2] = da1.sum(0)
    return loss, g


def adam(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (step counts from 1); returns new (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v


def sgs_target(ub, uu, du):
    """ub[3], uu[6] (00,01,02,11,12,22) filtered fields, du[i][j] = d ub_i/dx_j."""
    g = grad_tensor(du)
    pairs = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    t = np.zeros(g.shape)
    for q, (a, b) in enumerate(pairs):
        t[..., a, b] = t[..., b, a] = uu[q] - ub[a] * ub[b]
    tr = np.einsum('...ii', t) / 3.0
    for a in range(3):
        t[..., a, a] -= tr
    S = 0.5 * (g + np.swapaxes(g, -1, -2))
    ss = strain_ss(g)
    with np.errstate(invalid='ignore', divide='ignore'):
        nu = np.where(ss > 1e-300, -np.einsum('...ij,...ij', t, S) / (2.0 * ss), 0.0)
    return L.zero_edges(nu)


def nu_mlp(p, du, gx, gy, gz, mean, istd, lo, hi, cscale, c_fallback):
    """Eddy viscosity with the network coefficient; returns (nu, fallback mask)."""
    du = [[L.zero_edges(du[i][j]) for j in range(3)] for i in range(3)]
    g = grad_tensor(du)
    shape = g.shape[:-2]
    f, valid = features(g)
    f32 = f.astype(np.float32).astype(np.float64)
    inside = valid & np.all((f32 >= lo) & (f32 <= hi), axis=-1)
    y, _ = forward(p, standardise(f32.reshape(-1, N_IN), mean, istd))
    c = np.where(inside, np.maximum(cscale * y.reshape(shape), 0.0), c_fallback)
    nu = c * np.sqrt(2.0 * strain_ss(g)) * delta2(gx, gy, gz)
    edge = L.zero_edges(np.ones(shape)) == 0
    return np.where(edge, 0.0, nu), (~inside) & (~edge)
