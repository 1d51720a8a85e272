"""Shared test helpers: seeded fields, boundary data, error norms."""
import numpy as np

from oracle import mesh


def rng(seed):
    return np.random.default_rng(seed)


def field(shape, seed, lo=-1.0, hi=1.0):
    return np.asfortranarray(rng(seed).uniform(lo, hi, size=shape))


def max_rel(a, b, mask=None):
    a = np.asarray(a)
    b = np.asarray(b)
    if mask is not None:
        a = a[mask]
        b = b[mask]
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale)


def rel_l2(a, b):
    return float(np.linalg.norm((np.asarray(a) - np.asarray(b)).ravel()) /
                 max(np.linalg.norm(np.asarray(b).ravel()), 1e-300))


def grids(nx, ny, nz, kind="tanh", alpha=1.5):
    if kind == "tanh":
        return (mesh.tanh_grid(nx, alpha), mesh.tanh_grid(ny, alpha), mesh.tanh_grid(nz, alpha))
    if kind == "arcsin":
        return (mesh.arcsin_grid(nx), mesh.arcsin_grid(ny), mesh.arcsin_grid(nz, -0.25, 0.25))
    return (mesh.uniform_grid(nx), mesh.uniform_grid(ny), mesh.uniform_grid(nz))


def bc_arrays(n1, n2, n3, seed):
    r = rng(seed)
    return (np.asfortranarray(r.uniform(-1, 1, (n2, n3, 2))),
            np.asfortranarray(r.uniform(-1, 1, (n1, n3, 2))),
            np.asfortranarray(r.uniform(-1, 1, (n1, n2, 2))))


def solf_mask(n1, n2, n3):
    """Interior + 6 faces of solf(0:n1+1,...) (edges/corners are not written)."""
    m = np.zeros((n1 + 2, n2 + 2, n3 + 2), dtype=bool)
    m[1:-1, 1:-1, 1:-1] = True
    m[0, 1:-1, 1:-1] = m[-1, 1:-1, 1:-1] = True
    m[1:-1, 0, 1:-1] = m[1:-1, -1, 1:-1] = True
    m[1:-1, 1:-1, 0] = m[1:-1, 1:-1, -1] = True
    return m
