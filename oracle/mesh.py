"""Oracle 1D grids (test infrastructure only; see ``oracle/__init__.py``).

``arcsin_grid`` follows ``src/class_mesh/class_mesh.f90:137-200`` (the grid
the reference generates: beta = 33.3, alpha = 1 - beta/n^2).
``tanh_grid`` follows the commented formula at ``class_mesh.f90:203``:
x = xa + (xb-xa) * (1 + tanh(a*(2*(xi-xa)/(xb-xa) - 1)) / tanh(a)) / 2.
"""
import numpy as np


def uniform_grid(n, xa=0.0, xb=1.0):
    pas = (xb - xa) / float(n - 1)
    return xa + np.arange(n, dtype=np.float64) * pas


def arcsin_grid(n, xa=-0.5, xb=0.5, beta=33.3):
    """Reference default grid, ``class_mesh.f90:181-200``."""
    pi = 4.0 * np.arctan(1.0)
    pas = (xb - xa) / float(n - 1)
    alpha = 1.0 - beta / float(n * n)
    xi = xa + np.arange(n, dtype=np.float64) * pas
    return xa + (xb - xa) * (np.arcsin(-alpha * np.cos(pi * (xi - xa) / (xb - xa)))
                             / np.arcsin(alpha) + 1.0) * 0.5


def tanh_grid(n, alpha, xa=0.0, xb=1.0):
    """Commented tanh stretching of ``class_mesh.f90:203``."""
    if alpha == 0.0:
        return uniform_grid(n, xa, xb)
    pas = (xb - xa) / float(n - 1)
    xi = xa + np.arange(n, dtype=np.float64) * pas
    return xa + (xb - xa) * (1.0 + np.tanh(alpha * (2.0 * (xi - xa) / (xb - xa) - 1.0))
                             / np.tanh(alpha)) / 2.0
