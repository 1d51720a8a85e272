"""Pins the CPU oracle to the reference's analytic known-answer recipes.

* src/main/test_solver_3d.f90:31-111,218-258,310-361 -- x^9+y^9+x*y, sigma=2,
  Dirichlet on the reference arcsin grid; relative L2 error over interior +
  faces must fall at the scheme's order under grid refinement.
* src/main/test_derivatives.f90:135-206 -- convergence order of the compact
  first/second derivatives by grid doubling.
"""
import numpy as np
import pytest

from oracle import derivatives as D
from oracle import mesh
from oracle import solver as S


def poly_kat(n, bct=(1, 1, 1, 1, 1, 1), sigma=2.0, so=6):
    gx, gy, gz = mesh.arcsin_grid(n), mesh.arcsin_grid(n), mesh.arcsin_grid(n, -0.25, 0.25)
    sc = S.Solver3D(gx, gy, gz, bct, so)
    X, Y, Z = np.meshgrid(gx, gy, gz, indexing="ij")
    p = 9
    uex = X ** p + Y ** p + X * Y
    g = (p - 1) * p * X ** (p - 2) + (p - 1) * p * Y ** (p - 2) + sigma * uex
    dx = p * X ** (p - 1) + Y
    dy = p * Y ** (p - 1) + X
    dz = 0.0 * Z

    def face(a, axis, idx):
        sl = [slice(1, -1)] * 3
        sl[axis] = idx
        return a[tuple(sl)]

    def pick(t, val, der):
        return val if t == 1 else der

    bcx = np.stack([face(pick(bct[0], uex, dx), 0, 0), face(pick(bct[1], uex, dx), 0, -1)], -1)
    bcy = np.stack([face(pick(bct[2], uex, dy), 1, 0), face(pick(bct[3], uex, dy), 1, -1)], -1)
    bcz = np.stack([face(pick(bct[4], uex, dz), 2, 0), face(pick(bct[5], uex, dz), 2, -1)], -1)
    u = S.solver_3d(sc, g, np.zeros_like(uex), bcx, bcy, bcz, sigma)
    m = np.zeros(uex.shape, bool)
    m[1:-1, 1:-1, 1:-1] = True
    for a in range(3):
        for idx in (0, -1):
            sl = [slice(1, -1)] * 3
            sl[a] = idx
            m[tuple(sl)] = True
    return np.linalg.norm((u - uex)[m]) / np.linalg.norm(uex[m])


def test_solver_polynomial_kat_converges():
    errs = [poly_kat(n) for n in (17, 33)]
    assert errs[0] < 5e-6 and errs[1] < 1e-7
    order = np.log(errs[0] / errs[1]) / np.log(32.0 / 16.0)
    assert order > 5.0, (errs, order)


def test_solver_neumann_faces_kat():
    # Neumann on x2,y1,y2 and z (the commented variant at test_solver_3d.f90:56)
    e = poly_kat(25, bct=(1, 2, 2, 2, 2, 2))
    assert e < 1e-4


@pytest.mark.parametrize("so,order_min", [(4, 3.5), (6, 5.5), (8, 4.0)])
def test_derivative_order(so, order_min):
    errs = []
    for n in (101, 201):
        g = mesh.uniform_grid(n)
        dc = D.DerCoeffs(g, so)
        f = np.sin(2 * np.pi * 2 * g) + np.cos(2 * np.pi * 3 * g)
        d1 = 2 * np.pi * 2 * np.cos(2 * np.pi * 2 * g) - 2 * np.pi * 3 * np.sin(2 * np.pi * 3 * g)
        errs.append(np.linalg.norm(dc.der(f) - d1) / np.linalg.norm(d1))
    assert np.log(errs[0] / errs[1]) / np.log(200.0 / 100.0) > order_min


def test_residual_of_oracle_solution_is_small():
    n = 19
    gx, gy, gz = mesh.tanh_grid(n, 1.5), mesh.tanh_grid(n + 2, 1.5), mesh.tanh_grid(n - 2, 1.5)
    sc = S.Solver3D(gx, gy, gz, (1, 1, 2, 1, 1, 2), 6)
    rng = np.random.default_rng(0)
    n1, n2, n3 = n - 2, n, n - 4
    g = rng.normal(size=(n1, n2, n3))
    bcx = rng.normal(size=(n2, n3, 2))
    bcy = rng.normal(size=(n1, n3, 2))
    bcz = rng.normal(size=(n1, n2, 2))
    solf = S.solve_3d(sc, g, -3.0, np.zeros((n1 + 2, n2 + 2, n3 + 2)), bcx, bcy, bcz)
    r = S.residual(sc, g, solf[1:-1, 1:-1, 1:-1], -3.0, bcx, bcy, bcz)
    assert np.max(np.abs(r)) < 1e-9 * np.max(np.abs(g)) * 1e3
