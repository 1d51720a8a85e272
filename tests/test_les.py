"""LES eddy viscosity (navier_LES / les_sigma, class_navier_3D.f90:1225-1502).

CPU: the oracle's models against closed forms (Smagorinsky on a uniform
strain, WALE zero in pure shear, sigma-model singular values against an SVD,
sigma model zero for two-component gradients).  GPU: the fused kernel on
random gradient fields and the whole velocity -> gradients -> nu chain
against the oracle.  Tolerance: max |a - b| <= 1e-12 * max |b| (1e-10 for
the sigma model, whose acos amplifies rounding near coincident singular
values)."""
import numpy as np
import pytest

from oracle import derivatives as D
from oracle import les as L

from helpers import field, grids, max_rel


def uniform_grad(G, shape):
    return [[np.full(shape, G[i, j]) for j in range(3)] for i in range(3)]


def test_oracle_smagorinsky_uniform_strain():
    shape = (6, 5, 7)
    G = np.array([[0.3, 0.1, -0.2], [0.4, -0.5, 0.0], [0.2, 0.7, 0.2]])
    gx, gy, gz = np.linspace(0, 1, 6), np.linspace(0, 2, 5), np.linspace(0, 3, 7)
    nu = L.les_nu(uniform_grad(G, shape), gx, gy, gz, 1, 0.17)
    S = 0.5 * (G + G.T)
    d2 = ((1 / 5) ** 2 + (2 / 4) ** 2 + (3 / 6) ** 2) / 3
    assert abs(nu[2, 2, 3] - 0.17 * np.sqrt(2 * np.sum(S * S)) * d2) < 1e-14
    assert nu[0, 0, 3] == 0.0 and nu[2, 0, 0] == 0.0 and nu[5, 2, 6] == 0.0
    assert nu[0, 2, 3] != 0.0  # faces keep their value, only edges are zeroed


def test_oracle_wale_zero_in_pure_shear():
    shape = (5, 5, 5)
    G = np.zeros((3, 3))
    G[0, 1] = 2.0
    g = np.linspace(0, 1, 5)
    assert np.all(L.les_nu(uniform_grad(G, shape), g, g, g, 2, 0.5) == 0.0)


def test_oracle_sigma_values_are_singular_values():
    rng = np.random.default_rng(4)
    A = rng.normal(size=(200, 3, 3))
    s1, s2, s3 = L.sigma_values(A)
    sv = np.linalg.svd(A, compute_uv=False)
    assert np.max(np.abs(np.stack([s1, s2, s3], -1) - sv)) < 1e-6 * np.max(sv)


def test_oracle_sigma_zero_for_two_component_flow():
    shape = (5, 5, 5)
    G = np.array([[0.3, 0.8, 0.0], [-0.4, -0.3, 0.0], [0.0, 0.0, 0.0]])
    g = np.linspace(0, 1, 5)
    nu = L.les_nu(uniform_grad(G, shape), g, g, g, 3, 1.0)
    assert np.max(np.abs(nu)) < 1e-7


def random_gradients(shape, seed):
    return [[field(shape, seed + 3 * i + j) for j in range(3)] for i in range(3)]


@pytest.mark.gpu
@pytest.mark.parametrize("les_type", [0, 1, 2, 3])
def test_les_nu_matches_oracle(mf, gpu, les_type):
    shape = (33, 20, 17)
    gx, gy, gz = grids(*shape, kind="tanh")
    du = random_gradients(shape, 11)
    ref = L.les_nu(du, gx, gy, gz, les_type, 0.1)
    les = mf.LesModel(gx, gy, gz)
    ddu = [[mf.to_device(du[i][j]) for j in range(3)] for i in range(3)]
    got = mf.to_host(les.nu(ddu, les_type, 0.1))
    if les_type == 0:
        assert np.all(got == 0.0)
        return
    tol = 1e-10 if les_type == 3 else 1e-12
    assert max_rel(got, ref) < tol


@pytest.mark.gpu
@pytest.mark.parametrize("les_type", [1, 2, 3])
def test_les_nu_from_velocity_matches_oracle(mf, gpu, les_type):
    shape = (40, 33, 24)
    gx, gy, gz = grids(*shape, kind="arcsin")
    x, y, z = np.meshgrid(gx, gy, gz, indexing="ij")
    vel = [np.asfortranarray(np.sin(2 * x + y) * np.cos(z) + 0.2 * np.cos(3 * y * z)),
           np.asfortranarray(np.cos(x - 2 * z) * np.sin(y)),
           np.asfortranarray(np.sin(x * y + z) + 0.1 * x * x)]
    dc = [D.DerCoeffs(g, so=6) for g in (gx, gy, gz)]
    ops = (D.derx, D.dery, D.derz)
    du = [[ops[j](dc[j], vel[i]) for j in range(3)] for i in range(3)]
    ref = L.les_nu(du, gx, gy, gz, les_type, 0.18)
    les = mf.LesModel(gx, gy, gz)
    dcs = [mf.DerivativesCoefficients(g, so=6) for g in (gx, gy, gz)]
    got = mf.to_host(les.nu_velocity(*dcs, *[mf.to_device(v) for v in vel], les_type, 0.18))
    tol = 1e-9 if les_type == 3 else 1e-11
    assert max_rel(got, ref) < tol
