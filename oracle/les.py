"""Oracle LES eddy viscosity (test infrastructure only).

Restates navier_LES (src/class_navier/class_navier_3D.f90:1225-1455) and
les_sigma (:1458-1502) in FP64 NumPy: from the nine velocity gradients
du[i][j] = d u_i / d x_j (edges zeroed, field_zero_edges :366-391) compute
  type 1 Smagorinsky  nu = C sqrt(2 S:S)
  type 2 WALE         nu = C (Sd:Sd)^(3/2) / ((S:S)^(5/2) + (Sd:Sd)^(5/4)), 0 if Sd:Sd < 1e-10
  type 3 sigma        nu = C s3 (s1 - s2)(s2 - s3) / s1^2, 0 if s1 < 1e-10
then multiply by Delta^2 = (dx^2 + dy^2 + dz^2)/3 (one-sided spacing at the
ends, centred inside) and zero the edges.  The reference's 1e-10 thresholds
are default-kind (single precision) literals.
"""
import numpy as np

THRESH = float(np.float32(1e-10))


def zero_edges(f):
    f = np.array(f, dtype=np.float64)
    f[0, 0, :] = f[-1, 0, :] = f[0, -1, :] = f[-1, -1, :] = 0.0
    f[0, :, 0] = f[-1, :, 0] = f[0, :, -1] = f[-1, :, -1] = 0.0
    f[:, 0, 0] = f[:, -1, 0] = f[:, 0, -1] = f[:, -1, -1] = 0.0
    return f


def spacing(g):
    g = np.asarray(g, dtype=np.float64)
    d = np.empty_like(g)
    d[0] = g[1] - g[0]
    d[-1] = g[-1] - g[-2]
    d[1:-1] = (g[2:] - g[:-2]) * 0.5
    return d


def sigma_values(g2):
    """les_sigma for a (..., 3, 3) array of gradient tensors."""
    pi = 4.0 * np.arctan(1.0)
    g = np.einsum('...ik,...jk->...ij', g2, g2)
    i1 = g[..., 0, 0] + g[..., 1, 1] + g[..., 2, 2]
    i2 = (g[..., 0, 0] * g[..., 1, 1] + g[..., 0, 0] * g[..., 2, 2] + g[..., 1, 1] * g[..., 2, 2]
          - g[..., 0, 1] * g[..., 1, 0] - g[..., 0, 2] * g[..., 2, 0] - g[..., 1, 2] * g[..., 2, 1])
    i3 = (g[..., 0, 0] * g[..., 1, 1] * g[..., 2, 2] + g[..., 1, 0] * g[..., 2, 1] * g[..., 0, 2]
          + g[..., 2, 0] * g[..., 0, 1] * g[..., 1, 2] - g[..., 0, 2] * g[..., 1, 1] * g[..., 2, 0]
          - g[..., 1, 2] * g[..., 2, 1] * g[..., 0, 0] - g[..., 2, 2] * g[..., 0, 1] * g[..., 1, 0])
    a1 = i1 ** 2 / 9.0 - i2 / 3.0
    a2 = i1 ** 3 / 27.0 - i1 * i2 / 6.0 + i3 / 2.0
    with np.errstate(invalid='ignore', divide='ignore'):
        a3 = np.where(a1 < THRESH, 0.0, np.arccos(a2 / np.maximum(a1, 1e-300) ** 1.5) / 3.0)
    s1 = i1 / 3.0 + 2.0 * np.sqrt(np.maximum(a1, 0)) * np.cos(a3)
    s2 = i1 / 3.0 - 2.0 * np.sqrt(np.maximum(a1, 0)) * np.cos(a3 + pi / 3.0)
    s3 = i1 - s1 - s2
    return (np.sqrt(np.maximum(s1, 0.0)), np.sqrt(np.maximum(s2, 0.0)), np.sqrt(np.maximum(s3, 0.0)))


def les_nu(du, gx, gy, gz, les_type, c):
    """du: 3x3 nested list of (nx,ny,nz) arrays, du[i][j] = d u_i / d x_j."""
    du = [[zero_edges(du[i][j]) for j in range(3)] for i in range(3)]
    shape = du[0][0].shape
    if les_type == 0:
        return np.zeros(shape)
    if les_type in (1, 2):
        ss = np.zeros(shape)
        for i in range(3):
            ss = ss + du[i][i] ** 2
            for j in range(i + 1, 3):
                ss = ss + 0.5 * (du[i][j] + du[j][i]) ** 2
        if les_type == 1:
            nu = c * np.sqrt(2.0 * ss)
        else:
            sd = np.zeros(shape)
            trg2 = sum(du[m][k] * du[k][m] for m in range(3) for k in range(3))
            for i in range(3):
                for j in range(3):
                    a = np.zeros(shape)
                    for k in range(3):
                        a = a + 0.5 * (du[i][k] * du[k][j] + du[j][k] * du[k][i])
                    if i == j:
                        a = a - trg2 / 3.0
                    sd = sd + a ** 2
            with np.errstate(invalid='ignore', divide='ignore'):
                nu = np.where(sd < THRESH, 0.0,
                              c * sd ** 1.5 / (ss ** 2.5 + sd ** 1.25))
    else:
        g2 = np.stack([np.stack([du[i][j] for j in range(3)], -1) for i in range(3)], -2)
        s1, s2, s3 = sigma_values(g2)
        with np.errstate(invalid='ignore', divide='ignore'):
            nu = np.where(s1 < THRESH, 0.0, c * s3 * (s1 - s2) * (s2 - s3) / s1 ** 2)
    dx, dy, dz = spacing(gx), spacing(gy), spacing(gz)
    delta2 = (dx[:, None, None] ** 2 + dy[None, :, None] ** 2 + dz[None, None, :] ** 2) / 3.0
    return zero_edges(nu * delta2)
