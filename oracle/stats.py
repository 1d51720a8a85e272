"""Oracle of the channel-flow statistics (test infrastructure only).

Restates the post-processing of src/main/post_prod.f90:40-238 on in-memory
snapshots (the reference reads them from NetCDF files):

* mean profiles moy{u,v,w,p}(j) (:63-91): sums over the interior points
  i = 2..nx-1, k = 2..nz-1 (1-based) and all snapshots with the weight
  s = (x(i+1) - x(i-1)) (z(k+1) - z(k-1)); a point counts only where the
  first snapshot's u exceeds 1e-10 (a default-kind, single-precision literal)
  or j is a wall plane (j = 1, ny); n sums s once per snapshot;
* symmetrisation across the centre plane (:92-101): u, w, p even, v odd,
  for j = 1..ny/2 (integer division);
* u_tau = sqrt((du/dy(1) - du/dy(ny)) / 2 / Re) with du/dy the compact
  derivative of the mean u along y (:103-110);
* normalisation of the fields by u_tau (p by u_tau^2) (:112-122) and rms /
  cross-correlation profiles (:124-158) with the same weights, where the
  mask now tests the normalised first-snapshot u; rms values are square
  roots, the cross terms are not;
* symmetrisation (:159-174): rms u, v, w, p and uw as sqrt of the mean of
  squares, uv and vw odd.
"""
import numpy as np

from oracle import derivatives as D

THRESH = float(np.float32(1e-10))


def weights(gx, gz):
    dx = gx[2:] - gx[:-2]
    dz = gz[2:] - gz[:-2]
    return dx[:, None] * dz[None, :]  # interior (i, k)


def channel_stats(us, vs, ws, ps, gx, gy, gz, re, so=6):
    """us, ... : lists of (nx, ny, nz) snapshots.  Returns dict of profiles."""
    nt = len(us)
    nx, ny, nz = us[0].shape
    s = weights(np.asarray(gx, float), np.asarray(gz, float))
    inner = (slice(1, nx - 1), slice(None), slice(1, nz - 1))

    def mask_of(u1):
        m = u1[inner] > THRESH  # (nx-2, ny, nz-2)
        m[:, 0, :] = True
        m[:, ny - 1, :] = True
        return m

    def plane_sums(vals, m):
        # sum over (i, k) of s * vals, masked, for every j
        w = np.where(m, s[:, None, :], 0.0)
        return np.einsum('ijk,ijk->j', w, vals)

    m = mask_of(us[0])
    nsum = nt * np.einsum('ijk->j', np.where(m, s[:, None, :], 0.0))
    moy = {}
    for name, f in (("u", us), ("v", vs), ("w", ws), ("p", ps)):
        moy[name] = sum(plane_sums(x[inner], m) for x in f) / nsum
    for j in range(ny // 2):
        jj = ny - 1 - j
        for name, sign in (("u", 1), ("v", -1), ("w", 1), ("p", 1)):
            a = 0.5 * (moy[name][j] + sign * moy[name][jj])
            moy[name][j] = a
            moy[name][jj] = sign * a
    dc = D.DerCoeffs(np.asarray(gy, float), so)
    deru = D.derx(dc, moy["u"].reshape(ny, 1, 1)).ravel()
    utau = np.sqrt((deru[0] - deru[ny - 1]) * 0.5 / re)
    scale = {"u": utau, "v": utau, "w": utau, "p": utau * utau}
    fields = {"u": us, "v": vs, "w": ws, "p": ps}
    norm = {k: [x / scale[k] for x in fields[k]] for k in fields}
    moyn = {k: moy[k] / scale[k] for k in moy}
    m2 = mask_of(norm["u"][0])
    nsum2 = nt * np.einsum('ijk->j', np.where(m2, s[:, None, :], 0.0))
    dev = {k: [x[inner] - moyn[k][None, :, None] for x in norm[k]] for k in norm}
    rms = {}
    for name in ("u", "v", "w", "p"):
        rms[name] = np.sqrt(sum(plane_sums(d * d, m2) for d in dev[name]) / nsum2)
    for a, b in (("u", "v"), ("u", "w"), ("v", "w")):
        rms[a + b] = sum(plane_sums(x * y, m2) for x, y in zip(dev[a], dev[b])) / nsum2
    for j in range(ny // 2):
        jj = ny - 1 - j
        for name in ("u", "v", "w", "p", "uw"):
            a = np.sqrt((rms[name][j] ** 2 + rms[name][jj] ** 2) * 0.5)
            rms[name][j] = rms[name][jj] = a
        for name in ("uv", "vw"):
            a = (rms[name][j] - rms[name][jj]) * 0.5
            rms[name][j] = a
            rms[name][jj] = -a
    out = {"moy" + k: moyn[k] for k in moyn}
    out.update({"rms" + k: rms[k] for k in rms})
    out["utau"] = utau
    return out
