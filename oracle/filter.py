"""Oracle least-squares B-spline filter (test infrastructure only).

Restates the reachable parts of the reference's spline filter:

* ``lsq_univariate_spline``  LSQUnivariateSpline, src/class_filter/class_filter.f90:104-174:
  knots = (k+1)*xb, xn(2:nn-1), (k+1)*xe; weighted least-squares fit with fixed
  knots (FITPACK curfit with iopt=-1 -> fpcurf: rows of the observation matrix
  from fpbspl, Givens rotations fpgivs/fprota into the band triangle, fpback),
  then splev (values) and splder (first derivative) at xo.
* ``interp_period``  interp_period, class_filter.f90:267-347: periodic quintic
  least-squares spline (FITPACK percur with iopt=-1 -> fpperi) with
  nn = ni-k-1 equispaced nodes xn(i) = (xi(ni)-xi(1))*(i-1)/(nn-1) (the
  reference does not add xi(1)), evaluated with splev at xos.

The algorithms are P. Dierckx's published ones ("Curve and Surface Fitting
with Splines", 1993), restated here; the vendored FITPACK sources are not used.
The periodic fit is restated from its mathematical definition (periodic
spline space, least squares) rather than fpperi's rotation order.
"""
import numpy as np


def bspline_row(t, k, x, l):
    """The k+1 non-zero B-splines of degree k at x, t[l] <= x < t[l+1]
    (0-based l), de Boor-Cox recursion (FITPACK fpbspl)."""
    h = np.zeros(k + 1)
    h[0] = 1.0
    hh = np.zeros(k + 1)
    for j in range(1, k + 1):
        hh[:j] = h[:j]
        h[0] = 0.0
        for i in range(j):
            li = l + i + 1
            lj = li - j
            f = hh[i] / (t[li] - t[lj])
            h[i] = h[i] + f * (t[li] - x)
            h[i + 1] = f * (x - t[lj])
    return h


def knot_interval(t, k, n, x):
    """l with t[l] <= x < t[l+1], clamped to [k, n-k-2] (0-based)."""
    l = k
    while x >= t[l + 1] and l != n - k - 2:
        l += 1
    return l


def givens(piv, ww):
    """FITPACK fpgivs: rotation making piv zero against ww."""
    store = abs(piv)
    if store >= ww:
        dd = store * np.sqrt(1.0 + (ww / piv) ** 2)
    else:
        dd = ww * np.sqrt(1.0 + (piv / ww) ** 2)
    cos = ww / dd
    sin = piv / dd
    return dd, cos, sin


def lsq_fit(xi, yi, wi, t, k):
    """Coefficients of the weighted least-squares spline with knots t
    (fpcurf with iopt=-1): minimise sum (w_i (y_i - s(x_i)))^2."""
    n = t.size
    nk1 = n - k - 1
    k1 = k + 1
    a = np.zeros((nk1, k1))
    z = np.zeros(nk1)
    for it in range(xi.size):
        w = wi[it]
        x = xi[it]
        yw = yi[it] * w
        l = knot_interval(t, k, n, x)
        h = bspline_row(t, k, x, l) * w
        j = l - k  # first coefficient index of the row
        for i in range(k1):
            piv = h[i]
            if piv == 0.0:
                j += 1
                continue
            a[j, 0], cos, sin = givens(piv, a[j, 0])
            # rotate the right-hand side and the rest of the row
            yw, z[j] = cos * yw - sin * z[j], sin * yw + cos * z[j]
            if i < k:
                i2 = 1
                for i1 in range(i + 1, k1):
                    h[i1], a[j, i2] = cos * h[i1] - sin * a[j, i2], sin * h[i1] + cos * a[j, i2]
                    i2 += 1
            j += 1
    # back substitution (fpback): a is upper triangular with bandwidth k1
    c = np.zeros(nk1)
    for i in range(nk1 - 1, -1, -1):
        s = z[i]
        for m in range(1, k1):
            if i + m < nk1:
                s -= a[i, m] * c[i + m]
        c[i] = s / a[i, 0]
    return c


def splev(t, c, k, x, nu=0):
    """Values (nu=0) or first derivatives (nu=1) of the spline (splev / splder)."""
    n = t.size
    out = np.zeros(np.size(x))
    for p, xv in enumerate(np.atleast_1d(x)):
        l = knot_interval(t, k, n, xv)
        if nu == 0:
            h = bspline_row(t, k, xv, l)
            out[p] = np.dot(h, c[l - k:l + 1])
        else:
            # derivative: spline of degree k-1 with coefficients k*(c_i - c_{i-1})/(t_{i+k} - t_i)
            h = bspline_row(t[1:-1], k - 1, xv, l - 1)
            d = np.zeros(k)
            for i in range(k):
                ii = l - k + 1 + i
                d[i] = k * (c[ii] - c[ii - 1]) / (t[ii + k] - t[ii])
            out[p] = np.dot(h, d)
    return out


def lsq_knots(xi, xn, k):
    """Knot vector of LSQUnivariateSpline (class_filter.f90:147-153)."""
    xb, xe = xi[0], xi[-1]
    return np.concatenate([np.full(k + 1, xb), np.asarray(xn)[1:-1], np.full(k + 1, xe)])


def lsq_univariate_spline(xi, yi, wi, xn, xo, k):
    """LSQUnivariateSpline(ni,xi,yi,wi,nn,xn,no,xo,yo,ypo,k) -> (yo, ypo)."""
    xi = np.asarray(xi, dtype=np.float64)
    t = lsq_knots(xi, xn, k)
    c = lsq_fit(xi, np.asarray(yi, dtype=np.float64), np.asarray(wi, dtype=np.float64), t, k)
    return splev(t, c, k, xo, 0), splev(t, c, k, xo, 1)


# ---------------------------------------------------------------------------
# periodic fit (percur, iopt=-1)
# ---------------------------------------------------------------------------

def periodic_knots(xi, k, interior):
    """Periodic knot vector: t[k] = xb, t[n-k-1] = xe, the k outer knots on
    each side are the interior ones shifted by the period (fpperi)."""
    xb, xe = xi[0], xi[-1]
    per = xe - xb
    inner = np.concatenate([[xb], np.asarray(interior), [xe]])
    n = inner.size + 2 * k
    t = np.zeros(n)
    t[k:n - k] = inner
    for j in range(1, k + 1):
        t[k - j] = t[n - k - 1 - j] - per
        t[n - k - 1 + j] = t[k + j] + per
    return t


def periodic_design(xi, t, k):
    """Observation matrix on the n-2k-1 free coefficients of the periodic
    spline space (c_{i + n-2k-1} = c_i, i < k); the last data point only
    defines the period and is not fitted (percur)."""
    n = t.size
    nfree = n - 2 * k - 1
    rows = []
    for x in xi[:-1]:
        l = knot_interval(t, k, n, x)
        h = bspline_row(t, k, x, l)
        r = np.zeros(nfree)
        for i in range(k + 1):
            r[(l - k + i) % nfree] += h[i]
        rows.append(r)
    return np.array(rows)


def periodic_fit(xi, yi, wi, t, k):
    n = t.size
    nfree = n - 2 * k - 1
    A = periodic_design(xi, t, k) * np.asarray(wi)[:-1, None]
    b = np.asarray(yi)[:-1] * np.asarray(wi)[:-1]
    q, r = np.linalg.qr(A)
    free = np.linalg.solve(r, q.T @ b)
    return np.concatenate([free, free[:n - k - 1 - nfree]])


def interp_period(xi, yi, xos, k=5):
    """interp_period(ni,xi,yi,nos,xos,yos): periodic quintic LSQ spline with
    nn = ni-k-1 equispaced nodes, evaluated at xos."""
    xi = np.asarray(xi, dtype=np.float64)
    ni = xi.size
    nn = ni - k - 1
    xn = (xi[-1] - xi[0]) * np.arange(nn, dtype=np.float64) / float(nn - 1)
    t = periodic_knots(xi, k, xn[1:-1])
    c = periodic_fit(xi, np.asarray(yi, dtype=np.float64), np.ones(ni), t, k)
    return splev(t, c, k, xos, 0), splev(t, c, k, xos, 1), t, c
