"""Oracle compact finite-difference derivatives (test infrastructure only).

Restates, in FP64 NumPy:

* ``der_coeffs_generic``     src/class_derivatives/class_derivatives_coefficient.f90:53-212
* ``der_coeffs_global``      src/class_derivatives/class_derivatives.f90:330-377 (``der_coeffs_generic_gobal``)
* ``pentalu``                class_derivatives.f90:379-423
* ``pentares``               class_derivatives.f90:425-466 (vectorised over pencils)
* ``derx_rhs``               class_derivatives.f90:262-295
* ``DerCoeffs``              type + ``der_coeffs_init`` class_derivatives.f90:30-45,111-184
* ``der/der_s/dder/dder_s``  class_derivatives.f90:186-260
* field drivers ``derx .. dderz``  src/class_field/class_field.f90:629-978

Arrays are NumPy arrays indexed like the Fortran ones, 0-based:
``f[i, j, k]`` with shape (nx, ny, nz).  Pencil routines act along axis 0 of
an array of shape (n, ...), vectorised over the trailing axes.
"""
import numpy as np

# (n1 implicit, n2 explicit) stencil sizes, class_derivatives_coefficient.f90:68-127
_STENCIL = {
    1: {8: (3, 6), 6: (1, 6), 4: (1, 4), 2: (0, 3)},
    2: {8: (1, 5), 6: (2, 6), 4: (1, 5), 2: (0, 3)},
    3: {8: (4, 5), 6: (2, 5), 4: (2, 3), 2: (0, 3)},
}


def cshift(a, shift):
    """Fortran CSHIFT: result(i) = a(i + shift) (circular)."""
    return np.roll(np.asarray(a), -shift)


def taylor_matrix(h, n1, nt, der):
    """Taylor-matching matrix shared by both coefficient modules
    (class_derivatives_coefficient.f90:150-168)."""
    a = np.zeros((nt, nt))
    # implicit columns: row der+1 = -1, then a(i,j) = a(i-1,j)*h(j)/(i-der-1)
    a[der, :n1] = -1.0
    for i in range(der + 1, nt):
        for j in range(n1):
            a[i, j] = a[i - 1, j] * h[j] / float(i - der)
    # explicit columns: row 1 = 1, then a(i,j) = a(i-1,j)*h(j)/(i-1)
    a[0, n1:nt] = 1.0
    for i in range(1, nt):
        for j in range(n1, nt):
            a[i, j] = a[i - 1, j] * h[j] / float(i)
    return a


def der_coeffs_generic(h0, cl, der, so):
    """Coefficients of one row of the compact scheme.

    h0: 7 offsets grid(i) - grid(stencil); cl: 1 edge, 2 near edge, 3 interior;
    der: derivative order.  Returns (coef_imp[5], coef_exp[7]).
    """
    h0 = np.asarray(h0, dtype=np.float64)
    n1, n2 = _STENCIL[cl][so]
    nt = n1 + n2
    h = np.zeros(10)
    if cl == 1:
        h[0:n1] = h0[1:n1 + 1]
        h[n1:nt] = h0[0:n2]
    elif cl == 2:
        h[0] = h0[0]
        if n1 >= 2:
            h[1:n1] = h0[2:n1 + 1]
        h[n1:nt] = h0[0:n2]
    else:
        s = (4 - n1) // 2
        h[0:2] = h0[s:2 + s]
        if n1 >= 3 - s:
            h[2 - s:n1] = h0[3:n1 + 1 + s]
        s2 = (5 - n2) // 2
        h[n1:nt] = h0[s2:n2 + s2]
    a = taylor_matrix(h, n1, nt, der)
    r = np.zeros(nt)
    r[der] = 1.0
    r = np.linalg.solve(a, r)  # LAPACK gesv, as dgesv at :180

    coef_imp = np.zeros(5)
    coef_exp = np.zeros(7)
    k = (4 - n1) // 2 if cl == 3 else 0
    l = n1 + 1 if n1 + k >= cl else n1
    j = 0
    for i in range(1, l + 1):
        if i != cl - k:
            coef_imp[i + k - 1] = r[j]
            j += 1
    coef_imp[cl - 1] = 1.0
    s = (5 - n2) // 2 if cl == 3 else 0
    coef_exp[s:n2 + s] = r[n1:nt]
    return coef_imp, coef_exp


def der_coeffs_global(grid, der, so):
    """Assemble dl(n,5), dr(n,7) for a full line (class_derivatives.f90:330-377)."""
    grid = np.asarray(grid, dtype=np.float64)
    n = grid.size
    dl = np.zeros((n, 5))
    dr = np.zeros((n, 7))
    ci, ce = der_coeffs_generic(grid[0] - grid[0:7], 1, der, so)
    dl[0] = cshift(ci, -2)
    dr[0] = -ce
    ci, ce = der_coeffs_generic(grid[1] - grid[0:7], 2, der, so)
    dl[1] = cshift(ci, -1)
    dr[1] = -ce
    for i in range(2, n - 2):
        h = np.zeros(7)
        h[0:5] = grid[i] - grid[i - 2:i + 3]
        ci, ce = der_coeffs_generic(h, 3, der, so)
        dl[i] = ci
        dr[i] = -ce
    rev = grid[n - 1:n - 8:-1] if n > 7 else grid[::-1][:7]
    ci, ce = der_coeffs_generic(grid[n - 2] - rev, 2, der, so)
    dl[n - 2] = cshift(ci[::-1], 1)
    dr[n - 2] = -ce[::-1]
    ci, ce = der_coeffs_generic(grid[n - 1] - rev, 1, der, so)
    dl[n - 1] = cshift(ci[::-1], 2)
    dr[n - 1] = -ce[::-1]
    if der == 2:
        dr = -dr
    return dl, dr


def pentalu(dl):
    """In-place quasi-pentadiagonal LU (class_derivatives.f90:379-423).

    Columns of dl are (p, f, c, d, e); alpha = p(1) is the (1,4) entry and
    beta = e(n) the (n, n-3) entry.  Returns the factored copy.
    """
    dl = np.array(dl, dtype=np.float64)
    n = dl.shape[0]
    p, f, c, d, e = (dl[:, m] for m in range(5))  # views
    alpha = dl[0, 0]
    # step 1
    f[1] = f[1] / c[0]
    c[1] = c[1] - d[0] * f[1]
    d[1] = d[1] - e[0] * f[1]
    e[1] = e[1] - alpha * f[1]
    # step 2
    i = 2
    p[i] = p[i] / c[i - 2]
    f[i] = (f[i] - p[i] * d[i - 2]) / c[i - 1]
    c[i] = c[i] - d[i - 1] * f[i] - e[i - 2] * p[i]
    d[i] = d[i] - e[i - 1] * f[i] - alpha * p[i]
    for i in range(3, n - 1):
        p[i] = p[i] / c[i - 2]
        f[i] = (f[i] - p[i] * d[i - 2]) / c[i - 1]
        c[i] = c[i] - e[i - 2] * p[i] - d[i - 1] * f[i]
        d[i] = d[i] - e[i - 1] * f[i]
    # step 3 (beta aliases e(n))
    beta = e[n - 1] / c[n - 4]
    e[n - 1] = beta
    p[n - 1] = p[n - 1] - beta * d[n - 4]
    f[n - 1] = f[n - 1] - beta * e[n - 4]
    p[n - 1] = p[n - 1] / c[n - 3]
    f[n - 1] = (f[n - 1] - p[n - 1] * d[n - 3]) / c[n - 2]
    c[n - 1] = c[n - 1] - e[n - 3] * p[n - 1] - d[n - 2] * f[n - 1]
    return dl


def pentares(dlf, b):
    """Forward/back substitution with a factored quasi-penta matrix
    (class_derivatives.f90:425-466), vectorised over trailing axes of b."""
    n = dlf.shape[0]
    p, f, c, d, e = (dlf[:, m] for m in range(5))
    alpha = dlf[0, 0]
    beta = dlf[n - 1, 4]
    x = np.empty_like(b)
    x[0] = b[0]
    x[1] = b[1] - x[0] * f[1]
    for i in range(2, n - 1):
        x[i] = b[i] - p[i] * x[i - 2] - f[i] * x[i - 1]
    i = n - 1
    x[i] = b[i] - p[i] * x[i - 2] - f[i] * x[i - 1] - beta * x[i - 3]
    x[n - 1] = x[n - 1] / c[n - 1]
    x[n - 2] = (x[n - 2] - d[n - 2] * x[n - 1]) / c[n - 2]
    for i in range(n - 3, 0, -1):
        x[i] = (x[i] - e[i] * x[i + 2] - d[i] * x[i + 1]) / c[i]
    x[0] = (x[0] - e[0] * x[2] - d[0] * x[1] - alpha * x[3]) / c[0]
    return x


def derx_rhs(dr, f):
    """Explicit right-hand side (class_derivatives.f90:262-295), along axis 0."""
    n = dr.shape[0]
    sh = (slice(None),) + (None,) * (f.ndim - 1)
    rhs = np.empty_like(f)
    rhs[0] = sum(dr[0, m] * f[m] for m in range(7))
    rhs[1] = sum(dr[1, m] * f[m] for m in range(7))
    acc = dr[2:n - 2, 0][sh] * f[0:n - 4]
    for m in range(1, 5):
        acc = acc + dr[2:n - 2, m][sh] * f[m:n - 4 + m]
    rhs[2:n - 2] = acc
    rhs[n - 2] = sum(dr[n - 2, m] * f[n - 7 + m] for m in range(7))
    rhs[n - 1] = sum(dr[n - 1, m] * f[n - 7 + m] for m in range(7))
    return rhs


class DerCoeffs:
    """``type(derivatives_coefficients)`` + ``der_coeffs_init``
    (class_derivatives.f90:30-45,111-184)."""

    def __init__(self, grid, so=6, solver=False):
        grid = np.asarray(grid, dtype=np.float64)
        self.n = grid.size
        self.so = so
        self.solver = bool(solver)
        self.dl_raw, self.dr = der_coeffs_global(grid, 1, so)
        self.dl = pentalu(self.dl_raw)
        self.ddl_raw, self.ddr = der_coeffs_global(grid, 2, so)
        self.ddl = pentalu(self.ddl_raw)
        if self.solver:
            self.n_s = self.n - 2
            self.dl_s_raw, self.dr_s = der_coeffs_global(grid[1:-1], 1, so)
            self.dl_s = pentalu(self.dl_s_raw)
            self.ddl_s_raw, self.ddr_s = der_coeffs_global(grid[1:-1], 2, so)
            self.ddl_s = pentalu(self.ddl_s_raw)

    def dertype(self):
        return self.solver

    # pencil operations along axis 0 -------------------------------------
    def der(self, x):
        return pentares(self.dl, derx_rhs(self.dr, x))

    def dder(self, x):
        return pentares(self.ddl, derx_rhs(self.ddr, x))

    def der_s(self, x):
        """Acts on x(2:n-1); out(1), out(n) are undefined in the reference
        (OMP-private ``out`` at class_field.f90:647-652) and set to 0 here."""
        out = np.zeros_like(x)
        out[1:-1] = pentares(self.dl_s, derx_rhs(self.dr_s, x[1:-1]))
        return out

    def dder_s(self, x):
        out = np.zeros_like(x)
        out[1:-1] = pentares(self.ddl_s, derx_rhs(self.ddr_s, x[1:-1]))
        return out


def _field_apply(dc, f, axis, order):
    """Pencil driver for derx..dderz (class_field.f90:629-978).

    With ``dertype(dc)`` the pencils lying on the two boundary faces
    orthogonal to the other axes use the ``_s`` variant, and the 4 corner
    lines are left at 0 (``field_init`` zeroes the result, :475)."""
    f = np.asarray(f, dtype=np.float64)
    g = np.moveaxis(f, axis, 0)
    plain = dc.der if order == 1 else dc.dder
    out = plain(g)
    if dc.dertype():
        sub = dc.der_s if order == 1 else dc.dder_s
        s = sub(g)
        # g has shape (n, a, b): boundary lines are a in {0,-1} or b in {0,-1}
        res = np.zeros_like(g)
        res[:, 1:-1, 1:-1] = out[:, 1:-1, 1:-1]
        res[:, 0, 1:-1] = s[:, 0, 1:-1]
        res[:, -1, 1:-1] = s[:, -1, 1:-1]
        res[:, 1:-1, 0] = s[:, 1:-1, 0]
        res[:, 1:-1, -1] = s[:, 1:-1, -1]
        out = res
    return np.ascontiguousarray(np.moveaxis(out, 0, axis))


def derx(dc, f):
    return _field_apply(dc, f, 0, 1)


def dery(dc, f):
    return _field_apply(dc, f, 1, 1)


def derz(dc, f):
    return _field_apply(dc, f, 2, 1)


def dderx(dc, f):
    return _field_apply(dc, f, 0, 2)


def ddery(dc, f):
    return _field_apply(dc, f, 1, 2)


def dderz(dc, f):
    return _field_apply(dc, f, 2, 2)
