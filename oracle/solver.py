"""Oracle matrix-diagonalisation Poisson/Helmholtz solver (test infrastructure only).

Restates, in FP64 NumPy/SciPy:

* ``der_coeffs_generic_bc``  src/class_solver/class_solver_coefficient_3d.f90:30-245
* ``dder_coeffs``            src/class_solver/class_solver_3d.f90:568-619
* ``solver_matrix_init``     class_solver_3d.f90:468-566 (LAPACK dgeev via scipy)
* ``extrapolation_coeffs``   class_solver_3d.f90:622-656
* ``SolverAxis/Solver3D``    types + ``solver_coeffs_init(_3d)`` class_solver_3d.f90:28-50,380-466
* ``solve_3d``               class_solver_3d.f90:83-299 (+ dgx/dgy/dgz :307-378,
                             extrapolation_neum_{x,y,z} :658-776)
* ``solver_3d``              src/class_field/class_field.f90:1072-1109

Boundary types ``bct``: 1 Dirichlet, 2 Neumann, 3 second derivative.
"""
import numpy as np
import scipy.linalg

from .derivatives import cshift, taylor_matrix, pentalu

# (n1, n2) per (cl, so[, bct]) -- class_solver_coefficient_3d.f90:57-167
_CL1 = {8: (3, 6), 6: (1, 6), 4: (1, 4), 2: (0, 3)}
_CL4 = {8: (0, 7), 6: (0, 7), 4: (0, 5), 2: (0, 3)}
_CL2 = {8: {1: (1, 5), 2: (1, 5), 3: (2, 7)},
        6: {1: (1, 5), 2: (1, 5), 3: (1, 3)},
        4: {1: (1, 5), 2: (1, 5), 3: (1, 3)},
        2: {1: (0, 3), 2: (0, 3), 3: (0, 3)}}
_CL3 = {8: (4, 5), 6: (2, 5), 4: (2, 3), 2: (0, 3)}


def der_coeffs_generic_bc(h0, cl, der, bct, so):
    """Row coefficients with boundary type; returns (coef_imp[5], coef_exp[8])."""
    h0 = np.asarray(h0, dtype=np.float64)
    h = np.zeros(10)
    if cl == 1:
        n1, n2 = _CL1[so]
        n3 = n1 + n2
        h[0:n1] = h0[2:n1 + 2]
        h[n1:n3] = h0[0:n2]
    elif cl == 4:
        n1, n2 = _CL4[so]
        n3 = n1 + n2
        h[0:n3] = h0[0:n3]
    elif cl == 2:
        n1, n2 = _CL2[so][bct]
        n3 = n1 + n2
        h[0] = h0[1]
        if n1 >= 2:
            h[1:n1] = h0[3:n1 + 2]
        s = max(0, int((5 - n2) / 2))  # Fortran integer division truncates
        h[n1:n3] = h0[s:n2 + s]
    else:
        n1, n2 = _CL3[so]
        n3 = n1 + n2
        s = (4 - n1) // 2
        h[0:2] = h0[s:2 + s]
        if n1 >= 3 - s:
            h[2 - s:n1] = h0[3:n1 + 1 + s]
        s2 = (5 - n2) // 2
        h[n1:n3] = h0[s2:n2 + s2]
    a = taylor_matrix(h, n1, n3, der)
    # boundary column (class_solver_coefficient_3d.f90:195-203)
    if (cl == 2 and n2 > 4) or cl == 1:
        a[0:bct - 1, n1] = 0.0
        a[bct - 1, n1] = -1.0 if bct == 3 else 1.0
        for i in range(bct, n3):
            a[i, n1] = a[i - 1, n1] * h[n1] / float(i + 1 - bct)
    r = np.zeros(n3)
    r[der] = 1.0
    r = np.linalg.solve(a, r)

    coef_imp = np.zeros(5)
    coef_exp = np.zeros(8)
    k = (4 - n1) // 2 if cl == 3 else 0
    l = n1 + 1 if n1 + k >= cl else n1
    j = 0
    for i in range(1, l + 1):
        if i != cl - k:
            coef_imp[i + k - 1] = r[j]
            j += 1
    if cl <= 5:
        coef_imp[cl - 1] = 1.0
    s = 0
    if cl == 3:
        s = (5 - n2) // 2
    if cl == 2:
        s = max(0, int((5 - n2) / 2))
    coef_exp[s:n2 + s] = r[n1:n3]
    return coef_imp, coef_exp


def dder_coeffs(grid, bct, so):
    """ddl(n,5), ddr(n,8) for the n = nall-2 interior rows (class_solver_3d.f90:568-619).

    grid has nall = n + 2 points (grid(0:n+1) in the reference)."""
    g = np.asarray(grid, dtype=np.float64)
    n = g.size - 2
    ddl = np.zeros((n, 5))
    ddr = np.zeros((n, 8))
    ci, ce = der_coeffs_generic_bc(g[1] - g[0:7], 1, 2, bct[0], so)
    ddl[0] = cshift(ci, -2)
    ddr[0] = -ce
    if bct[0] == 2:
        ddr[0, 0] = -ddr[0, 0]
    ci, ce = der_coeffs_generic_bc(g[2] - g[0:7], 2, 2, bct[0], so)
    ddl[1] = cshift(ci, -1)
    ddr[1] = -ce
    if bct[0] == 2:
        ddr[1, 0] = -ddr[1, 0]
    for i in range(3, n - 1):  # Fortran rows 3..n-2 (grid index i)
        h = np.zeros(7)
        h[0:5] = g[i] - g[i - 2:i + 3]
        ci, ce = der_coeffs_generic_bc(h, 3, 2, 0, so)
        ddl[i - 1] = ci
        ddr[i - 1] = -ce
    rev = g[n + 1:n - 6:-1] if n - 6 >= 0 else g[n + 1::-1][:7]
    ci, ce = der_coeffs_generic_bc(g[n - 1] - rev, 2, 2, bct[1], so)
    ddl[n - 2] = cshift(ci[::-1], 1)
    ddr[n - 2] = -ce[::-1]
    if bct[1] == 2:
        ddr[n - 2, 7] = -ddr[n - 2, 7]
    ci, ce = der_coeffs_generic_bc(g[n] - rev, 1, 2, bct[1], so)
    ddl[n - 1] = cshift(ci[::-1], 2)
    ddr[n - 1] = -cshift(ce[::-1], 1)
    if bct[1] == 2:
        ddr[n - 1, 6] = -ddr[n - 1, 6]
    ddr = -ddr
    return ddl, ddr


def lhs_rhs_matrices(ddl, ddr):
    """Dense lhs and rhs of the interior operator (class_solver_3d.f90:484-521)."""
    n = ddl.shape[0]
    lhs = np.zeros((n, n))
    rhs = np.zeros((n, n))
    lhs[0, 0:3] = ddl[0, 2:5]
    lhs[0, 3] = ddl[0, 0]
    lhs[1, 0:4] = ddl[1, 1:5]
    for i in range(2, n - 2):
        lhs[i, i - 2:i + 3] = ddl[i, 0:5]
    lhs[n - 2, n - 4:n] = ddl[n - 2, 0:4]
    lhs[n - 1, n - 4] = ddl[n - 1, 4]
    lhs[n - 1, n - 3:n] = ddl[n - 1, 0:3]
    rhs[0, 0:6] = ddr[0, 1:7]
    rhs[1, 0:7] = ddr[1, 1:8]
    for i in range(2, n - 2):
        rhs[i, i - 2:i + 3] = ddr[i, 0:5]
    rhs[n - 2, n - 7:n] = ddr[n - 2, 0:7]
    rhs[n - 1, n - 6:n] = ddr[n - 1, 0:6]
    return lhs, rhs


class EigenError(RuntimeError):
    """Complex eigenvalues (the reference stops at class_solver_3d.f90:537-540)."""


def solver_matrix_init(ddl, ddr):
    lhs, rhs = lhs_rhs_matrices(ddl, ddr)
    inv_lhs = np.linalg.inv(lhs)
    temp = inv_lhs @ rhs
    w, vr = scipy.linalg.eig(temp)
    if np.max(np.abs(w.imag)) > 1e-13:
        raise EigenError("complex eigenvalues: max |imag| = %g" % np.max(np.abs(w.imag)))
    wr = w.real.copy()
    vr = vr.real.copy()
    inv_vect = np.linalg.inv(vr)
    return inv_lhs, wr, vr, inv_vect


def extrapolation_coeffs(grid, bct, so):
    """neum(2,7) (class_solver_3d.f90:622-656); always first derivative."""
    g = np.asarray(grid, dtype=np.float64)
    n = g.size - 2
    neum = np.zeros((2, 7))
    _, ce = der_coeffs_generic_bc(g[0] - g[0:7], 4, 1, bct[0], so)
    neum[0] = -ce[0:7]
    rev = g[n + 1:n - 6:-1] if n - 6 >= 0 else g[n + 1::-1][:7]
    _, ce = der_coeffs_generic_bc(g[n + 1] - rev, 4, 1, bct[1], so)
    neum[1] = -ce[6::-1]
    return neum


class SolverAxis:
    """``type(solver_coeffs)`` for one direction (class_solver_3d.f90:28-44,413-466)."""

    def __init__(self, grid, bct, so=6):
        grid = np.asarray(grid, dtype=np.float64)
        self.nall = grid.size
        self.n = grid.size - 2
        self.so = so
        self.bc = (int(bct[0]), int(bct[1]))
        self.ddl, self.ddr = dder_coeffs(grid, self.bc, so)
        self.inv_lhs, self.eigen, self.vect, self.inv_vect = solver_matrix_init(self.ddl, self.ddr)
        self.neum = extrapolation_coeffs(grid, self.bc, so)
        # quasi-penta factor of the lhs (used by the FP64 residual oracle)
        self.ddl_lu = pentalu(self.ddl)


class Solver3D:
    """``type(solver_coeffs_3d)`` + ``solver_coeffs_init_3d`` (class_solver_3d.f90:47-50,380-411).

    The reference stores the y/z eigenvector matrices transposed; here all
    three are kept untransposed and the transforms use the matching einsum."""

    def __init__(self, gx, gy, gz, bct, so=6):
        self.cx = SolverAxis(gx, bct[0:2], so)
        self.cy = SolverAxis(gy, bct[2:4], so)
        self.cz = SolverAxis(gz, bct[4:6], so)


def _fold_rows(ax, bc_t):
    """The four boundary columns ddr(1,1), ddr(2,1), ddr(n-1,8), ddr(n,7)
    times the boundary values (class_solver_3d.f90:113-116); bc_t is the
    C-ordered view (2, b, a) of a Fortran bc(a, b, 2) array.  Returns the
    (4, a*b) rows and the matching (n, 4) columns of inv_lhs."""
    n = ax.n
    coef = (ax.ddr[0, 0], ax.ddr[1, 0], ax.ddr[n - 2, 7], ax.ddr[n - 1, 6])
    side = (0, 0, 1, 1)
    rows = np.stack([coef[c] * bc_t[side[c]].reshape(-1) for c in range(4)])
    cols = ax.inv_lhs[:, [0, 1, n - 2, n - 1]]
    return rows, cols


def fold_bc(sc, rhs, bcx, bcy, bcz):
    """rhs minus inv_lhs(:,{1,2,n-1,n}) * (ddr_bc * bc) along x, y and z
    (class_solver_3d.f90:104-175).  Works on the C-ordered (n3,n2,n1) view of
    the Fortran array; returns a Fortran-ordered result."""
    R = np.array(np.asarray(rhs, dtype=np.float64).T, order='C')  # (n3, n2, n1)
    n3, n2, n1 = R.shape
    rows, cols = _fold_rows(sc.cx, np.asarray(bcx).T)            # rows: (4, n3*n2)
    R -= (rows.T @ cols.T).reshape(n3, n2, n1)
    rows, cols = _fold_rows(sc.cy, np.asarray(bcy).T)            # rows: (4, n3*n1)
    R -= np.matmul(cols, rows.reshape(4, n3, n1).transpose(1, 0, 2))
    rows, cols = _fold_rows(sc.cz, np.asarray(bcz).T)            # rows: (4, n2*n1)
    R -= (cols @ rows).reshape(n3, n2, n1)
    return R.T


def transform(sc, u, which):
    """Apply inv_vect ('inv') or vect ('fwd') along x, then y, then z
    (dgx/dgy/dgz, class_solver_3d.f90:307-378), as BLAS products on the
    C-ordered (n3,n2,n1) view of the Fortran array."""
    mats = [getattr(c, 'inv_vect' if which == 'inv' else 'vect') for c in (sc.cx, sc.cy, sc.cz)]
    U = np.ascontiguousarray(np.asarray(u).T)                     # (n3, n2, n1)
    n3, n2, n1 = U.shape
    U = (U.reshape(n3 * n2, n1) @ mats[0].T).reshape(n3, n2, n1)  # x: c = V1 b
    U = np.matmul(mats[1], U)                                     # y: per k-plane
    U = (mats[2] @ U.reshape(n3, n2 * n1)).reshape(n3, n2, n1)    # z
    return U.T


def eigen_divide(sc, aux, sigma):
    """sol = aux/(lx+ly+lz+sigma), 0 where max(|sigma|,|l|) < 1e-11 (class_solver_3d.f90:202-225).
    The reference's threshold is the default-kind literal 1e-11."""
    thresh = float(np.float32(1e-11))
    A = np.asarray(aux).T                                         # (n3, n2, n1)
    out = np.empty(A.shape)
    lx, ly, lz = sc.cx.eigen, sc.cy.eigen, sc.cz.eigen
    lxy = lx[None, :] + ly[:, None]                               # (n2, n1): lx(i)+ly(j)
    bxy = np.maximum(np.maximum(abs(sigma), np.abs(lx))[None, :], np.abs(ly)[:, None])
    for k in range(A.shape[0]):
        den = (lxy + lz[k]) + sigma
        null = np.maximum(bxy, abs(lz[k])) < thresh
        with np.errstate(divide='ignore', invalid='ignore'):
            out[k] = np.where(null, 0.0, A[k] / den)
    return out.T


def insert_bc(sc, sol, solf, bcx, bcy, bcz):
    """Copy interior and apply Dirichlet / Neumann extrapolation (class_solver_3d.f90:250-297,658-776)."""
    n1, n2, n3 = sol.shape
    solf = np.array(solf, dtype=np.float64)
    solf[1:n1 + 1, 1:n2 + 1, 1:n3 + 1] = sol
    for axis, ax, bc in ((0, sc.cx, bcx), (1, sc.cy, bcy), (2, sc.cz, bcz)):
        v = np.moveaxis(solf, axis, 0)  # view (n+2, a+2, b+2)
        inner = (slice(1, -1), slice(1, -1))
        n = v.shape[0] - 2
        if ax.bc[0] == 1:
            v[(0,) + inner] = bc[:, :, 0]
        elif ax.bc[0] in (2, 3):
            d = ax.neum[0]
            acc = bc[:, :, 0]
            for m in range(1, 7):
                acc = acc - d[m] * v[(m,) + inner]
            v[(0,) + inner] = acc * (1.0 / d[0])
        if ax.bc[1] == 1:
            v[(n + 1,) + inner] = bc[:, :, 1]
        elif ax.bc[1] in (2, 3):
            d = ax.neum[1]
            acc = bc[:, :, 1]
            for m in range(5, -1, -1):
                acc = acc - d[m] * v[(n - 5 + m,) + inner]
            v[(n + 1,) + inner] = acc * (1.0 / d[6])
    return solf


def solve_3d(sc, rhs, sigma, solf, bcx, bcy, bcz):
    """Full ``solve_3d``: returns the updated solf (rhs is not modified here)."""
    r = fold_bc(sc, rhs, np.asarray(bcx), np.asarray(bcy), np.asarray(bcz))
    aux = transform(sc, r, 'inv')
    sol = eigen_divide(sc, aux, sigma)
    sol = transform(sc, sol, 'fwd')
    return insert_bc(sc, sol, solf, bcx, bcy, bcz)


def solver_3d(sc, g, u, bcx, bcy, bcz, sigma):
    """Field-level wrapper (class_field.f90:1072-1109): interior of g, result into u."""
    gr = np.asarray(g)[1:-1, 1:-1, 1:-1]
    return solve_3d(sc, gr, sigma, u, bcx, bcy, bcz)


# ---------------------------------------------------------------------------
# FP64 residual of the interior operator, used to check iterative refinement
# ---------------------------------------------------------------------------

def apply_axis_operator(ax, u_line, bc_lo, bc_hi):
    """lhs^{-1} (rhs * u + bc column) along axis 0 of u_line (n, ...)."""
    from .derivatives import pentares
    n = ax.n
    sh = (slice(None),) + (None,) * (u_line.ndim - 1)
    lhs, rhs = lhs_rhs_matrices(ax.ddl, ax.ddr)
    b = np.tensordot(rhs, u_line, axes=([1], [0]))
    b[0] += ax.ddr[0, 0] * bc_lo
    b[1] += ax.ddr[1, 0] * bc_lo
    b[n - 2] += ax.ddr[n - 2, 7] * bc_hi
    b[n - 1] += ax.ddr[n - 1, 6] * bc_hi
    return pentares(ax.ddl_lu, b)


def residual(sc, g, u, sigma, bcx, bcy, bcz):
    """r = g - (Lx + Ly + Lz + sigma) u on the interior, boundary data included."""
    r = np.array(g, dtype=np.float64) - sigma * u
    r -= apply_axis_operator(sc.cx, u, bcx[:, :, 0], bcx[:, :, 1])
    r -= np.moveaxis(apply_axis_operator(sc.cy, np.moveaxis(u, 1, 0), bcy[:, :, 0], bcy[:, :, 1]), 0, 1)
    r -= np.moveaxis(apply_axis_operator(sc.cz, np.moveaxis(u, 2, 0), bcz[:, :, 0], bcz[:, :, 1]), 0, 2)
    return r
