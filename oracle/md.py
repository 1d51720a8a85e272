"""Oracle influence-matrix multidomain coupling (test infrastructure only).

Restates, in FP64 NumPy:

* ``Topology``            md_influence_matrix_param, src/class_md/class_md.f90:1450-1680
                          (interface numbering with periodic wrap, row offsets, ninf)
* ``MultiDomain.influence_matrix``  md_influence_matrix_set, src/class_field/class_field.f90:1396-1510
                          + md_influence_matrix_setvalues, class_md.f90:1049-1095
* ``MultiDomain.solve``   multidomain_solve, class_field.f90:1295-1388, with
                          md_vector_setvalues / md_vector_getvalues (class_md.f90:663-708,
                          445-550) and the interface solve of md_solve (class_md.f90:379-438)
                          done by a dense direct solve instead of a PETSc KSP.

Subdomain (i,j,k) of an (nd1,nd2,nd3) decomposition owns the x-grid of slab
i, the y-grid of slab j and the z-grid of slab k, so faces always match
(the reference uses one size for every subdomain; uneven slab sizes are a
conforming generalisation).  Neighbouring subdomains share their interface
nodes.  Boundary types: physical faces keep the caller's ``bct``; interface
faces are Dirichlet (md_bc_init, class_md.f90:275-293).

Null-space modes of the interface system (class_field.f90:1339-1354):
``null=0`` none; ``null=1`` the rhs is made mean-free and the solution is
the one orthogonal to the constant vector (KSP with a null space);
``null=2`` row 0 of the matrix is replaced by 5*e_0 and rhs(0) by 0
(md_add_pert, class_md.f90:223-249; md_vector_zero_lastpoint :251-268).
"""
import numpy as np

from . import derivatives as D
from . import solver as S


class Topology:
    """Interface numbering of md_influence_matrix_param (class_md.f90:1450-1680).

    ``dm_int[i,j,k,l,m]``: interface id (1-based, -1 = none) of face l
    (0 x, 1 y, 2 z) side m (0 left, 1 right) of subdomain (i,j,k).
    ``kind[p]`` is the axis of interface p, ``offset[p]`` its first row and
    ``size[p]`` its number of points."""

    def __init__(self, nd, periods, nint):
        """nint[l][s] = interior points of slab s along axis l."""
        self.nd = tuple(int(v) for v in nd)
        self.periods = tuple(bool(v) for v in periods)
        nd1, nd2, nd3 = self.nd
        dm = -np.ones((nd1, nd2, nd3, 3, 2), dtype=int)
        kind = []
        count = 0
        for i in range(nd1):
            for j in range(nd2):
                for k in range(nd3):
                    idx = (i, j, k)
                    for l in range(3):
                        if idx[l] < self.nd[l] - 1 or self.periods[l]:
                            count += 1
                            dm[i, j, k, l, 1] = count
                            kind.append(l)
        # left face = right face of the left neighbour (with periodic wrap)
        dm[1:, :, :, 0, 0] = dm[:-1, :, :, 0, 1]
        if self.periods[0]:
            dm[0, :, :, 0, 0] = dm[-1, :, :, 0, 1]
        dm[:, 1:, :, 1, 0] = dm[:, :-1, :, 1, 1]
        if self.periods[1]:
            dm[:, 0, :, 1, 0] = dm[:, -1, :, 1, 1]
        dm[:, :, 1:, 2, 0] = dm[:, :, :-1, 2, 1]
        if self.periods[2]:
            dm[:, :, 0, 2, 0] = dm[:, :, -1, 2, 1]
        dm[dm == 0] = -1
        self.dm_int = dm
        self.it = count
        self.kind = np.array(kind, dtype=int)
        # sizes: tangential interior points of the owning (left) subdomain
        self.size = np.zeros(count, dtype=int)
        for i in range(nd1):
            for j in range(nd2):
                for k in range(nd3):
                    for l in range(3):
                        p = dm[i, j, k, l, 1]
                        if p > 0:
                            n = [nint[0][i], nint[1][j], nint[2][k]]
                            t = [a for a in range(3) if a != l]
                            self.size[p - 1] = n[t[0]] * n[t[1]]
        self.offset = np.concatenate([[0], np.cumsum(self.size)[:-1]]).astype(int)
        self.ninf = int(self.size.sum())


class MultiDomain:
    """All subdomains of a decomposition with their solver and derivative
    coefficients (solver-type derivatives, as the reference's MD test uses)."""

    def __init__(self, nd, periods, gx, gy, gz, bct, so=6, der_so=6):
        self.nd = tuple(nd)
        self.grids = (list(gx), list(gy), list(gz))
        nint = [[g.size - 2 for g in self.grids[l]] for l in range(3)]
        self.topo = Topology(nd, periods, nint)
        self.bct = tuple(bct)
        self.sub = {}
        for i in range(nd[0]):
            for j in range(nd[1]):
                for k in range(nd[2]):
                    inter = self.topo.dm_int[i, j, k]
                    b = list(bct)
                    for l in range(3):
                        for m in range(2):
                            if inter[l, m] > 0:
                                b[2 * l + m] = 1
                    g3 = (gx[i], gy[j], gz[k])
                    self.sub[(i, j, k)] = {
                        "sc": S.Solver3D(*g3, tuple(b), so),
                        "dc": [D.DerCoeffs(g, der_so, True) for g in g3],
                        "shape": tuple(g.size for g in g3),
                    }
        self.M = None

    def subdomains(self):
        return sorted(self.sub, key=lambda c: (c[2], c[1], c[0]))

    # face helpers -------------------------------------------------------
    @staticmethod
    def face_of(f, l, m):
        """Interior points of face (l, m) of a full field f(nx,ny,nz)."""
        sl = [slice(1, -1)] * 3
        sl[l] = 0 if m == 0 else -1
        return f[tuple(sl)]

    def face_derivatives(self, c, u):
        """Signed normal derivatives on the interface faces of subdomain c:
        left faces -d/dn, right faces +d/dn (multidomain_solve,
        class_field.f90:1322-1331).  Returns {(l,m): array}."""
        dc = self.sub[c]["dc"]
        out = {}
        ders = [D.derx(dc[0], u), D.dery(dc[1], u), D.derz(dc[2], u)]
        for l in range(3):
            for m in range(2):
                if self.topo.dm_int[c + (l, m)] > 0:
                    v = self.face_of(ders[l], l, m)
                    out[(l, m)] = -v if m == 0 else v
        return out

    def _solve_sub(self, c, g, bcs, sigma):
        sc = self.sub[c]["sc"]
        nx, ny, nz = self.sub[c]["shape"]
        u = np.zeros((nx, ny, nz))
        return S.solver_3d(sc, g, u, bcs[0], bcs[1], bcs[2], sigma)

    def _bc_arrays(self, c):
        nx, ny, nz = self.sub[c]["shape"]
        return [np.zeros((ny - 2, nz - 2, 2)), np.zeros((nx - 2, nz - 2, 2)),
                np.zeros((nx - 2, ny - 2, 2))]

    # assembly -----------------------------------------------------------
    def influence_matrix(self, sigma, null=0):
        """Dense influence matrix (md_influence_matrix_set): a Dirac on each
        interface point of each subdomain, the subdomain solved with g = 0,
        and the normal derivatives on all its interface faces (left faces
        +d/dn, right faces -d/dn) added to the rows of those interfaces."""
        topo = self.topo
        M = np.zeros((topo.ninf, topo.ninf))
        for c in self.subdomains():
            inter = topo.dm_int[c]
            shape = self.sub[c]["shape"]
            g = np.zeros(shape)
            for m in range(2):
                for l in range(3):
                    p = inter[l, m]
                    if p <= 0:
                        continue
                    npts = topo.size[p - 1]
                    col0 = topo.offset[p - 1]
                    for q in range(npts):
                        bcs = self._bc_arrays(c)
                        n1f = bcs[l].shape[0]
                        bcs[l][q % n1f, q // n1f, m] = 1.0   # face point q, Fortran order
                        u = self._solve_sub(c, g, bcs, sigma)
                        d = self.face_derivatives(c, u)
                        for (l2, m2), v in d.items():
                            p2 = inter[l2, m2]
                            rows = topo.offset[p2 - 1] + np.arange(topo.size[p2 - 1])
                            # column sign convention of the matrix: -(rhs sign)
                            M[rows, col0 + q] += -v.reshape(-1, order='F')
        if null == 2:
            M[0, :] = 0.0
            M[0, 0] = 5.0
        self.M = M
        self.null = null
        self.sigma = sigma
        return M

    # solve ----------------------------------------------------------------
    def solve(self, g, bc, sigma):
        """multidomain_solve: g[c] full fields, bc[c] = [bcx, bcy, bcz] of
        the physical faces (interface faces are ignored).  Returns u[c]."""
        topo = self.topo
        rhs = np.zeros(topo.ninf)
        for c in self.subdomains():
            inter = topo.dm_int[c]
            bcs = [np.array(b, dtype=np.float64) for b in bc[c]]
            for l in range(3):
                for m in range(2):
                    if inter[l, m] > 0:
                        bcs[l][:, :, m] = 0.0
            u0 = self._solve_sub(c, g[c], bcs, sigma)
            for (l, m), v in self.face_derivatives(c, u0).items():
                p = inter[l, m]
                rows = topo.offset[p - 1] + np.arange(topo.size[p - 1])
                rhs[rows] += v.reshape(-1, order='F')
        lam = self.interface_solve(rhs)
        out = {}
        for c in self.subdomains():
            inter = topo.dm_int[c]
            bcs = [np.array(b, dtype=np.float64) for b in bc[c]]
            for l in range(3):
                for m in range(2):
                    p = inter[l, m]
                    if p > 0:
                        vals = lam[topo.offset[p - 1]:topo.offset[p - 1] + topo.size[p - 1]]
                        bcs[l][:, :, m] = vals.reshape(bcs[l].shape[:2], order='F')
            out[c] = self._solve_sub(c, g[c], bcs, sigma)
        return out, lam

    def interface_solve(self, rhs):
        rhs = np.array(rhs, dtype=np.float64)
        if self.null == 1:
            rhs -= rhs.mean()
            Mp = self.M.copy()
            Mp[0, :] = 0.0
            Mp[0, 0] = 5.0
            r = rhs.copy()
            r[0] = 0.0
            lam = np.linalg.solve(Mp, r)
            return lam - lam.mean()
        if self.null == 2:
            rhs[0] = 0.0
        return np.linalg.solve(self.M, rhs)
