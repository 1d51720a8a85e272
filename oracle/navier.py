"""Oracle of the single-domain Navier-Stokes time step (test infrastructure only).

Restates, in FP64 NumPy, one subdomain (``mpid%dims == 0``), no mapping
(``mapt = 0``: ``derxm`` = ``derx``, the ``_nc`` terms are zero,
src/class_mapping/class_mapping.f90:61-129) and ``nsubite`` sub-iterations
(convergence test ``testconv``, navier3d.f90:366-412; from the second
sub-iteration on every extrapolation returns the current iterate it(1)), the
time loop of src/main/navier3d.f90:48-274 built from
src/class_navier/class_navier_3D.f90:

* state ``type(navier3d)`` (:13-44): nt = 4 time levels u, v, w, p, phi in
  slots addressed through the permutation ``it``; BDF factors ``fac`` for
  tou = 1, 2, 3 and sigmau = -Re fac(1), sigmap = 0 (:2133-2155); velocity
  Dirichlet on all faces, pressure Neumann on all faces (:2157-2160);
  derivatives with solver-type coefficients, so = (6, 6) (:2273-2278);
* ``navier_time`` (:2052-2064), ``navier_bc_velocity`` with boundary values
  from the exact solution ``sol`` (:395-433, 848-925, 927-1041),
  ``navier_presolve_{u,v,w}`` (:1528-1595) with ``navier_nonlinear``
  (:1169-1222, nlt = 0, 1, 2) and the forcing ``f`` (:1043-1167, the
  exact-solution source, the LES term and the flow-rate term for u),
  ``add_boundary_gradient`` for pt = 1 (:695-791), ``navier_solve_{u,v,w}``
  (:1597-1761, before the pressure for pt = 1, 2, after the projection for
  pt = 3, 4: navier3d.f90:78-102), ``navier_presolve_phi`` /
  ``navier_phi_rhs`` (:1764-1785, 1961-2007), ``navier_solve_phi`` with
  ``navier_bc_pressure`` (:1787-1845, 342-393) and ``add_boundary_rotrot``
  for pt = 3 (:793-846), ``navier_projection`` (:1847-1959),
  ``navier_extrapol`` (:2010-2050) and the slot rotation
  (navier3d.f90:256-261);
* the driver's per-step diagnostics (navier3d.f90:120-254) with
  ``integrale`` / ``norme2`` (class_navier_3D.f90:2419-2603); they report the
  level it(nt) and remove the weighted mean of its pressure, as the driver
  does.

``navier_LES`` (:1225-1455) runs before the presolve: the nine gradients of
the newest velocity level (edges zeroed) and, for les_type 1, 2, 3, the eddy
viscosity of oracle.les with the coefficient les_c**2 (:2138) -- for
les_type 4 the learned coefficient of oracle.mlp.nu_mlp with that
Smagorinsky value as the fallback (no reference counterpart); the forcing
then subtracts les_f = -sum_j d/dx_j (nu (du_ij + du_ji)) (:1083-1099) before
the flow-rate term.  The 1e-10 of the flow-rate term is a default-kind
(single precision) literal.
"""
import numpy as np

from oracle import derivatives as D
from oracle import les as L
from oracle import mlp as M
from oracle import solver as S
from oracle.les import zero_edges

NT = 4
THRESH = float(np.float32(1e-10))
NMODES = 5


def sol(x, y, z, t, kind, rey, nmodes=NMODES):
    """Exact solution and source terms (class_navier_3D.f90:927-1041): a sum
    of 5 steady modes (wt = 0).  The sources carry each mode's own advection
    only, so the sum is an exact solution for one mode (nmodes = 1), not for
    the reference's five."""
    x, y, z = np.broadcast_arrays(np.asarray(x, float), np.asarray(y, float), np.asarray(z, float))
    out = np.zeros(x.shape)
    pi = 4.0 * np.arctan(1.0)
    for i in range(1, nmodes + 1):
        a = b = 1.0
        wx = wy = wp = pi * i
        wt = 0.0 * i * pi
        ct, st = np.cos(wt * t), np.sin(wt * t)
        if kind == "u":
            out = out + a * np.sin(wx * x) * np.cos(wy * y) * ct / wx
        elif kind == "v":
            out = out - a * np.cos(wx * x) * np.sin(wy * y) * ct / wy
        elif kind == "p":
            out = out + b * np.sin(wp * (x - y)) * ct
        elif kind == "rhsu":
            out = out + (b * wp * ct * np.cos(wp * (y - x))
                         + a ** 2 * ct ** 2 * np.cos(wx * x) * np.sin(wx * x)
                         * (np.sin(wy * y) ** 2 + np.cos(wy * y) ** 2) / wx
                         + a * ct * np.sin(wx * x) * np.cos(wy * y) * (wy ** 2 / wx + wx) / rey
                         - a * wt * st * np.sin(wx * x) * np.cos(wy * y) / wx)
        elif kind == "rhsv":
            out = out + (-b * wp * ct * np.cos(wp * (y - x))
                         + a ** 2 * ct ** 2 * np.cos(wy * y) * np.sin(wy * y)
                         * (np.sin(wx * x) ** 2 + np.cos(wx * x) ** 2) / wy
                         - a * ct * np.cos(wx * x) * np.sin(wy * y) * (wy + wx ** 2 / wy) / rey
                         + a * wt * st * np.cos(wx * x) * np.sin(wy * y) / wy)
    return out


def bdf_factors(tou, ts):
    """fac(1:4) of navier_initialization (class_navier_3D.f90:2133-2152)."""
    if tou == 1:
        return np.array([1.0 / ts, -1.0 / ts, 0.0, 0.0])
    if tou == 2:
        return np.array([1.5 / ts, -2.0 / ts, 0.5 / ts, 0.0])
    if tou == 3:
        return np.array([11.0 / (6.0 * ts), -18.0 / (6.0 * ts), 9.0 / (6.0 * ts), -2.0 / (6.0 * ts)])
    raise ValueError("tou must be 1, 2 or 3")


def half_widths(g):
    """Integration widths of integrale/norme2: (g(i+1)-g(i-1))/2 inside,
    (g(2)-g(1))/2 and (g(n)-g(n-1))/2 at the ends."""
    g = np.asarray(g, float)
    w = np.empty_like(g)
    w[1:-1] = (g[2:] - g[:-2]) * 0.5
    w[0] = (g[1] - g[0]) * 0.5
    w[-1] = (g[-1] - g[-2]) * 0.5
    return w


def quad_weights(gx, gy, gz):
    """Weights of integrale / norme2 (class_navier_3D.f90:2419-2603): interior
    points and face points, edges and corners excluded."""
    wx, wy, wz = half_widths(gx), half_widths(gy), half_widths(gz)
    W = wx[:, None, None] * wy[None, :, None] * wz[None, None, :]
    bx = np.zeros(len(gx), int); bx[[0, -1]] = 1
    by = np.zeros(len(gy), int); by[[0, -1]] = 1
    bz = np.zeros(len(gz), int); bz[[0, -1]] = 1
    nb = bx[:, None, None] + by[None, :, None] + bz[None, None, :]
    return np.where(nb <= 1, W, 0.0)


def _ratio(a, b):
    """a / b in IEEE arithmetic (inf or NaN for b = 0, as the reference's
    Fortran division gives when there is no manufactured solution)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        return float(np.float64(a) / np.float64(b))


class Navier:
    """Single-domain state and time step; fields are (nx, ny, nz) arrays."""

    def __init__(self, gx, gy, gz, ts, rey, nlt=2, pt=1, tou=2, top=2, so=(6, 6), flow_rate=True,
                 nmodes=NMODES, les_type=0, les_c=0.0, nsubite=1):
        if pt not in (1, 2, 3, 4):
            raise ValueError("pressure types 1 to 4")
        self.gx, self.gy, self.gz = (np.asarray(g, float) for g in (gx, gy, gz))
        self.nx, self.ny, self.nz = len(gx), len(gy), len(gz)
        self.ts, self.rey = float(ts), float(rey)
        self.nlt, self.pt, self.tou, self.top = nlt, pt, tou, top
        self.flow_rate = flow_rate
        self.nmodes = nmodes
        self.les_type, self.les_c = les_type, float(les_c)
        self.nsubite, self.subite, self.subiterations = int(nsubite), 1, 0
        self.sub = None
        self.du = None
        self.les_nu = None
        self.les_network = None  # les_type 4: dict(params, mean, istd, lo, hi, cscale)
        self.fac = bdf_factors(tou, ts)
        self.sigmau = -self.rey * self.fac[0]
        self.sigmap = 0.0
        self.scu = S.Solver3D(self.gx, self.gy, self.gz, (1,) * 6, so[0])
        self.scp = S.Solver3D(self.gx, self.gy, self.gz, (2,) * 6, so[0])
        self.dcx = D.DerCoeffs(self.gx, so[1], solver=True)
        self.dcy = D.DerCoeffs(self.gy, so[1], solver=True)
        self.dcz = D.DerCoeffs(self.gz, so[1], solver=True)
        shape = (self.nx, self.ny, self.nz)
        z = lambda: np.zeros(shape)
        self.u, self.v, self.w = [z() for _ in range(NT)], [z() for _ in range(NT)], [z() for _ in range(NT)]
        self.p, self.phi = [z() for _ in range(NT)], [z() for _ in range(NT)]
        self.rhs = {c: [z(), z()] for c in "uvw"}
        self.it = list(range(NT))
        self.time = 0.0
        self.g = None          # flow-rate term (the saved field g of f), uniform
        self.debit = None
        self.W = quad_weights(self.gx, self.gy, self.gz)
        self.err_vts_t = 0.0
        self.err_pre_t = 0.0

    # -- helpers ------------------------------------------------------------
    def derx(self, f):
        return D.derx(self.dcx, f)

    def dery(self, f):
        return D.dery(self.dcy, f)

    def derz(self, f):
        return D.derz(self.dcz, f)

    def integrale(self, f):
        return float(np.sum(self.W * f))

    def norme(self, f):
        return float(np.sqrt(np.sum(self.W * f * f)))

    def points(self):
        return np.meshgrid(self.gx, self.gy, self.gz, indexing="ij")

    def extrapol(self, var, kind):
        """navier_extrapol with subite = 1 (class_navier_3D.f90:2010-2050)."""
        order = self.tou if kind == "v" else self.top - 1
        it = self.it
        if self.subite > 1:
            out = 1.0 * var[it[0]]
        elif order == -1:
            out = 1.0 * var[it[0]]
        elif order == 1:
            out = 1.0 * var[it[NT - 1]]
        elif order == 2:
            out = 2.0 * var[it[NT - 1]] - 1.0 * var[it[NT - 2]]
        elif order == 3:
            out = 3.0 * var[it[NT - 1]] - 3.0 * var[it[NT - 2]] + 1.0 * var[it[NT - 3]]
        else:
            out = np.zeros((self.nx, self.ny, self.nz))
        return zero_edges(out)

    def nonlinear(self, x):
        """navier_nonlinear: the advection term of every slot, extrapolated."""
        tmp = []
        for i in range(NT):
            if self.nlt == 1:
                t = self.u[i] * self.derx(x[i]) + self.v[i] * self.dery(x[i]) + self.w[i] * self.derz(x[i])
            elif self.nlt == 2:
                t = (self.u[i] * self.derx(x[i]) + self.v[i] * self.dery(x[i])
                     + self.w[i] * self.derz(x[i])) * 0.5
                t = t + self.derx(x[i] * self.u[i]) * 0.5
                t = t + self.dery(x[i] * self.v[i]) * 0.5
                t = t + self.derz(x[i] * self.w[i]) * 0.5
            else:
                t = np.zeros((self.nx, self.ny, self.nz))
            tmp.append(t)
        return self.extrapol(tmp, "v")

    def flow_update(self, isum, reft):
        """Flow-rate term of f (class_navier_3D.f90:1140-1164) from the
        integral of extrapol(u) and of 1 (over all subdomains)."""
        err = isum / reft
        if self.g is None:
            self.debit = err
            if self.debit <= THRESH:
                self.debit = 1.0
            self.g = 3.0 * self.debit
        err = err - self.debit
        self.g = self.g - err * self.fac[0]
        return self.g

    def forcing(self, c, g=None):
        """f(nav,mpid,'rhs'//c); g is the flow-rate term (u only)."""
        X, Y, Z = self.points()
        F = sol(X, Y, Z, self.time, "rhs" + c, self.rey, self.nmodes)
        if self.les_type:
            F = F - self.les_forcing(c)
        if c == "u" and self.flow_rate:
            F = F + g
        return F

    def les_forcing(self, c):
        """les_f of f() for component c (class_navier_3D.f90:1083-1099)."""
        i = "uvw".index(c)
        grads = (self.derx, self.dery, self.derz)
        lf = np.zeros((self.nx, self.ny, self.nz))
        for j in range(3):
            aux = self.les_nu * (self.du[i][j] + self.du[j][i])
            lf = lf - grads[j](aux)
        return lf

    def bc_exact(self, c):
        """navier_bc_velocity_utils: face values of sol (interior tangential points)."""
        gx, gy, gz, t = self.gx, self.gy, self.gz, self.time
        m = self.nmodes
        bcx = np.stack([sol(g, gy[1:-1, None], gz[None, 1:-1], t, c, self.rey, m) for g in (gx[0], gx[-1])], -1)
        bcy = np.stack([sol(gx[1:-1, None], g, gz[None, 1:-1], t, c, self.rey, m) for g in (gy[0], gy[-1])], -1)
        bcz = np.stack([sol(gx[1:-1, None], gy[None, 1:-1], g, t, c, self.rey, m) for g in (gz[0], gz[-1])], -1)
        return [bcx, bcy, bcz]

    # -- the time step, in stages (a multidomain driver interleaves them with
    # the collective solves and sums) ------------------------------------
    def step(self):
        """One pass of the step for one domain."""
        g = None
        if self.flow_rate:
            ones = np.ones((self.nx, self.ny, self.nz))
            g = self.flow_update(self.integrale(self.extrapol(self.u, "v")), self.integrale(ones))
        self.stage_presolve(g)
        if self.pt <= 2:
            self.velocity_solves()
        self.stage_phi()
        self.set_phi(S.solver_3d(self.scp, self.fphi, self.phi[self.it[0]], *self.bcphi, self.sigmap))
        self.stage_projection()
        if self.pt >= 3:
            self.velocity_solves()

    def velocity_solves(self):
        new = self.it[0]
        levels = (self.u, self.v, self.w)
        for q in range(3):
            fu, bc = self.velocity_rhs(q)
            levels[q][new] = S.solver_3d(self.scu, fu, levels[q][new], *bc, self.sigmau)

    def stage_presolve(self, g):
        """Boundary values, navier_LES, presolve u, v, w and (pt = 1) the
        boundary gradient (navier3d.f90:63-80)."""
        it, fac = self.it, self.fac
        n0 = it[NT - 1]
        self.bc = {c: self.bc_exact(c) for c in "uvw"}
        bc = self.bc
        levels = {"u": self.u, "v": self.v, "w": self.w}
        if self.les_type:  # navier_LES on the newest level
            grads = (self.derx, self.dery, self.derz)
            vel = (self.u[n0], self.v[n0], self.w[n0])
            self.du = [[zero_edges(grads[j](vel[i])) for j in range(3)] for i in range(3)]
            if self.les_type == 4:
                # the learned coefficient (network parameters and scaling in
                # self.les_network, oracle.mlp.nu_mlp), Smagorinsky with
                # les_c**2 outside the training range
                net = self.les_network
                self.les_nu, _ = M.nu_mlp(net["params"], self.du, self.gx, self.gy, self.gz, net["mean"],
                                          net["istd"], net["lo"], net["hi"], net["cscale"], self.les_c ** 2)
            else:
                self.les_nu = L.les_nu(self.du, self.gx, self.gy, self.gz, self.les_type, self.les_c ** 2)
        for c in "uvw":
            self.rhs[c][1] = self.rhs[c][0]
            nl = self.nonlinear(levels[c])
            self.rhs[c][0] = zero_edges(self.forcing(c, g) - nl)
        if self.pt == 1:
            e = self.extrapol(self.phi, "p")
            dx, dy, dz = self.derx(e), self.dery(e), self.derz(e)
            for m, (i, j, k) in enumerate(((0, 0, 0), (-1, -1, -1))):
                bc["v"][0][:, :, m] += dy[i, 1:-1, 1:-1] / fac[0]
                bc["w"][0][:, :, m] += dz[i, 1:-1, 1:-1] / fac[0]
                bc["u"][1][:, :, m] += dx[1:-1, j, 1:-1] / fac[0]
                bc["w"][1][:, :, m] += dz[1:-1, j, 1:-1] / fac[0]
                bc["u"][2][:, :, m] += dx[1:-1, 1:-1, k] / fac[0]
                bc["v"][2][:, :, m] += dy[1:-1, 1:-1, k] / fac[0]

    def velocity_rhs(self, q):
        """navier_solve_{u,v,w} (:1597-1761): the right-hand side field and
        the boundary arrays of component q."""
        it, fac = self.it, self.fac
        new, n0, n1, n2 = it[0], it[NT - 1], it[NT - 2], it[NT - 3]
        c = "uvw"[q]
        lev = (self.u, self.v, self.w)[q]
        grads = (self.derx, self.dery, self.derz)
        fu = np.zeros((self.nx, self.ny, self.nz))
        fu = fu + fac[1] * lev[n0] + fac[2] * lev[n1]
        if self.tou == 3:
            fu = fu + fac[3] * lev[n2]
        if self.pt == 2:
            fu = fu + grads[q](self.extrapol(self.p, "p"))
        elif self.pt >= 3:
            fu = fu + grads[q](self.p[new])
        fu = fu - self.rhs[c][0]
        fu = self.rey * fu
        return fu, self.bc[c]

    def set_velocity(self, q, field):
        (self.u, self.v, self.w)[q][self.it[0]] = field

    def set_phi(self, field):
        self.phi[self.it[0]] = field

    def stage_phi(self):
        """Presolve phi, the right-hand side and the Neumann data of the
        phi solve (:1764-1845, 342-393, 793-846)."""
        fac = self.fac
        levels = {"u": self.u, "v": self.v, "w": self.w}
        bc = self.bc
        rp = [self.phi_rhs(levels[c], self.rhs[c]) for c in "uvw"]
        fphi = self.sigmap * self.extrapol(self.phi, "p")
        fphi = fphi + self.derx(rp[0]) + self.dery(rp[1]) + self.derz(rp[2])
        nx, ny, nz = self.nx, self.ny, self.nz
        bcphi = [np.stack([rp[0][m * (nx - 1), 1:-1, 1:-1] - fac[0] * bc["u"][0][:, :, m] for m in (0, 1)], -1),
                 np.stack([rp[1][1:-1, m * (ny - 1), 1:-1] - fac[0] * bc["v"][1][:, :, m] for m in (0, 1)], -1),
                 np.stack([rp[2][1:-1, 1:-1, m * (nz - 1)] - fac[0] * bc["w"][2][:, :, m] for m in (0, 1)], -1)]
        if self.pt == 3:
            self.add_boundary_rotrot(bcphi)
        self.rp, self.fphi, self.bcphi = rp, fphi, bcphi

    def stage_projection(self):
        """navier_projection (:1847-1959)."""
        new, fac = self.it[0], self.fac
        levels = {"u": self.u, "v": self.v, "w": self.w}
        grads = (self.derx, self.dery, self.derz)
        rp = self.rp
        self.phi[new] = zero_edges(self.phi[new])
        if self.pt in (2, 4):
            aux = self.extrapol(self.p, "p")
        self.p[new] = self.phi[new].copy()
        if self.pt in (2, 4):
            self.p[new] = self.p[new] + aux
        self.p[new] = zero_edges(self.p[new])
        if self.pt <= 2:
            div = (self.derx(self.u[new]) + self.dery(self.v[new]) + self.derz(self.w[new])) / self.rey
            self.p[new] = self.p[new] - div
        elif self.pt == 4:
            div = (self.derx(self.extrapol(self.u, "p")) + self.dery(self.extrapol(self.v, "p"))
                   + self.derz(self.extrapol(self.w, "p"))) / self.rey
            self.p[new] = self.p[new] - div
        self.p[new] = zero_edges(self.p[new])
        for q, c in enumerate("uvw"):
            levels[c][new] = zero_edges((rp[q] - grads[q](self.phi[new])) / fac[0])

    def phi_rhs(self, var, fvar):
        """navier_phi_rhs with subite = 1 (class_navier_3D.f90:1961-2007)."""
        it, fac = self.it, self.fac
        if self.pt <= 2:
            out = fac[0] * var[it[0]]
        else:
            out = fvar[0] - fac[1] * var[it[NT - 1]] - fac[2] * var[it[NT - 2]] - fac[3] * var[it[NT - 3]]
            if self.pt == 4 and self.subite > 1:
                out = fvar[0] - fvar[1] + fac[0] * var[it[0]]
            elif self.pt == 4:
                out = (out - fvar[1] + fac[0] * var[it[NT - 1]] + fac[1] * var[it[NT - 2]]
                       + fac[2] * var[it[NT - 3]] + fac[3] * var[it[0]])
        return zero_edges(out)

    def add_boundary_rotrot(self, bcphi):
        """add_boundary_rotrot (class_navier_3D.f90:793-846): the normal
        component of curl curl of the extrapolated velocity, over Re, taken
        from the Neumann data of phi (pt = 3)."""
        eu, ev, ew = (self.extrapol(f, "p") for f in (self.u, self.v, self.w))
        dd = (lambda f: D.dderx(self.dcx, f), lambda f: D.ddery(self.dcy, f), lambda f: D.dderz(self.dcz, f))
        ax = self.derx(self.dery(ev) + self.derz(ew)) - dd[1](eu) - dd[2](eu)
        ay = self.dery(self.derx(eu) + self.derz(ew)) - dd[0](ev) - dd[2](ev)
        az = self.derz(self.derx(eu) + self.dery(ev)) - dd[0](ew) - dd[1](ew)
        nx, ny, nz = self.nx, self.ny, self.nz
        for m in (0, 1):
            bcphi[0][:, :, m] = bcphi[0][:, :, m] - ax[m * (nx - 1), 1:-1, 1:-1] / self.rey
            bcphi[1][:, :, m] = bcphi[1][:, :, m] - ay[1:-1, m * (ny - 1), 1:-1] / self.rey
            bcphi[2][:, :, m] = bcphi[2][:, :, m] - az[1:-1, 1:-1, m * (nz - 1)] / self.rey

    def diagnostics(self):
        """navier3d.f90:120-254 on level it(nt) (before the rotation), which
        removes the weighted mean of that level's pressure.  Returns the
        printed numbers."""
        it = self.it
        cur, prev = it[NT - 1], it[NT - 2]
        ones = np.ones((self.nx, self.ny, self.nz))
        out = {}
        ref = self.norme(ones)
        div = self.derx(self.u[cur]) + self.dery(self.v[cur]) + self.derz(self.w[cur])
        out["div"] = self.norme(div) / ref
        X, Y, Z = self.points()
        ue = [sol(X, Y, Z, self.time, c, self.rey, self.nmodes) for c in "uv"] + [np.zeros_like(X)]
        pex = sol(X, Y, Z, self.time, "p", self.rey, self.nmodes)
        ref = self.norme(np.sqrt(ue[0] ** 2 + ue[1] ** 2 + ue[2] ** 2))
        err = self.norme(np.sqrt((ue[0] - self.u[cur]) ** 2 + (ue[1] - self.v[cur]) ** 2
                                 + (ue[2] - self.w[cur]) ** 2))
        self.err_vts_t += err ** 2 * self.ts
        out["vel"] = (err, _ratio(err, ref), np.sqrt(self.err_vts_t))
        ref = self.integrale(ones)
        mean = self.integrale(self.p[cur])
        self.p[cur] = self.p[cur] - mean / ref
        pex = pex - self.integrale(pex) / ref
        refp = self.norme(pex)
        err = self.norme(self.p[cur] - pex)
        self.err_pre_t += err ** 2 * self.ts
        out["pres"] = (err, _ratio(err, refp), np.sqrt(self.err_pre_t))
        reft = self.integrale(ones)
        ek = 0.5 * (self.norme(self.u[cur]) ** 2 + self.norme(self.v[cur]) ** 2 + self.norme(self.w[cur]))
        out["kinetic"] = ek / reft
        aux = self.p[cur] - self.p[prev]
        aux = aux - self.integrale(aux) / reft
        e = self.norme(aux)
        out["station_p"] = (e, e / reft)
        e2 = (self.norme(self.u[cur] - self.u[prev]) ** 2 + self.norme(self.v[cur] - self.v[prev]) ** 2
              + self.norme(self.w[cur] - self.w[prev]))
        out["station_v"] = (np.sqrt(e2), np.sqrt(e2) / reft)
        return out

    def rotate(self):
        """Slot rotation at the end of a time step (navier3d.f90:256-261)."""
        self.it = self.it[1:] + self.it[:1]

    def testconv(self, eps=1e-9):
        """testconv (navier3d.f90:366-412): relative change of the velocity
        and of the mean-corrected pressure since the last sub-iteration."""
        new = self.it[0]
        u, v, w, p = self.u[new], self.v[new], self.w[new], self.p[new]
        su, sv, sw, sp = self.sub
        ref = self.norme(np.sqrt(u ** 2 + v ** 2 + w ** 2))
        e1 = self.norme(np.sqrt((su - u) ** 2 + (sv - v) ** 2 + (sw - w) ** 2)) / ref
        refi = self.integrale(np.ones((self.nx, self.ny, self.nz)))
        sp = sp + self.integrale(p - sp) / refi
        e2 = self.norme(p - sp) / self.norme(sp)
        return e1 < eps and e2 < eps

    def advance(self, diagnostics=False):
        """One iteration of the time loop (navier3d.f90:48-261): navier_time,
        the sub-iterations (step, convergence test, driver diagnostics), the
        slot rotation.  Returns the last sub-iteration's diagnostics."""
        self.time += self.ts
        d = None
        for subite in range(1, self.nsubite + 1):
            self.subite = subite
            self.step()
            test = subite > 1 and self.testconv()
            self.sub = [f[self.it[0]].copy() for f in (self.u, self.v, self.w, self.p)]
            if diagnostics:
                d = self.diagnostics()
            self.subiterations = subite
            if test:
                break
        self.subite = 1
        self.rotate()
        return d


class NavierMD:
    """Multidomain branch of the step (``mpid%dims /= 0``, navier3d.f90 with
    class_navier_3D.f90): one ``Navier`` per subdomain for the local stages;
    the velocity solves and the phi solve through ``multidomain_solve``
    (oracle.md.MultiDomain; velocity Dirichlet on the outer faces with
    sigmau, pressure Neumann with sigma 0 and the constant null space,
    psm = 1: class_navier_3D.f90:1641-1648, 1829-1834, 2157-2160); sums over
    all subdomains for the flow-rate term, the diagnostics and testconv
    (md_mpi_reduce_double_sum).  Interface faces take no boundary values
    (erase_boundary_inter :626-648): the solve ignores them."""

    def __init__(self, nd, periods, gx, gy, gz, ts, rey, so=(6, 6), **kw):
        from oracle import md as omd
        self.mdu = omd.MultiDomain(nd, periods, gx, gy, gz, (1,) * 6, so[0], so[1])
        self.mdp = omd.MultiDomain(nd, periods, gx, gy, gz, (2,) * 6, so[0], so[1])
        self.subs = self.mdu.subdomains()
        self.dom = {c: Navier(gx[c[0]], gy[c[1]], gz[c[2]], ts, rey, so=so, **kw) for c in self.subs}
        d0 = self.dom[self.subs[0]]
        self.pt, self.flow_rate, self.nsubite, self.ts = d0.pt, d0.flow_rate, d0.nsubite, d0.ts
        self.sigmau = d0.sigmau
        self.mdu.influence_matrix(self.sigmau, 0)
        self.mdp.influence_matrix(0.0, 1)
        self.err_vts_t = 0.0
        self.err_pre_t = 0.0
        self.subiterations = 0

    def doms(self):
        return [self.dom[c] for c in self.subs]

    def sum_integrale(self, fields):
        return sum(d.integrale(f) for d, f in zip(self.doms(), fields))

    def sum_norme(self, fields):
        return float(np.sqrt(sum(float(np.sum(d.W * f * f)) for d, f in zip(self.doms(), fields))))

    def ones(self):
        return [np.ones((d.nx, d.ny, d.nz)) for d in self.doms()]

    def velocity_solves(self):
        for q in range(3):
            rhs, bc = {}, {}
            for c in self.subs:
                rhs[c], bc[c] = self.dom[c].velocity_rhs(q)
            sol, _ = self.mdu.solve(rhs, bc, self.sigmau)
            for c in self.subs:
                self.dom[c].set_velocity(q, sol[c])

    def step(self):
        doms = self.doms()
        g = None
        if self.flow_rate:
            isum = self.sum_integrale([d.extrapol(d.u, "v") for d in doms])
            g = doms[0].flow_update(isum, self.sum_integrale(self.ones()))
            for d in doms[1:]:
                d.g, d.debit = doms[0].g, doms[0].debit
        for d in doms:
            d.stage_presolve(g)
        if self.pt <= 2:
            self.velocity_solves()
        for d in doms:
            d.stage_phi()
        sol, _ = self.mdp.solve({c: self.dom[c].fphi for c in self.subs},
                                {c: self.dom[c].bcphi for c in self.subs}, 0.0)
        for c in self.subs:
            self.dom[c].set_phi(sol[c])
        for d in doms:
            d.stage_projection()
        if self.pt >= 3:
            self.velocity_solves()

    def testconv(self, eps=1e-9):
        doms = self.doms()
        new = doms[0].it[0]
        vel = [(d.u[new], d.v[new], d.w[new]) for d in doms]
        ref = self.sum_norme([np.sqrt(u ** 2 + v ** 2 + w ** 2) for u, v, w in vel])
        e1 = self.sum_norme([np.sqrt((d.sub[0] - u) ** 2 + (d.sub[1] - v) ** 2 + (d.sub[2] - w) ** 2)
                             for d, (u, v, w) in zip(doms, vel)]) / ref
        refi = self.sum_integrale(self.ones())
        m = self.sum_integrale([d.p[new] - d.sub[3] for d in doms]) / refi
        sp = [d.sub[3] + m for d in doms]
        e2 = self.sum_norme([d.p[new] - s for d, s in zip(doms, sp)]) / self.sum_norme(sp)
        return e1 < eps and e2 < eps

    def diagnostics(self):
        """navier3d.f90:120-254 with the sums over all subdomains."""
        doms = self.doms()
        cur, prev = doms[0].it[NT - 1], doms[0].it[NT - 2]
        out = {}
        ones = self.ones()
        ref = self.sum_norme(ones)
        out["div"] = self.sum_norme([d.derx(d.u[cur]) + d.dery(d.v[cur]) + d.derz(d.w[cur]) for d in doms]) / ref
        ue, pex = [], []
        for d in doms:
            X, Y, Z = d.points()
            ue.append([sol(X, Y, Z, d.time, c, d.rey, d.nmodes) for c in "uv"] + [np.zeros_like(X)])
            pex.append(sol(X, Y, Z, d.time, "p", d.rey, d.nmodes))
        ref = self.sum_norme([np.sqrt(e[0] ** 2 + e[1] ** 2 + e[2] ** 2) for e in ue])
        err = self.sum_norme([np.sqrt((e[0] - d.u[cur]) ** 2 + (e[1] - d.v[cur]) ** 2 + (e[2] - d.w[cur]) ** 2)
                              for d, e in zip(doms, ue)])
        self.err_vts_t += err ** 2 * self.ts
        out["vel"] = (err, _ratio(err, ref), np.sqrt(self.err_vts_t))
        ref = self.sum_integrale(ones)
        mean = self.sum_integrale([d.p[cur] for d in doms])
        for d in doms:
            d.p[cur] = d.p[cur] - mean / ref
        pm = self.sum_integrale(pex)
        pex = [x - pm / ref for x in pex]
        refp = self.sum_norme(pex)
        err = self.sum_norme([d.p[cur] - x for d, x in zip(doms, pex)])
        self.err_pre_t += err ** 2 * self.ts
        out["pres"] = (err, _ratio(err, refp), np.sqrt(self.err_pre_t))
        reft = ref
        nu_, nv_, nw_ = (self.sum_norme([getattr(d, a)[cur] for d in doms]) for a in "uvw")
        out["kinetic"] = 0.5 * (nu_ ** 2 + nv_ ** 2 + nw_) / reft
        aux = [d.p[cur] - d.p[prev] for d in doms]
        am = self.sum_integrale(aux)
        e = self.sum_norme([a - am / reft for a in aux])
        out["station_p"] = (e, e / reft)
        e2 = (self.sum_norme([d.u[cur] - d.u[prev] for d in doms]) ** 2
              + self.sum_norme([d.v[cur] - d.v[prev] for d in doms]) ** 2
              + self.sum_norme([d.w[cur] - d.w[prev] for d in doms]))
        out["station_v"] = (np.sqrt(e2), np.sqrt(e2) / reft)
        return out

    def advance(self, diagnostics=False):
        doms = self.doms()
        for d in doms:
            d.time += d.ts
        out = None
        for subite in range(1, self.nsubite + 1):
            for d in doms:
                d.subite = subite
            self.step()
            test = subite > 1 and self.testconv()
            for d in doms:
                d.sub = [f[d.it[0]].copy() for f in (d.u, d.v, d.w, d.p)]
            if diagnostics:
                out = self.diagnostics()
            self.subiterations = subite
            if test:
                break
        for d in doms:
            d.subite = 1
            d.rotate()
        return out
