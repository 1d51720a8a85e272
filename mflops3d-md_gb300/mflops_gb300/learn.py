"""Learned LES coefficient: training data from a fine FP64 box flow, filtered
to the LES grid by the spline filter, and the training loop of the network
(no reference counterpart; the plain models of navier_LES,
class_navier_3D.f90:1225-1455, are the fallback and the baseline).

Pipeline, every step on the GPU through the library's entry points:

1. ``BoxFlow``: a decaying flow in the no-slip unit box on a uniform fine
   grid.  Initial condition u = curl(e psi), psi = two Helmholtz smoothings
   of white noise (the 3-D solver with Dirichlet faces) and e a wall envelope;
   time stepping by explicit three-stage SSP Runge-Kutta with a projection
   after each stage (compact derivatives, Neumann Poisson solve).
2. ``PairMaker.pairs``: F(u_i) and F(u_i u_j) on the LES grid (a
   differential filter on the fine grid through the Helmholtz solver, then
   the least-squares spline filter with knots at the LES nodes), the gradients of
   F(u) with the LES grid's compact derivatives, then the features, the
   factor b = Delta^2 sqrt(2 S:S) and the target nu = -tau^d:S / (2 S:S).
3. ``fit``: standardisation from the training pairs, cscale = the best
   constant coefficient (least squares), Adam steps on random mini-batches.
"""
import numpy as np

import mflops_gb300 as mf


def uniform_grid(n):
    return np.linspace(0.0, 1.0, n)


class BoxFlow:
    """Fine-grid decaying flow in the no-slip unit box (FP64, device fields)."""

    def __init__(self, n, nu, seed, k0=30.0, so=6):
        import torch
        self.n = n
        self.nu = nu
        self.grid = uniform_grid(n)
        g = self.grid
        self.dc = mf.DerivativesCoefficients(g, so=so)
        self.poisson = mf.SolverCoeffs3D(g, g, g, (2,) * 6, so)     # Neumann faces
        self.smooth = mf.SolverCoeffs3D(g, g, g, (1,) * 6, so)      # Dirichlet faces
        shape = (n, n, n)
        m = n - 2
        self.zero_bc = [mf.empty_device((m, m, 2)) for _ in range(3)]
        self.rhs = mf.empty_device((m, m, m))
        self.phi = mf.empty_device(shape)
        f = lambda: mf.empty_device(shape)
        self.du = [[f() for _ in range(3)] for _ in range(3)]
        self.ddu = [[f() for _ in range(3)] for _ in range(3)]
        self.dphi = [f() for _ in range(3)]
        self.u = [f() for _ in range(3)]
        self.u1 = [f() for _ in range(3)]
        self.u2 = [f() for _ in range(3)]
        self.time = 0.0
        # initial condition: u = curl(e psi)
        gen = torch.Generator(device="cuda").manual_seed(int(seed))
        x = torch.tensor(g, device="cuda")
        e1 = 16.0 * x * x * (1.0 - x) * (1.0 - x)
        env = e1[:, None, None] * e1[None, :, None] * e1[None, None, :]
        psi = []
        r = mf.empty_device((m, m, m))
        p = f()
        for _ in range(3):
            w = torch.randn(shape[::-1], dtype=torch.float64, device="cuda",
                            generator=gen).permute(2, 1, 0)
            for _ in range(2):
                # (lap - k0^2) p = w: a low-pass filter of w, rescaled by -k0^2
                r.copy_(w[1:-1, 1:-1, 1:-1])
                self.smooth.solve_3d(r, -k0 * k0, p, *self.zero_bc)
                w = p * (-k0 * k0)
            psi.append(f())
            psi[-1].copy_(w * env)
        dpsi = [[f() for _ in range(3)] for _ in range(3)]
        for i in range(3):
            for j in range(3):
                self.dc.apply(j, 1, psi[i], out=dpsi[i][j])
        mf.flow_curl(dpsi, out=self.u)
        self.project(self.u)
        urms = float(torch.sqrt(sum((c * c).mean() for c in self.u) / 3.0))
        for c in self.u:
            c.mul_(1.0 / urms)

    def project(self, u):
        """u <- u - grad(phi), lap(phi) = div(u) with Neumann faces."""
        for j in range(3):
            self.dc.apply(j, 1, u[j], out=self.dphi[j])
        mf.flow_divergence(1.0, *self.dphi, out=self.rhs)
        # a small negative shift keeps the constant mode regular; constants
        # have no gradient, so the correction does not depend on it
        self.poisson.solve_3d(self.rhs, -1e-3, self.phi, *self.zero_bc)
        for j in range(3):
            self.dc.apply(j, 1, self.phi, out=self.dphi[j])
        mf.flow_correct(1.0, u, self.dphi)

    def divergence_norm(self):
        """RMS of div(u) over the interior, relative to RMS |grad u|."""
        for j in range(3):
            self.dc.apply(j, 1, self.u[j], out=self.dphi[j])
        d = sum(self.dphi)[1:-1, 1:-1, 1:-1]
        g = sum(c[1:-1, 1:-1, 1:-1] ** 2 for c in self.dphi)
        return float((d ** 2).mean().sqrt() / g.mean().sqrt())

    def _grads(self, u):
        for i in range(3):
            for j in range(3):
                self.dc.apply(j, 1, u[i], out=self.du[i][j])
                self.dc.apply(j, 2, u[i], out=self.ddu[i][j])

    def step(self, dt):
        """Three-stage strong-stability-preserving Runge-Kutta (Shu & Osher):
        u1 = P(u + dt R(u)), u2 = P(3/4 u + 1/4 (u1 + dt R(u1))),
        u <- P(1/3 u + 2/3 (u2 + dt R(u2))); stable for centred advection up
        to |lambda dt| = sqrt(3), where two-stage methods are not."""
        self._grads(self.u)
        mf.flow_stage(self.nu, dt, 0.0, 1.0, self.u, None, self.du, self.ddu, self.u1)
        self.project(self.u1)
        self._grads(self.u1)
        mf.flow_stage(self.nu, dt, 0.75, 0.25, self.u1, self.u, self.du, self.ddu, self.u2)
        self.project(self.u2)
        self._grads(self.u2)
        mf.flow_stage(self.nu, dt, 1.0 / 3.0, 2.0 / 3.0, self.u2, self.u, self.du, self.ddu, self.u1)
        self.project(self.u1)
        self.u, self.u1 = self.u1, self.u
        self.time += dt

    def run(self, steps, cfl=0.3, every=0, callback=None):
        """Advance `steps` steps at the given CFL number; callback(self, step)
        every `every` steps.  Raises when the flow leaves its decaying regime
        (a grid too coarse for the viscosity)."""
        ke0 = self.stats()[0]
        for it in range(1, steps + 1):
            self.step(self.cfl_dt(cfl))
            if every and it % every == 0:
                ke = self.stats()[0]
                if not np.isfinite(ke) or ke > 2.0 * ke0:
                    raise RuntimeError("box flow unstable at step %d (kinetic energy %g)" % (it, ke))
                if callback is not None:
                    callback(self, it)

    def cfl_dt(self, cfl=0.3):
        umax = max(float(c.abs().max()) for c in self.u)
        return cfl * (self.grid[1] - self.grid[0]) / max(umax, 1e-12)

    def stats(self):
        """(kinetic energy, skewness of du/dx over the interior)."""
        self.dc.apply(0, 1, self.u[0], out=self.dphi[0])
        d = self.dphi[0][2:-2, 2:-2, 2:-2]
        ke = float(sum((c * c).mean() for c in self.u) / 2.0)
        return ke, float((d ** 3).mean() / (d ** 2).mean() ** 1.5)


class PairMaker:
    """Filters fine fields to an LES grid and forms training pairs there.

    The filter is a positive smoothing kernel followed by the transfer to the
    LES grid: the differential filter v = (1 - Delta^2/24 lap)^-1 f on the
    fine grid (one Helmholtz solve, (lap + s) v = s f with s = -24/Delta^2,
    zero on the no-slip walls where velocities and their products vanish),
    Delta = width x the LES spacing, then the least-squares spline filter to
    the LES nodes.  The spline filter alone is a projection whose kernel has
    negative lobes: on a cascading flow its subgrid dissipation comes out
    with either sign at about half of the points and uncorrelated with the
    strain, which leaves nothing to learn."""

    def __init__(self, fine_grid, nc, margin=3, k=3, width=2.0):
        self.fine = np.asarray(fine_grid, dtype=np.float64)
        self.nc = nc
        self.coarse = uniform_grid(nc)
        self.filt = mf.SplineFilter(self.fine, self.coarse, xn=self.coarse, k=k)
        self.dc = mf.DerivativesCoefficients(self.coarse, so=6)
        self.les = mf.LesModel(self.coarse, self.coarse, self.coarse)
        self.margin = margin
        g = self.fine
        delta = width * (self.coarse[1] - self.coarse[0])
        self.sigma = -24.0 / (delta * delta)
        self.smoother = mf.SolverCoeffs3D(g, g, g, (1,) * 6, 6)
        n, m = g.size, g.size - 2
        self.zero_bc = [mf.empty_device((m, m, 2)) for _ in range(3)]
        self.r = mf.empty_device((m, m, m))
        self.v = mf.empty_device((n, n, n))

    def smooth(self, f):
        self.r.copy_(f[1:-1, 1:-1, 1:-1])
        self.r.mul_(self.sigma)
        self.smoother.solve_3d(self.r, self.sigma, self.v, *self.zero_bc)
        return self.v

    def filter3(self, f):
        a = self.filt.apply(self.smooth(f), 0)
        b = self.filt.apply(a, 1)
        return self.filt.apply(b, 2)

    def gradients(self, ub):
        n = self.nc
        du = [[mf.empty_device((n, n, n)) for _ in range(3)] for _ in range(3)]
        for i in range(3):
            for j in range(3):
                self.dc.apply(j, 1, ub[i], out=du[i][j])
        return du

    def pairs(self, u):
        """(X (M, 6), base (M,), target (M,)) float32 on the GPU for the
        interior LES points (margin points from the walls) with b > 0."""
        import torch
        ub = [self.filter3(c) for c in u]
        uu = [self.filter3(p) for p in mf.flow_products(u)]
        du = self.gradients(ub)
        X, b = self.les.features(du)
        t = self.les.sgs_target(ub, uu, du)
        n, m = self.nc, self.margin
        keep = torch.zeros((n, n, n), dtype=torch.bool, device="cuda")
        keep[m:n - m, m:n - m, m:n - m] = True
        keep = keep.permute(2, 1, 0).reshape(-1) & (b > 0)
        sel = torch.nonzero(keep).squeeze(1)
        return X[sel].contiguous(), b[sel].contiguous(), t[sel].contiguous()


def scaling_from(X, base, target):
    """Standardisation, training range, best constant and loss scale."""
    Xd = X.double()
    mean = Xd.mean(0).cpu().numpy()
    std = Xd.std(0).cpu().numpy()
    lo = X.min(0).values.cpu().numpy()
    hi = X.max(0).values.cpu().numpy()
    b, t = base.double(), target.double()
    c0 = float((t * b).sum() / (b * b).sum())
    loss_scale = float(1.0 / (t * t).mean())
    return dict(mean=mean, istd=1.0 / np.maximum(std, 1e-6), lo=lo, hi=hi,
                cscale=max(c0, 1e-8), loss_scale=loss_scale, c0=c0)


def fit(mlp, X, base, target, steps=2000, batch=8192, lr=2e-3, seed=0, log_every=0):
    """Adam on random mini-batches; returns (scaling, loss history)."""
    import torch
    s = scaling_from(X, base, target)
    mlp.set_scaling(s["mean"], s["istd"], s["lo"], s["hi"], s["cscale"], s["loss_scale"])
    gen = torch.Generator(device="cuda").manual_seed(int(seed))
    n = base.numel()
    hist = []
    for it in range(steps):
        idx = torch.randint(0, n, (min(batch, n),), device="cuda", generator=gen, dtype=torch.int32)
        want = bool(log_every) and (it % log_every == 0 or it == steps - 1)
        loss, _ = mlp.train_step(X, base, target, idx=idx, lr=lr, want_loss=want)
        if want:
            hist.append((it, loss))
    return s, hist


def evaluate(mlp, scaling, X, base, target):
    """Held-out mean squared error of nu for the network (best constant where
    a point leaves the training range) and for the best constant coefficient,
    with nu = 0 and the correlations for reference."""
    import torch
    c = mlp.predict(X).double().clamp_min(0.0)
    lo = torch.tensor(scaling["lo"], device="cuda")
    hi = torch.tensor(scaling["hi"], device="cuda")
    inside = ((X >= lo) & (X <= hi)).all(1)
    c = torch.where(inside, c, torch.full_like(c, scaling["c0"]))
    b, t = base.double(), target.double()
    nu_m = c * b
    nu_c = scaling["c0"] * b
    mse = lambda a: float(((a - t) ** 2).mean())
    corr = lambda a: float(torch.corrcoef(torch.stack([a, t]))[0, 1])
    return dict(mse_mlp=mse(nu_m), mse_const=mse(nu_c), mse_zero=float((t * t).mean()),
                corr_mlp=corr(nu_m), corr_const=corr(nu_c), inside=float(inside.double().mean()),
                n=int(t.numel()))
