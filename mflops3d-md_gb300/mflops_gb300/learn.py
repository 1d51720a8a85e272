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

    def __init__(self, n, nu, seed, k0=30.0, so=6, precision=None, refine=2):
        import torch
        self.n = n
        self.nu = nu
        # projection solves: plain FP64 by default, or a mixed mode with
        # `refine` FP64-residual refinement steps (axes up to 256 points)
        self.precision = mf.MF_PREC_FP64 if precision is None else precision
        self.refine = refine
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
        self.poisson.solve_3d(self.rhs, -1e-3, self.phi, *self.zero_bc, precision=self.precision,
                              refine=self.refine if self.precision != mf.MF_PREC_FP64 else -1)
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


# ---------------------------------------------------------------------------
# A-posteriori judgement: LES runs of the time step against the filtered fine run
# ---------------------------------------------------------------------------

def profile_and_spectrum(u, margin=1):
    """(mean profile, spectrum) of a velocity field on a box grid: the
    kinetic energy averaged over x-z planes as a function of y, and the
    energy spectrum along x (squared moduli of the FFT of each interior x
    line, averaged over the interior y, z points and the three components).
    Both as float64 torch tensors."""
    import torch
    m = margin
    ke = sum(c * c for c in u) * 0.5
    prof = ke[:, m:ke.shape[1] - m, :].mean(dim=(0, 2))
    spec = 0.0
    for c in u:
        inner = c[1:-1, m:c.shape[1] - m, m:c.shape[2] - m]
        spec = spec + (torch.fft.rfft(inner, dim=0).abs() ** 2).mean(dim=(1, 2))
    return prof, spec / 3.0


def profile_error(a, b):
    """rel-L2 distance of two mean profiles."""
    return float((a - b).norm() / b.norm())


def spectrum_error(a, b, kmax=None):
    """Mean |log(E_a(k) / E_b(k))| over the wavenumbers 1..kmax."""
    import torch
    k = slice(1, kmax) if kmax else slice(1, None)
    return float(torch.log(a[k] / b[k]).abs().mean())


class APosteriori:
    """LES runs of the Navier-Stokes time step (mf_navier_step, one domain,
    no-slip walls, no forcing: nmodes = 0, no flow-rate term) on the LES grid,
    started from the filtered fine field and compared with the filtered fine
    run at the same times.  Models: none (les_type 0), Smagorinsky with the
    training's best constant (les_c^2 = c0), and the learned coefficient
    (les_type 4, Smagorinsky with c0 where the features leave the training
    range).  The plain model is the yardstick: the network's errors are
    reported next to it."""

    def __init__(self, fine_flow, pairs, mlp, scaling, precision=None, refine=1):
        self.fine = fine_flow
        self.pairs = pairs
        self.mlp = mlp
        self.c0 = scaling["c0"]
        self.precision = mf.MF_PREC_3XTF32 if precision is None else precision
        self.refine = refine

    def filtered(self):
        """The fine velocity filtered to the LES grid, its wall values set to
        the no-slip data the time step imposes (the filter leaves them at
        ~1% of the velocity scale)."""
        out = [self.pairs.filter3(c).clone() for c in self.fine.u]
        for c in out:
            c[0].zero_(); c[-1].zero_()
            c[:, 0].zero_(); c[:, -1].zero_()
            c[:, :, 0].zero_(); c[:, :, -1].zero_()
        return out

    def _les(self, start, les_type, dt):
        g = self.pairs.coarse
        kw = dict(ts=dt, reynolds=1.0 / self.fine.nu, nmodes=0, flow_rate=0, precision=self.precision,
                  refine=self.refine)
        if les_type:
            kw.update(les_type=les_type, les_c=float(np.sqrt(max(self.c0, 0.0))))
        nav = mf.NavierStokes3D(g, g, g, **kw)
        if les_type == mf.MF_LES_LEARNED:
            nav.set_les_network(self.mlp)
        for lev in range(4):
            for q, var in enumerate("uvw"):
                nav.set_field(var, lev, start[q])
        return nav

    def run(self, t_end, checkpoints=4, dt_les=None, cfl=0.1, fine_cfl=0.3, models=(0, 1, 4)):
        """Advance the fine flow (RK3 at fine_cfl) and the LES runs (the
        time step at `cfl` on the LES grid: its explicit extrapolated
        advection needs a smaller CFL number than the Runge-Kutta fine run)
        to t_end; at `checkpoints` equally spaced times compare mean profile
        and spectrum.  Returns a dict per model: lists of (time, profile
        error, spectrum error) and the final divergence norm, plus the LES
        step time in ms."""
        import torch
        start = self.filtered()
        h = self.pairs.coarse[1] - self.pairs.coarse[0]
        umax = max(float(c.abs().max()) for c in start)
        dt = dt_les or cfl * h / max(umax, 1e-12)
        per = max(1, int(round(t_end / checkpoints / dt)))
        dt = t_end / checkpoints / per
        runs = {m: self._les(start, m, dt) for m in models}
        out = {m: {"errors": []} for m in models}
        t = self.fine.time
        t0 = t
        step_ms = {m: 0.0 for m in models}
        for c in range(1, checkpoints + 1):
            target = t0 + c * t_end / checkpoints
            while self.fine.time < target - 1e-12:
                self.fine.step(min(self.fine.cfl_dt(fine_cfl), target - self.fine.time))
            ref = profile_and_spectrum(self.filtered())
            for m, nav in runs.items():
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                for _ in range(per):
                    nav.step()
                b.record()
                torch.cuda.synchronize()
                step_ms[m] += a.elapsed_time(b) / per / checkpoints
                les = profile_and_spectrum([nav.field(v, 3) for v in "uvw"])
                kmax = les[1].numel() // 2
                out[m]["errors"].append((target, profile_error(les[0], ref[0]),
                                         spectrum_error(les[1], ref[1], kmax)))
        for m, nav in runs.items():
            d = nav.step(diagnostics=True)
            out[m]["divergence"] = d["div"]
            out[m]["step_ms"] = step_ms[m]
            out[m]["profile_error_mean"] = float(np.mean([e[1] for e in out[m]["errors"]]))
            out[m]["spectrum_error_mean"] = float(np.mean([e[2] for e in out[m]["errors"]]))
            nav.close()
        out["dt_les"] = dt
        return out
