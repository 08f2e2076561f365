"""Samplers on the GPU that drive the fused kernels: an ensemble swap sampler
(the caller of the swap likelihood), an affine-invariant stretch-move
ensemble (the fused likelihood) and HMC (the fused likelihood + gradient).

Swap sampler:

Each of W walkers holds K sources and a residual r_w = d - sum_k h(theta_wk)
restricted to a frequency band.  One proposal step replaces, in every walker,
source k_s by a proposed one, computes dlogL with the swap kernel, accepts
with probability min(1, exp(dlogL)) and updates the residual of accepted
walkers by adding h_old - h_new (a template fill with amplitudes +-amp, exact
because h is linear in amp).  All proposals and uniform draws are prepared on
the device beforehand, so a block of steps is captured and replayed as one
CUDA graph.  Sources in a walker are assumed not to change the N that the
batch is evaluated with.
"""

import math

import torch


class SwapSampler:
    """Ensemble swap sampler over W walkers of K sources each (see the module
    docstring): one swap-likelihood launch and one residual update per step,
    any number of steps captured as one CUDA graph."""

    def __init__(self, gb, params, data, psd, N, T, dt, start_freq_ind, tdi2=False,
                 precision="mixed"):
        """``params``: (nparams, W, K) FP64 CUDA tensor of the current sources;
        ``data``: [A, E] (Lb,) complex128 band of the data; ``psd``: [A, E] (Lb,)."""
        self.gb = gb
        self.params = params.contiguous()
        self.nparams, self.W, self.K = params.shape
        self.kw = dict(N=N, T=T, dt=dt, tdi2=tdi2, precision=precision)
        self.s0 = int(start_freq_ind)
        self.psd = [p.contiguous() for p in psd]
        Lb = data[0].shape[0]
        dev = params.device
        # residuals as (channel, walker, bin): each channel is a contiguous
        # (W, Lb) array whose rows the likelihood selects with data_index
        self.res = torch.empty((2, self.W, Lb), dtype=torch.complex128, device=dev)
        self.res[0] = data[0]
        self.res[1] = data[1]
        # r_w = d - sum_k h(theta_wk): add every source with amplitude -amp
        allp = self.params.reshape(self.nparams, self.W * self.K).clone()
        allp[0] = -allp[0]
        gw = torch.arange(self.W, device=dev, dtype=torch.int32).repeat_interleave(self.K)
        gb.add_to_templates(allp.contiguous(), gw, (self.res[0], self.res[1]),
                            start_freq_ind=self.s0, **self.kw)
        self.walkers = torch.arange(self.W, device=dev, dtype=torch.int32)
        self.accepted = torch.zeros(self.W, dtype=torch.int64, device=dev)
        self.graph = None

    def step(self, k, proposal, log_u):
        """One Metropolis swap step for source ``k`` of every walker.

        ``proposal``: (nparams, W) proposed sources; ``log_u``: (W,) log uniforms.
        Returns dlogL (W,).
        """
        old = self.params[:, :, k].contiguous()
        dl = self.gb.swap_likelihood(old, proposal, [self.res[0], self.res[1]], self.psd,
                                     data_index=self.walkers, start_freq_ind=self.s0,
                                     return_tensor=True, **self.kw)
        acc = log_u < dl
        accf = acc.to(torch.float64)
        # residual += h_old - h_new for accepted walkers (amplitudes zeroed otherwise)
        upd = torch.cat([old, proposal], dim=1).clone()
        upd[0, :self.W] = old[0] * accf
        upd[0, self.W:] = -proposal[0] * accf
        groups = torch.cat([self.walkers, self.walkers])
        self.gb.add_to_templates(upd.contiguous(), groups, (self.res[0], self.res[1]),
                                 start_freq_ind=self.s0, **self.kw)
        self.params[:, :, k] = torch.where(acc[None, :], proposal, old)
        self.accepted += acc
        return dl

    def capture(self, ks, proposals, log_us):
        """Capture len(ks) steps (proposals (S, nparams, W), log_us (S, W)) as one graph."""
        self.ks = list(ks)
        self.proposals = proposals
        self.log_us = log_us
        # warm-up outside capture: builds plans, workspaces and cached kernels
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self._snapshot = (self.params.clone(), self.res.clone(), self.accepted.clone())
            self.step(self.ks[0], self.proposals[0], self.log_us[0])
            self.params.copy_(self._snapshot[0])
            self.res.copy_(self._snapshot[1])
            self.accepted.copy_(self._snapshot[2])
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.dls = [self.step(k, self.proposals[i], self.log_us[i])
                        for i, k in enumerate(self.ks)]
        # the graph holds raw pointers into the plans' tile lists, queues and
        # workspaces: keep those plans alive for as long as the graph
        self._graph_plans = list(self.gb._plans.values())
        return self.graph

    def replay(self):
        """Replay the captured graph (all its steps)."""
        self.graph.replay()

    def log_likelihood(self):
        """-1/2 <r_w|r_w> of every walker's residual (the band's contribution)."""
        Tu = int(self.kw["T"] / self.kw["dt"]) * self.kw["dt"]
        w = 4.0 / Tu
        out = torch.zeros(self.W, dtype=torch.float64, device=self.res.device)
        for ch in range(2):
            out += w * (self.res[ch].abs() ** 2 / self.psd[ch][None, :]).sum(1)
        return -0.5 * out


def random_proposals(params_k, scale, gen):
    """Gaussian moves of (nparams, W) sources: relative for amp, absolute otherwise."""
    p = params_k.clone()
    z = torch.randn(p.shape, generator=gen, device=p.device, dtype=p.dtype)
    p[0] = p[0] * (1 + scale[0] * z[0])
    for i in range(1, p.shape[0]):
        p[i] = p[i] + scale[i] * z[i]
    return p


def log_uniforms(W, steps, gen, device):
    """(steps, W) logs of uniforms in (0, 1], clamped away from log 0."""
    u = torch.rand((steps, W), generator=gen, device=device, dtype=torch.float64)
    return torch.log(u.clamp_min(math.ldexp(1.0, -60)))


class HMCSampler:
    """Hamiltonian Monte Carlo over the source parameters of a batch of
    independent binaries, driven by the fused likelihood + gradient kernel.

    Every binary is its own chain with target logL (the mixed fused
    likelihood, the one the gradient belongs to).  The free parameters
    (default amp, f0, fdot, phi0, iota, psi, lam, beta; fddot is held fixed)
    move in whitened coordinates x = theta / scale with unit mass, so
    ``scales`` (e.g. Fisher-diagonal standard deviations) set the metric.  A
    transition is ``n_leapfrog`` leapfrog steps (one kernel launch each: the
    gradient at the end of a step is the one the next step starts with)
    followed by a Metropolis test on H = -logL + |p|^2 / 2.  Momenta and
    uniform draws are prepared on the device beforehand, so any number of
    transitions is captured and replayed as one CUDA graph.  The reference
    has no counterpart (its derivatives are finite differences).
    """

    FREE = (0, 1, 2, 4, 5, 6, 7, 8)

    def __init__(self, gb, params, data, psd, N, T, dt, scales, step_size, n_leapfrog,
                 start_freq_ind=0, tdi2=False, data_index=None, noise_index=None, free=FREE):
        import ctypes
        from . import _native as nat
        self._nat, self._ctypes = nat, ctypes
        self.gb = gb
        dev = gb.device
        self.params = params.to(device=dev, dtype=torch.float64).clone().contiguous()
        npar, B = self.params.shape
        if npar != gb.NPARAMS:
            raise ValueError(f"params must be ({gb.NPARAMS}, B)")
        if gb.d_d is None:
            raise ValueError("set gb.d_d before sampling")
        self.B = B
        self.free = torch.as_tensor(list(free), device=dev, dtype=torch.long)
        nf = len(free)
        s = torch.as_tensor(scales, device=dev, dtype=torch.float64)
        self.scale = (s[:, None].expand(nf, B) if s.ndim == 1 else s).contiguous()
        self.eps = float(step_size)
        self.n_leapfrog = int(n_leapfrog)
        Tu = int(T / dt) * dt
        dd, pp, L, di, ni = gb._prepare_data(data, psd, data_index, noise_index, B)
        self.la = gb._ll_args(dd, pp, L, di, ni, Tu)
        self.d_h = torch.zeros(B, dtype=torch.complex128, device=dev)
        self.h_h = torch.zeros(B, dtype=torch.complex128, device=dev)
        self.grad = torch.zeros((npar, B), dtype=torch.float64, device=dev)
        self.d_d = torch.as_tensor(gb.d_d, dtype=torch.float64, device=dev)
        self._lib = nat.lib()

        def bind(tile, bps):
            plan = gb._plan(N, Tu, "mixed", tdi2, npar, tile, bps)
            self.args = plan.args(self.params, start_freq_ind, gb._status, grad=True)

        def run(tile, bps):
            bind(tile, bps)
            self._evaluate()
        self.args = None
        bind(*gb._launch_shape("grad", N, B, "mixed", tdi2, npar, run))
        # state at the current point
        self._evaluate()
        self.logL = self._like().clone()
        self.g = self.grad[self.free].clone()
        self.accepted = torch.zeros(B, dtype=torch.int64, device=dev)
        self.dH = torch.zeros(B, dtype=torch.float64, device=dev)
        self.graph = None

    def _evaluate(self):
        nat, ct = self._nat, self._ctypes
        rc = self._lib.gbx_waveform_ll_grad(ct.byref(self.args), ct.byref(self.la),
                                            nat.ptr(self.d_h), nat.ptr(self.h_h),
                                            nat.ptr(self.grad), nat.stream_handle())
        nat.check(rc, "gbx_waveform_ll_grad")

    def _like(self):
        return -0.5 * (self.d_d + self.h_h.real - 2.0 * self.d_h.real)

    def leapfrog(self, p, g):
        """``n_leapfrog`` leapfrog steps from the current parameters (moved in
        place) with whitened momenta ``p`` and free-parameter gradient ``g``
        there.  Returns (p, g, logL) at the end point."""
        f, s, eps = self.free, self.scale, self.eps
        for _ in range(self.n_leapfrog):
            p = p + (0.5 * eps) * (g * s)
            self.params[f] = self.params[f] + eps * (s * p)
            self._evaluate()
            g = self.grad[f]
            p = p + (0.5 * eps) * (g * s)
        return p, g, self._like()

    def transition(self, mom, log_u):
        """One HMC transition of every chain: ``mom`` (nfree, B) standard normal
        momenta, ``log_u`` (B,) log uniforms.  Returns the accept mask."""
        f = self.free
        q0 = self.params[f].clone()
        H0 = -self.logL + 0.5 * (mom * mom).sum(0)
        p, g, like = self.leapfrog(mom.clone(), self.g)
        dH = (-like + 0.5 * (p * p).sum(0)) - H0
        acc = (log_u < -dH) & torch.isfinite(dH)
        self.params[f] = torch.where(acc[None, :], self.params[f], q0)
        self.logL.copy_(torch.where(acc, like, self.logL))
        self.g.copy_(torch.where(acc[None, :], g, self.g))
        self.accepted += acc
        self.dH.copy_(dH)
        return acc

    def capture(self, moms, log_us):
        """Capture len(moms) transitions (moms (S, nfree, B), log_us (S, B)) as one graph."""
        self.moms, self.log_us = moms, log_us
        snap = (self.params.clone(), self.logL.clone(), self.g.clone(), self.accepted.clone())
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):                 # warm-up outside capture
            self.transition(moms[0], log_us[0])
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        for dst, src in zip((self.params, self.logL, self.g, self.accepted), snap):
            dst.copy_(src)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            for i in range(moms.shape[0]):
                self.transition(moms[i], log_us[i])
        self._graph_keep = (self.args, self.la)
        return self.graph

    def replay(self):
        """Replay the captured graph (all its steps)."""
        self.graph.replay()


# ---------------------------------------------------------------------------
# affine-invariant ensemble (stretch move)
# ---------------------------------------------------------------------------

def stretch_z(u, a=2.0):
    """Stretch factors z with density g(z) proportional to 1/sqrt(z) on
    [1/a, a], from uniforms u by the inverse CDF: z = ((a - 1) u + 1)^2 / a
    (Goodman & Weare 2010, eq. 9)."""
    return ((a - 1.0) * u + 1.0) ** 2 / a


def stretch_draws(steps, B, Wh, gen, device, dtype=torch.float64):
    """Random numbers for ``steps`` stretch-move steps of B ensembles of 2 Wh
    walkers: uniforms for z, partner indices into the other half, and log
    uniforms for the accept test, each (steps, 2, B, Wh)."""
    u = torch.rand((steps, 2, B, Wh), generator=gen, device=device, dtype=dtype)
    j = torch.randint(0, Wh, (steps, 2, B, Wh), generator=gen, device=device)
    lu = torch.rand((steps, 2, B, Wh), generator=gen, device=device, dtype=dtype)
    return u, j, torch.log(lu.clamp_min(math.ldexp(1.0, -60)))


def stretch_update(x, logL, accepted, h, u, j, log_u, loglike, free, a=2.0, bounds=None):
    """Update half ``h`` (0 or 1) of every ensemble in place by one stretch
    move (Goodman & Weare 2010; the move of emcee and Eryn).

    ``x`` (npar, B, W) walkers of B independent ensembles, W even; ``logL``
    (B, W) their log-likelihoods; ``accepted`` (B, W) counters.  Walker k of
    the half moves to Y = C_j + z (X_k - C_j) in the ``free`` coordinates,
    with C_j the partner ``j`` (B, W/2) of the other half and z = stretch_z(u),
    and is accepted when log_u < (n_free - 1) log z + logL(Y) - logL(X) and Y
    lies inside ``bounds`` ((n_free, 2) lower/upper, optional).  ``loglike``
    maps (npar, B, W/2) points to (B, W/2) log-likelihoods.  Returns the
    accept mask (B, W/2)."""
    npar, B, W = x.shape
    Wh = W // 2
    sl = slice(h * Wh, (h + 1) * Wh)
    X = x[:, :, sl]
    C = x[:, :, Wh:] if h == 0 else x[:, :, :Wh]
    z = stretch_z(u, a)
    Cj = torch.gather(C, 2, j[None].expand(npar, B, Wh))
    Y = X.clone()
    Y[free] = Cj[free] + z[None] * (X[free] - Cj[free])
    ll = loglike(Y)
    cur = logL[:, sl]
    lp = (len(free) - 1) * torch.log(z) + ll - cur
    if bounds is not None:
        yf = Y[free]
        ok = ((yf >= bounds[:, 0, None, None]) & (yf <= bounds[:, 1, None, None])).all(0)
        lp = torch.where(ok, lp, torch.full_like(lp, -math.inf))
    acc = (log_u < lp) & torch.isfinite(ll)
    X.copy_(torch.where(acc[None], Y, X))
    cur.copy_(torch.where(acc, ll, cur))
    accepted[:, sl] += acc
    return acc


class StretchSampler:
    """Affine-invariant ensemble sampler (stretch move) over B independent
    binaries with W walkers each, driven by the fused likelihood kernel.

    A step updates the two halves of every ensemble in turn; each half-update
    evaluates the B W/2 proposed points in one fused waveform + likelihood
    launch (the plan is bound once to a fixed proposal buffer), so the random
    numbers of any number of steps (``stretch_draws``) are prepared on the
    device and the steps are captured and replayed as one CUDA graph.  The
    target is the likelihood (flat prior inside optional ``bounds`` on the
    free parameters); fddot is held fixed by default.  The reference's
    sampler-facing caller is an ensemble sampler of this kind (Eryn, its
    optional ``sampling`` dependency); the move itself follows Goodman &
    Weare (2010).
    """

    FREE = (0, 1, 2, 4, 5, 6, 7, 8)

    def __init__(self, gb, params, data, psd, N, T, dt, a=2.0, start_freq_ind=0, tdi2=False,
                 free=FREE, bounds=None, precision="mixed"):
        import ctypes
        from . import _native as nat
        self._nat, self._ctypes = nat, ctypes
        self.gb = gb
        dev = gb.device
        x = params.to(device=dev, dtype=torch.float64)
        if x.ndim != 3:
            raise ValueError("params must be (nparams, B, W)")
        npar, B, W = x.shape
        if npar != gb.NPARAMS:
            raise ValueError(f"params must be ({gb.NPARAMS}, B, W)")
        if W < 4 or W % 2:
            raise ValueError("the number of walkers per ensemble must be even and >= 4")
        self.x = x.clone().contiguous()
        self.B, self.W, self.Wh = B, W, W // 2
        self.a = float(a)
        self.free = torch.as_tensor(list(free), device=dev, dtype=torch.long)
        self.bounds = None if bounds is None else \
            torch.as_tensor(bounds, device=dev, dtype=torch.float64).reshape(len(free), 2)
        n = B * self.Wh
        self.prop = torch.empty((npar, n), dtype=torch.float64, device=dev)
        Tu = int(T / dt) * dt
        dd, pp, L, di, ni = gb._prepare_data(data, psd, None, None, n)
        self.la = gb._ll_args(dd, pp, L, di, ni, Tu)
        self.d_h = torch.zeros(n, dtype=torch.complex128, device=dev)
        self.h_h = torch.zeros(n, dtype=torch.complex128, device=dev)
        self.d_d = 0.0 if gb.d_d is None else float(gb.d_d)
        self._lib = nat.lib()
        self.prop.copy_(self.x[:, :, :self.Wh].reshape(npar, n))

        def bind(tile, bps):
            plan = gb._plan(N, Tu, precision, tdi2, npar, tile, bps)
            self.args = plan.args(self.prop, start_freq_ind, gb._status)
            self._plan_keep = plan

        def run(tile, bps):
            bind(tile, bps)
            self._evaluate()
        self.args = None
        bind(*gb._launch_shape("ll", N, n, precision, tdi2, npar, run))
        self.logL = torch.empty((B, W), dtype=torch.float64, device=dev)
        for h in (0, 1):
            self.logL[:, h * self.Wh:(h + 1) * self.Wh] = self._loglike(
                self.x[:, :, h * self.Wh:(h + 1) * self.Wh])
        self.accepted = torch.zeros((B, W), dtype=torch.int64, device=dev)
        self.graph = None

    def _evaluate(self):
        nat, ct = self._nat, self._ctypes
        rc = self._lib.gbx_waveform_ll(ct.byref(self.args), ct.byref(self.la), nat.ptr(self.d_h),
                                       nat.ptr(self.h_h), nat.stream_handle())
        nat.check(rc, "gbx_waveform_ll")

    def _loglike(self, Y):
        """log-likelihoods (B, W/2) of the points Y (npar, B, W/2)."""
        self.prop.copy_(Y.reshape(self.prop.shape))
        self._evaluate()
        like = -0.5 * (self.d_d + self.h_h.real - 2.0 * self.d_h.real)
        return like.reshape(self.B, self.Wh)

    def step(self, u, j, log_u):
        """One step: both halves of every ensemble, ``u``/``j``/``log_u`` of
        shape (2, B, W/2) as made by ``stretch_draws``."""
        for h in (0, 1):
            stretch_update(self.x, self.logL, self.accepted, h, u[h], j[h], log_u[h],
                           self._loglike, self.free, self.a, self.bounds)

    def capture(self, us, js, log_us):
        """Capture len(us) steps (arrays (S, 2, B, W/2)) as one CUDA graph."""
        self.us, self.js, self.log_us = us, js, log_us
        snap = (self.x.clone(), self.logL.clone(), self.accepted.clone())
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):                 # warm-up outside capture
            self.step(us[0], js[0], log_us[0])
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        for dst, src in zip((self.x, self.logL, self.accepted), snap):
            dst.copy_(src)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            for i in range(us.shape[0]):
                self.step(us[i], js[i], log_us[i])
        self._graph_keep = (self.args, self.la, self._plan_keep)
        return self.graph

    def replay(self):
        """Replay the captured graph (all its steps)."""
        self.graph.replay()
