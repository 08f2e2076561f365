"""Stretch-move ensemble sampler (gbgpu_gb300.mcmc.StretchSampler) on the
fused likelihood kernel.

Self-consistency (the reference's own sampler is the external Eryn package):
a captured CUDA graph of steps reproduces the eager steps exactly, the
cached log-likelihoods equal a fresh GBGPU.get_ll of the walkers, and
ensembles started in a small ball around injected sources spread out,
accept at a healthy rate and stay on the posterior.  The move itself is
checked against known targets on CPU (tests/test_stretch_cpu.py).
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

T_OBS = 4 * 31557600.0
DT = 10.0
FREE = (0, 1, 2, 4, 5, 6, 7, 8)


def _setup(B=16, W=32, N=256, seed=7):
    from gbgpu_gb300 import GBGPU
    from gbgpu_gb300.mcmc import StretchSampler
    from gbgpu_gb300.sensitivity import A1TDISens
    rng = np.random.default_rng(seed)
    Tu = int(T_OBS / DT) * DT
    q0 = np.rint(rng.uniform(3.0e-3, 3.2e-3, B) * Tu)
    fdot = 10 ** rng.uniform(-17, -16, B)
    f0 = (q0 + rng.uniform(-0.3, 0.3, B)) / Tu
    truth = np.array([10 ** rng.uniform(-22.0, -21.5, B), f0, fdot, 11 / 3 * fdot ** 2 / f0,
                      rng.uniform(0.5, 5.5, B), np.arccos(rng.uniform(-0.9, 0.9, B)),
                      rng.uniform(0.3, 2.8, B), rng.uniform(0.5, 5.5, B),
                      np.arcsin(rng.uniform(-0.9, 0.9, B))])
    s0 = int(q0.min()) - 2 * N
    L = int(q0.max()) + 2 * N - s0
    S = A1TDISens.get_Sn((np.arange(L) + s0) / Tu)
    gb = GBGPU(precision="mixed")
    tmpl = torch.zeros((1, 2, L), dtype=torch.complex128, device="cuda")
    gb.generate_global_template(truth.T, np.zeros(B, np.int32), tmpl, N=N, T=T_OBS, dt=DT,
                                start_freq_ind=s0)
    noise = np.sqrt(S * Tu / 4) * (rng.standard_normal((2, L)) + 1j * rng.standard_normal((2, L)))
    data = [tmpl[0, c] + torch.as_tensor(noise[c], device="cuda") for c in range(2)]
    Sd = torch.as_tensor(S, device="cuda")
    gb.d_d = 0.0
    F = GBGPU(precision="fp64").fisher_matrices(truth, N=N, T=T_OBS, dt=DT, inds=FREE,
                                                return_gpu=True)
    sig = (1.0 / torch.sqrt(torch.diagonal(F, dim1=1, dim2=2))).T          # (8, B)
    g = torch.Generator(device="cuda").manual_seed(seed)
    x = torch.as_tensor(truth, device="cuda")[:, :, None].repeat(1, 1, W)
    x[list(FREE)] += 0.1 * sig[:, :, None] * torch.randn((len(FREE), B, W), generator=g,
                                                         device="cuda", dtype=torch.float64)

    def make():
        return StretchSampler(gb, x, data, [Sd, Sd], N=N, T=T_OBS, dt=DT, start_freq_ind=s0,
                              free=FREE)
    return gb, make, truth, sig, g, (data, Sd, s0, N)


def test_graph_replay_matches_eager_steps():
    from gbgpu_gb300.mcmc import stretch_draws
    gb, make, truth, sig, g, _ = _setup()
    a, b = make(), make()
    u, j, lu = stretch_draws(6, a.B, a.Wh, g, "cuda")
    for s in range(6):
        a.step(u[s], j[s], lu[s])
    b.capture(u, j, lu)
    b.replay()
    torch.cuda.synchronize()
    assert torch.equal(a.x, b.x)
    assert torch.equal(a.logL, b.logL)
    assert torch.equal(a.accepted, b.accepted)
    assert int(a.accepted.sum()) > 0


def test_cached_loglike_matches_fresh_get_ll():
    from gbgpu_gb300.mcmc import stretch_draws
    gb, make, truth, sig, g, (data, Sd, s0, N) = _setup()
    smp = make()
    u, j, lu = stretch_draws(20, smp.B, smp.Wh, g, "cuda")
    for s in range(20):
        smp.step(u[s], j[s], lu[s])
    flat = smp.x.reshape(smp.x.shape[0], -1).contiguous()
    like = gb.get_ll(flat, data, [Sd, Sd], N=N, T=T_OBS, dt=DT, start_freq_ind=s0)
    hh = np.abs(gb.h_h.real.cpu().numpy())
    cached = smp.logL.reshape(-1).cpu().numpy()
    # the two evaluations may pack binaries into tiles differently (summation order)
    assert np.all(np.abs(like - cached) <= 1e-6 * np.maximum(1.0, hh))


def test_ensembles_spread_and_stay_on_the_posterior():
    from gbgpu_gb300.mcmc import stretch_draws
    gb, make, truth, sig, g, _ = _setup()
    smp = make()
    steps = 150
    u, j, lu = stretch_draws(steps, smp.B, smp.Wh, g, "cuda")
    smp.capture(u, j, lu)
    smp.replay()
    torch.cuda.synchronize()
    frac = smp.accepted.sum().item() / (smp.B * smp.W * steps)
    assert 0.1 < frac < 0.9, frac
    assert bool(torch.isfinite(smp.logL).all())
    xf = smp.x[list(FREE)]                                    # (8, B, W)
    spread = xf.std(2) / sig                                  # in Fisher sigmas
    assert float(spread.median()) > 0.3                       # grew from the 0.1-sigma ball
    off = (xf.mean(2) - torch.as_tensor(truth[list(FREE)], device="cuda")).abs() / sig
    # noise shifts the posterior by ~1 sigma; weakly constrained (iota, psi) directions
    # may wander further than their Fisher sigma
    assert float(off.median()) < 2.0 and bool(torch.isfinite(off).all())


def test_stretch_sampler_in_the_pair_form():
    """The stretch-move ensemble on the pair form's fused likelihood (the same
    graph-captured steps): the cached log-likelihoods equal a fresh pair-form
    get_ll of the final walkers to 1e-9 of <h|h> (the mixed form: 1e-6)."""
    from gbgpu_gb300 import GBGPU
    from gbgpu_gb300.mcmc import StretchSampler, stretch_draws
    _, make, truth, sig, g, (data, Sd, s0, N) = _setup(B=8, W=16)
    gb = GBGPU(precision="pair")
    smp = StretchSampler(gb, make().x.clone(), data, [Sd, Sd], N=N, T=T_OBS, dt=DT,
                         start_freq_ind=s0, free=FREE, precision="pair")
    u, j, lu = stretch_draws(6, smp.B, smp.Wh, g, "cuda")
    smp.capture(u, j, lu)
    smp.replay()
    torch.cuda.synchronize()
    assert int(smp.accepted.sum()) > 0
    flat = smp.x.reshape(smp.x.shape[0], -1).contiguous()
    gb.d_d = 0.0
    like = gb.get_ll(flat, data, [Sd, Sd], N=N, T=T_OBS, dt=DT, start_freq_ind=s0,
                     precision="pair")
    hh = np.abs(gb.h_h.real.cpu().numpy())
    cached = smp.logL.reshape(-1).cpu().numpy()
    err = np.max(np.abs(like - cached) / np.maximum(1.0, hh))
    print(f"pair stretch sampler: cached vs fresh logL, max error / <h|h> {err:.2e}")
    assert err < 1e-9
