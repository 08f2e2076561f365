"""Swap sampler (gbgpu_gb300.mcmc) -- the caller of the swap likelihood.

Checks that a block of proposal steps replayed as a CUDA graph gives the same
state as the same steps run eagerly, that the incrementally updated walker
residuals equal d minus the sum of the current sources recomputed from
scratch, and that dlogL of accepted swaps equals the change of the band's
-1/2 <r|r>.
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

T_OBS = 4 * 31557600.0
DT = 5.0


def _setup(W=6, K=12, N=256, seed=3):
    from gbgpu_gb300 import GBGPUThirdBody
    from gbgpu_gb300.sensitivity import A1TDISens
    rng = np.random.default_rng(seed)
    Tu = int(T_OBS / DT) * DT
    s0 = int(2e-3 * Tu)
    Lb = 4096
    f0 = (s0 + 600 + rng.uniform(0, Lb - 1200, (W, K))) / Tu
    fdot = 10 ** rng.uniform(-18, -16, (W, K))
    P2 = 10 ** rng.uniform(0, np.log10(40), (W, K))
    p = np.stack([10 ** rng.uniform(-22.3, -21.7, (W, K)), f0, fdot, 11 / 3 * fdot ** 2 / f0,
                  rng.uniform(0, 2 * np.pi, (W, K)), np.arccos(rng.uniform(-1, 1, (W, K))),
                  rng.uniform(0, np.pi, (W, K)), rng.uniform(0, 2 * np.pi, (W, K)),
                  np.arcsin(rng.uniform(-1, 1, (W, K))), 10 ** rng.uniform(-2, 2, (W, K)),
                  rng.uniform(0, 2 * np.pi, (W, K)), rng.uniform(0, 0.9, (W, K)), P2,
                  rng.uniform(0, 1, (W, K)) * P2])
    S = A1TDISens.get_Sn((np.arange(Lb) + s0) / Tu)
    noise = np.sqrt(S * Tu / 4) * (rng.standard_normal((2, Lb)) + 1j * rng.standard_normal((2, Lb)))
    data = [torch.as_tensor(noise[c], device="cuda") for c in range(2)]
    psd = [torch.as_tensor(S, device="cuda")] * 2
    gb = GBGPUThirdBody(precision="mixed")
    return gb, torch.as_tensor(p, device="cuda"), data, psd, s0, N, rng


def _proposals(sampler, steps, seed):
    from gbgpu_gb300.mcmc import random_proposals, log_uniforms
    g = torch.Generator(device="cuda").manual_seed(seed)
    scale = torch.tensor([0.05, 2e-9, 0, 0, 0.2, 0.1, 0.1, 0.02, 0.02, 0.05, 0.1, 0.02, 0.01, 0.01],
                         dtype=torch.float64, device="cuda")
    ks = [i % sampler.K for i in range(steps)]
    props = torch.stack([random_proposals(sampler.params[:, :, k], scale, g) for k in ks])
    props[:, 11].clamp_(0.0, 0.9)
    return ks, props, log_uniforms(sampler.W, steps, g, "cuda")


def test_graph_replay_equals_eager_and_residuals_stay_consistent():
    from gbgpu_gb300.mcmc import SwapSampler
    gb, p, data, psd, s0, N, rng = _setup()
    kw = dict(N=N, T=T_OBS, dt=DT, start_freq_ind=s0)
    eager = SwapSampler(gb, p.clone(), data, psd, **kw)
    graph = SwapSampler(gb, p.clone(), data, psd, **kw)
    ks, props, lus = _proposals(eager, 8, 11)
    before = eager.log_likelihood()
    dls = []
    for i, k in enumerate(ks):
        ll0 = eager.log_likelihood()
        dl = eager.step(k, props[i], lus[i])
        acc_now = (lus[i] < dl)
        ll1 = eager.log_likelihood()
        # accepted walkers: dlogL equals the change of -1/2 <r|r>; others unchanged
        d_ll = (ll1 - ll0).cpu().numpy()
        dl_n = dl.cpu().numpy()
        a = acc_now.cpu().numpy()
        scale = 1e-5 * np.maximum(1.0, np.abs(ll0.cpu().numpy()))
        assert np.all(np.abs(d_ll[a] - dl_n[a]) < scale[a])
        assert np.all(np.abs(d_ll[~a]) < scale[~a])
        dls.append(dl)
    assert int(eager.accepted.sum()) > 0
    del before
    graph.capture(ks, props, lus)
    graph.replay()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(graph.params.cpu().numpy(), eager.params.cpu().numpy())
    np.testing.assert_array_equal(graph.accepted.cpu().numpy(), eager.accepted.cpu().numpy())
    for d1, d2 in zip(graph.dls, dls):
        np.testing.assert_allclose(d1.cpu().numpy(), d2.cpu().numpy(), rtol=1e-12, atol=1e-9)
    # residual == d - sum_k h(current sources), recomputed from scratch
    fresh = SwapSampler(gb, eager.params.clone(), data, psd, **kw)
    err = (fresh.res - eager.res).abs().max().item()
    assert err < 1e-6 * eager.res.abs().max().item()
    np.testing.assert_allclose(graph.res.cpu().numpy(), eager.res.cpu().numpy(), rtol=0,
                               atol=1e-9 * eager.res.abs().max().item())


def test_swap_sampler_in_the_pair_form():
    """The same sampler on the 9-parameter model in the pair form (swap
    likelihood and residual updates both in pairs): accepted swaps' dlogL
    equals the change of -1/2 <r|r> to 1e-8 of |logL| (the FP32 form: 1e-5),
    and the incrementally updated residuals equal d minus the sum of the
    current sources recomputed from scratch."""
    from gbgpu_gb300 import GBGPU
    from gbgpu_gb300.mcmc import SwapSampler, random_proposals, log_uniforms
    _, p, data, psd, s0, N, _ = _setup(seed=5)
    gb = GBGPU()
    kw = dict(N=N, T=T_OBS, dt=DT, start_freq_ind=s0, precision="pair")
    s = SwapSampler(gb, p[:9].contiguous().clone(), data, psd, **kw)
    g = torch.Generator(device="cuda").manual_seed(17)
    scale = torch.tensor([0.05, 2e-9, 0, 0, 0.2, 0.1, 0.1, 0.02, 0.02], dtype=torch.float64,
                         device="cuda")
    steps = 8
    lus = log_uniforms(s.W, steps, g, "cuda")
    accepted = 0
    for i in range(steps):
        k = i % s.K
        prop = random_proposals(s.params[:, :, k], scale, g)
        ll0 = s.log_likelihood()
        dl = s.step(k, prop, lus[i])
        ll1 = s.log_likelihood()
        a = (lus[i] < dl).cpu().numpy()
        d_ll, dl_n = (ll1 - ll0).cpu().numpy(), dl.cpu().numpy()
        tol = 1e-8 * np.maximum(1.0, np.abs(ll0.cpu().numpy()))
        assert np.all(np.abs(d_ll[a] - dl_n[a]) < tol[a])
        assert np.all(np.abs(d_ll[~a]) < tol[~a])
        accepted += int(a.sum())
    assert accepted > 0
    fresh = SwapSampler(gb, s.params.clone(), data, psd, **kw)
    assert (fresh.res - s.res).abs().max().item() < 1e-9 * s.res.abs().max().item()
