"""HMC sampler (gbgpu_gb300.mcmc.HMCSampler) on the fused likelihood + gradient.

Self-consistency only (the reference has no counterpart): the leapfrog
integrator is time-reversible, its energy error shrinks as step^2, chains
accept at a high rate at a moderate step, and a captured CUDA graph of
transitions reproduces the eager run exactly (the kernel is deterministic).
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

T_OBS = 4 * 31557600.0
DT = 10.0
FREE = (0, 1, 2, 4, 5, 6, 7, 8)


def _setup(B=48, N=256, seed=5, step=0.25, n_leapfrog=8):
    from gbgpu_gb300 import GBGPU
    from gbgpu_gb300.mcmc import HMCSampler
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
    # whitening scales: Fisher-diagonal standard deviations at the truth, from
    # the FP64 waveform (one binary per call: the reference's information_matrix
    # wants one start bin; it differentiates by relative steps, d h / d ln theta)
    gbf = GBGPU(precision="fp64")
    sig = np.zeros((len(FREE), B))
    for b in range(B):
        F = gbf.information_matrix(truth[:, b:b + 1], inds=list(FREE), N=N, T=T_OBS, dt=DT,
                                   psd_func=A1TDISens.get_Sn)
        sig[:, b] = np.abs(truth[list(FREE), b]) / np.sqrt(np.diag(F[0]))
    assert np.all(np.isfinite(sig)) and np.all(sig > 0)
    smp = HMCSampler(gb, torch.as_tensor(truth, device="cuda"), data, [Sd, Sd], N=N, T=T_OBS,
                     dt=DT, scales=sig, step_size=step, n_leapfrog=n_leapfrog,
                     start_freq_ind=s0, free=FREE)
    return smp, truth, rng


def test_leapfrog_is_reversible():
    smp, truth, rng = _setup(step=0.2, n_leapfrog=6)
    q0 = smp.params.clone()
    p0 = torch.as_tensor(rng.standard_normal((len(FREE), smp.B)), device="cuda")
    p1, g1, _ = smp.leapfrog(p0.clone(), smp.g.clone())
    p2, _, _ = smp.leapfrog(-p1, g1)
    f = smp.free
    rel = ((smp.params[f] - q0[f]).abs() / smp.scale).max().item()
    assert rel < 1e-4, rel                              # back within 1e-4 sigma
    assert torch.allclose(-p2, p0, atol=1e-3)


def test_energy_error_is_second_order_and_acceptance_high():
    med = []
    for step in (0.2, 0.1):
        smp, _, rng = _setup(step=step, n_leapfrog=int(round(1.6 / step)))
        mom = torch.as_tensor(rng.standard_normal((len(FREE), smp.B)), device="cuda")
        lu = torch.log(torch.as_tensor(rng.uniform(size=smp.B), device="cuda"))
        acc = smp.transition(mom, lu)
        med.append(float(smp.dH.abs().median()))
        if step == 0.2:
            assert acc.float().mean().item() > 0.7
    ratio = med[0] / med[1]
    assert 2.5 < ratio < 6.5, (med, ratio)              # ~4 for a second-order integrator


def test_graph_replay_matches_eager():
    smp, truth, rng = _setup(step=0.25, n_leapfrog=5)
    S = 6
    moms = torch.as_tensor(rng.standard_normal((S, len(FREE), smp.B)), device="cuda")
    lus = torch.log(torch.as_tensor(rng.uniform(size=(S, smp.B)), device="cuda"))
    start = (smp.params.clone(), smp.logL.clone(), smp.g.clone())
    for i in range(S):
        smp.transition(moms[i], lus[i])
    eager = (smp.params.clone(), smp.accepted.clone())
    smp.params.copy_(start[0])
    smp.logL.copy_(start[1])
    smp.g.copy_(start[2])
    smp.accepted.zero_()
    smp.capture(moms, lus)
    smp.replay()
    torch.cuda.synchronize()
    assert torch.equal(smp.params, eager[0])
    assert torch.equal(smp.accepted, eager[1])
    assert eager[1].float().mean().item() > 0.5 * S
