"""Swap log-likelihood (gbx_swap_ll) against the oracle's composition.

The reference has no swap call; its definition here (dlogL = Re<r|Dh> -
<Dh|Dh>/2 with the reference's inner product) is restated in
oracle/fastgb_oracle.py:swap_ll.  Tolerances: FP64 form 1e-10, pair form 1e-9
and mixed form 1e-6, all relative to max(1, <h_old|h_old> + <h_new|h_new>).
"""

import numpy as np
import pytest

import fastgb_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

T_OBS = 4 * 31557600.0


def _draw(rng, B):
    f0 = rng.uniform(2.0e-3, 2.02e-3, B)
    fdot = 10 ** rng.uniform(-18, -15, B)
    p = np.array([10 ** rng.uniform(-22.5, -21.5, B), f0, fdot, 11 / 3 * fdot ** 2 / f0,
                  rng.uniform(0, 2 * np.pi, B), np.arccos(rng.uniform(-1, 1, B)),
                  rng.uniform(0, np.pi, B), rng.uniform(0, 2 * np.pi, B),
                  np.arcsin(rng.uniform(-1, 1, B))])
    return p


def _residuals(rng, p, N, T, dt, nwalk):
    from gbgpu_gb300.sensitivity import A1TDISens
    si = O.start_indices(p[1], N, T, dt)
    s0 = int(si.min()) - 3 * N
    L = int(si.max()) + 4 * N - s0
    Tu = int(T / dt) * dt
    S = A1TDISens.get_Sn((np.arange(L) + s0) / Tu)
    data = [np.sqrt(S * Tu / 4) * (rng.standard_normal((nwalk, L)) + 1j * rng.standard_normal((nwalk, L)))
            for _ in range(2)]
    return data, S, s0


@pytest.mark.parametrize("precision,N", [("fp64", 128), ("mixed", 128), ("fp64", 512),
                                         ("mixed", 1024), ("pair", 128), ("pair", 1024)])
def test_swap_matches_oracle(precision, N):
    from gbgpu_gb300 import GBGPU
    rng = np.random.default_rng(60 + N)
    B, nwalk = 48, 3
    po = _draw(rng, B)
    pn = po.copy()
    # mixed proposals: small moves (overlapping windows), large f0 jumps
    # (disjoint windows), identical sources (dlogL = 0)
    pn[1, :16] += rng.uniform(-3, 3, 16) / T_OBS
    pn[1, 16:32] += rng.uniform(2 * N, 3 * N, 16) / T_OBS
    pn[4:, :32] += rng.uniform(-0.1, 0.1, (5, 32))
    pn[0, :32] *= 1 + rng.uniform(-0.2, 0.2, 32)
    data, S, s0 = _residuals(rng, np.concatenate([po, pn], 1), N, T_OBS, 10.0, nwalk)
    di = rng.integers(0, nwalk, B).astype(np.int32)
    ref = O.swap_ll(po, pn, data, [S, S], N, T_OBS, 10.0, data_index=di, start_freq_ind=s0)
    wo = O.waveform(po, N, T=T_OBS, dt=10.0)
    wn = O.waveform(pn, N, T=T_OBS, dt=10.0)
    Tu = int(T_OBS / 10.0) * 10.0
    scale = np.ones(B)
    for b in range(B):
        for w in (wo, wn):
            k = int(w["start_inds"][b]) - s0
            for ch in range(2):
                scale[b] += 4 / Tu * np.sum(np.abs(w["AETf"][b, ch]) ** 2 / S[k:k + N])
    gb = GBGPU()
    got = gb.swap_likelihood(po, pn, [torch.as_tensor(x, device="cuda") for x in data],
                             [torch.as_tensor(S, device="cuda")] * 2, N=N, T=T_OBS, dt=10.0,
                             data_index=di, start_freq_ind=s0, precision=precision)
    tol = {"fp64": 1e-10, "pair": 1e-9}.get(precision, 1e-6)
    err = np.abs(got - ref) / scale
    assert np.max(err) < tol, np.max(err)
    assert np.all(np.abs(got[32:]) <= tol * scale[32:])       # identical pairs


def test_swap_third_body():
    from gbgpu_gb300 import GBGPUThirdBody
    rng = np.random.default_rng(71)
    B, N = 20, 512
    po = _draw(rng, B)
    pn = po.copy()
    pn[1] += rng.uniform(-2, 2, B) / T_OBS
    P2 = 10 ** rng.uniform(0, np.log10(40), B)
    third_o = (10 ** rng.uniform(-2, 2, B), rng.uniform(0, 2 * np.pi, B), rng.uniform(0, 0.9, B),
               P2, rng.uniform(0, 1, B) * P2)
    third_n = tuple(x.copy() for x in third_o)
    third_n[0][:] *= 1.3
    data, S, s0 = _residuals(rng, np.concatenate([po, pn], 1), N, T_OBS, 5.0, 1)
    d1 = [x[0] for x in data]
    ref = O.swap_ll(po, pn, d1, [S, S], N, T_OBS, 5.0, start_freq_ind=s0, third_old=third_o,
                    third_new=third_n)
    gb = GBGPUThirdBody()
    full_o = np.concatenate([po, np.array(third_o)])
    full_n = np.concatenate([pn, np.array(third_n)])
    for precision, tol in (("fp64", 1e-9), ("mixed", 1e-5)):
        got = gb.swap_likelihood(full_o, full_n, [torch.as_tensor(x, device="cuda") for x in d1],
                                 [torch.as_tensor(S, device="cuda")] * 2, N=N, T=T_OBS, dt=5.0,
                                 start_freq_ind=s0, precision=precision)
        np.testing.assert_allclose(got, ref, rtol=tol, atol=tol * np.max(np.abs(ref)))
