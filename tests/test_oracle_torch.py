"""Pins the differentiable torch restatement (oracle/fastgb_torch.py).

Values against the NumPy oracle (itself pinned to the reference's golden
vectors); the forward-mode gradient against five-point central differences of
the NumPy oracle's likelihood.  CPU only, small sizes.
"""

import numpy as np
import pytest

import fastgb_oracle as O

torch = pytest.importorskip("torch")
import fastgb_torch as FT  # noqa: E402

T_OBS = 4 * 31557600.0


def _params(rng, B, fmin=2.0e-3, fmax=2.2e-3):
    # f0 within 0.3 bins of an integer bin, so a finite-difference stencil of
    # f0 never moves the carrier bin rint(f0 T)
    f0 = (np.rint(rng.uniform(fmin, fmax, B) * T_OBS) + rng.uniform(-0.3, 0.3, B)) / T_OBS
    fdot = 10 ** rng.uniform(-17, -16, B)
    return np.array([10 ** rng.uniform(-22.3, -21.7, B), f0, fdot, 11 / 3 * fdot ** 2 / f0,
                     rng.uniform(0.5, 5.5, B), np.arccos(rng.uniform(-0.9, 0.9, B)),
                     rng.uniform(0.3, 2.8, B), rng.uniform(0.5, 5.5, B),
                     np.arcsin(rng.uniform(-0.9, 0.9, B))])


def _third(rng, B):
    P2 = 10 ** rng.uniform(0.3, 1.0, B)
    return np.array([10 ** rng.uniform(0, 1.5, B), rng.uniform(0, 2 * np.pi, B),
                     rng.uniform(0.1, 0.8, B), P2, rng.uniform(0, 1, B) * P2])


@pytest.mark.parametrize("tdi2,third", [(False, False), (True, False), (False, True)])
def test_torch_waveform_matches_numpy_oracle(tdi2, third):
    rng = np.random.default_rng(3)
    p = _params(rng, 5)
    th = _third(rng, 5) if third else None
    w = O.waveform(p, 128, T=T_OBS, dt=10.0, tdi2=tdi2, third=None if th is None else tuple(th))
    AE = FT.waveform_aet(torch.as_tensor(p), 128, T_OBS, 10.0, tdi2=tdi2,
                         third=None if th is None else torch.as_tensor(th))
    ref = w["AETf"][:, :2]
    err = np.abs(AE.numpy() - ref).max() / np.abs(ref).max()
    assert err < 1e-11, err


def _data(rng, p, N, dt, th=None):
    si = O.start_indices(p[1], N, T_OBS, dt)
    s0 = int(si.min()) - N
    L = int(si.max()) + 2 * N - s0
    Tu = int(T_OBS / dt) * dt
    f = (np.arange(L) + s0) / Tu
    S = 1e-40 * (1 + (2e-3 / f) ** 4)
    d = [np.sqrt(S * Tu / 4) * (rng.standard_normal(L) + 1j * rng.standard_normal(L)) for _ in range(2)]
    w = O.waveform(p, N, T=T_OBS, dt=dt, third=None if th is None else tuple(th))
    for b in range(p.shape[1]):
        k = int(w["start_inds"][b]) - s0
        for ch in range(2):
            d[ch][k:k + N] += w["AETf"][b, ch] * 1.02
    return d, [S, S], s0


@pytest.mark.parametrize("third", [False, True])
def test_forward_gradient_matches_central_differences(third):
    rng = np.random.default_rng(11)
    B, N, dt = 3, 64, 10.0
    p = _params(rng, B)
    th = _third(rng, B) if third else None
    data, psd, s0 = _data(rng, p, N, dt, th)
    g = FT.forward_gradient(p, data, psd, N, T_OBS, dt, third=th, start_freq_ind=s0)
    full = p if th is None else np.concatenate([p, th])
    for k in range(full.shape[0]):
        h = (1e-7 if k == 1 else 1e-6) * np.maximum(np.abs(full[k]), 1.0 if k >= 4 else 0.0)
        if k == 3:
            h = np.full(B, 1e-3 / (np.pi / 3 * T_OBS ** 3))
        vals = []
        for m in (2, 1, -1, -2):
            q = full.copy()
            q[k] = q[k] + m * h
            vals.append(O.get_ll(q[:9], data, psd, N, T=T_OBS, dt=dt, start_freq_ind=s0,
                                 third=None if th is None else tuple(q[9:])))
        fd = (-vals[0] + 8 * vals[1] - 8 * vals[2] + vals[3]) / (12 * h)
        scale = np.abs(fd) + np.sqrt(np.mean(fd ** 2))
        assert np.all(np.abs(g[k] - fd) <= 1e-4 * scale), (k, g[k], fd)
