"""Swap log-likelihood gradient (gbx_swap_ll_grad) against FP64 references.

d dlogL / d theta_new = Re<r + h_old - h_new | d h_new>, the likelihood
gradient at the proposal against the data r + h_old (the reference has no
swap call; its inner product is gbgpu_utils.cu:172-183).  Checked two ways:

* forward mode (oracle/fastgb_torch.py, torch.func.jvp) of the FP64 torch
  likelihood at the proposal against r + h_old, h_old the oracle waveform of
  the current source placed on the grid;
* five-point central differences of the FP64 swap kernel itself
  (gbx_swap_ll, within 1e-10 of the oracle's swap_ll) in the proposal's
  parameters (steps as in tests/test_gpu_grad.py).

Tolerances per parameter, |g - g_ref| <= tol (|g_ref| + rms_b g_ref): 3e-5
against forward mode, 5e-5 against the differences, as for the likelihood
gradient.  Pairs cover overlapping windows, disjoint windows and identical
sources; f0 sits within 0.3 bin of a bin centre so that no stencil point
moves a window.
"""

import numpy as np
import pytest

import fastgb_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

T_OBS = 4 * 31557600.0
FD_TOL = 5e-5
FWD_TOL = 3e-5
NAMES = ["amp", "f0", "fdot", "fddot", "phi0", "iota", "psi", "lam", "beta",
         "A2", "varpi", "e2", "P2", "T2"]


def _worst(grad, ref):
    out = []
    for k in range(ref.shape[0]):
        rms = np.sqrt(np.mean(ref[k] ** 2))
        out.append(float(np.max(np.abs(grad[k] - ref[k]) / (np.abs(ref[k]) + rms))))
    return np.array(out)


def _check(grad, ref, tol, what):
    w = _worst(grad, ref)
    print(f"{what} worst normalised error per parameter: " +
          ", ".join(f"{NAMES[k]} {w[k]:.1e}" for k in range(len(w))))
    assert np.all(w <= tol), dict(zip(NAMES, w))


def _pairs(rng, B, N, dt):
    """(old, new) pairs: a third small moves, a third jumps by 2N-3N bins, a
    third identical; f0 within 0.3 bin of a bin centre."""
    T = int(T_OBS / dt) * dt
    q0 = np.rint(rng.uniform(2.0e-3, 2.02e-3, B) * T)
    fdot = 10 ** rng.uniform(-17, -16, B)
    po = np.array([10 ** rng.uniform(-22.3, -21.7, B), (q0 + rng.uniform(-0.3, 0.3, B)) / T, fdot,
                   np.zeros(B), rng.uniform(0.5, 5.5, B), np.arccos(rng.uniform(-0.9, 0.9, B)),
                   rng.uniform(0.3, 2.8, B), rng.uniform(0.5, 5.5, B),
                   np.arcsin(rng.uniform(-0.9, 0.9, B))])
    po[3] = 11 / 3 * po[2] ** 2 / po[1]
    pn = po.copy()
    a, b = B // 3, 2 * B // 3
    pn[1, :a] = (q0[:a] + rng.integers(-2, 3, a) + rng.uniform(-0.3, 0.3, a)) / T
    pn[1, a:b] = (q0[a:b] + rng.integers(2 * N, 3 * N, b - a) + rng.uniform(-0.3, 0.3, b - a)) / T
    pn[0, :b] *= 1 + rng.uniform(-0.2, 0.2, b)
    pn[2, :b] *= 1 + rng.uniform(-0.05, 0.05, b)
    pn[4:, :b] += rng.uniform(-0.1, 0.1, (5, b))
    pn[3] = 11 / 3 * pn[2] ** 2 / pn[1]
    return po, pn


def _residuals(rng, p, N, dt, nwalk):
    from gbgpu_gb300.sensitivity import A1TDISens
    T = int(T_OBS / dt) * dt
    si = O.start_indices(p[1], N, T_OBS, dt)
    s0 = int(si.min()) - 3 * N
    L = int(si.max()) + 4 * N - s0
    S = A1TDISens.get_Sn((np.arange(L) + s0) / T)
    data = [np.sqrt(S * T / 4) * (rng.standard_normal((nwalk, L)) + 1j * rng.standard_normal((nwalk, L)))
            for _ in range(2)]
    return data, S, s0


def _with_old(data, di, wo, s0, N):
    """One data row per pair: its residual row plus the current source."""
    rows = []
    for ch in range(2):
        r = data[ch][di].copy()
        for b in range(len(di)):
            k = int(wo["start_inds"][b]) - s0
            r[b, k:k + N] += wo["AETf"][b, ch]
        rows.append(r)
    return rows


def _fd(gb, po, pn, dd, Sd, s0, N, dt, di, third=None):
    out = np.zeros_like(pn)
    for k in range(pn.shape[0]):
        h = 1e-7 * np.maximum(np.abs(pn[k]), 1.0 if k >= 4 else 0.0)
        if k == 3:
            h = np.full_like(h, 1e-4 / (np.pi / 3 * T_OBS ** 3))
        h = np.where(h == 0, 1e-7, h)
        vals = []
        for m in (2, 1, -1, -2):
            q = pn.copy()
            q[k] = q[k] + m * h
            vals.append(gb.swap_likelihood(po, q, dd, [Sd, Sd], N=N, T=T_OBS, dt=dt, data_index=di,
                                           start_freq_ind=s0, precision="fp64"))
        out[k] = (-vals[0] + 8 * vals[1] - 8 * vals[2] + vals[3]) / (12 * h)
    return out


@pytest.mark.parametrize("N", [128, 512])
def test_swap_gradient_matches_forward_mode_and_differences(N):
    import fastgb_torch as FT
    from gbgpu_gb300 import GBGPU
    dt = 10.0
    rng = np.random.default_rng(300 + N)
    B, nwalk = 24, 3
    po, pn = _pairs(rng, B, N, dt)
    data, S, s0 = _residuals(rng, np.concatenate([po, pn], 1), N, dt, nwalk)
    di = rng.integers(0, nwalk, B).astype(np.int32)
    gb = GBGPU()
    dd = [torch.as_tensor(x, device="cuda") for x in data]
    Sd = torch.as_tensor(S, device="cuda")
    dl, g = gb.swap_likelihood(po, pn, dd, [Sd, Sd], N=N, T=T_OBS, dt=dt, data_index=di,
                               start_freq_ind=s0, grad=True)
    assert g.shape == (9, B) and np.all(np.isfinite(g))
    # the change of log-likelihood is the mixed swap kernel's
    dl_m = gb.swap_likelihood(po, pn, dd, [Sd, Sd], N=N, T=T_OBS, dt=dt, data_index=di,
                              start_freq_ind=s0, precision="mixed")
    np.testing.assert_array_equal(dl, dl_m)
    wo = O.waveform(po, N, T=T_OBS, dt=dt)
    rows = _with_old(data, di, wo, s0, N)
    ref = FT.forward_gradient(pn, rows, [S, S], N, T_OBS, dt, start_freq_ind=s0,
                              data_index=np.arange(B))
    _check(g, ref, FWD_TOL, f"swap N={N} vs forward mode:")
    _check(g, _fd(gb, po, pn, dd, Sd, s0, N, dt, di), FD_TOL, f"swap N={N} vs FD:")


def test_swap_gradient_third_body():
    import fastgb_torch as FT
    from gbgpu_gb300 import GBGPUThirdBody
    dt, N = 5.0, 512
    rng = np.random.default_rng(77)
    B = 16
    po, pn = _pairs(rng, B, N, dt)
    P2 = 10 ** rng.uniform(0.3, 1.0, B)
    to = np.array([10 ** rng.uniform(0.5, 1.5, B), rng.uniform(0.3, 6.0, B), rng.uniform(0.1, 0.8, B),
                   P2, rng.uniform(0.1, 0.9, B) * P2])
    tn = to.copy()
    tn[0] *= 1 + rng.uniform(-0.05, 0.05, B)
    tn[1] += rng.uniform(-0.02, 0.02, B)
    full_o, full_n = np.concatenate([po, to]), np.concatenate([pn, tn])
    data, S, s0 = _residuals(rng, np.concatenate([po, pn], 1), N, dt, 1)
    di = np.zeros(B, np.int32)
    gb = GBGPUThirdBody()
    dd = [torch.as_tensor(x, device="cuda") for x in data]
    Sd = torch.as_tensor(S, device="cuda")
    dl, g = gb.swap_likelihood(full_o, full_n, dd, [Sd, Sd], N=N, T=T_OBS, dt=dt, data_index=di,
                               start_freq_ind=s0, grad=True)
    assert g.shape == (14, B)
    wo = O.waveform(po, N, T=T_OBS, dt=dt, third=to)
    rows = _with_old(data, di, wo, s0, N)
    ref = FT.forward_gradient(pn, rows, [S, S], N, T_OBS, dt, third=tn, start_freq_ind=s0,
                              data_index=np.arange(B))
    _check(g, ref, FWD_TOL, "third-body swap vs forward mode:")


def test_swap_gradient_rejects_other_precisions():
    from gbgpu_gb300 import GBGPU
    rng = np.random.default_rng(5)
    po, pn = _pairs(rng, 4, 128, 10.0)
    data, S, s0 = _residuals(rng, np.concatenate([po, pn], 1), 128, 10.0, 1)
    gb = GBGPU()
    with pytest.raises(ValueError, match="mixed form"):
        gb.swap_likelihood(po, pn, [torch.as_tensor(x[0], device="cuda") for x in data],
                           [torch.as_tensor(S, device="cuda")] * 2, N=128, T=T_OBS, dt=10.0,
                           start_freq_ind=s0, grad=True, precision="fp64")
