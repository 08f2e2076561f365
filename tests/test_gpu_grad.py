"""Gradient kernel (gbx_waveform_ll_grad) against FP64 references.

The reference has no gradients; the checks are (1) the forward-mode FP64
gradient of the torch restatement (oracle/fastgb_torch.py, torch.func.jvp)
and (2) the five-point central difference (relative step 1e-7 -- for fddot a
step moving its phase term by 1e-4 rad -- with the stencil of the
reference's information_matrix, gbgpu.py:1108-1110) of the plain FP64 fused
likelihood, which itself matches the reference's likelihood to 1e-10.
Tolerances, per parameter: |g - g_ref| <= tol (|g_ref| + rms_b g_ref) with
tol = 3e-5 against forward mode (only the mixed form's rounding: its ~1e-7
relative template error amplified by cancellation in the residual; measured
worst 1.1e-5, amp and iota of the third-body case) and tol = 5e-5 against
the differences (their FP64 rounding and truncation; measured worst 1.3e-5,
f0).  Each test prints the measured worst value per parameter.  The
third-body model (14 parameters) is checked the same way.
"""

import numpy as np
import pytest

import fastgb_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

T_OBS = 4 * 31557600.0
FD_TOL = 5e-5        # five-point differences (measured worst: 1.3e-5)
FWD_TOL = 3e-5       # forward mode: only the mixed form's rounding (measured worst: 1.1e-5)


def _case(B, N, seed, dt=10.0, tdi2=False, third=False):
    from gbgpu_gb300 import GBGPU, GBGPUThirdBody
    from gbgpu_gb300.sensitivity import A1TDISens
    rng = np.random.default_rng(seed)
    T = int(T_OBS / dt) * dt
    q0 = np.rint(rng.uniform(2.0e-3, 2.4e-3, B) * T)
    truth = np.array([10 ** rng.uniform(-22.3, -21.7, B), (q0 + rng.uniform(-0.3, 0.3, B)) / T,
                      10 ** rng.uniform(-17, -16, B), np.zeros(B), rng.uniform(0.5, 5.5, B),
                      np.arccos(rng.uniform(-0.9, 0.9, B)), rng.uniform(0.3, 2.8, B),
                      rng.uniform(0.5, 5.5, B), np.arcsin(rng.uniform(-0.9, 0.9, B))])
    truth[3] = 11 / 3 * truth[2] ** 2 / truth[1]
    if third:
        # A2 [m/s], varpi, e2, P2 [yr], T2 [yr]: a Doppler phase of O(1) rad
        P2 = 10 ** rng.uniform(0.3, 1.0, B)
        truth = np.concatenate([truth, np.array([10 ** rng.uniform(0.5, 1.5, B),
                                                 rng.uniform(0.3, 6.0, B), rng.uniform(0.1, 0.8, B),
                                                 P2, rng.uniform(0.1, 0.9, B) * P2])])
    si = O.start_indices(truth[1], N, T, dt)
    s0 = int(si.min()) - N
    L = int(si.max()) + 2 * N - s0
    S = A1TDISens.get_Sn((np.arange(L) + s0) / T)
    gb = GBGPUThirdBody(precision="fp64") if third else GBGPU(precision="fp64")
    tmpl = torch.zeros((1, 2, L), dtype=torch.complex128, device="cuda")
    gb.generate_global_template(truth.T, np.zeros(B, np.int32), tmpl, N=N, T=T_OBS, dt=dt,
                                tdi2=tdi2, start_freq_ind=s0)
    noise = np.sqrt(S * T / 4) * (rng.standard_normal((2, L)) + 1j * rng.standard_normal((2, L)))
    data = [tmpl[0, 0] + torch.as_tensor(noise[0], device="cuda"),
            tmpl[0, 1] + torch.as_tensor(noise[1], device="cuda")]
    # evaluate away from the truth so every gradient component is well away from 0
    ev = truth.copy()
    ev[0] *= 1 + rng.uniform(-0.05, 0.05, B)
    ev[1] += rng.uniform(-0.05, 0.05, B) / T
    ev[2] *= 1 + rng.uniform(-0.05, 0.05, B)
    for k in (4, 5, 6, 7, 8):
        ev[k] += rng.uniform(-0.02, 0.02, B)
    if third:
        ev[9] *= 1 + rng.uniform(-0.05, 0.05, B)
        ev[10] += rng.uniform(-0.05, 0.05, B)
        ev[11] += rng.uniform(-0.02, 0.02, B)
        ev[12] *= 1 + rng.uniform(-0.02, 0.02, B)
        ev[13] += rng.uniform(-0.02, 0.02, B)
    return gb, ev, data, torch.as_tensor(S, device="cuda"), s0, dt


def _fd(gb, p, data, Sd, s0, N, dt, tdi2):
    out = np.zeros_like(p)
    for k in range(p.shape[0]):
        h = 1e-7 * np.maximum(np.abs(p[k]), 1.0 if k >= 4 else 0.0)
        if k == 3:
            # a relative step of fddot (~1e-31) moves logL by ~1e-11, at FP64
            # round-off; step so that the phase term pi/3 fddot T^3 moves 1e-4 rad
            h = np.full_like(h, 1e-4 / (np.pi / 3 * T_OBS ** 3))
        h = np.where(h == 0, 1e-7, h)
        vals = []
        for m in (2, 1, -1, -2):
            q = p.copy()
            q[k] = q[k] + m * h
            vals.append(gb.get_ll(q, data, [Sd, Sd], N=N, T=T_OBS, dt=dt, tdi2=tdi2,
                                  start_freq_ind=s0, precision="fp64"))
        out[k] = (-vals[0] + 8 * vals[1] - 8 * vals[2] + vals[3]) / (12 * h)
    return out


@pytest.mark.parametrize("N,tdi2", [(256, True), (128, False), (1024, False)])
def test_gradient_matches_fp64_finite_differences(N, tdi2):
    gb, p, data, Sd, s0, dt = _case(24, N, 40 + N, tdi2=tdi2)
    gb.d_d = 0.0
    like, grad = gb.get_ll_grad(p, data, [Sd, Sd], N=N, T=T_OBS, dt=dt, tdi2=tdi2,
                                start_freq_ind=s0)
    _check(grad, _fd(gb, p, data, Sd, s0, N, dt, tdi2), FD_TOL, f"N={N} tdi2={tdi2} vs FD:")
    # the likelihood returned with the gradient is the mixed fused likelihood
    like_m = gb.get_ll(p, data, [Sd, Sd], N=N, T=T_OBS, dt=dt, tdi2=tdi2, start_freq_ind=s0,
                       precision="mixed")
    np.testing.assert_allclose(like, like_m, rtol=1e-12, atol=1e-9)


def test_gradient_uneven_N_and_autograd():
    from gbgpu_gb300.autodiff import log_likelihood
    gb, p, data, Sd, s0, dt = _case(40, 2048, 77)
    gb.d_d = 0.0
    rng = np.random.default_rng(5)
    Ns = 2 ** rng.integers(6, 12, 40)
    like, grad = gb.get_ll_grad(p, data, [Sd, Sd], N=Ns, T=T_OBS, dt=dt, start_freq_ind=s0)
    for n in np.unique(Ns):
        sel = Ns == n
        l1, g1 = gb.get_ll_grad(p[:, sel], data, [Sd, Sd], N=int(n), T=T_OBS, dt=dt,
                                start_freq_ind=s0)
        np.testing.assert_allclose(like[sel], l1, rtol=1e-12, atol=1e-9)
        np.testing.assert_allclose(grad[:, sel], g1, rtol=1e-12, atol=0)
    pt = torch.as_tensor(p, device="cuda").requires_grad_(True)
    ll = log_likelihood(gb, pt, data, [Sd, Sd], N=Ns, T=T_OBS, dt=dt, start_freq_ind=s0)
    w = torch.linspace(0.5, 1.5, 40, device="cuda", dtype=torch.float64)
    (ll * w).sum().backward()
    np.testing.assert_allclose(pt.grad.cpu().numpy(), grad * w.cpu().numpy()[None, :],
                               rtol=1e-12, atol=0)
    np.testing.assert_allclose(ll.detach().cpu().numpy(), like, rtol=1e-12, atol=1e-9)


NAMES14 = ["amp", "f0", "fdot", "fddot", "phi0", "iota", "psi", "lam", "beta",
           "A2", "varpi", "e2", "P2", "T2"]


def _worst(grad, ref):
    """Per parameter: max_b |g - g_ref| / (|g_ref| + rms_b g_ref)."""
    out = []
    for k in range(ref.shape[0]):
        rms = np.sqrt(np.mean(ref[k] ** 2))
        out.append(float(np.max(np.abs(grad[k] - ref[k]) / (np.abs(ref[k]) + rms))))
    return np.array(out)


def _check(grad, ref, tol=FD_TOL, what=""):
    w = _worst(grad, ref)
    print(f"{what} worst normalised error per parameter: " +
          ", ".join(f"{NAMES14[k]} {w[k]:.1e}" for k in range(len(w))))
    assert np.all(w <= tol), dict(zip(NAMES14, w))


def _forward_mode(p, data, Sd, s0, N, dt, tdi2):
    import fastgb_torch as FT
    d = [x.cpu().numpy() for x in data]
    S = Sd.cpu().numpy()
    third = p[9:] if p.shape[0] > 9 else None
    return FT.forward_gradient(p[:9], d, [S, S], N, T_OBS, dt, tdi2=tdi2, third=third,
                               start_freq_ind=s0)


@pytest.mark.parametrize("N,tdi2", [(256, True), (512, False)])
def test_gradient_matches_forward_mode(N, tdi2):
    gb, p, data, Sd, s0, dt = _case(16, N, 90 + N, tdi2=tdi2)
    gb.d_d = 0.0
    _, grad = gb.get_ll_grad(p, data, [Sd, Sd], N=N, T=T_OBS, dt=dt, tdi2=tdi2, start_freq_ind=s0)
    _check(grad, _forward_mode(p, data, Sd, s0, N, dt, tdi2), FWD_TOL,
           f"N={N} tdi2={tdi2} vs forward mode:")


@pytest.mark.parametrize("N", [256, 512])
def test_third_body_gradient(N):
    gb, p, data, Sd, s0, dt = _case(16, N, 120 + N, dt=5.0, third=True)
    gb.d_d = 0.0
    like, grad = gb.get_ll_grad(p, data, [Sd, Sd], N=N, T=T_OBS, dt=dt, start_freq_ind=s0)
    assert grad.shape == (14, 16)
    _check(grad, _forward_mode(p, data, Sd, s0, N, dt, False), FWD_TOL,
           f"third body N={N} vs forward mode:")
    _check(grad, _fd(gb, p, data, Sd, s0, N, dt, False), FD_TOL, f"third body N={N} vs FD:")
    like_m = gb.get_ll(p, data, [Sd, Sd], N=N, T=T_OBS, dt=dt, start_freq_ind=s0, precision="mixed")
    np.testing.assert_allclose(like, like_m, rtol=1e-12, atol=1e-9)
