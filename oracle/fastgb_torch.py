"""Differentiable FP64 restatement of the FastGB likelihood -- TEST INFRASTRUCTURE ONLY.

The same arithmetic as ``fastgb_oracle.waveform`` / ``get_ll`` (which restate
gbgpu/gbgpu.py:178-316, 348-540, gbgpu/thirdbody.py:155-428 and the inner
product of gbgpu/cutils/gbgpu_utils.cu:124-185) written in torch FP64 /
complex128 so that ``torch.func.jvp`` gives a forward-mode reference gradient
of log L.  The reference itself has no derivatives; this module is the
forward-mode checker for the adjoint kernel.  It is pinned against the NumPy
oracle (values) and against its central finite differences
(``tests/test_oracle_torch.py``).

The integer carrier bin q = rint(f0 T) and start_inds are piecewise constant
in the parameters, so their derivative is zero here exactly as in the adjoint.
"""

import math

import numpy as np
import torch

import fastgb_oracle as O

C_SI = O.C_SI
YRSID_SI = O.YRSID_SI


def kepler_u(l, e):
    """Eccentric anomaly; torch transcription of fastgb_oracle.kepler_u
    (gbgpu/thirdbody.py:228-320: Mikkola start + one 4th-order Newton step)."""
    two_pi = 2.0 * math.pi
    neg = l < 0
    l = torch.abs(l)
    over2pi = l > two_pi
    mult = torch.where(over2pi, torch.floor(l.detach() / two_pi), torch.zeros_like(l))
    l = torch.where(over2pi, l - mult * two_pi, l)
    overpi = l > math.pi
    l = torch.where(overpi, two_pi - l, l)
    alpha = (1.0 - e) / (4.0 * e + 0.5)
    beta = 0.5 * l / (4.0 * e + 0.5)
    z = torch.sqrt(beta * beta + alpha * alpha * alpha)
    z = torch.where(neg, beta - z, beta + z)
    cz = torch.abs(z) ** (1.0 / 3.0)
    z = torch.where(z < 0, -cz, cz)
    s = z - alpha / z
    w = s - 0.078 * s ** 5 / (1.0 + e)
    u0 = l + e * (3.0 * w - 4.0 * w ** 3)
    f = u0 - e * torch.sin(u0) - l
    f1 = 1.0 - e * torch.cos(u0)
    f2 = u0 - f - l
    f3 = 1.0 - f1
    f4 = -f2
    f2 = f2 * 0.5
    f3 = f3 * 0.166666666666667
    f4 = f4 * 0.0416666666666667
    u1 = -f / f1
    u2 = -f / (f1 + f2 * u1)
    u3 = -f / (f1 + f2 * u2 + f3 * u2 * u2)
    u4 = -f / (f1 + f2 * u3 + f3 * u3 * u3 + f4 * u3 * u3 * u3)
    u = u0 + u4
    u = torch.where(overpi, two_pi - u, u)
    u = torch.where(over2pi, two_pi * mult + u, u)
    return torch.where(neg, -u, u)


def third_body_vlos(t, A2, varpi, e2, n2, T2):
    """v_LOS = A2 (sin(phi + varpi) + e2 sin varpi); gbgpu/thirdbody.py:322-380."""
    u = kepler_u(n2 * (t - T2), e2.expand_as(t))
    e = e2.expand_as(t)
    adjust = e > 1e-6
    safe_e = torch.where(adjust, e, torch.ones_like(e))
    bet = (1.0 - torch.sqrt(1.0 - safe_e * safe_e)) / safe_e
    phi = torch.where(adjust, u + 2.0 * torch.atan2(bet * torch.sin(u), 1.0 - bet * torch.cos(u)), u)
    return A2 * (torch.sin(phi + varpi) + e2 * torch.sin(varpi))


def waveform_aet(params, N, T, dt, tdi2=False, orbits=None, third=None):
    """A and E channels (B, 2, N) complex128 for one N (start_inds are
    ``fastgb_oracle.start_indices`` of the f0 values).

    ``params`` (9, B) and ``third`` (5, B) = (A2, varpi, e2, P2[yr], T2[yr])
    are torch FP64 tensors; every step follows fastgb_oracle.waveform.
    """
    if orbits is None:
        orbits = O.OracleOrbits()
    amp, f0, fdot, fddot, phi0, iota, psi, lam, beta = [x[:, None] for x in params]
    T = int(T / dt) * dt
    L = orbits.armlength
    fstar = C_SI / (L * 2 * np.pi)
    theta = np.pi / 2 - beta
    ci = torch.cos(iota)
    c2p, s2p = torch.cos(2.0 * psi), torch.sin(2.0 * psi)
    Ap = amp * (1.0 + ci * ci)
    Ac = -2.0 * amp * ci
    DP = torch.complex(Ap * c2p, -Ac * s2p)
    DC = torch.complex(-Ap * s2p, -Ac * c2p)
    st, ct, sp, cp = torch.sin(theta), torch.cos(theta), torch.sin(lam), torch.cos(lam)
    u = torch.stack([ct * cp, ct * sp, -st], dim=-1)[:, 0]         # (B,3)
    v = torch.stack([sp, -cp, torch.zeros_like(cp)], dim=-1)[:, 0]
    k = torch.stack([-st * cp, -st * sp, -ct], dim=-1)[:, 0]
    eplus = v[:, :, None] * v[:, None, :] - u[:, :, None] * u[:, None, :]
    ecross = u[:, :, None] * v[:, None, :] + v[:, :, None] * u[:, None, :]

    tm_np = np.linspace(0, T, num=N, endpoint=False)
    tm = torch.as_tensor(tm_np, dtype=torch.float64)
    P = [torch.as_tensor(orbits.get_pos(tm_np, np.full(N, s, dtype=np.int32))) for s in (1, 2, 3)]
    r = {"12": (P[1] - P[0]) / L, "13": (P[2] - P[0]) / L, "23": (P[2] - P[1]) / L}
    r["31"] = -r["13"]
    kdotr = {}
    for ij in ("12", "13", "23"):
        kdotr[ij] = k @ r[ij].T
        kdotr[ij[1] + ij[0]] = -kdotr[ij]
    kdotP = torch.stack([k @ Ps.T for Ps in P], dim=1) / C_SI       # (B,3,N)
    xi = tm[None, None, :] - kdotP
    f0_, fdot_, fddot_ = f0[:, :, None], fdot[:, :, None], fddot[:, :, None]
    fi = f0_ + fdot_ * xi + 0.5 * fddot_ * xi ** 2
    if third is not None:
        A2, varpi, e2, P2, T2 = [x[:, None, None] for x in third]
        n2 = 2 * np.pi / (P2 * YRSID_SI)
        T2s = T2 * YRSID_SI
        vlos = third_body_vlos(xi, A2, varpi, e2, n2, T2s)
        fi = fi * (1 + vlos / C_SI)
    fonfs = fi / fstar
    q = torch.round(f0.detach() * T)
    dfa = 2.0 * np.pi * (q / T)
    om = 2.0 * np.pi * f0
    Aij = {}
    for ij in ("12", "23", "31"):
        rr = r[ij]
        pp = torch.einsum("na,bac,nc->bn", rr, eplus, rr)
        cc = torch.einsum("na,bac,nc->bn", rr, ecross, rr)
        Aij[ij] = pp * DP + cc * DC
    argS = (phi0[:, :, None] + (om - dfa)[:, :, None] * tm[None, None, :]
            + np.pi * fdot_ * xi ** 2 + 1 / 3 * np.pi * fddot_ * xi ** 3)
    if third is not None:
        fgw = f0_ + fdot_ * xi + 0.5 * fddot_ * xi * xi
        g = vlos * fgw
        step = (xi[:, :, 1:] - xi[:, :, :-1]) * (g[:, :, :-1] + g[:, :, 1:]) / 2.0 * np.pi * 2 / C_SI
        argS = argS + torch.cat([torch.zeros_like(step[:, :, :1]), torch.cumsum(step, dim=-1)], -1)
    kp = om[:, :, None] * kdotP - argS
    G = {}
    for ij, sym, s in (("12", "12", 0), ("23", "23", 1), ("31", "31", 2),
                       ("21", "12", 1), ("32", "23", 2), ("13", "31", 0)):
        a = 0.5 * fonfs[:, s, :] * (1 + kdotr[ij])
        G[ij] = 0.25 * torch.sin(a) / a * torch.exp(-1.0j * (a + kp[:, s])) * Aij[sym]
    f = f0 + fdot * tm[None, :] + 0.5 * fddot * tm[None, :] ** 2
    omL = f / fstar
    fc = torch.exp(-1.0j * omL)
    fc2 = 4.0 * omL * torch.sin(omL) * fc / amp
    X = G["21"] - G["31"] + (G["12"] - G["13"]) * fc
    Y = G["32"] - G["12"] + (G["23"] - G["21"]) * fc
    Z = G["13"] - G["23"] + (G["31"] - G["32"]) * fc
    sl = fc2[:, None, :] * torch.stack([X, Y, Z], dim=1)
    XYZf = torch.fft.fftshift(amp[:, :, None] * torch.fft.fft(sl, dim=-1), dim=-1)
    fctr = torch.full_like(amp, 0.5 * T / N).to(torch.complex128)
    if tdi2:
        omegaL = 2 * np.pi * f0 * (L / C_SI)
        fctr = fctr * (2.0j * torch.sin(2 * omegaL) * torch.exp(-2j * omegaL))
    XYZf = XYZf * fctr[:, :, None]
    Xf, Yf, Zf = XYZf[:, 0], XYZf[:, 1], XYZf[:, 2]
    return torch.stack([(Zf - Xf) / np.sqrt(2.0), (Xf - 2.0 * Yf + Zf) / np.sqrt(6.0)], dim=1)


def log_likelihood(params, data, psd, N, T, dt, start, tdi2=False, d_d=0.0, start_freq_ind=0,
                   data_index=None, noise_index=None, third=None):
    """-1/2 (d_d + <h|h> - 2 Re<d|h>) per binary (gbgpu.py:580-735 with the
    inner product of gbgpu_utils.cu:124-185), differentiable in params/third;
    ``start`` = start_inds of the undifferentiated f0."""
    AE = waveform_aet(params, N, T, dt, tdi2=tdi2, third=third)
    Tu = int(T / dt) * dt
    df = 1.0 / Tu
    B = AE.shape[0]
    data = [torch.as_tensor(np.asarray(x)).reshape(-1, np.asarray(x).shape[-1]) for x in data]
    psd = [torch.as_tensor(np.asarray(x)).reshape(-1, np.asarray(x).shape[-1]) for x in psd]
    di = np.zeros(B, np.int64) if data_index is None else np.asarray(data_index, np.int64)
    ni = np.zeros(B, np.int64) if noise_index is None else np.asarray(noise_index, np.int64)
    j = torch.as_tensor((start - start_freq_ind)[:, None] + np.arange(N)[None, :])
    d_h = torch.zeros(B, dtype=torch.complex128)
    h_h = torch.zeros(B, dtype=torch.float64)
    for ch in range(2):
        d = data[ch][torch.as_tensor(di)[:, None], j]
        S = psd[ch][torch.as_tensor(ni)[:, None], j]
        h = AE[:, ch]
        d_h = d_h + 4.0 * df * torch.sum(torch.conj(d) * h / S, dim=-1)
        h_h = h_h + 4.0 * df * torch.sum((torch.conj(h) * h).real / S, dim=-1)
    return -0.5 * (d_d + h_h - 2.0 * d_h.real)


def forward_gradient(params, data, psd, N, T, dt, tdi2=False, third=None, **kw):
    """d logL_b / d theta_b for every binary by forward mode: one jvp per
    parameter row (binaries are independent).  Returns (np+nt, B) NumPy."""
    p = torch.as_tensor(np.asarray(params, dtype=np.float64))
    th = None if third is None else torch.as_tensor(np.asarray(third, dtype=np.float64))
    rows = p.shape[0] + (0 if th is None else th.shape[0])
    start = O.start_indices(np.asarray(params[1], dtype=np.float64), N, T, dt)
    out = np.zeros((rows, p.shape[1]))
    for k in range(rows):
        tp = torch.zeros_like(p)
        tt = None if th is None else torch.zeros_like(th)
        if k < p.shape[0]:
            tp[k] = 1.0
        else:
            tt[k - p.shape[0]] = 1.0
        if th is None:
            fn = lambda x: log_likelihood(x, data, psd, N, T, dt, start, tdi2=tdi2, **kw)
            _, jv = torch.func.jvp(fn, (p,), (tp,))
        else:
            fn = lambda x, y: log_likelihood(x, data, psd, N, T, dt, start, tdi2=tdi2, third=y,
                                             **kw)
            _, jv = torch.func.jvp(fn, (p, th), (tp, tt))
        out[k] = jv.numpy()
    return out
