"""NumPy FP64 oracle for the FastGB hot path -- TEST INFRASTRUCTURE ONLY.

A CPU restatement of the reference's waveform, likelihood, global-template
fill, third-body hooks and the swap-likelihood composition.  It is imported
only by ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py``, to compare against; the product never calls it.  Each function
cites the reference lines it restates (paths relative to the reference's
project root).  The native inner loops (get_ll / fill_global) are restated in
C in ``oracle/gbgpu_oracle.c`` and bound here through ctypes.

Pinning: ``tests/test_oracle_golden.py`` checks every function here against
golden vectors produced by running the reference's own Python and its C++
``gbgpu_utils.cu`` (``tests/golden/make_golden.py``).  The orbit and the
constants are stand-ins for ``lisatools`` (see ``oracle/stubs``); both the
oracle and the product consume the same orbit arrays, so parity of the
FastGB arithmetic is exact while fidelity to the ``lisatools`` orbit files is
not claimed.
"""

import ctypes
import os
import subprocess

import numpy as np

C_SI = 299792458.0
PI = np.pi
YRSID_SI = 31558149.763545603

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


# ----------------------------------------------------------------------------
# Analytic orbit (same published formula as oracle/stubs/lisatools/detector.py)
# ----------------------------------------------------------------------------
class OracleOrbits:
    """Cornish & Rubbo (2003) first-order-eccentricity constellation."""

    def __init__(self, armlength=2.5e9):
        self.armlength = float(armlength)
        self.t_base = np.linspace(0.0, 10.0 * YRSID_SI, 1001)
        self._R = 149597870700.0
        self._ecc = self.armlength / (2.0 * np.sqrt(3.0) * self._R)
        self._fm = 1.0 / YRSID_SI

    def get_pos(self, t, sc):
        t = np.asarray(t, dtype=np.float64)
        sc = np.asarray(sc)
        alpha = 2.0 * np.pi * self._fm * t
        beta = 2.0 * np.pi * (sc - 1) / 3.0
        R = self._R
        eR = self._ecc * R
        x = R * np.cos(alpha) + 0.5 * eR * (np.cos(2.0 * alpha - beta) - 3.0 * np.cos(beta))
        y = R * np.sin(alpha) + 0.5 * eR * (np.sin(2.0 * alpha - beta) - 3.0 * np.sin(beta))
        z = -np.sqrt(3.0) * eR * np.cos(alpha - beta)
        return np.stack([x, y, z], axis=-1)


# ----------------------------------------------------------------------------
# Third-body line-of-sight velocity (gbgpu/thirdbody.py:228-428)
# ----------------------------------------------------------------------------
def kepler_u(l, e):
    """Eccentric anomaly by Mikkola's cubic start + one 4th-order Newton step.

    Restates gbgpu/thirdbody.py:228-320 elementwise, including its handling of
    negative mean anomalies (z = beta - sqrt(...)) and its 2 pi reductions.
    """
    l = np.array(l, dtype=np.float64, copy=True)
    e = np.broadcast_to(np.asarray(e, dtype=np.float64), l.shape)
    neg = l < 0
    l = l * np.sign(l)
    over2pi = l > 2 * np.pi
    mult = np.where(over2pi, np.floor(l / (2 * np.pi)), 0.0)
    l = np.where(over2pi, l - mult * 2.0 * np.pi, l)
    overpi = l > np.pi
    l = np.where(overpi, 2.0 * np.pi - l, l)

    alpha = (1.0 - e) / (4.0 * e + 0.5)
    beta = 0.5 * l / (4.0 * e + 0.5)
    z = np.sqrt(beta * beta + alpha * alpha * alpha)
    z = np.where(neg, beta - z, beta + z)
    cz = np.abs(z) ** (1 / 3)
    z = np.where(z < 0, -cz, cz)
    s = z - alpha / z
    w = s - 0.078 * s * s * s * s * s / (1.0 + e)
    u0 = l + e * (3.0 * w - 4.0 * w * w * w)

    f = u0 - e * np.sin(u0) - l
    f1 = 1.0 - e * np.cos(u0)
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
    u = np.where(overpi, 2.0 * np.pi - u, u)
    u = np.where(over2pi, 2.0 * np.pi * mult + u, u)
    u = np.where(neg, -u, u)
    return u


def third_body_vlos(t, A2, varpi, e2, n2, T2):
    """v_LOS(t) = A2 (sin(phi2 + varpi) + e2 sin varpi); gbgpu/thirdbody.py:322-380."""
    sh = (-1,) + (1,) * (t.ndim - 1)
    e = e2.reshape(sh)
    u = kepler_u(n2.reshape(sh) * (t - T2.reshape(sh)), np.broadcast_to(e, t.shape))
    ecc = np.broadcast_to(e, t.shape)
    adjust = ecc > 1e-6
    safe_e = np.where(adjust, ecc, 1.0)
    bet = (1.0 - np.sqrt(1.0 - safe_e * safe_e)) / safe_e
    phi = np.where(adjust, u + 2.0 * np.arctan2(bet * np.sin(u), 1.0 - bet * np.cos(u)), u)
    return A2.reshape(sh) * (np.sin(phi + varpi.reshape(sh)) + e * np.sin(varpi.reshape(sh)))


def third_body_phase(f0, fdot, fddot, xi, A2, varpi, e2, n2, T2):
    """Cumulative trapezoid phase from the LOS Doppler shift.

    Restates add_to_argS + parab_step_ET (gbgpu/thirdbody.py:182-226,
    382-428): term[..., 0] = 0 and term[..., k] = sum_{m<=k}
    (xi_m - xi_{m-1}) (g_{m-1} + g_m) / 2 * 2 pi / c with g = v_LOS * f_GW.
    """
    sh = (-1, 1, 1)
    fgw = f0.reshape(sh) + fdot.reshape(sh) * xi + 0.5 * fddot.reshape(sh) * xi * xi
    g = third_body_vlos(xi, A2, varpi, e2, n2, T2) * fgw
    dtt = xi[:, :, 1:] - xi[:, :, :-1]
    step = dtt * (g[:, :, :-1] + g[:, :, 1:]) / 2.0 * PI * 2 / C_SI
    out = np.zeros_like(xi)
    out[:, :, 1:] = np.cumsum(step, axis=-1)
    return out


# ----------------------------------------------------------------------------
# Waveform (gbgpu/gbgpu.py:108-540)
# ----------------------------------------------------------------------------
def waveform(params, N, T=4 * YRSID_SI, dt=10.0, tdi2=False, orbits=None,
             third=None, unequal_arms=False):
    """FastGB X/Y/Z and A/E/T for a batch sharing one N.

    ``params`` is (9, B): amp, f0, fdot, fddot, phi0, iota, psi, lam, beta.
    ``third`` is None or (A2, varpi, e2, P2[yr], T2[yr]) arrays of length B.
    ``unequal_arms``: the library's unequal-arm model (no counterpart in the
    reference, whose TDI takes one armlength, gbgpu.py:167-170): arm a has
    length ell_a L with ell_a = |r_a| at each sample; transfer argument
    (f/f*)(ell_a +- k.r_a)/2, antenna pattern r.e.r / ell_a^2 times ell_a,
    delays D_a = exp(-i omL ell_a),
    X = -2i omL [(1 - D31^2)(G21 + D12 G12) - (1 - D12^2)(G31 + D31 G13)]
    (Y, Z cyclic), TDI-2 per sample: X (1 - D12^2 D31^2) (cyclic).
    Returns dict(XYZf=(B,3,N) c128, AETf=(B,3,N) c128, start_inds=(B,) int64,
    T=T_used, df=1/T_used).
    """
    if orbits is None:
        orbits = OracleOrbits()
    params = np.asarray(params, dtype=np.float64)
    amp, f0, fdot, fddot, phi0, iota, psi, lam, beta = params
    B = amp.shape[0]
    T = int(T / dt) * dt                                  # gbgpu.py:178-179
    df = 1 / T
    L = orbits.armlength
    fstar = C_SI / (L * 2 * np.pi)                       # gbgpu.py:243
    theta = np.pi / 2 - beta

    # polarisation amplitudes and sky basis (gbgpu.py:240-266)
    ci = np.cos(iota)
    c2p, s2p = np.cos(2.0 * psi), np.sin(2.0 * psi)
    Ap = amp * (1.0 + ci * ci)
    Ac = -2.0 * amp * ci
    DP = Ap * c2p - 1.0j * Ac * s2p
    DC = -Ap * s2p - 1.0j * Ac * c2p
    st, ct, sp, cp = np.sin(theta), np.cos(theta), np.sin(lam), np.cos(lam)
    u = np.stack([ct * cp, ct * sp, -st], axis=-1)           # (B,3)
    v = np.stack([sp, -cp, np.zeros_like(cp)], axis=-1)
    k = np.stack([-st * cp, -st * sp, -ct], axis=-1)
    eplus = v[:, :, None] * v[:, None, :] - u[:, :, None] * u[:, None, :]
    ecross = u[:, :, None] * v[:, None, :] + v[:, :, None] * u[:, None, :]

    # sample times and spacecraft (gbgpu.py:269-272, 390-397)
    tm = np.linspace(0, T, num=N, endpoint=False)
    P = [orbits.get_pos(tm, np.full(N, s, dtype=np.int32)) for s in (1, 2, 3)]
    r = {"12": (P[1] - P[0]) / L, "13": (P[2] - P[0]) / L, "23": (P[2] - P[1]) / L}
    r["31"] = -r["13"]

    # slow part (gbgpu.py:399-540)
    kdotr = {}
    for ij in ("12", "13", "23"):
        kdotr[ij] = k @ r[ij].T                              # (B,N)
        kdotr[ij[1] + ij[0]] = -kdotr[ij]
    kdotP = np.stack([k @ Ps.T for Ps in P], axis=1) / C_SI  # (B,3,N)
    xi = tm[None, None, :] - kdotP
    fi = f0[:, None, None] + fdot[:, None, None] * xi + 1 / 2.0 * fddot[:, None, None] * xi ** 2
    if third is not None:
        A2, varpi, e2, P2, T2 = [np.asarray(a, dtype=np.float64) for a in third]
        n2 = 2 * np.pi / (P2 * YRSID_SI)                     # thirdbody.py:68-70
        T2s = T2 * YRSID_SI
        fi = fi * (1 + third_body_vlos(xi, A2, varpi, e2, n2, T2s) / C_SI)
    fonfs = fi / fstar
    q = np.rint(f0 * T)
    dfa = 2.0 * np.pi * (q / T)
    om = 2.0 * np.pi * f0

    Aij = {}
    for ij in ("12", "23", "31"):
        rr = r[ij]                                           # (N,3)
        pp = np.einsum("na,bac,nc->bn", rr, eplus, rr)
        cc = np.einsum("na,bac,nc->bn", rr, ecross, rr)
        Aij[ij] = pp * DP[:, None] + cc * DC[:, None]

    argS = (phi0[:, None, None] + (om[:, None, None] - dfa[:, None, None]) * tm[None, None, :]
            + np.pi * fdot[:, None, None] * xi ** 2
            + 1 / 3 * np.pi * fddot[:, None, None] * xi ** 3)
    if third is not None:
        argS = argS + third_body_phase(f0, fdot, fddot, xi, A2, varpi, e2, n2, T2s)
    kp = om[:, None, None] * kdotP - argS

    ell = {ij: (np.linalg.norm(r[ij], axis=-1) if unequal_arms else np.ones(N))
           for ij in ("12", "23", "31")}
    G = {}
    for ij, sym, s in (("12", "12", 0), ("23", "23", 1), ("31", "31", 2),
                       ("21", "12", 1), ("32", "23", 2), ("13", "31", 0)):
        a = 0.5 * fonfs[:, s, :] * (ell[sym] + kdotr[ij])
        G[ij] = 0.25 * np.sin(a) / a * np.exp(-1.0j * (a + kp[:, s])) * Aij[sym] / ell[sym]

    # TDI assembly + FFT (gbgpu.py:348-388)
    f = f0[:, None] + fdot[:, None] * tm[None, :] + 1 / 2 * fddot[:, None] * tm[None, :] ** 2
    omL = f / fstar
    if unequal_arms:
        D = {a: np.exp(-1.0j * omL * ell[a]) for a in ("12", "23", "31")}
        X = ((1 - D["31"] ** 2) * (G["21"] + D["12"] * G["12"])
             - (1 - D["12"] ** 2) * (G["31"] + D["31"] * G["13"]))
        Y = ((1 - D["12"] ** 2) * (G["32"] + D["23"] * G["23"])
             - (1 - D["23"] ** 2) * (G["12"] + D["12"] * G["21"]))
        Z = ((1 - D["23"] ** 2) * (G["13"] + D["31"] * G["31"])
             - (1 - D["31"] ** 2) * (G["23"] + D["23"] * G["32"]))
        if tdi2:
            X = X * (1 - D["12"] ** 2 * D["31"] ** 2)
            Y = Y * (1 - D["23"] ** 2 * D["12"] ** 2)
            Z = Z * (1 - D["31"] ** 2 * D["23"] ** 2)
        pre = -2.0j * omL / amp[:, None]
        sl = pre[:, None, :] * np.stack([X, Y, Z], axis=1)
    else:
        fc = np.exp(-1.0j * omL)
        fc2 = 4.0 * omL * np.sin(omL) * fc / amp[:, None]
        X = G["21"] - G["31"] + (G["12"] - G["13"]) * fc
        Y = G["32"] - G["12"] + (G["23"] - G["21"]) * fc
        Z = G["13"] - G["23"] + (G["31"] - G["32"]) * fc
        sl = fc2[:, None, :] * np.stack([X, Y, Z], axis=1)
    XYZf = np.fft.fftshift(amp[:, None, None] * np.fft.fft(sl, axis=-1), axes=-1)
    fmin = (q - N / 2) / T
    start_inds = np.round(fmin / df).astype(int)            # gbgpu.py:296-297

    fctr = np.full(B, 0.5 * T / N, dtype=np.complex128)      # gbgpu.py:298-309
    if tdi2 and not unequal_arms:
        omegaL = 2 * np.pi * f0 * (L / C_SI)
        fctr = fctr * (2.0j * np.sin(2 * omegaL) * np.exp(-2j * omegaL))
    XYZf = XYZf * fctr[:, None, None]
    Xf, Yf, Zf = XYZf[:, 0], XYZf[:, 1], XYZf[:, 2]
    AETf = np.stack([(Zf - Xf) / np.sqrt(2.0), (Xf - 2.0 * Yf + Zf) / np.sqrt(6.0),
                     (Xf + Yf + Zf) / np.sqrt(3.0)], axis=1)  # utility.py:24-38
    return {"XYZf": XYZf, "AETf": AETf, "start_inds": start_inds, "T": T, "df": df, "N": N}


def start_indices(f0, N, T, dt):
    """start_inds = round(((rint(f0 T) - N/2) / T) / (1/T)); gbgpu.py:296, 387, 462."""
    T = int(T / dt) * dt
    q = np.rint(np.asarray(f0, dtype=np.float64) * T)
    return np.round(((q - N / 2) / T) / (1 / T)).astype(np.int64)


# ----------------------------------------------------------------------------
# Native loops (C restatement in gbgpu_oracle.c)
# ----------------------------------------------------------------------------
def _lib():
    global _LIB
    if _LIB is None:
        so = os.path.join(_HERE, "_build", "liboracle.so")
        if not os.path.isfile(so):
            subprocess.run(["make", "-C", _HERE, "oracle"], check=True,
                           stdout=subprocess.DEVNULL)
        lib = ctypes.CDLL(so)
        vp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        for name in ("oracle_get_ll", "oracle_get_ll_par"):
            fn = getattr(lib, name)
            fn.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, d, vp, i, i, vp, vp, i]
            fn.restype = None
        lib.oracle_fill_global.argtypes = [vp, vp, vp, vp, vp, i, i, vp, i]
        lib.oracle_fill_global.restype = None
        lib.oracle_num_threads.restype = i
        _LIB = lib
    return _LIB


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def get_ll_native(A_pm, E_pm, A_data, E_data, A_psd, E_psd, df, start_ind, M,
                  num_bin, data_index, noise_index, data_length, parallel=False):
    """(d_h, h_h) from point-major templates; restates gbgpu_utils.cu:124-185."""
    A_pm = np.ascontiguousarray(A_pm, dtype=np.complex128)
    E_pm = np.ascontiguousarray(E_pm, dtype=np.complex128)
    A_data = np.ascontiguousarray(A_data, dtype=np.complex128)
    E_data = np.ascontiguousarray(E_data, dtype=np.complex128)
    A_psd = np.ascontiguousarray(A_psd, dtype=np.float64)
    E_psd = np.ascontiguousarray(E_psd, dtype=np.float64)
    si = np.ascontiguousarray(start_ind, dtype=np.int32)
    di = np.ascontiguousarray(data_index, dtype=np.int32)
    ni = np.ascontiguousarray(noise_index, dtype=np.int32)
    d_h = np.zeros(num_bin, np.complex128)
    h_h = np.zeros(num_bin, np.complex128)
    fn = _lib().oracle_get_ll_par if parallel else _lib().oracle_get_ll
    fn(_p(d_h), _p(h_h), _p(A_pm), _p(E_pm), _p(A_data), _p(E_data), _p(A_psd),
       _p(E_psd), float(df), _p(si), int(M), int(num_bin), _p(di), _p(ni),
       int(data_length))
    return d_h, h_h


def fill_global_native(A_glob, E_glob, A_pm, E_pm, start_ind, M, num_bin,
                       group_index, data_length):
    """Accumulate into flat (G*L,) buffers in place; gbgpu_utils.cu:54-101."""
    A_pm = np.ascontiguousarray(A_pm, dtype=np.complex128)
    E_pm = np.ascontiguousarray(E_pm, dtype=np.complex128)
    si = np.ascontiguousarray(start_ind, dtype=np.int32)
    gi = np.ascontiguousarray(group_index, dtype=np.int32)
    assert A_glob.flags["C_CONTIGUOUS"] and A_glob.dtype == np.complex128
    assert E_glob.flags["C_CONTIGUOUS"] and E_glob.dtype == np.complex128
    _lib().oracle_fill_global(_p(A_glob), _p(E_glob), _p(A_pm), _p(E_pm), _p(si),
                              int(M), int(num_bin), _p(gi), int(data_length))


def point_major(X):
    """(B, N) -> reference flat layout index i*B + b (gbgpu.py:333-346)."""
    return np.ascontiguousarray(np.asarray(X).T).reshape(-1)


# ----------------------------------------------------------------------------
# API-level compositions
# ----------------------------------------------------------------------------
def get_ll(params, data, psd, N, T=4 * YRSID_SI, dt=10.0, tdi2=False, d_d=0.0,
           start_freq_ind=0, data_index=None, noise_index=None, orbits=None,
           third=None, phase_marginalize=False, return_terms=False, parallel=False,
           unequal_arms=False):
    """GBGPUBase.get_ll semantics (gbgpu.py:580-735) on the oracle waveform."""
    w = waveform(params, N, T=T, dt=dt, tdi2=tdi2, orbits=orbits, third=third,
                 unequal_arms=unequal_arms)
    B = w["AETf"].shape[0]
    data = [np.asarray(x) for x in data]
    psd = [np.asarray(x) for x in psd]
    L = data[0].shape[-1]
    data = [x.reshape(-1) for x in data]
    psd = [x.reshape(-1) for x in psd]
    di = np.zeros(B, np.int32) if data_index is None else np.asarray(data_index, np.int32)
    ni = np.zeros(B, np.int32) if noise_index is None else np.asarray(noise_index, np.int32)
    si = (w["start_inds"] - start_freq_ind).astype(np.int32)
    d_h, h_h = get_ll_native(point_major(w["AETf"][:, 0]), point_major(w["AETf"][:, 1]),
                             data[0], data[1], psd[0], psd[1], w["df"], si, N, B,
                             di, ni, L, parallel=parallel)
    if phase_marginalize:
        d_h = np.abs(d_h)
    like = -1.0 / 2.0 * (d_d + h_h - 2 * d_h).real
    if return_terms:
        return like, d_h, h_h, w
    return like


def fill_global_template(group_index, templates, A, E, start_inds, start_freq_ind=0):
    """fill_global_template semantics (gbgpu.py:737-837): overwrites channels 0, 1."""
    G, nch, L = templates.shape
    A = np.asarray(A)
    E = np.asarray(E)
    N = A.shape[1]
    B = A.shape[0]
    tA = np.zeros(G * L, np.complex128)
    tE = np.zeros(G * L, np.complex128)
    si = (np.asarray(start_inds) - start_freq_ind).astype(np.int32)
    fill_global_native(tA, tE, point_major(A), point_major(E), si, N, B,
                       np.asarray(group_index, np.int32), L)
    templates[:, 0] = tA.reshape(G, L)
    templates[:, 1] = tE.reshape(G, L)


def inner(a, b, psd, df):
    """4 df sum conj(a) b / S over a window; the convention of gbgpu_utils.cu:172-183."""
    return 4.0 * df * np.sum(np.conj(a) * b / psd)


def swap_ll(params_old, params_new, data, psd, N, T, dt, tdi2=False, orbits=None,
            data_index=None, noise_index=None, start_freq_ind=0, third_old=None,
            third_new=None):
    """Swap log-likelihood difference (no counterpart in the reference).

    For a residual r = d - (sum of the current sources) held in ``data`` and a
    proposal replacing source h_old by h_new, logL = -1/2 <r|r> changes by
        dlogL = -1/2 <r - dh | r - dh> + 1/2 <r|r> = Re<r|dh> - 1/2 <dh|dh>,
    dh = h_new - h_old, with <a|b> = 4 df sum_A,E conj(a) b / S over the union of both windows and
    the data/PSD rows chosen by data_index / noise_index as in get_ll.
    """
    wo = waveform(params_old, N, T=T, dt=dt, tdi2=tdi2, orbits=orbits, third=third_old)
    wn = waveform(params_new, N, T=T, dt=dt, tdi2=tdi2, orbits=orbits, third=third_new)
    B = wo["AETf"].shape[0]
    data = [np.asarray(x) for x in data]
    psd = [np.asarray(x) for x in psd]
    L = data[0].shape[-1]
    d2 = [x.reshape(-1, L) for x in data]
    p2 = [x.reshape(-1, L) for x in psd]
    di = np.zeros(B, np.int64) if data_index is None else np.asarray(data_index)
    ni = np.zeros(B, np.int64) if noise_index is None else np.asarray(noise_index)
    out = np.zeros(B)
    df = wo["df"]
    for b in range(B):
        so = int(wo["start_inds"][b]) - start_freq_ind
        sn = int(wn["start_inds"][b]) - start_freq_ind
        lo, hi = min(so, sn), max(so, sn) + N
        tot = 0.0
        for ch in range(2):
            dh = np.zeros(hi - lo, np.complex128)
            dh[sn - lo:sn - lo + N] += wn["AETf"][b, ch]
            dh[so - lo:so - lo + N] -= wo["AETf"][b, ch]
            r = d2[ch][di[b], lo:hi]
            S = p2[ch][ni[b], lo:hi]
            tot += (inner(r, dh, S, df).real - 0.5 * inner(dh, dh, S, df).real)
        out[b] = tot
    return out
