"""Generate golden vectors by running the reference's own FastGB code.

Run where the reference project is checked out beside this repository
(../reference; override with GBGPU_REFERENCE_ROOT) after
``make -C oracle all``:

    python tests/golden/make_golden.py

It imports the reference's unmodified ``gbgpu/gbgpu.py``,
``gbgpu/thirdbody.py`` and ``gbgpu/utils/utility.py`` through
``oracle/refload.py`` (stub ``lisatools``/``gpubackendtools``; native
``get_ll``/``fill_global`` from the reference's ``gbgpu_utils.cu`` compiled as
C++), evaluates a set of small seeded cases and writes one compressed
``.npz`` per case next to this script.  The fixtures are small (tens to
hundreds of KB) and are what the CPU and GPU parity tests compare against;
the tests themselves never read the reference tree.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import refload  # noqa: E402

ref_gbgpu, ref_third, ref_util, lisatools = refload.load_reference()
YRSID_SI = lisatools.utils.constants.YRSID_SI
TJ4 = 4 * 31557600.0


def draw_params(rng, B, f_lo=1e-3, f_hi=5e-3, fdot_lo=-18, fdot_hi=-15):
    """Config-0 style draws: amp log-U(1e-23,1e-21), f0 U, fdot log-U,
    fddot = 11/3 fdot^2/f0, phi0, lam U[0,2pi), psi U[0,pi),
    iota = arccos U[-1,1], beta = arcsin U[-1,1]."""
    amp = 10 ** rng.uniform(-23, -21, B)
    f0 = rng.uniform(f_lo, f_hi, B)
    fdot = 10 ** rng.uniform(fdot_lo, fdot_hi, B)
    fddot = 11.0 / 3.0 * fdot ** 2 / f0
    phi0 = rng.uniform(0, 2 * np.pi, B)
    iota = np.arccos(rng.uniform(-1, 1, B))
    psi = rng.uniform(0, np.pi, B)
    lam = rng.uniform(0, 2 * np.pi, B)
    beta = np.arcsin(rng.uniform(-1, 1, B))
    return np.array([amp, f0, fdot, fddot, phi0, iota, psi, lam, beta])


def save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    print("wrote", path, os.path.getsize(path), "bytes")


def case_wave(name, seed, B, N, T, dt, tdi2, **kw):
    rng = np.random.default_rng(seed)
    p = draw_params(rng, B, **kw)
    gb = ref_gbgpu.GBGPU()
    gb.run_wave(*p, N=N, T=T, dt=dt, tdi2=tdi2)
    save(name, params=p, N=N, T=T, dt=dt, tdi2=tdi2, XYZf=gb.XYZf, AETf=gb.AETf,
         start_inds=np.asarray(gb.start_inds), A_out=gb.A_out, freqs=gb.freqs,
         df=gb.df)


def case_ll(name, seed, B, N, T, dt, tdi2, ndata=1, npsd=1, phase_marginalize=False):
    rng = np.random.default_rng(seed)
    p = draw_params(rng, B, f_lo=2.0e-3, f_hi=2.006e-3)
    gb = ref_gbgpu.GBGPU()
    gb.run_wave(*p, N=N, T=T, dt=dt, tdi2=tdi2)
    si = np.asarray(gb.start_inds)
    start_freq_ind = int(si.min()) - 37
    L = int(si.max()) + N + 41 - start_freq_ind
    f = (np.arange(L) + start_freq_ind) / (int(T / dt) * dt)
    S = lisatools.sensitivity.A1TDISens.get_Sn(f)
    # data: sum of the sources in their windows + seeded noise, per stream
    data = []
    for ch in range(2):
        rows = []
        for k in range(ndata):
            d = np.zeros(L, np.complex128)
            for b in range(B):
                o = si[b] - start_freq_ind
                d[o:o + N] += gb.AETf[b, ch] * (1.0 + 0.1 * k)
            sig = np.sqrt(S * (int(T / dt) * dt) / 4.0)
            d += sig * (rng.standard_normal(L) + 1j * rng.standard_normal(L)) / np.sqrt(2.0)
            rows.append(d)
        data.append(np.array(rows) if ndata > 1 else rows[0])
    psd = []
    for ch in range(2):
        rows = [S * (1.0 + 0.25 * k) for k in range(npsd)]
        psd.append(np.array(rows) if npsd > 1 else rows[0])
    data_index = rng.integers(0, ndata, B).astype(np.int32) if ndata > 1 else None
    noise_index = rng.integers(0, npsd, B).astype(np.int32) if npsd > 1 else None
    d_d = 123.0
    gb.d_d = d_d
    kwargs = {}
    if data_index is not None:
        kwargs["data_index"] = data_index
        # the reference requires 2-D psd whenever it takes a noise_index
    if noise_index is not None:
        kwargs["noise_index"] = noise_index
    if ndata > 1 and npsd == 1:
        kwargs["noise_index"] = np.zeros(B, np.int32)
        psd = [np.atleast_2d(x) for x in psd]
    like = gb.get_ll(p, data, psd, N=N, T=T, dt=dt, tdi2=tdi2,
                     start_freq_ind=start_freq_ind,
                     phase_marginalize=phase_marginalize, **kwargs)
    out = dict(params=p, N=N, T=T, dt=dt, tdi2=tdi2, like=like,
               d_h=np.asarray(gb.d_h), h_h=np.asarray(gb.h_h), d_d=d_d,
               start_freq_ind=start_freq_ind, A_data=data[0], E_data=data[1],
               A_psd=psd[0], E_psd=psd[1], start_inds=si,
               phase_marginalize=phase_marginalize)
    if phase_marginalize:
        out["non_marg_d_h"] = np.asarray(gb.non_marg_d_h)
    if "data_index" in kwargs:
        out["data_index"] = kwargs["data_index"]
    if "noise_index" in kwargs:
        out["noise_index"] = kwargs["noise_index"]
    save(name, **out)


def case_fill(name, seed):
    rng = np.random.default_rng(seed)
    B, N, G = 12, 128, 3
    T, dt = TJ4, 10.0
    p = draw_params(rng, B, f_lo=2.0e-3, f_hi=2.004e-3)
    gb = ref_gbgpu.GBGPU()
    gb.run_wave(*p, N=N, T=T, dt=dt)
    si = np.asarray(gb.start_inds)
    # the template window cuts through the first and last waveforms so the
    # out-of-range skip (gbgpu_utils.cu:88-91) is exercised
    start_freq_ind = int(si.min()) + 20
    L = int(si.max()) + N - 30 - start_freq_ind
    group_index = rng.integers(0, G, B).astype(np.int32)
    templates = (rng.standard_normal((G, 3, L)) + 1j * rng.standard_normal((G, 3, L)))
    before = templates.copy()
    gb.fill_global_template(group_index, templates, gb.A, gb.E, si, N=N,
                            start_freq_ind=start_freq_ind)
    # generate_global_template takes params as (B, nparams)
    templates2 = np.zeros((G, 2, L), np.complex128)
    gb.generate_global_template(p.T, group_index, templates2, N=N, T=T, dt=dt,
                                start_freq_ind=start_freq_ind)
    save(name, params=p, N=N, T=T, dt=dt, group_index=group_index,
         templates_before=before, templates_after=templates,
         generated=templates2, start_freq_ind=start_freq_ind, start_inds=si,
         A=gb.A, E=gb.E)


def case_ll_third(name, seed, B, N, T, dt, tdi2):
    """GBGPUThirdBody.get_ll with (14, B) parameters against injected data."""
    rng = np.random.default_rng(seed)
    p = draw_params(rng, B, f_lo=2.0e-3, f_hi=2.006e-3)
    A2 = 10 ** rng.uniform(-2, 2, B)
    P2 = 10 ** rng.uniform(0, np.log10(40), B)
    e2 = rng.uniform(0, 0.9, B)
    varpi = rng.uniform(0, 2 * np.pi, B)
    T2 = rng.uniform(0, 1, B) * P2
    third = np.array([A2, varpi, e2, P2, T2])
    gb = ref_third.GBGPUThirdBody()
    gb.run_wave(*p, *third.copy(), N=N, T=T, dt=dt, tdi2=tdi2)
    si = np.asarray(gb.start_inds)
    start_freq_ind = int(si.min()) - 29
    L = int(si.max()) + N + 33 - start_freq_ind
    f = (np.arange(L) + start_freq_ind) / (int(T / dt) * dt)
    S = lisatools.sensitivity.A1TDISens.get_Sn(f)
    data = []
    for ch in range(2):
        d = np.zeros(L, np.complex128)
        for b in range(B):
            o = si[b] - start_freq_ind
            d[o:o + N] += gb.AETf[b, ch]
        sig = np.sqrt(S * (int(T / dt) * dt) / 4.0)
        d += sig * (rng.standard_normal(L) + 1j * rng.standard_normal(L)) / np.sqrt(2.0)
        data.append(d)
    gb.d_d = 77.0
    params = np.concatenate([p, third])
    like = gb.get_ll(params.copy(), data, [S, S], N=N, T=T, dt=dt, tdi2=tdi2,
                     start_freq_ind=start_freq_ind)
    save(name, params=params, N=N, T=T, dt=dt, tdi2=tdi2, like=like,
         d_h=np.asarray(gb.d_h), h_h=np.asarray(gb.h_h), d_d=77.0,
         start_freq_ind=start_freq_ind, A_data=data[0], E_data=data[1], A_psd=S, E_psd=S,
         start_inds=si)


def case_third(name, seed, B, N, T, dt, tdi2=False):
    rng = np.random.default_rng(seed)
    p = draw_params(rng, B)
    A2 = 10 ** rng.uniform(-2, 2, B)
    P2 = 10 ** rng.uniform(0, np.log10(40), B)
    e2 = rng.uniform(0, 0.9, B)
    e2[0] = 0.0          # circular branch (no true-anomaly correction)
    e2[1] = 5e-7         # below the 1e-6 threshold
    varpi = rng.uniform(0, 2 * np.pi, B)
    T2 = rng.uniform(0, 1, B) * P2
    T2[2] = 3.5 * P2[2]  # pericentre after the window: negative mean anomaly
    gb = ref_third.GBGPUThirdBody()
    gb.run_wave(*p, A2, varpi, e2, P2, T2.copy(), N=N, T=T, dt=dt, tdi2=tdi2)
    save(name, params=p, A2=A2, varpi=varpi, e2=e2, P2=P2, T2=T2, N=N, T=T,
         dt=dt, tdi2=tdi2, XYZf=gb.XYZf, AETf=gb.AETf, start_inds=np.asarray(gb.start_inds))


def case_third_converters(name, seed):
    """The reference's third_body_factors and get_T2 on seeded inputs (copies:
    the reference scales its M, mc and P2 arguments in place)."""
    rng = np.random.default_rng(seed)
    n = 16
    M = rng.uniform(0.3, 1.5, n)
    mc = 10 ** rng.uniform(0, 3, n)
    P2 = 10 ** rng.uniform(-0.5, 1.5, n)
    e2 = rng.uniform(0, 0.9, n)
    iota = np.arccos(rng.uniform(-1, 1, n))
    Omega2 = rng.uniform(0, 2 * np.pi, n)
    omega2 = rng.uniform(0, 2 * np.pi, n)
    phi2 = rng.uniform(-np.pi, np.pi, n)
    lam = rng.uniform(0, 2 * np.pi, n)
    beta = np.arcsin(rng.uniform(-1, 1, n))
    A2, varpi, T2 = ref_third.third_body_factors(M.copy(), mc.copy(), P2.copy(), e2, iota,
                                                 Omega2, omega2, phi2, lam, beta)
    A2s, varpis, T2s = ref_third.third_body_factors(M.copy(), mc.copy() * 1e-3, P2.copy() * YRSID_SI,
                                                    e2, iota, Omega2, omega2, phi2, lam, beta,
                                                    third_mass_unit="MSUN",
                                                    third_period_unit="sec")
    T2_yrs = ref_third.get_T2(P2.copy(), e2, phi2)
    save(name, M=M, mc=mc, P2=P2, e2=e2, iota=iota, Omega2=Omega2, omega2=omega2, phi2=phi2,
         lam=lam, beta=beta, A2=A2, varpi=varpi, T2=T2, A2_msun=A2s, varpi_msun=varpis,
         T2_msun=T2s, T2_yrs=T2_yrs)


def case_kepler(name, seed):
    rng = np.random.default_rng(seed)
    gb = ref_third.GBGPUThirdBody()
    l = np.concatenate([rng.uniform(-40, 40, 200), [0.0, np.pi, -np.pi, 2 * np.pi + 1e-3,
                                                    -7.0, 13.0]])
    e = np.concatenate([rng.uniform(0, 0.95, 200), [0.3, 0.5, 0.1, 0.9, 0.0, 0.7]])
    # the reference works on (B, 3, n) arrays
    u = gb.get_u(l.reshape(-1, 1, 1).copy(), e.reshape(-1, 1, 1))
    save(name, l=l, e=e, u=u.reshape(-1))


def case_get_n(name, seed):
    rng = np.random.default_rng(seed)
    amp = 10 ** rng.uniform(-24, -20, 64)
    f0 = 10 ** rng.uniform(-4, -0.5, 64)
    outs = {}
    for T in (0.5 * YRSID_SI, 1.5 * YRSID_SI, 3.0 * YRSID_SI, 4.0 * YRSID_SI, 6 * YRSID_SI, 9 * YRSID_SI):
        for os_ in (1, 2, 4):
            outs[f"N_{T:.1f}_{os_}"] = ref_util.get_N(amp, f0, T, oversample=os_)
    gb = ref_third.GBGPUThirdBody()
    P2 = 10 ** rng.uniform(-1.5, 1.6, 64)
    third_N = gb.special_get_N(amp, f0, 4 * YRSID_SI, np.ones(64), np.zeros(64),
                               np.zeros(64), P2, np.zeros(64), oversample=2)
    save(name, amp=amp, f0=f0, P2=P2, third_N=third_N,
         keys=np.array(list(outs.keys())), **outs)


def case_misc(name):
    rng = np.random.default_rng(5)
    X = rng.standard_normal((4, 3)) + 1j * rng.standard_normal((4, 3))
    Y = rng.standard_normal((4, 3)) + 1j * rng.standard_normal((4, 3))
    Z = rng.standard_normal((4, 3)) + 1j * rng.standard_normal((4, 3))
    A, E, Tc = ref_util.AET(X, Y, Z)
    f0 = rng.uniform(1e-3, 2e-3, 5)
    fdot = rng.uniform(1e-17, 2e-17, 5)
    fddot = rng.uniform(1e-28, 2e-28, 5)
    t = np.linspace(0, 3e8, 7)[None, :]
    fgw = ref_util.get_fGW(f0, fdot, fddot, t)
    m1 = np.array([0.2, 0.6, 1.0])
    m2 = np.array([0.1, 0.3, 0.5])
    amp = ref_util.get_amplitude(m1, m2, np.array([0.1, 0.01, 0.003]), np.array([6.0, 1.0, 10.0]))
    fd = ref_util.get_fdot(np.array([1e-3, 2e-3, 5e-3]), m1=m1, m2=m2)
    Mc = ref_util.get_chirp_mass_from_f_fdot(np.array([1e-3, 2e-3, 5e-3]), fd)
    # inject_signal: only the non-zero window of the 0..fmax grid is stored
    gb = ref_gbgpu.GBGPU()
    p = draw_params(np.random.default_rng(9), 1)
    Ai, Ei = gb.inject_signal(*[x[0] for x in p], N=128, T=TJ4, dt=10.0)
    s0 = int(gb.start_inds[0])
    save(name, X=X, Y=Y, Z=Z, A=A, E=E, T=Tc, f0=f0, fdot=fdot, fddot=fddot, t=t,
         fgw=fgw, m1=m1, m2=m2, amp=amp, fdotout=fd, Mc=Mc, inj_params=p,
         inj_len=len(Ai), inj_start=s0, inj_A=Ai[s0:s0 + 128], inj_E=Ei[s0:s0 + 128],
         inj_nnz=int(np.count_nonzero(Ai)))


def case_fisher(name):
    gb = ref_gbgpu.GBGPU()
    B = 3
    rng = np.random.default_rng(11)
    p = draw_params(rng, B, fdot_lo=-17, fdot_hi=-16)
    # the 4-point branch requires every binary to sit on the first binary's
    # start index (gbgpu.py:1092-1095), so all f0 share one Fourier bin
    p[1] = (252460.0 + rng.uniform(-0.3, 0.3, B)) / TJ4
    inds = np.array([0, 1, 2, 4, 5, 6, 7, 8])
    fm = gb.information_matrix(p.copy(), eps=1e-9, inds=inds, N=256, T=TJ4, dt=10.0,
                               psd_func=lisatools.sensitivity.A1TDISens.get_Sn)
    fm2 = gb.information_matrix(p.copy(), eps=1e-9, inds=inds, N=256, T=TJ4, dt=10.0,
                                easy_central_difference=True,
                                psd_func=lisatools.sensitivity.A1TDISens.get_Sn)
    save(name, params=p, inds=inds, fisher=fm, fisher_easy=fm2, N=256, T=TJ4, dt=10.0)


if __name__ == "__main__":
    case_wave("wave_n128", 1, B=8, N=128, T=TJ4, dt=10.0, tdi2=False)
    case_wave("wave_n256_tdi2", 2, B=6, N=256, T=TJ4, dt=5.0, tdi2=True)
    case_wave("wave_n64_1yr", 3, B=5, N=64, T=0.95 * YRSID_SI, dt=15.0, tdi2=False)
    case_wave("wave_n512_hf", 4, B=3, N=512, T=TJ4, dt=5.0, tdi2=False,
              f_lo=1e-2, f_hi=2.5e-2)
    case_wave("wave_n2048_hf", 14, B=2, N=2048, T=TJ4, dt=5.0, tdi2=True,
              f_lo=1.5e-2, f_hi=2.5e-2)
    case_wave("wave_b1", 15, B=1, N=128, T=TJ4, dt=10.0, tdi2=False)
    case_ll("ll_basic", 6, B=8, N=128, T=TJ4, dt=10.0, tdi2=False)
    case_ll("ll_multi", 7, B=10, N=256, T=TJ4, dt=5.0, tdi2=True, ndata=3, npsd=2)
    case_ll("ll_phasemarg", 8, B=6, N=128, T=TJ4, dt=10.0, tdi2=False,
            phase_marginalize=True)
    case_fill("fill_basic", 9)
    case_third("third_n256", 10, B=6, N=256, T=TJ4, dt=5.0)
    case_third("third_n512_1yr", 16, B=4, N=512, T=YRSID_SI, dt=15.0)
    case_third("third_n128_tdi2", 17, B=4, N=128, T=TJ4, dt=10.0, tdi2=True)
    case_ll_third("ll_third", 18, B=6, N=256, T=TJ4, dt=5.0, tdi2=True)
    case_wave("wave_n4096", 19, B=1, N=4096, T=TJ4, dt=5.0, tdi2=False,
              f_lo=2.0e-2, f_hi=2.5e-2)
    case_third_converters("third_converters", 20)
    case_kepler("kepler", 12)
    case_get_n("get_n", 13)
    case_misc("misc")
    case_fisher("fisher")
