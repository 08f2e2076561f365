"""CUDA path against the reference's golden vectors and the CPU oracle.

Tolerances: start indices bit-exact; the FP64 form within 1e-10 relative
(normwise per binary for waveform windows, per value for <d|h>, <h|h>,
templates); the pair form within 1e-10 normwise on the waveform windows and
1e-9 relative on <d|h> and <h|h>, with |dlogL| <= 1e-8 max(1, SNR^2); the
mixed form within |dlogL| <= 1e-6
max(1, SNR^2) with SNR^2 = <h|h>, plus a stated per-output bound on the raw
terms.
"""

import numpy as np
import pytest

import fastgb_oracle as O
from conftest import load_golden, rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

WAVE_CASES = ["wave_n128", "wave_n256_tdi2", "wave_n64_1yr", "wave_n512_hf",
              "wave_n2048_hf", "wave_b1", "wave_n4096"]
FP64_TOL = 1e-10
MIXED_LL_TOL = 1e-6
PAIR_LL_TOL = 1e-8


def dev(x, dtype=None):
    t = torch.as_tensor(np.asarray(x), device="cuda")
    return t.to(dtype) if dtype is not None else t


@pytest.fixture(scope="module")
def gbgpu():
    from gbgpu_gb300 import GBGPU
    return GBGPU


@pytest.mark.parametrize("precision", ["fp64", "pair"])
@pytest.mark.parametrize("case", WAVE_CASES)
def test_run_wave_matches_reference(gbgpu, case, precision):
    g = load_golden(case)
    gb = gbgpu()
    gb.run_wave(*g["params"], N=int(g["N"]), T=float(g["T"]), dt=float(g["dt"]),
                tdi2=bool(g["tdi2"]), precision=precision)
    np.testing.assert_array_equal(gb.start_inds.cpu().numpy(), g["start_inds"])
    assert np.max(rel_err(gb.XYZf.cpu().numpy(), g["XYZf"], axis=(1, 2))) < FP64_TOL
    assert np.max(rel_err(gb.AETf.cpu().numpy(), g["AETf"], axis=(1, 2))) < FP64_TOL
    assert rel_err(gb.A_out.cpu().numpy(), g["A_out"]) < FP64_TOL
    np.testing.assert_allclose(gb.freqs.cpu().numpy(), g["freqs"], rtol=1e-15)
    assert gb.A.shape == (len(g["start_inds"]), int(g["N"]))


@pytest.mark.parametrize("case", ["ll_basic", "ll_multi", "ll_phasemarg"])
@pytest.mark.parametrize("precision", ["fp64", "pair", "mixed"])
def test_get_ll_matches_reference(gbgpu, case, precision):
    g = load_golden(case)
    gb = gbgpu()
    gb.d_d = float(g["d_d"])
    kw = {}
    if "data_index" in g:
        kw["data_index"] = dev(g["data_index"], torch.int32)
    if "noise_index" in g:
        kw["noise_index"] = dev(g["noise_index"], torch.int32)
    like = gb.get_ll(g["params"], [dev(g["A_data"]), dev(g["E_data"])],
                     [dev(g["A_psd"]), dev(g["E_psd"])], N=int(g["N"]), T=float(g["T"]),
                     dt=float(g["dt"]), tdi2=bool(g["tdi2"]),
                     start_freq_ind=int(g["start_freq_ind"]),
                     phase_marginalize=bool(g["phase_marginalize"]), precision=precision, **kw)
    d_h = gb.d_h.cpu().numpy()
    h_h = gb.h_h.cpu().numpy()
    snr2 = np.abs(g["h_h"].real)
    if precision == "fp64":
        np.testing.assert_allclose(d_h, g["d_h"], rtol=FP64_TOL, atol=0)
        np.testing.assert_allclose(h_h.real, g["h_h"].real, rtol=FP64_TOL, atol=0)
        np.testing.assert_allclose(like, g["like"], rtol=FP64_TOL)
    elif precision == "pair":
        np.testing.assert_allclose(d_h, g["d_h"], rtol=1e-9, atol=0)
        np.testing.assert_allclose(h_h.real, g["h_h"].real, rtol=1e-9, atol=0)
        assert np.max(np.abs(like - g["like"]) / np.maximum(1.0, snr2)) < PAIR_LL_TOL
    else:
        assert np.max(np.abs(like - g["like"]) / np.maximum(1.0, snr2)) < MIXED_LL_TOL
        # stated per-output bound of the mixed form: |d(h_h)| <= 1e-6 h_h
        assert np.max(np.abs(h_h.real - g["h_h"].real) / snr2) < 1e-6
    if bool(g["phase_marginalize"]):
        np.testing.assert_allclose(gb.non_marg_d_h, g["non_marg_d_h"],
                                   rtol={"fp64": FP64_TOL, "pair": 1e-9}.get(precision, 1e-5))
    # the waveform attributes are produced on demand after the fused call
    np.testing.assert_array_equal(gb.start_inds.cpu().numpy(), g["start_inds"])


@pytest.mark.parametrize("precision", ["fp64", "pair", "mixed"])
def test_get_ll_one_psd_array_for_both_channels(gbgpu, precision):
    """The same PSD tensor for A and E (the kernels then form one weight per
    bin): the oracle's likelihood with that PSD in both channels."""
    g = load_golden("ll_multi")
    S = dev(g["A_psd"])
    kw = dict(N=int(g["N"]), T=float(g["T"]), dt=float(g["dt"]), tdi2=bool(g["tdi2"]),
              start_freq_ind=int(g["start_freq_ind"]))
    _, d_h, h_h, _ = O.get_ll(g["params"], [g["A_data"], g["E_data"]], [g["A_psd"], g["A_psd"]],
                              data_index=g["data_index"], noise_index=g["noise_index"],
                              return_terms=True, **kw)
    gb = gbgpu()
    gb.d_d = 0.0
    gb.get_ll(g["params"], [dev(g["A_data"]), dev(g["E_data"])], [S, S], precision=precision,
              data_index=dev(g["data_index"], torch.int32),
              noise_index=dev(g["noise_index"], torch.int32), **kw)
    tol = {"fp64": FP64_TOL, "pair": 1e-9, "mixed": 1e-5}[precision]
    np.testing.assert_allclose(gb.d_h.cpu().numpy(), d_h, rtol=tol, atol=tol * np.abs(d_h).max())
    np.testing.assert_allclose(gb.h_h.real.cpu().numpy(), h_h.real, rtol=tol, atol=0)


def test_backend_get_ll_dropin_matches_oracle(gbgpu):
    """backend.get_ll with the reference's 15-argument list (gbgpu_utils_wrap.pyx:20-48)."""
    g = load_golden("ll_multi")
    W = O.waveform(g["params"], int(g["N"]), T=float(g["T"]), dt=float(g["dt"]), tdi2=True)
    B = W["AETf"].shape[0]
    L = g["A_data"].shape[-1]
    si = (W["start_inds"] - int(g["start_freq_ind"])).astype(np.int32)
    di, ni = g["data_index"], g["noise_index"]
    A_pm, E_pm = O.point_major(W["AETf"][:, 0]), O.point_major(W["AETf"][:, 1])
    ref_dh, ref_hh = O.get_ll_native(A_pm, E_pm, g["A_data"].ravel(), g["E_data"].ravel(),
                                     g["A_psd"].ravel(), g["E_psd"].ravel(), W["df"], si,
                                     int(g["N"]), B, di, ni, L)
    gb = gbgpu()
    d_h = torch.zeros(B, dtype=torch.complex128, device="cuda")
    h_h = torch.zeros(B, dtype=torch.complex128, device="cuda")
    gb.backend.get_ll(d_h, h_h, dev(A_pm), dev(E_pm), dev(g["A_data"].ravel()),
                      dev(g["E_data"].ravel()), dev(g["A_psd"].ravel()),
                      dev(g["E_psd"].ravel()), W["df"], dev(si), int(g["N"]), B, dev(di),
                      dev(ni), L)
    np.testing.assert_allclose(d_h.cpu().numpy(), ref_dh, rtol=1e-12)
    np.testing.assert_allclose(h_h.cpu().numpy().real, ref_hh.real, rtol=1e-12)
    # one PSD array for both channels (the kernel then forms one weight per bin)
    ref_dh, ref_hh = O.get_ll_native(A_pm, E_pm, g["A_data"].ravel(), g["E_data"].ravel(),
                                     g["A_psd"].ravel(), g["A_psd"].ravel(), W["df"], si,
                                     int(g["N"]), B, di, ni, L)
    S = dev(g["A_psd"].ravel())
    gb.backend.get_ll(d_h, h_h, dev(A_pm), dev(E_pm), dev(g["A_data"].ravel()),
                      dev(g["E_data"].ravel()), S, S, W["df"], dev(si), int(g["N"]), B, dev(di),
                      dev(ni), L)
    np.testing.assert_allclose(d_h.cpu().numpy(), ref_dh, rtol=1e-12)
    np.testing.assert_allclose(h_h.cpu().numpy().real, ref_hh.real, rtol=1e-12)
    # the FP64 variant: the reference's arithmetic, to FP64 rounding
    gb.backend.get_ll(d_h, h_h, dev(A_pm), dev(E_pm), dev(g["A_data"].ravel()),
                      dev(g["E_data"].ravel()), S, S, W["df"], dev(si), int(g["N"]), B, dev(di),
                      dev(ni), L, fp64=True)
    np.testing.assert_allclose(d_h.cpu().numpy(), ref_dh, rtol=1e-14, atol=1e-14 * np.abs(ref_dh).max())
    np.testing.assert_allclose(h_h.cpu().numpy().real, ref_hh.real, rtol=1e-14)


def test_backend_get_ll_edges_odd_batch(gbgpu):
    """Drop-in get_ll on windows that cross both ends of the data (those bins
    count as zero and raise GBX_FLAG_WINDOW), an odd batch, two data and noise
    rows, a PSD bin at infinity (contributes zero, as 1/inf in FP64) and an
    all-zero template; then data_length = 0.  Reference sums in NumPy FP64;
    bound 1e-12 of sum |terms| per output."""
    from gbgpu_gb300 import _native as nat
    rng = np.random.default_rng(7)
    L, M, B = 600, 128, 5
    s = np.array([-40, 10, 300, 520, 472], dtype=np.int32)
    di = np.array([0, 1, 1, 0, 1], dtype=np.int32)
    ni = np.array([1, 0, 1, 1, 0], dtype=np.int32)
    cplx = lambda *shape: rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    A_d, E_d = 1e-20 * cplx(2, L), 1e-20 * cplx(2, L)
    A_p = 1e-40 * (1 + rng.random((2, L)))
    E_p = 2e-40 * (1 + rng.random((2, L)))
    A_p[1, 350] = np.inf
    A_t, E_t = 1e-21 * cplx(B, M), 1e-21 * cplx(B, M)
    A_t[2] = E_t[2] = 0.0
    df = 1.0 / 3.15e7
    ref_dh = np.zeros(B, complex)
    ref_hh = np.zeros(B)
    bound_dh = np.zeros(B)
    bound_hh = np.zeros(B)
    for b in range(B):
        j = s[b] + np.arange(M)
        ok = (j >= 0) & (j < L)
        jj = j[ok]
        for d, p, t in ((A_d, A_p, A_t), (E_d, E_p, E_t)):
            dh = np.conj(d[di[b], jj]) * t[b, ok] / p[ni[b], jj]
            hh = np.abs(t[b, ok]) ** 2 / p[ni[b], jj]
            ref_dh[b] += 4 * df * dh.sum()
            ref_hh[b] += 4 * df * hh.sum()
            bound_dh[b] += 4 * df * np.abs(dh).sum()
            bound_hh[b] += 4 * df * hh.sum()
    gb = gbgpu()
    d_h = torch.zeros(B, dtype=torch.complex128, device="cuda")
    h_h = torch.zeros(B, dtype=torch.complex128, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    gb.backend.get_ll(d_h, h_h, dev(O.point_major(A_t)), dev(O.point_major(E_t)),
                      dev(A_d.ravel()), dev(E_d.ravel()), dev(A_p.ravel()), dev(E_p.ravel()),
                      df, dev(s), M, B, dev(di), dev(ni), L, status=st)
    got_dh, got_hh = d_h.cpu().numpy(), h_h.cpu().numpy()
    assert np.all(np.abs(got_dh - ref_dh) <= 1e-12 * bound_dh + 1e-300)
    assert np.all(np.abs(got_hh.real - ref_hh) <= 1e-12 * bound_hh + 1e-300)
    assert got_dh[2] == 0 and got_hh[2] == 0
    assert int(st.item()) & nat.GBX_FLAG_WINDOW
    # the FP64 variant under the same edges: FP64 rounding of the same sums
    st.zero_()
    gb.backend.get_ll(d_h, h_h, dev(O.point_major(A_t)), dev(O.point_major(E_t)),
                      dev(A_d.ravel()), dev(E_d.ravel()), dev(A_p.ravel()), dev(E_p.ravel()),
                      df, dev(s), M, B, dev(di), dev(ni), L, status=st, fp64=True)
    f_dh, f_hh = d_h.cpu().numpy(), h_h.cpu().numpy()
    assert np.all(np.abs(f_dh - ref_dh) <= 1e-14 * bound_dh + 1e-300)
    assert np.all(np.abs(f_hh.real - ref_hh) <= 1e-14 * bound_hh + 1e-300)
    assert f_dh[2] == 0 and f_hh[2] == 0
    assert int(st.item()) & nat.GBX_FLAG_WINDOW
    # windows inside the data raise no flag
    st.zero_()
    sel = [1, 2, 4]
    gb.backend.get_ll(d_h[:3], h_h[:3], dev(O.point_major(A_t[sel])), dev(O.point_major(E_t[sel])),
                      dev(A_d.ravel()), dev(E_d.ravel()), dev(A_p.ravel()), dev(E_p.ravel()),
                      df, dev(s[sel]), M, 3, dev(di[sel]), dev(ni[sel]), L, status=st)
    assert int(st.item()) == 0
    np.testing.assert_allclose(d_h[:3].cpu().numpy(), got_dh[sel], rtol=0, atol=0)
    # no data at all: every bin is outside, sums are zero
    gb.backend.get_ll(d_h, h_h, dev(O.point_major(A_t)), dev(O.point_major(E_t)),
                      dev(A_d.ravel()), dev(E_d.ravel()), dev(A_p.ravel()), dev(E_p.ravel()),
                      df, dev(s), M, B, dev(di), dev(ni), 0, status=st)
    assert not torch.any(d_h != 0) and not torch.any(h_h != 0)
    assert int(st.item()) & nat.GBX_FLAG_WINDOW


@pytest.mark.parametrize("L", [400, 401])
def test_backend_get_ll_rows_outside_the_arrays_are_flagged(gbgpu, L):
    """Drop-in get_ll with a data_index row past the data array and a
    negative noise_index row: those binaries are flagged GBX_FLAG_INDEX, not
    read, and get zero outputs; the other binaries match the FP64 sums.  An
    odd data length puts odd PSD rows at odd element offsets (the staged
    copies start at the even element below)."""
    from gbgpu_gb300 import _native as nat
    rng = np.random.default_rng(11)
    M, B = 64, 4
    cplx = lambda *shape: rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    A_d, E_d = 1e-20 * cplx(2, L), 1e-20 * cplx(2, L)
    A_p = 1e-40 * (1 + rng.random((2, L)))
    E_p = 1e-40 * (1 + rng.random((2, L)))
    A_t, E_t = 1e-20 * cplx(B, M), 1e-20 * cplx(B, M)
    s = np.array([10, 100, 200, 300], dtype=np.int32)
    di = np.array([0, 5, 1, 1], dtype=np.int32)        # row 5 is past the two data rows
    ni = np.array([1, 0, -1, 0], dtype=np.int32)       # row -1 is before the first
    df = 1e-8
    gb = gbgpu()
    d_h = torch.full((B,), 7.0, dtype=torch.complex128, device="cuda")
    h_h = torch.full((B,), 7.0, dtype=torch.complex128, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    gb.backend.get_ll(d_h, h_h, dev(O.point_major(A_t)), dev(O.point_major(E_t)),
                      dev(A_d.ravel()), dev(E_d.ravel()), dev(A_p.ravel()), dev(E_p.ravel()),
                      df, dev(s), M, B, dev(di), dev(ni), L, status=st)
    assert int(st.item()) & nat.GBX_FLAG_INDEX
    got = d_h.cpu().numpy()
    assert got[1] == 0 and got[2] == 0 and h_h[1].item() == 0 and h_h[2].item() == 0
    for b in (0, 3):
        j = s[b] + np.arange(M)
        ref = 4 * df * sum((np.conj(d[di[b], j]) * t[b] / p[ni[b], j]).sum()
                           for d, p, t in ((A_d, A_p, A_t), (E_d, E_p, E_t)))
        np.testing.assert_allclose(got[b], ref, rtol=1e-12)


def test_fill_global_template_matches_reference(gbgpu):
    g = load_golden("fill_basic")
    gb = gbgpu()
    t = dev(g["templates_before"]).clone()
    gb.fill_global_template(dev(g["group_index"]), t, dev(g["A"]), dev(g["E"]),
                            dev(g["start_inds"]), start_freq_ind=int(g["start_freq_ind"]))
    t = t.cpu().numpy()
    ref = g["templates_after"]
    np.testing.assert_array_equal(t[:, 2], ref[:, 2])          # untouched channel
    assert rel_err(t[:, :2], ref[:, :2]) < 1e-13
    # NumPy templates are filled in place as well
    tn = g["templates_before"].copy()
    gb.fill_global_template(g["group_index"], tn, g["A"], g["E"], g["start_inds"],
                            start_freq_ind=int(g["start_freq_ind"]))
    assert rel_err(tn, ref) < 1e-13


def test_backend_fill_global_dropin(gbgpu):
    g = load_golden("fill_basic")
    A, E = g["A"], g["E"]
    B, N = A.shape
    G = g["templates_after"].shape[0]
    L = g["templates_after"].shape[-1]
    si = (g["start_inds"] - int(g["start_freq_ind"])).astype(np.int32)
    rA = np.zeros(G * L, np.complex128)
    rE = np.zeros(G * L, np.complex128)
    O.fill_global_native(rA, rE, O.point_major(A), O.point_major(E), si, N, B,
                         g["group_index"], L)
    gb = gbgpu()
    tA = torch.zeros(G * L, dtype=torch.complex128, device="cuda")
    tE = torch.zeros(G * L, dtype=torch.complex128, device="cuda")
    gb.backend.fill_global(tA, tE, dev(O.point_major(A)), dev(O.point_major(E)), dev(si), N, B,
                           dev(g["group_index"]), L)
    assert rel_err(tA.cpu().numpy(), rA) < 1e-13
    assert rel_err(tE.cpu().numpy(), rE) < 1e-13


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_generate_global_template_matches_reference(gbgpu, precision):
    g = load_golden("fill_basic")
    gb = gbgpu()
    t = torch.zeros(g["generated"].shape, dtype=torch.complex128, device="cuda")
    gb.generate_global_template(g["params"].T, dev(g["group_index"]), t, N=int(g["N"]),
                                T=float(g["T"]), dt=float(g["dt"]),
                                start_freq_ind=int(g["start_freq_ind"]), precision=precision)
    err = rel_err(t.cpu().numpy(), g["generated"])
    assert err < (FP64_TOL if precision == "fp64" else 2e-6), err


@pytest.mark.parametrize("case", ["third_n256", "third_n512_1yr", "third_n128_tdi2"])
def test_third_body_matches_reference(case):
    from gbgpu_gb300 import GBGPUThirdBody
    g = load_golden(case)
    gb = GBGPUThirdBody()
    gb.run_wave(*g["params"], g["A2"], g["varpi"], g["e2"], g["P2"], g["T2"], N=int(g["N"]),
                T=float(g["T"]), dt=float(g["dt"]), tdi2=bool(g["tdi2"]))
    np.testing.assert_array_equal(gb.start_inds.cpu().numpy(), g["start_inds"])
    assert np.max(rel_err(gb.XYZf.cpu().numpy(), g["XYZf"], axis=(1, 2))) < FP64_TOL
    assert np.max(rel_err(gb.AETf.cpu().numpy(), g["AETf"], axis=(1, 2))) < FP64_TOL


def test_pair_form_declines_the_third_body():
    """The pair form covers the 9-parameter model; the third body's 14 raise."""
    from gbgpu_gb300 import GBGPUThirdBody
    g = load_golden("ll_third")
    gb = GBGPUThirdBody()
    gb.d_d = float(g["d_d"])
    with pytest.raises(RuntimeError, match="pair form"):
        gb.get_ll(g["params"], [dev(g["A_data"]), dev(g["E_data"])],
                  [dev(g["A_psd"]), dev(g["E_psd"])], N=int(g["N"]), T=float(g["T"]),
                  dt=float(g["dt"]), tdi2=bool(g["tdi2"]),
                  start_freq_ind=int(g["start_freq_ind"]), precision="pair")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_third_body_get_ll_matches_reference(precision):
    """GBGPUThirdBody.get_ll, (14, B) parameters, TDI-2, against the reference's."""
    from gbgpu_gb300 import GBGPUThirdBody
    g = load_golden("ll_third")
    gb = GBGPUThirdBody()
    gb.d_d = float(g["d_d"])
    like = gb.get_ll(g["params"], [dev(g["A_data"]), dev(g["E_data"])],
                     [dev(g["A_psd"]), dev(g["E_psd"])], N=int(g["N"]), T=float(g["T"]),
                     dt=float(g["dt"]), tdi2=bool(g["tdi2"]),
                     start_freq_ind=int(g["start_freq_ind"]), precision=precision)
    snr2 = np.abs(g["h_h"].real)
    if precision == "fp64":
        np.testing.assert_allclose(gb.d_h.cpu().numpy(), g["d_h"], rtol=FP64_TOL, atol=0)
        np.testing.assert_allclose(gb.h_h.cpu().numpy().real, g["h_h"].real, rtol=FP64_TOL)
        np.testing.assert_allclose(like, g["like"], rtol=FP64_TOL)
    else:
        assert np.max(np.abs(like - g["like"]) / np.maximum(1.0, snr2)) < MIXED_LL_TOL
    np.testing.assert_array_equal(gb.start_inds.cpu().numpy(), g["start_inds"])


def _ll_setup(B, N, seed, f_lo=2e-3, f_hi=2.02e-3, T=4 * 31557600.0, dt=10.0, third=False):
    from gbgpu_gb300.sensitivity import A1TDISens
    rng = np.random.default_rng(seed)
    p = np.array([10 ** rng.uniform(-23, -21, B), rng.uniform(f_lo, f_hi, B),
                  10 ** rng.uniform(-18, -15, B), np.zeros(B), rng.uniform(0, 2 * np.pi, B),
                  np.arccos(rng.uniform(-1, 1, B)), rng.uniform(0, np.pi, B),
                  rng.uniform(0, 2 * np.pi, B), np.arcsin(rng.uniform(-1, 1, B))])
    p[3] = 11 / 3 * p[2] ** 2 / p[1]
    extra = None
    if third:
        P2 = 10 ** rng.uniform(0, np.log10(40), B)
        extra = (10 ** rng.uniform(-2, 2, B), rng.uniform(0, 2 * np.pi, B),
                 rng.uniform(0, 0.9, B), P2, rng.uniform(0, 1, B) * P2)
    Nmax = int(np.max(N))
    si = O.start_indices(p[1], Nmax, T, dt)
    s0 = int(si.min()) - Nmax
    L = int(si.max()) + 2 * Nmax - s0
    f = (np.arange(L) + s0) / (int(T / dt) * dt)
    S = A1TDISens.get_Sn(f)
    Tu = int(T / dt) * dt
    data = [np.sqrt(S * Tu / 4) * (rng.standard_normal(L) + 1j * rng.standard_normal(L))
            for _ in range(2)]
    return p, extra, data, S, s0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_uneven_N_persistent_kernel(gbgpu, precision):
    """Per-binary N in one launch == the oracle run one N-group at a time."""
    B = 300
    rng = np.random.default_rng(3)
    Ns = 2 ** rng.integers(5, 12, B)
    p, _, data, S, s0 = _ll_setup(B, Ns, 4)
    gb = gbgpu()
    gb.d_d = 0.0
    like = gb.get_ll(p, [dev(x) for x in data], [dev(S), dev(S)], N=Ns, T=4 * 31557600.0,
                     dt=10.0, start_freq_ind=s0, precision=precision)
    hh = gb.h_h.cpu().numpy().real
    ref = np.zeros(B)
    ref_hh = np.zeros(B)
    for N in np.unique(Ns):
        sel = Ns == N
        r, _, h, _ = O.get_ll(p[:, sel], data, [S, S], int(N), T=4 * 31557600.0, dt=10.0,
                              start_freq_ind=s0, return_terms=True)
        ref[sel] = r
        ref_hh[sel] = h.real
    scale = np.maximum(1.0, ref_hh)
    tol = FP64_TOL if precision == "fp64" else MIXED_LL_TOL
    assert np.max(np.abs(like - ref) / scale) < tol
    assert np.max(np.abs(hh - ref_hh) / scale) < tol


@pytest.mark.parametrize("N,precision", [(32, "fp64"), (4096, "fp64"), (8192, "mixed"),
                                         (1024, "mixed"), (32, "pair"), (4096, "pair")])
def test_ll_extreme_N(gbgpu, N, precision):
    B = 5
    p, _, data, S, s0 = _ll_setup(B, N, 7, f_lo=1e-2, f_hi=1.001e-2)
    gb = gbgpu()
    gb.d_d = 0.0
    like = gb.get_ll(p, [dev(x) for x in data], [dev(S), dev(S)], N=N, T=4 * 31557600.0,
                     dt=5.0, start_freq_ind=s0, precision=precision)
    ref, _, hh, _ = O.get_ll(p, data, [S, S], N, T=4 * 31557600.0, dt=5.0, start_freq_ind=s0,
                             return_terms=True)
    tol = {"fp64": FP64_TOL, "pair": PAIR_LL_TOL}.get(precision, MIXED_LL_TOL)
    assert np.max(np.abs(like - ref) / np.maximum(1.0, hh.real)) < tol


@pytest.mark.parametrize("N,B", [(32, 5), (64, 3), (32, 1)])
def test_pair_waveform_small_N_odd_batch(gbgpu, N, B):
    """The pair transform's last five stages run on half-warps, one 32-element
    block each: an odd number of blocks (three channels, odd batches at N = 32,
    64) leaves a spare half-warp that repeats the last block and stores
    nothing.  Windows against the oracle, start indices bit-exact."""
    rng = np.random.default_rng(40 + N + B)
    f0 = rng.uniform(2e-4, 4e-4, B)
    fd = 10 ** rng.uniform(-18, -17, B)
    p = np.array([10 ** rng.uniform(-23, -21, B), f0, fd, 11 / 3 * fd ** 2 / f0,
                  rng.uniform(0, 2 * np.pi, B), np.arccos(rng.uniform(-1, 1, B)),
                  rng.uniform(0, np.pi, B), rng.uniform(0, 2 * np.pi, B),
                  np.arcsin(rng.uniform(-1, 1, B))])
    gb = gbgpu()
    gb.run_wave(*p, N=N, T=4 * 31557600.0, dt=10.0, precision="pair")
    W = O.waveform(p, N, T=4 * 31557600.0, dt=10.0)
    np.testing.assert_array_equal(gb.start_inds.cpu().numpy(), W["start_inds"])
    assert np.max(rel_err(gb.XYZf.cpu().numpy(), W["XYZf"], axis=(1, 2))) < 1e-10
    assert np.max(rel_err(gb.AETf.cpu().numpy(), W["AETf"], axis=(1, 2))) < 1e-10


@pytest.mark.parametrize("N,tdi2", [(64, False), (256, True), (1024, False), (4096, True)])
def test_pair_waveform_across_the_band(gbgpu, N, tdi2):
    """Pair windows against the oracle for binaries spread log-uniformly over
    1e-4 .. 2.5e-2 Hz (omega L from 0.005 to 1.3), all angles random, fdot up
    to 1e-15: the stated 1e-10 normwise bound over the whole band."""
    rng = np.random.default_rng(900 + N)
    B = 60
    f0 = 10 ** rng.uniform(-4, np.log10(2.5e-2), B)
    fd = 10 ** rng.uniform(-19, -15, B)
    p = np.array([10 ** rng.uniform(-23, -21, B), f0, fd, 11 / 3 * fd ** 2 / f0,
                  rng.uniform(0, 2 * np.pi, B), np.arccos(rng.uniform(-1, 1, B)),
                  rng.uniform(0, np.pi, B), rng.uniform(0, 2 * np.pi, B),
                  np.arcsin(rng.uniform(-1, 1, B))])
    if tdi2:
        p[2], p[3] = 0.0, 0.0      # the reference's TDI-2 factor is taken at f0
    gb = gbgpu()
    gb.run_wave(*p, N=N, T=4 * 31557600.0, dt=5.0, tdi2=tdi2, precision="pair")
    W = O.waveform(p, N, T=4 * 31557600.0, dt=5.0, tdi2=tdi2)
    np.testing.assert_array_equal(gb.start_inds.cpu().numpy(), W["start_inds"])
    err = rel_err(gb.XYZf.cpu().numpy(), W["XYZf"], axis=(1, 2))
    print(f"pair N={N} tdi2={tdi2}: worst window error {err.max():.2e} "
          f"(f0 {p[1][np.argmax(err)]:.2e} Hz)")
    assert np.max(err) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_third_body_ll(precision):
    from gbgpu_gb300 import GBGPUThirdBody
    B, N = 40, 512
    p, extra, data, S, s0 = _ll_setup(B, N, 11, dt=5.0, third=True)
    gb = GBGPUThirdBody()
    gb.d_d = 0.0
    full = np.concatenate([p, np.array(extra)])
    like = gb.get_ll(full, [dev(x) for x in data], [dev(S), dev(S)], N=N, T=4 * 31557600.0,
                     dt=5.0, start_freq_ind=s0, precision=precision)
    ref, _, hh, _ = O.get_ll(p, data, [S, S], N, T=4 * 31557600.0, dt=5.0, start_freq_ind=s0,
                             third=extra, return_terms=True)
    tol = FP64_TOL if precision == "fp64" else MIXED_LL_TOL
    assert np.max(np.abs(like - ref) / np.maximum(1.0, hh.real)) < tol


def test_window_outside_data_flags_and_counts_zero(gbgpu):
    p, _, data, S, s0 = _ll_setup(4, 128, 12)
    gb = gbgpu()
    gb.d_d = 0.0
    cut = 200    # data arrays end inside the last windows
    d = [x[:-cut] for x in data]
    with pytest.warns(UserWarning, match="extend past"):
        gb.get_ll(p, [dev(x) for x in d], [dev(S[:-cut])] * 2, N=128, T=4 * 31557600.0,
                  dt=10.0, start_freq_ind=s0)


def test_empty_batch(gbgpu):
    gb = gbgpu()
    gb.d_d = 0.0
    z = np.zeros(0)
    like = gb.get_ll(np.zeros((9, 0)), [dev(np.zeros(10, complex))] * 2, [dev(np.ones(10))] * 2,
                     N=128, T=4 * 31557600.0, dt=10.0)
    assert like.shape == (0,)
    del z


def test_inject_signal_matches_reference(gbgpu):
    g = load_golden("misc")
    gb = gbgpu()
    A, E = gb.inject_signal(*[x[0] for x in g["inj_params"]], N=128, T=4 * 31557600.0, dt=10.0)
    assert len(A) == int(g["inj_len"])
    s = int(g["inj_start"])
    assert np.count_nonzero(A) == int(g["inj_nnz"])
    assert rel_err(A[s:s + 128], g["inj_A"]) < FP64_TOL
    assert rel_err(E[s:s + 128], g["inj_E"]) < FP64_TOL


def test_information_matrix_matches_reference(gbgpu):
    from gbgpu_gb300.sensitivity import A1TDISens
    g = load_golden("fisher")
    gb = gbgpu()
    fm = gb.information_matrix(g["params"].copy(), eps=1e-9, inds=g["inds"], N=int(g["N"]),
                               T=float(g["T"]), dt=float(g["dt"]), psd_func=A1TDISens.get_Sn)
    # finite differences with eps = 1e-9 amplify 1e-13 waveform differences
    # by 1/eps, so the matrices agree to about 1e-3 relative
    for b in range(fm.shape[0]):
        assert rel_err(fm[b], g["fisher"][b]) < 5e-3


def test_errors_like_the_reference(gbgpu):
    gb = gbgpu()
    with pytest.raises(ValueError, match="d_d"):
        gb.get_ll(np.zeros((9, 1)), [dev(np.zeros(4, complex))] * 2, [dev(np.ones(4))] * 2, N=64)
    gb.d_d = 0.0
    with pytest.raises(ValueError, match="data_index"):
        gb.get_ll(np.ones((9, 1)) * 1e-3, [dev(np.zeros(4, complex))] * 2,
                  [dev(np.ones(4))] * 2, N=64, data_index=dev(np.zeros(1), torch.int32))
    with pytest.raises(ValueError, match="Observation time"):
        gb.run_wave(*np.ones((9, 1)) * 1e-3, N=64, T=1e10)
    t = torch.zeros((2, 1, 10), dtype=torch.complex128, device="cuda")
    with pytest.raises(ValueError, match="A and E"):
        gb.fill_global_template(np.zeros(1, np.int32), t, np.zeros((1, 64)), np.zeros((1, 64)),
                                np.zeros(1, np.int32))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_workspace_and_in_tile_setup_agree(gbgpu, precision):
    """gbx_waveform_ll with a prep workspace and with workspace=NULL (per-tile
    set-up) evaluate the same per-binary constants: results are identical."""
    import ctypes
    from gbgpu_gb300 import _native as nat
    B = 257
    rng = np.random.default_rng(21)
    Ns = 2 ** rng.integers(5, 12, B)
    p, _, data, S, s0 = _ll_setup(B, Ns, 22)
    gb = gbgpu()
    dd = [dev(x) for x in data]
    Sd = dev(S)
    prm = dev(p).contiguous()
    plan = gb._plan(Ns, int(4 * 31557600.0 / 10.0) * 10.0, precision, False, 9)
    la = nat.LLArgs()
    la.A_data, la.E_data = dd[0].data_ptr(), dd[1].data_ptr()
    la.A_psd = la.E_psd = Sd.data_ptr()
    la.data_length, la.num_data, la.num_psd = len(S), 1, 1
    la.df = 1.0 / (4 * 31557600.0)
    outs = []
    for use_ws in (True, False):
        a = plan.args(prm, s0)
        if not use_ws:
            a.workspace = None
            a.workspace_bytes = 0
        d_h = torch.zeros(B, dtype=torch.complex128, device="cuda")
        h_h = torch.zeros(B, dtype=torch.complex128, device="cuda")
        rc = nat.lib().gbx_waveform_ll(ctypes.byref(a), ctypes.byref(la), nat.ptr(d_h),
                                       nat.ptr(h_h), nat.stream_handle())
        nat.check(rc, "gbx_waveform_ll")
        outs.append((d_h.cpu().numpy(), h_h.cpu().numpy()))
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


class _CudaArrayOnly:
    """A device array of another library (CuPy, Numba, ...): only the CUDA array
    interface, no torch type."""

    def __init__(self, t):
        self._t = t

    @property
    def __cuda_array_interface__(self):
        return self._t.__cuda_array_interface__

    @property
    def shape(self):
        return tuple(self._t.shape)


def test_cuda_array_interface_inputs(gbgpu):
    """get_ll, fill_global_template (in place) and backend.get_ll take device
    arrays of other libraries without copies, with results identical to torch
    inputs."""
    g = load_golden("ll_multi")
    gb = gbgpu()
    gb.d_d = float(g["d_d"])
    kw = dict(N=int(g["N"]), T=float(g["T"]), dt=float(g["dt"]), tdi2=bool(g["tdi2"]),
              start_freq_ind=int(g["start_freq_ind"]),
              data_index=dev(g["data_index"], torch.int32),
              noise_index=dev(g["noise_index"], torch.int32))
    prm, dA, dE = dev(g["params"]), dev(g["A_data"]), dev(g["E_data"])
    pA, pE = dev(g["A_psd"]), dev(g["E_psd"])
    ref = gb.get_ll(prm, [dA, dE], [pA, pE], **kw)
    kw["data_index"] = _CudaArrayOnly(kw["data_index"])
    got = gb.get_ll(_CudaArrayOnly(prm), [_CudaArrayOnly(dA), _CudaArrayOnly(dE)],
                    [_CudaArrayOnly(pA), _CudaArrayOnly(pE)], **kw)
    np.testing.assert_array_equal(got, ref)
    # templates of another library are filled in place
    f = load_golden("fill_basic")
    t = dev(f["templates_before"]).clone()
    gb.fill_global_template(dev(f["group_index"]), _CudaArrayOnly(t), dev(f["A"]), dev(f["E"]),
                            dev(f["start_inds"]), start_freq_ind=int(f["start_freq_ind"]),
                            mode="deterministic")
    assert rel_err(t.cpu().numpy()[:, :2], f["templates_after"][:, :2]) < 1e-13
    # the backend method table takes them as well
    d_h = torch.zeros(3, dtype=torch.complex128, device="cuda")
    h_h = torch.zeros(3, dtype=torch.complex128, device="cuda")
    W = O.waveform(g["params"][:, :3], int(g["N"]), T=float(g["T"]), dt=float(g["dt"]), tdi2=True)
    si = (W["start_inds"] - int(g["start_freq_ind"])).astype(np.int32)
    A_pm, E_pm = O.point_major(W["AETf"][:, 0]), O.point_major(W["AETf"][:, 1])
    L = g["A_data"].shape[-1]
    z = torch.zeros(3, dtype=torch.int32, device="cuda")
    args = (dev(A_pm), dev(E_pm), dev(g["A_data"][0]), dev(g["E_data"][0]), dev(g["A_psd"][0]),
            dev(g["E_psd"][0]))
    gb.backend.get_ll(d_h, h_h, *args, W["df"], dev(si), int(g["N"]), 3, z, z, L)
    ref_dh = d_h.clone()
    gb.backend.get_ll(_CudaArrayOnly(d_h), h_h, *[_CudaArrayOnly(a) for a in args], W["df"],
                      _CudaArrayOnly(dev(si)), int(g["N"]), 3, z, z, L)
    assert torch.equal(d_h, ref_dh)


def test_tabulated_orbits_match_the_analytic_orbit(gbgpu):
    """GBGPU(orbits=TabulatedOrbits(...)) with 6-hourly samples of the analytic
    orbit gives the analytic orbit's waveforms (spline error ~1 m)."""
    from gbgpu_gb300.orbits import EqualArmlengthOrbits, TabulatedOrbits
    g = load_golden("wave_n256_tdi2")
    ana = EqualArmlengthOrbits()
    t = np.arange(0.0, 5 * 31557600.0, 21600.0)
    tab = TabulatedOrbits(t, np.stack([ana.get_pos(t, np.full(t.size, s)) for s in (1, 2, 3)]),
                          ana.armlength)
    a, b = gbgpu(), gbgpu(orbits=tab)
    kw = dict(N=int(g["N"]), T=float(g["T"]), dt=float(g["dt"]), tdi2=bool(g["tdi2"]))
    a.run_wave(*g["params"], **kw)
    b.run_wave(*g["params"], **kw)
    np.testing.assert_array_equal(b.start_inds.cpu().numpy(), a.start_inds.cpu().numpy())
    assert np.max(rel_err(b.AETf.cpu().numpy(), a.AETf.cpu().numpy(), axis=(1, 2))) < 1e-6


def test_out_of_range_rows_raise_and_leave_other_binaries_intact(gbgpu):
    """A data_index / noise_index row outside the data or PSD arrays, or a
    group_index outside the templates, is caught in the kernel (that binary is
    skipped, GBX_FLAG_INDEX is set) and raised on the host as ValueError; the
    other binaries' results are those of a call without the bad row."""
    g = load_golden("ll_multi")                      # 3 data rows, 2 PSD rows, 10 binaries
    gb = gbgpu()
    gb.d_d = float(g["d_d"])
    data = [dev(g["A_data"]), dev(g["E_data"])]
    psd = [dev(g["A_psd"]), dev(g["E_psd"])]
    kw = dict(N=int(g["N"]), T=float(g["T"]), dt=float(g["dt"]), tdi2=bool(g["tdi2"]),
              start_freq_ind=int(g["start_freq_ind"]))
    di, ni = g["data_index"].astype(np.int32), g["noise_index"].astype(np.int32)
    gb.get_ll(g["params"], data, psd, data_index=dev(di), noise_index=dev(ni), **kw)
    good = gb.d_h.cpu().numpy()
    bad_di, bad_ni = di.copy(), ni.copy()
    bad_di[3] = 7
    bad_ni[3] = 7
    for d_rows, n_rows in ((bad_di, ni), (di, bad_ni)):
        with pytest.raises(ValueError, match="out of range"):
            gb.get_ll(g["params"], data, psd, data_index=dev(d_rows), noise_index=dev(n_rows),
                      **kw)
        np.testing.assert_array_equal(np.delete(gb.d_h.cpu().numpy(), 3), np.delete(good, 3))
    f = load_golden("fill_basic")
    gi = f["group_index"].astype(np.int32).copy()
    gi[0] = 99
    t = dev(f["templates_before"]).clone()
    with pytest.raises(ValueError, match="out of range"):
        gb.fill_global_template(dev(gi), t, dev(f["A"]), dev(f["E"]), dev(f["start_inds"]),
                                start_freq_ind=int(f["start_freq_ind"]))
