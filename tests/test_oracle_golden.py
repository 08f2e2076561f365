"""The CPU oracle against golden vectors from the reference's own code.

The fixtures in tests/golden were produced by tests/golden/make_golden.py,
which runs the reference's gbgpu.py / thirdbody.py / utility.py and its
gbgpu_utils.cu (compiled as C++).  These tests pin the oracle before it is
compared against the CUDA path.
"""

import numpy as np
import pytest

import fastgb_oracle as O
from conftest import load_golden, rel_err

WAVE_CASES = ["wave_n128", "wave_n256_tdi2", "wave_n64_1yr", "wave_n512_hf",
              "wave_n2048_hf", "wave_b1", "wave_n4096"]


@pytest.mark.parametrize("case", WAVE_CASES)
def test_waveform_matches_reference(case):
    g = load_golden(case)
    w = O.waveform(g["params"], int(g["N"]), T=float(g["T"]), dt=float(g["dt"]),
                   tdi2=bool(g["tdi2"]))
    np.testing.assert_array_equal(w["start_inds"], g["start_inds"])
    assert np.max(rel_err(w["XYZf"], g["XYZf"], axis=(1, 2))) < 1e-12
    assert np.max(rel_err(w["AETf"], g["AETf"], axis=(1, 2))) < 1e-12
    np.testing.assert_allclose(O.point_major(w["AETf"][:, 0]), g["A_out"], rtol=0,
                               atol=1e-11 * np.abs(g["A_out"]).max())


@pytest.mark.parametrize("case", ["ll_basic", "ll_multi", "ll_phasemarg"])
def test_get_ll_matches_reference(case):
    g = load_golden(case)
    like, d_h, h_h, w = O.get_ll(
        g["params"], [g["A_data"], g["E_data"]], [g["A_psd"], g["E_psd"]], int(g["N"]),
        T=float(g["T"]), dt=float(g["dt"]), tdi2=bool(g["tdi2"]), d_d=float(g["d_d"]),
        start_freq_ind=int(g["start_freq_ind"]),
        data_index=g.get("data_index"), noise_index=g.get("noise_index"),
        phase_marginalize=bool(g["phase_marginalize"]), return_terms=True)
    np.testing.assert_array_equal(w["start_inds"], g["start_inds"])
    assert rel_err(d_h, g["d_h"]) < 1e-11
    assert rel_err(h_h, g["h_h"]) < 1e-11
    np.testing.assert_allclose(like, g["like"], rtol=1e-10)


def test_native_ll_bit_exact_on_reference_templates():
    """Same inputs as the reference C++ call -> identical bits."""
    g = load_golden("ll_basic")
    w = load_golden("ll_basic")
    # rebuild the exact arrays the reference passed to get_ll_wrap
    W = O.waveform(g["params"], int(g["N"]), T=float(g["T"]), dt=float(g["dt"]))
    si = (W["start_inds"] - int(g["start_freq_ind"])).astype(np.int32)
    B = W["AETf"].shape[0]
    args = (O.point_major(W["AETf"][:, 0]), O.point_major(W["AETf"][:, 1]),
            g["A_data"], g["E_data"], g["A_psd"], g["E_psd"], W["df"], si,
            int(g["N"]), B, np.zeros(B, np.int32), np.zeros(B, np.int32),
            g["A_data"].shape[-1])
    d1, h1 = O.get_ll_native(*args)
    d2, h2 = O.get_ll_native(*args, parallel=True)
    np.testing.assert_array_equal(d1, d2)
    np.testing.assert_array_equal(h1, h2)
    del w


def test_fill_global_matches_reference():
    g = load_golden("fill_basic")
    t = g["templates_before"].copy()
    O.fill_global_template(g["group_index"], t, g["A"], g["E"], g["start_inds"],
                           start_freq_ind=int(g["start_freq_ind"]))
    # channels 0/1 are overwritten with the fresh sums, channel 2 untouched
    np.testing.assert_array_equal(t, g["templates_after"])
    gen = np.zeros_like(g["generated"])
    W = O.waveform(g["params"], int(g["N"]), T=float(g["T"]), dt=float(g["dt"]))
    O.fill_global_template(g["group_index"], gen, W["AETf"][:, 0], W["AETf"][:, 1],
                           W["start_inds"], start_freq_ind=int(g["start_freq_ind"]))
    assert rel_err(gen, g["generated"]) < 1e-12


@pytest.mark.parametrize("case", ["third_n256", "third_n512_1yr", "third_n128_tdi2"])
def test_third_body_matches_reference(case):
    g = load_golden(case)
    w = O.waveform(g["params"], int(g["N"]), T=float(g["T"]), dt=float(g["dt"]),
                   tdi2=bool(g["tdi2"]),
                   third=(g["A2"], g["varpi"], g["e2"], g["P2"], g["T2"]))
    np.testing.assert_array_equal(w["start_inds"], g["start_inds"])
    assert np.max(rel_err(w["XYZf"], g["XYZf"], axis=(1, 2))) < 1e-11
    assert np.max(rel_err(w["AETf"], g["AETf"], axis=(1, 2))) < 1e-11


def test_third_body_get_ll_matches_reference():
    """GBGPUThirdBody.get_ll with (14, B) parameters, TDI-2, injected data."""
    g = load_golden("ll_third")
    p = g["params"]
    like, d_h, h_h, w = O.get_ll(
        p[:9], [g["A_data"], g["E_data"]], [g["A_psd"], g["E_psd"]], int(g["N"]),
        T=float(g["T"]), dt=float(g["dt"]), tdi2=bool(g["tdi2"]), d_d=float(g["d_d"]),
        start_freq_ind=int(g["start_freq_ind"]), third=tuple(p[9:14]), return_terms=True)
    np.testing.assert_array_equal(w["start_inds"], g["start_inds"])
    assert rel_err(d_h, g["d_h"]) < 1e-11
    assert rel_err(h_h, g["h_h"]) < 1e-11
    np.testing.assert_allclose(like, g["like"], rtol=1e-10)


def test_kepler_matches_reference():
    g = load_golden("kepler")
    u = O.kepler_u(g["l"], g["e"])
    np.testing.assert_allclose(u, g["u"], rtol=1e-13, atol=1e-13)


def test_start_indices_bit_exact():
    for case in WAVE_CASES:
        g = load_golden(case)
        si = O.start_indices(g["params"][1], int(g["N"]), float(g["T"]), float(g["dt"]))
        np.testing.assert_array_equal(si, g["start_inds"])
