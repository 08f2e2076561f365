"""The plain-FP64 workload at its full size against the oracle.

1,000 binaries (amp log-U(1e-23, 1e-21), f0 U(1e-3, 5e-3) Hz, fdot
log-U(1e-18, 1e-15), fddot = 11/3 fdot^2/f0, isotropic angles), N = 128,
T = 4 x 31,557,600 s, dt = 10 s, oversample 1, no TDI-2; data = the injected
sum of all 1,000 (the oracle's scatter-add) + Gaussian noise from the
analytic A/E PSD on the 4-yr grid from 0 to 0.1 Hz (12,623,041 bins).
run_wave (reference gbgpu.py:108-316) and get_ll (gbgpu.py:580-735) are
compared with the oracle: start indices bit-exact, A/E/T and X/Y/Z within
1e-10 normwise per binary, <d|h> and <h|h> within 1e-10 (FP64 form) or
1e-9 (pair form) of max(|term|, 1), and the mixed form within |dlogL| <=
1e-6 max(1, <h|h>).
"""

import numpy as np
import pytest

import fastgb_oracle as O
from conftest import rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

T_OBS, DT, N = 4 * 31557600.0, 10.0, 128


@pytest.fixture(scope="module")
def cfg0():
    import bench
    p = bench.draw_config0(2026)
    dA, dE, S = bench.host_noise(2027)
    W = O.waveform(p, N, T=T_OBS, dt=DT)
    B = p.shape[1]
    O.fill_global_native(dA, dE, O.point_major(W["AETf"][:, 0]), O.point_major(W["AETf"][:, 1]),
                         W["start_inds"].astype(np.int32), N, B, np.zeros(B, np.int32), len(S))
    _, d_h, h_h, _ = O.get_ll(p, [dA, dE], [S, S], N, T=T_OBS, dt=DT, return_terms=True)
    return p, dA, dE, S, W, d_h, h_h


def test_config0_run_wave_matches_the_oracle(cfg0):
    from gbgpu_gb300 import GBGPU
    p, _, _, _, W, _, _ = cfg0
    gb = GBGPU()
    gb.run_wave(*p, N=N, T=T_OBS, dt=DT)
    np.testing.assert_array_equal(gb.start_inds.cpu().numpy(), W["start_inds"])
    assert np.max(rel_err(gb.AETf.cpu().numpy(), W["AETf"], axis=(1, 2))) < 1e-10
    assert np.max(rel_err(gb.XYZf.cpu().numpy(), W["XYZf"], axis=(1, 2))) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "pair", "mixed"])
def test_config0_get_ll_matches_the_oracle(cfg0, precision):
    from gbgpu_gb300 import GBGPU
    p, dA, dE, S, _, d_h, h_h = cfg0
    gb = GBGPU()
    gb.d_d = 0.0
    dev = lambda x: torch.as_tensor(x, device="cuda")
    gb.get_ll(p, [dev(dA), dev(dE)], [dev(S), dev(S)], N=N, T=T_OBS, dt=DT, precision=precision)
    got_dh, got_hh = gb.d_h.cpu().numpy(), gb.h_h.real.cpu().numpy()
    if precision == "mixed":
        dl = np.abs((got_dh.real - d_h.real) - 0.5 * (got_hh - h_h.real))
        assert np.max(dl / np.maximum(1.0, h_h.real)) < 1e-6
    else:
        tol = 1e-10 if precision == "fp64" else 1e-9
        assert np.all(np.abs(got_dh - d_h) <= tol * np.maximum(np.abs(d_h), 1.0))
        assert np.all(np.abs(got_hh - h_h.real) <= tol * np.maximum(h_h.real, 1.0))
