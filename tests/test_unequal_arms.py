"""Unequal arms: per-sample arm lengths in the link transfer functions,
antenna patterns and TDI delays (no counterpart in the reference, whose TDI
takes one armlength, gbgpu.py:167-170).

Pinned two ways: (1) with equal arms the model is the reference's TDI
exactly (CPU: the oracle's unequal-arm form against its equal-arm form, which
the reference's golden vectors pin; GPU: the kernels' unequal-arm path
against their equal-arm path), and (2) on orbits whose arms breathe by about
1 % the FP64 and pair kernels match the oracle's restatement of the same
formulas to 1e-10 (windows, normwise per binary) and their likelihoods to
1e-10 of max(|term|, 1).
"""

import numpy as np
import pytest

import fastgb_oracle as O
from conftest import rel_err

T_OBS, DT = 4 * 31557600.0, 10.0


class BreathingOrbits:
    """The analytic constellation with each spacecraft moved radially from
    the centroid by 1 % x sin(2 pi t / yr + 2 pi (s - 1)/3 + 0.3 s): arms of
    different, time-varying lengths (up to ~2 % apart), smooth in time."""

    def __init__(self):
        self.base = O.OracleOrbits()
        self.armlength = self.base.armlength
        self.t_base = self.base.t_base

    def configure(self, *args, **kwargs):
        return None

    def get_pos(self, t, sc):
        t = np.asarray(t, dtype=np.float64)
        sc = np.asarray(sc)
        C = sum(self.base.get_pos(t, np.full(t.shape, s)) for s in (1, 2, 3)) / 3.0
        own = self.base.get_pos(t, sc)
        eps = 0.01 * np.sin(2 * np.pi * t / O.YRSID_SI + 2 * np.pi * (sc - 1) / 3 + 0.3 * sc)
        return C + (1.0 + eps)[..., None] * (own - C)


def _params(B, seed, fdot=True, lo=1e-3, hi=2e-2):
    rng = np.random.default_rng(seed)
    f0 = 10 ** rng.uniform(np.log10(lo), np.log10(hi), B)
    fd = 10 ** rng.uniform(-18, -15, B) if fdot else np.zeros(B)
    return np.array([10 ** rng.uniform(-23, -21, B), f0, fd, 11 / 3 * fd ** 2 / f0,
                     rng.uniform(0, 2 * np.pi, B), np.arccos(rng.uniform(-1, 1, B)),
                     rng.uniform(0, np.pi, B), rng.uniform(0, 2 * np.pi, B),
                     np.arcsin(rng.uniform(-1, 1, B))])


@pytest.mark.parametrize("tdi2", [False, True])
def test_oracle_unequal_form_is_the_reference_tdi_with_equal_arms(tdi2):
    # TDI-2 of the reference is a constant factor at f0: compare at fdot = 0
    p = _params(12, 3, fdot=not tdi2)
    eq = O.waveform(p, 256, T=T_OBS, dt=DT, tdi2=tdi2)
    un = O.waveform(p, 256, T=T_OBS, dt=DT, tdi2=tdi2, unequal_arms=True)
    assert np.max(rel_err(un["XYZf"], eq["XYZf"], axis=(1, 2))) < 1e-11


def test_oracle_breathing_arms_change_the_windows():
    p = _params(12, 4)
    orb = BreathingOrbits()
    eq = O.waveform(p, 256, T=T_OBS, dt=DT, orbits=orb)
    un = O.waveform(p, 256, T=T_OBS, dt=DT, orbits=orb, unequal_arms=True)
    d = rel_err(un["XYZf"], eq["XYZf"], axis=(1, 2))
    assert np.all(d > 1e-4) and np.all(np.isfinite(d))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "pair"])
@pytest.mark.parametrize("tdi2", [False, True])
def test_kernels_unequal_path_equals_equal_path_on_equal_arms(precision, tdi2):
    pytest.importorskip("torch")
    from gbgpu_gb300 import GBGPU
    # against the FP64 equal-arm path (within 1e-13 of the reference): each form
    # keeps its own bound, so two pair results may differ by up to twice it
    p = _params(24, 5, fdot=not tdi2)
    out = []
    for unequal, prec in ((False, "fp64"), (True, precision)):
        gb = GBGPU(unequal_arms=unequal)
        gb.run_wave(*p, N=256, T=T_OBS, dt=DT, tdi2=tdi2, precision=prec)
        out.append(gb.XYZf.cpu().numpy())
    assert np.max(rel_err(out[1], out[0], axis=(1, 2))) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "pair"])
@pytest.mark.parametrize("N,tdi2", [(128, False), (256, True), (1024, False)])
def test_unequal_arm_windows_match_the_oracle(precision, N, tdi2):
    pytest.importorskip("torch")
    from gbgpu_gb300 import GBGPU
    p = _params(20, 6 + N)
    orb = BreathingOrbits()
    gb = GBGPU(orbits=orb, unequal_arms=True)
    gb.run_wave(*p, N=N, T=T_OBS, dt=DT, tdi2=tdi2, precision=precision)
    W = O.waveform(p, N, T=T_OBS, dt=DT, tdi2=tdi2, orbits=orb, unequal_arms=True)
    np.testing.assert_array_equal(gb.start_inds.cpu().numpy(), W["start_inds"])
    assert np.max(rel_err(gb.XYZf.cpu().numpy(), W["XYZf"], axis=(1, 2))) < 1e-10
    assert np.max(rel_err(gb.AETf.cpu().numpy(), W["AETf"], axis=(1, 2))) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "pair"])
def test_unequal_arm_likelihood_matches_the_oracle(precision):
    torch = pytest.importorskip("torch")
    from gbgpu_gb300 import GBGPU
    from gbgpu_gb300.sensitivity import A1TDISens
    N = 256
    p = _params(32, 21, lo=2e-3, hi=4e-3)
    orb = BreathingOrbits()
    T = int(T_OBS / DT) * DT
    si = O.start_indices(p[1], N, T_OBS, DT)
    s0 = int(si.min()) - N
    L = int(si.max()) + 2 * N - s0
    S = A1TDISens.get_Sn((np.arange(L) + s0) / T)
    rng = np.random.default_rng(22)
    data = [np.sqrt(S * T / 4) * (rng.standard_normal(L) + 1j * rng.standard_normal(L))
            for _ in range(2)]
    _, d_h, h_h, _ = O.get_ll(p, data, [S, S], N, T=T_OBS, dt=DT, tdi2=True, orbits=orb,
                              start_freq_ind=s0, return_terms=True, unequal_arms=True)
    gb = GBGPU(orbits=orb, unequal_arms=True)
    gb.d_d = 0.0
    dev = lambda x: torch.as_tensor(x, device="cuda")
    gb.get_ll(p, [dev(x) for x in data], [dev(S), dev(S)], N=N, T=T_OBS, dt=DT, tdi2=True,
              start_freq_ind=s0, precision=precision)
    tol = 1e-10 if precision == "fp64" else 1e-9
    assert np.all(np.abs(gb.d_h.cpu().numpy() - d_h) <= tol * np.maximum(np.abs(d_h), 1.0))
    assert np.all(np.abs(gb.h_h.real.cpu().numpy() - h_h.real) <=
                  tol * np.maximum(h_h.real, 1.0))


@pytest.mark.gpu
def test_unequal_arms_are_declined_by_the_fp32_form():
    torch = pytest.importorskip("torch")
    from gbgpu_gb300 import GBGPU
    p = _params(4, 9)
    gb = GBGPU(unequal_arms=True)
    gb.d_d = 0.0
    L = 4096
    d = torch.zeros(L, dtype=torch.complex128, device="cuda")
    S = torch.ones(L, dtype=torch.float64, device="cuda")
    with pytest.raises(RuntimeError, match="unequal arms"):
        gb.get_ll(p, [d, d], [S, S], N=128, T=T_OBS, dt=DT, precision="mixed",
                  start_freq_ind=int(O.start_indices(p[1], 128, T_OBS, DT).min()) - 100)
