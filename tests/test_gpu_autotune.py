"""Launch shapes (samples per tile, blocks per SM) and the autotuner.

Every shape must give the same likelihood as the oracle (the shapes differ
only in the summation order of FP32 partial sums); the autotuner must pick a
shape that runs, cache it, and reuse it.
"""

import json

import numpy as np
import pytest

import fastgb_oracle as O
from test_gpu_parity import FP64_TOL, MIXED_LL_TOL, _ll_setup, dev

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

T_OBS = 4 * 31557600.0


@pytest.mark.parametrize("tile,bps", [(64, 0), (256, 1), (1024, 2), (2048, 0), (4096, 1)])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_every_launch_shape_matches_oracle(tile, bps, precision):
    from gbgpu_gb300 import GBGPU
    B = 200
    rng = np.random.default_rng(21)
    Ns = 2 ** rng.integers(5, 12, B)
    p, _, data, S, s0 = _ll_setup(B, Ns, 22)
    gb = GBGPU()
    gb.d_d = 0.0
    ref = np.zeros(B)
    ref_hh = np.zeros(B)
    for N in np.unique(Ns):
        sel = Ns == N
        r, _, h, _ = O.get_ll(p[:, sel], data, [S, S], int(N), T=T_OBS, dt=10.0,
                              start_freq_ind=s0, return_terms=True)
        ref[sel] = r
        ref_hh[sel] = h.real
    gb._launch_shape = lambda *a, **k: (tile, bps)
    like = gb.get_ll(p, [dev(x) for x in data], [dev(S), dev(S)], N=Ns, T=T_OBS, dt=10.0,
                     start_freq_ind=s0, precision=precision)
    tol = FP64_TOL if precision == "fp64" else MIXED_LL_TOL
    assert np.max(np.abs(like - ref) / np.maximum(1.0, ref_hh)) < tol
    # uniform N with the same shape
    like1 = gb.get_ll(p[:, :40], [dev(x) for x in data], [dev(S), dev(S)], N=256, T=T_OBS,
                      dt=10.0, start_freq_ind=s0, precision=precision)
    r1, _, h1, _ = O.get_ll(p[:, :40], data, [S, S], 256, T=T_OBS, dt=10.0, start_freq_ind=s0,
                            return_terms=True)
    assert np.max(np.abs(like1 - r1) / np.maximum(1.0, h1.real)) < tol


def test_gradient_launch_shapes_agree():
    from gbgpu_gb300 import GBGPU
    B = 64
    rng = np.random.default_rng(31)
    Ns = 2 ** rng.integers(6, 11, B)
    p, _, data, S, s0 = _ll_setup(B, Ns, 32)
    gb = GBGPU()
    gb.d_d = 0.0
    out = {}
    for shape in ((0, 0), (256, 1), (2048, 0)):
        gb._launch_shape = lambda *a, **k: shape
        out[shape] = gb.get_ll_grad(p, [dev(x) for x in data], [dev(S), dev(S)], N=Ns, T=T_OBS,
                                    dt=10.0, start_freq_ind=s0)
    l0, g0 = out[(0, 0)]
    for shape, (l1, g1) in out.items():
        # shapes differ only in the order of FP32 partial sums
        np.testing.assert_allclose(l1, l0, rtol=1e-6, atol=1e-6)
        scale = np.sqrt(np.mean(g0 ** 2, axis=1, keepdims=True))
        assert np.max(np.abs(g1 - g0) / (np.abs(g0) + scale)) < 1e-4, shape


def test_autotuner_picks_caches_and_reuses(tmp_path, monkeypatch):
    from gbgpu_gb300 import GBGPU, autotune
    path = tmp_path / "tune.json"
    tuner = autotune.Autotuner(path=str(path), reps=2)
    monkeypatch.setattr(autotune, "_TUNER", tuner)
    B = 300
    rng = np.random.default_rng(41)
    Ns = 2 ** rng.integers(5, 12, B)
    p, _, data, S, s0 = _ll_setup(B, Ns, 42)
    gb = GBGPU(precision="mixed", autotune=True)
    gb.d_d = 0.0
    d = [dev(x) for x in data]
    like = gb.get_ll(p, d, [dev(S), dev(S)], N=Ns, T=T_OBS, dt=10.0, start_freq_ind=s0)
    saved = json.loads(path.read_text())
    assert len(saved) == 1
    (key, shape), = saved.items()
    assert "ll|" in key and tuple(shape) in tuner.candidates
    assert len(tuner.last_timings) >= len(autotune.TILES)
    # a second call reuses the cached shape: no timing run
    tuner.last_timings = None
    like2 = gb.get_ll(p, d, [dev(S), dev(S)], N=Ns, T=T_OBS, dt=10.0, start_freq_ind=s0)
    assert tuner.last_timings is None
    np.testing.assert_array_equal(like, like2)
    # a fresh tuner reads the file
    t2 = autotune.Autotuner(path=str(path))
    assert t2.lookup(key.split("|", 3)[3]) == tuple(shape)
    ref = O.get_ll(p[:, Ns == 256], data, [S, S], 256, T=T_OBS, dt=10.0, start_freq_ind=s0)
    assert np.allclose(like[Ns == 256], ref, rtol=1e-5, atol=1e-4)


def test_args_outlive_plan_cache_eviction():
    """A gbx_wave_args keeps its plan's device buffers alive after the plan
    leaves the cache (the tuner builds many plans per workload)."""
    import ctypes
    from gbgpu_gb300 import GBGPU
    from gbgpu_gb300 import _native as nat
    from gbgpu_gb300.gbgpu import _PLAN_CACHE
    B = 120
    rng = np.random.default_rng(51)
    Ns = 2 ** rng.integers(5, 11, B)
    p, _, data, S, s0 = _ll_setup(B, Ns, 52)
    gb = GBGPU()
    gb.d_d = 0.0
    T = int(T_OBS / 10.0) * 10.0
    prm = torch.as_tensor(p, device="cuda")
    d = [dev(x) for x in data]
    Sd = dev(S)
    zi = torch.zeros(B, dtype=torch.int32, device="cuda")
    la = gb._ll_args(d, [Sd, Sd], d[0].shape[0], zi, zi, T)
    a = gb._plan(Ns, T, "mixed", False, 9, 1024, 1).args(prm, s0)
    for k in range(_PLAN_CACHE + 4):                 # evict it
        gb._plan(int(2 ** (5 + k % 6)), T, "mixed", False, 9, 64 << (k % 7), k // 7)
    junk = torch.full((1 << 22,), -1, dtype=torch.int32, device="cuda")   # reuse freed memory
    d_h = torch.empty(B, dtype=torch.complex128, device="cuda")
    h_h = torch.empty(B, dtype=torch.complex128, device="cuda")
    rc = nat.lib().gbx_waveform_ll(ctypes.byref(a), ctypes.byref(la), nat.ptr(d_h), nat.ptr(h_h),
                                   nat.stream_handle())
    assert rc == 0
    ref = gb.get_ll(p, d, [Sd, Sd], N=Ns, T=T_OBS, dt=10.0, start_freq_ind=s0, precision="mixed")
    like = (-0.5 * (h_h.real - 2 * d_h.real)).cpu().numpy()
    np.testing.assert_allclose(like, ref, rtol=1e-6, atol=1e-6)
    del junk


def test_invalid_launch_shapes_are_rejected():
    """Bad tile values and shapes the shared memory cannot hold return errors
    (the autotuner skips such candidates)."""
    from gbgpu_gb300 import GBGPU, GBGPUThirdBody
    p, extra, data, S, s0 = _ll_setup(8, 256, 61, third=True)
    d = [dev(x) for x in data]
    for tile in (100, 32, 8192):
        gb = GBGPU()
        gb.d_d = 0.0
        gb._launch_shape = lambda *a, _t=tile, **k: (_t, 0)
        with pytest.raises(RuntimeError, match="tile"):
            gb.get_ll(p, d, [dev(S), dev(S)], N=256, T=T_OBS, dt=10.0, start_freq_ind=s0)
    # third-body gradient with N = 2048 and 4096-sample tiles: too much shared memory
    gb3 = GBGPUThirdBody()
    gb3.d_d = 0.0
    gb3._launch_shape = lambda *a, **k: (4096, 0)
    full = np.concatenate([p, np.array(extra)])
    with pytest.raises(RuntimeError, match="shared memory"):
        gb3.get_ll_grad(full, d, [dev(S), dev(S)], N=2048, T=T_OBS, dt=10.0, start_freq_ind=s0)
    # the default shape works for the same call
    gb3._launch_shape = lambda *a, **k: (0, 0)
    like, grad = gb3.get_ll_grad(full, d, [dev(S), dev(S)], N=2048, T=T_OBS, dt=10.0,
                                 start_freq_ind=s0)
    assert grad.shape == (14, 8) and np.all(np.isfinite(grad))


def test_n_array_changed_in_place_is_detected():
    """get_ll reuses the previous call's N-array key when the same buffer comes
    back with the same sampled entries, and verifies it after the launch: a
    buffer changed in place at an entry the quick check does not sample must
    still give the new assignment's likelihoods (those of a fresh object)."""
    from gbgpu_gb300 import GBGPU
    B = 200
    rng = np.random.default_rng(51)
    Ns = (2 ** rng.integers(7, 10, B)).astype(np.int64)
    p, _, data, S, s0 = _ll_setup(B, Ns, 52)
    kw = dict(T=T_OBS, dt=10.0, start_freq_ind=s0, precision="mixed")
    dd, SS = [dev(x) for x in data], [dev(S), dev(S)]
    gb = GBGPU()
    gb.d_d = 0.0
    first = gb.get_ll(p, dd, SS, N=Ns, **kw)
    again = gb.get_ll(p, dd, SS, N=Ns, **kw)                 # unchanged: same key, same bits
    np.testing.assert_array_equal(again, first)
    k = 1                                                    # the quick check samples 0, 3, 6, ...
    Ns[k] = 64
    second = gb.get_ll(p, dd, SS, N=Ns, **kw)
    fresh = GBGPU()
    fresh.d_d = 0.0
    np.testing.assert_array_equal(second, fresh.get_ll(p, dd, SS, N=Ns.copy(), **kw))
    assert second[k] != first[k]
