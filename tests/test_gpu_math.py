"""The mixed kernels' own math helpers (through gbx_math_selftest).

sincos_mod (Cody-Waite reduction + Taylor series) is used for the reduced
carrier phase (|x| <= pi), omega L and large link arguments (|x| < 8); the
link helper gives sin(a)/a and cos(a).  Bounds: absolute error of sin/cos
below 3 FP32 ulps of 1 (3.6e-7), relative error of sin(a)/a below 3e-7.  The
integer-pipe FP64 -> FP32 conversion with a power-of-two scaling must equal a
host restatement bit for bit (round to nearest, ties away from zero; flush
below the normal range, infinity above).
"""

import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _run(x, which):
    from gbgpu_gb300 import _native as nat
    xd = torch.as_tensor(x, dtype=torch.float32, device="cuda")
    out = torch.empty(2 * xd.numel(), dtype=torch.float32, device="cuda")
    rc = nat.lib().gbx_math_selftest(ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                     int(xd.numel()), int(which), 0, nat.stream_handle())
    nat.check(rc, "gbx_math_selftest")
    torch.cuda.synchronize()
    o = out.cpu().numpy().astype(np.float64).reshape(-1, 2)
    return xd.cpu().numpy().astype(np.float64), o[:, 0], o[:, 1]


def test_sincos_mod_against_fp64():
    x = np.concatenate([np.linspace(-8.0, 8.0, 400001),
                        np.pi / 2 * np.arange(-5, 6) + 1e-7, np.pi / 4 * np.arange(-10, 11)])
    xs, s, c = _run(x, 0)
    assert np.max(np.abs(s - np.sin(xs))) < 3.6e-7
    assert np.max(np.abs(c - np.cos(xs))) < 3.6e-7
    # CUDA's own sincosf, for comparison of the error level
    t = torch.as_tensor(xs, dtype=torch.float32, device="cuda")
    s_ref = torch.sin(t).double().cpu().numpy()
    assert np.max(np.abs(s - np.sin(xs))) <= 4 * max(np.max(np.abs(s_ref - np.sin(xs))), 6e-8)


def test_link_sinc_cos_against_fp64():
    a = np.concatenate([np.linspace(-6.0, 6.0, 200001), [1e-6, -1e-6, 0.1599, 0.1601, 0.4999,
                                                         0.5001, 1.5999, 1.6001]])
    a = a[a != 0]
    xs, S, C = _run(a, 1)
    ref = np.sin(xs) / xs
    assert np.max(np.abs(S - ref) / np.maximum(np.abs(ref), 1e-3)) < 3e-7
    assert np.max(np.abs(C - np.cos(xs))) < 3.6e-7


def _d2f_host(x, e):
    """x * 2^e to FP32: 24 significant bits rounded to nearest, ties away;
    signed zero when the unrounded value is below FP32's normal range,
    infinity above (the rule the kernels implement)."""
    import math
    out = np.empty(x.shape, np.float32)
    for k, v in enumerate(x):
        if v == 0.0:
            out[k] = np.float32(math.copysign(0.0, v))
            continue
        if not np.isfinite(v):
            out[k] = np.float32(math.copysign(np.inf, v))
            continue
        m, ex = math.frexp(abs(v))                 # |v| = m 2^ex, m in [0.5, 1)
        E = ex - 1 + e                             # unbiased exponent of |v| 2^e
        if E < -126:
            val = 0.0
        elif E > 127:
            val = np.inf
        else:
            q = math.floor(m * 2 ** 24 + 0.5)       # ties away from zero
            val = q * 2.0 ** (ex + e - 24)
            if val >= 2.0 ** 128:
                val = np.inf
        out[k] = np.float32(math.copysign(val, v))
    return out


def test_d2f_scaled_bit_exact():
    from gbgpu_gb300 import _native as nat
    rng = np.random.default_rng(2)
    x = np.concatenate([10.0 ** rng.uniform(-60, 60, 4000) * rng.choice([-1, 1], 4000),
                        [0.0, -0.0, np.inf, -np.inf, 1.0, 1.5, 1.0 + 2.0 ** -24,
                         1.0 + 2.0 ** -24 + 2.0 ** -40, 1.0 - 2.0 ** -25, 2.0 ** -126,
                         2.0 ** -127, 3.4e38, 3.41e38, 1e-45]])
    for e in (0, 60, -60, 140):
        xd = torch.as_tensor(x, dtype=torch.float64, device="cuda")
        out = torch.empty(x.size, dtype=torch.float32, device="cuda")
        rc = nat.lib().gbx_math_selftest(ctypes.c_void_p(xd.data_ptr()),
                                         ctypes.c_void_p(out.data_ptr()), int(x.size), 2, e,
                                         nat.stream_handle())
        nat.check(rc, "gbx_math_selftest")
        got = out.cpu().numpy()
        want = _d2f_host(x, e)
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
