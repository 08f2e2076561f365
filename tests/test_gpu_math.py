"""The mixed kernels' own FP32 math helpers against FP64 (through gbx_math_selftest).

sincos_mod (Cody-Waite reduction + Taylor series) is used for the reduced
carrier phase (|x| <= pi), omega L and large link arguments (|x| < 8); the
link helper gives sin(a)/a and cos(a).  Bounds: absolute error of sin/cos
below 3 FP32 ulps of 1 (3.6e-7), relative error of sin(a)/a below 3e-7.
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
                                     int(xd.numel()), int(which), nat.stream_handle())
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
    a = np.concatenate([np.linspace(-6.0, 6.0, 200001), [1e-6, -1e-6, 0.4999, 0.5001, 1.5999,
                                                         1.6001]])
    a = a[a != 0]
    xs, S, C = _run(a, 1)
    ref = np.sin(xs) / xs
    assert np.max(np.abs(S - ref) / np.maximum(np.abs(ref), 1e-3)) < 3e-7
    assert np.max(np.abs(C - np.cos(xs))) < 3.6e-7
