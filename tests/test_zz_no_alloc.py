"""The allocation-free entry point gbx_waveform_ll_noalloc.

It serves callers that may not allocate device memory (a plug-in whose host
application owns all device allocations, an FFI binding without a CUDA
allocator): its scratch is a static device array instead of a caller
workspace.  Checked through the C ABI against gbx_waveform_ll with a
workspace, twice in a row so the shared array's leftover contents and the
work-queue counter reset are exercised, and against the CPU oracle (the
reference's algorithm) per N class; runs alone or after the other tests.
"""

import ctypes

import numpy as np
import pytest

import fastgb_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _case(seed, B):
    from gbgpu_gb300.sensitivity import A1TDISens
    rng = np.random.default_rng(seed)
    T, dt = 4 * 31557600.0, 10.0
    p = np.array([10 ** rng.uniform(-23, -21, B), rng.uniform(2e-3, 2.02e-3, B),
                  10 ** rng.uniform(-18, -15, B), np.zeros(B), rng.uniform(0, 2 * np.pi, B),
                  np.arccos(rng.uniform(-1, 1, B)), rng.uniform(0, np.pi, B),
                  rng.uniform(0, 2 * np.pi, B), np.arcsin(rng.uniform(-1, 1, B))])
    p[3] = 11 / 3 * p[2] ** 2 / p[1]
    Ns = 2 ** rng.integers(5, 12, B)
    si = O.start_indices(p[1], 2048, T, dt)
    s0 = int(si.min()) - 2048
    L = int(si.max()) + 4096 - s0
    S = A1TDISens.get_Sn((np.arange(L) + s0) / T)
    data = [np.sqrt(S * T / 4) * (rng.standard_normal(L) + 1j * rng.standard_normal(L))
            for _ in range(2)]
    return p, Ns, data, S, s0, T


def _run(fn, gb, p, Ns, data, S, s0, T, precision):
    from gbgpu_gb300 import _native as nat
    B = p.shape[1]
    dd = [torch.as_tensor(x, device="cuda") for x in data]
    Sd = torch.as_tensor(S, device="cuda")
    prm = torch.as_tensor(p, device="cuda").contiguous()
    plan = gb._plan(Ns, T, precision, False, 9)
    a = plan.args(prm, s0)
    la = nat.LLArgs()
    la.A_data, la.E_data = dd[0].data_ptr(), dd[1].data_ptr()
    la.A_psd = la.E_psd = Sd.data_ptr()
    la.data_length, la.num_data, la.num_psd = len(S), 1, 1
    la.df = 1.0 / T
    d_h = torch.full((B,), np.nan, dtype=torch.complex128, device="cuda")
    h_h = torch.full((B,), np.nan, dtype=torch.complex128, device="cuda")
    rc = fn(ctypes.byref(a), ctypes.byref(la), nat.ptr(d_h), nat.ptr(h_h), nat.stream_handle())
    nat.check(rc, fn.__name__)
    torch.cuda.synchronize()
    return d_h.cpu().numpy(), h_h.cpu().numpy()


def _oracle(p, Ns, data, S, s0, T):
    """(d_h, h_h) of the CPU oracle, one N class at a time."""
    B = p.shape[1]
    d_h = np.zeros(B, np.complex128)
    h_h = np.zeros(B, np.complex128)
    for n in np.unique(Ns):
        sel = Ns == n
        _, dh, hh, _ = O.get_ll(p[:, sel], data, [S, S], int(n), T=T, dt=10.0,
                                start_freq_ind=s0, return_terms=True)
        d_h[sel], h_h[sel] = dh, hh
    return d_h, h_h


@pytest.mark.parametrize("precision", ["fp64", "pair", "mixed"])
def test_noalloc_matches_workspace_entry_point_twice(precision):
    from gbgpu_gb300 import GBGPU
    from gbgpu_gb300 import _native as nat
    gb = GBGPU()
    lib = nat.lib()
    for seed, B in ((31, 700), (32, 333)):
        p, Ns, data, S, s0, T = _case(seed, B)
        ref = _run(lib.gbx_waveform_ll, gb, p, Ns, data, S, s0, T, precision)
        got = _run(lib.gbx_waveform_ll_noalloc, gb, p, Ns, data, S, s0, T, precision)
        # same kernels on the same inputs; 1e-12 relative leaves room for nothing
        # but the identical result
        np.testing.assert_allclose(got[0], ref[0], rtol=1e-12, atol=0)
        np.testing.assert_allclose(got[1], ref[1], rtol=1e-12, atol=0)
        assert np.all(np.isfinite(got[0])) and np.all(np.isfinite(got[1]))
        # and the reference's algorithm: FP64 and pair forms to 1e-10 / 1e-9
        # relative per term, the mixed form to |dlogL| <= 1e-6 max(1, <h|h>)
        odh, ohh = _oracle(p, Ns, data, S, s0, T)
        if precision == "mixed":
            dl = np.abs((got[0].real - odh.real) - 0.5 * (got[1].real - ohh.real))
            assert np.max(dl / np.maximum(1.0, ohh.real)) < 1e-6
        else:
            tol = 1e-10 if precision == "fp64" else 1e-9
            np.testing.assert_allclose(got[0], odh, rtol=tol, atol=0)
            np.testing.assert_allclose(got[1].real, ohh.real, rtol=tol, atol=0)


def test_noalloc_rejects_batches_above_the_static_size():
    from gbgpu_gb300 import _native as nat
    a = nat.WaveArgs()
    a.num_bin = 8193
    la = nat.LLArgs()
    rc = nat.lib().gbx_waveform_ll_noalloc(ctypes.byref(a), ctypes.byref(la), None, None, None)
    assert rc == 1
    assert b"8192" in nat.lib().gbx_last_error()
