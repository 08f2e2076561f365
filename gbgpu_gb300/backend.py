"""Backend method table -- the GB300 counterpart of the reference's
``GBGPUBackendMethods(get_ll, fill_global, xp)`` (gbgpu/cutils/__init__.py:13-31)
and of its Cython wrappers (gbgpu/cutils/gbgpu_utils_wrap.pyx:20-69).

The two methods take the reference's argument lists unchanged; arrays are
torch CUDA tensors (or raw device addresses as ints, like the Cython layer's
``size_t`` pointers) and the work is queued on the current torch stream.
"""

import ctypes

import torch

from . import _native as nat


def _addr(x):
    if x is None:
        return None
    if isinstance(x, int):
        return ctypes.c_void_p(x)
    if not isinstance(x, torch.Tensor) and hasattr(x, "__cuda_array_interface__"):
        x = torch.as_tensor(x, device="cuda")            # CuPy, Numba, ...: no copy
    if isinstance(x, torch.Tensor):
        if not x.is_cuda:
            raise TypeError("backend arrays must be CUDA tensors")
        if not x.is_contiguous():
            raise ValueError("backend arrays must be contiguous")
        return ctypes.c_void_p(x.data_ptr())
    raise TypeError(f"unsupported array type {type(x)!r}")


def _numel(x):
    """Elements of an array argument (0 for a raw address: size unknown)."""
    if isinstance(x, int) or x is None:
        return 0
    if not isinstance(x, torch.Tensor) and hasattr(x, "__cuda_array_interface__"):
        shape = x.__cuda_array_interface__["shape"]
        n = 1
        for d in shape:
            n *= int(d)
        return n
    return int(x.numel()) if isinstance(x, torch.Tensor) else 0


class GB300Backend:
    """``backend.get_ll`` / ``backend.fill_global`` / ``backend.xp``."""

    name = "gpu"
    xp = torch

    def __init__(self):
        self._lib = nat.lib()
        nat.check(self._lib.gbx_init(), "gbx_init")

    def get_ll(self, d_h, h_h, A_template, E_template, A_data, E_data, A_psd, E_psd, df,
               start_ind, M, num_bin, data_index, noise_index, data_length, status=None,
               fp64=False):
        """gbx_get_ll with the reference's method-table arguments (gbgpu_utils_wrap.pyx:20-48).

        When the data and PSD arrive as arrays (not raw addresses) their row
        counts are passed on, so out-of-range data_index / noise_index rows are
        flagged in ``status`` and skipped instead of being read.  ``fp64=True``
        sums in FP64 as the reference does (gbx_get_ll_fp64) instead of in
        float pairs (within 1e-12 of sum |terms|)."""
        rows = lambda x: (_numel(x) // int(data_length)) if data_length else 0
        nd = min(rows(A_data), rows(E_data))
        npsd = min(rows(A_psd), rows(E_psd))
        fn = self._lib.gbx_get_ll_fp64 if fp64 else self._lib.gbx_get_ll_ex
        rc = fn(
            _addr(d_h), _addr(h_h), _addr(A_template), _addr(E_template), _addr(A_data),
            _addr(E_data), _addr(A_psd), _addr(E_psd), float(df), _addr(start_ind), int(M),
            int(num_bin), _addr(data_index), _addr(noise_index), int(data_length),
            int(num_bin), 1, int(nd), int(npsd), _addr(status), nat.stream_handle())
        nat.check(rc, "gbx_get_ll")

    def fill_global(self, A_glob, E_glob, A_template, E_template, start_ind, M, num_bin,
                    group_index, data_length, status=None):
        """gbx_fill_global with the reference's method-table arguments (gbgpu_utils_wrap.pyx:51-69)."""
        rc = self._lib.gbx_fill_global(
            _addr(A_glob), _addr(E_glob), _addr(A_template), _addr(E_template),
            _addr(start_ind), int(M), int(num_bin), _addr(group_index), int(data_length),
            _addr(status), nat.stream_handle())
        nat.check(rc, "gbx_fill_global")


_BACKEND = None


def get_backend(name=None):
    """The single backend of this package (CUDA on sm_103a); no CPU fallback."""
    global _BACKEND
    if name not in (None, "gpu", "cuda", "gb300", "cuda13x"):
        raise ValueError(f"backend {name!r} is not available: this package only runs on the GPU")
    if _BACKEND is None:
        if not torch.cuda.is_available():
            raise RuntimeError("gbgpu_gb300 needs a CUDA GPU; no CPU fallback exists")
        _BACKEND = GB300Backend()
    return _BACKEND


def has_backend(name):
    """True when get_backend(name) succeeds (a CUDA device and the library)."""
    try:
        get_backend(name)
        return True
    except (RuntimeError, ValueError):
        return False
