"""ctypes binding of ``libgbgpu_gb300.so`` (the C ABI in include/gbgpu_gb300.h).

There is no fallback: if the library is missing or a call returns a non-zero
status, a RuntimeError is raised.
"""

import ctypes
import os

import torch

from .build import LIB

GBX_OK = 0
GBX_FP64 = 0
GBX_MIXED = 1
GBX_PAIR = 2
GBX_MAX_LOG2N = 13
GBX_TDI2_BIT = 1
GBX_TDI_UNEQUAL = 2
GBX_FLAG_WINDOW = 1
GBX_FLAG_INDEX = 2
GBX_FLAG_TILE = 4

EXPORTS = (
    "gbx_version", "gbx_last_error", "gbx_device_info", "gbx_init",
    "gbx_get_ll", "gbx_get_ll_ex", "gbx_get_ll_fp64", "gbx_fill_global", "gbx_fill_global_ex",
    "gbx_orbit_table_bytes", "gbx_orbit_table",
    "gbx_waveform", "gbx_waveform_ll", "gbx_waveform_fill", "gbx_wave_workspace_bytes",
    "gbx_waveform_ll_noalloc", "gbx_waveform_ll_grad", "gbx_grad_workspace_bytes",
    "gbx_swap_ll", "gbx_swap_ll_grad", "gbx_fisher", "gbx_fill_global_det", "gbx_math_selftest",
)

_vp = ctypes.c_void_p
_i = ctypes.c_int
_d = ctypes.c_double
_ll = ctypes.c_longlong


class WaveArgs(ctypes.Structure):
    """Mirror of ``gbx_wave_args``."""
    _fields_ = [
        ("params", _vp), ("num_bin", _i), ("nparams", _i), ("N", _i), ("precision", _i),
        ("tdi2", _i), ("start_freq_ind", _i), ("T", _d), ("armlength", _d), ("year", _d),
        ("orbit", _vp * (GBX_MAX_LOG2N + 1)), ("order", _vp), ("tiles", _vp), ("ntiles", _i),
        ("queue", _vp), ("status", _vp), ("workspace", _vp), ("workspace_bytes", ctypes.c_size_t),
        ("tile", _i), ("blocks_per_sm", _i),
    ]


class LLArgs(ctypes.Structure):
    """Mirror of ``gbx_ll_args``."""
    _fields_ = [
        ("A_data", _vp), ("E_data", _vp), ("A_psd", _vp), ("E_psd", _vp),
        ("data_length", _i), ("num_data", _i), ("num_psd", _i),
        ("data_index", _vp), ("noise_index", _vp), ("df", _d),
    ]


_lib = None


def lib():
    """Load the library once; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        raise RuntimeError(
            f"{LIB} is missing: build it with `python -m gbgpu_gb300.build` "
            "(or __graft_entry__.build()); there is no CPU fallback")
    L = ctypes.CDLL(LIB)
    L.gbx_version.restype = _i
    L.gbx_last_error.restype = ctypes.c_char_p
    L.gbx_device_info.argtypes = [ctypes.POINTER(_i), ctypes.POINTER(_i)]
    L.gbx_init.restype = _i
    L.gbx_get_ll.argtypes = [_vp] * 8 + [_d, _vp, _i, _i, _vp, _vp, _i, _vp, _vp]
    L.gbx_get_ll_ex.argtypes = [_vp] * 8 + [_d, _vp, _i, _i, _vp, _vp, _i, _ll, _ll, _i, _i,
                                            _vp, _vp]
    L.gbx_get_ll_fp64.argtypes = L.gbx_get_ll_ex.argtypes
    L.gbx_fill_global.argtypes = [_vp] * 5 + [_i, _i, _vp, _i, _vp, _vp]
    L.gbx_fill_global_ex.argtypes = [_vp] * 5 + [_i, _i, _vp, _i, _i, _ll, _ll, _ll, _vp, _vp]
    L.gbx_fill_global_det.argtypes = [_vp] * 5 + [_i, _i, _vp, _vp, _i, _i, _ll, _ll, _ll, _vp]
    L.gbx_orbit_table_bytes.argtypes = [_i]
    L.gbx_orbit_table_bytes.restype = ctypes.c_size_t
    L.gbx_orbit_table.argtypes = [_vp, _vp, _i, _d, _vp]
    L.gbx_wave_workspace_bytes.argtypes = [_i]
    L.gbx_wave_workspace_bytes.restype = ctypes.c_size_t
    L.gbx_waveform.argtypes = [ctypes.POINTER(WaveArgs), _vp, _vp, _vp, _vp]
    L.gbx_waveform_ll.argtypes = [ctypes.POINTER(WaveArgs), ctypes.POINTER(LLArgs), _vp, _vp, _vp]
    L.gbx_waveform_ll_noalloc.argtypes = [ctypes.POINTER(WaveArgs), ctypes.POINTER(LLArgs),
                                          _vp, _vp, _vp]
    L.gbx_waveform_ll_grad.argtypes = [ctypes.POINTER(WaveArgs), ctypes.POINTER(LLArgs),
                                       _vp, _vp, _vp, _vp]
    L.gbx_grad_workspace_bytes.argtypes = [_i]
    L.gbx_grad_workspace_bytes.restype = ctypes.c_size_t
    L.gbx_swap_ll.argtypes = [ctypes.POINTER(WaveArgs), ctypes.POINTER(LLArgs), _vp, _vp]
    L.gbx_swap_ll_grad.argtypes = [ctypes.POINTER(WaveArgs), ctypes.POINTER(LLArgs), _vp, _vp, _vp]
    L.gbx_fisher.argtypes = [ctypes.POINTER(WaveArgs), _vp, _vp, _i, _i, _vp, ctypes.c_double,
                             _vp, _vp]
    L.gbx_waveform_fill.argtypes = [ctypes.POINTER(WaveArgs), _vp, _vp, _vp, _i, _i, _ll, _vp]
    L.gbx_math_selftest.argtypes = [_vp, _vp, _i, _i, _i, _vp]
    for name in EXPORTS:
        if name not in ("gbx_last_error", "gbx_orbit_table_bytes", "gbx_wave_workspace_bytes",
                        "gbx_grad_workspace_bytes"):
            getattr(L, name).restype = _i
    _lib = L
    return L


def check(rc, what):
    if rc != GBX_OK:
        msg = lib().gbx_last_error().decode(errors="replace")
        raise RuntimeError(f"{what} failed (status {rc}): {msg}")


def ptr(t):
    """Device address of a tensor (None -> NULL)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise TypeError("expected a CUDA tensor")
    return ctypes.c_void_p(t.data_ptr())


def stream_handle(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)
