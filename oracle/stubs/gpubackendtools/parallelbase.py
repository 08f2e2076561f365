"""``ParallelModuleBase`` stand-in backed by the reference C++ build."""

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_REF_SO = os.path.join(_HERE, "..", "..", "_ref", "libgbgpu_ref.so")


def _ptr(x):
    if isinstance(x, np.ndarray):
        if not x.flags["C_CONTIGUOUS"]:
            raise ValueError("reference backend needs C-contiguous arrays")
        return ctypes.c_void_p(x.ctypes.data)
    return x


def wrapper(*args, **kwargs):
    """Same role as gpubackendtools.wrapper: arrays -> raw pointers."""
    return tuple(_ptr(a) for a in args), kwargs


class _RefBackend:
    name = "cpu"

    def __init__(self):
        lib = ctypes.CDLL(os.path.abspath(_REF_SO))
        vp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        lib.ref_get_ll.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, d, vp, i, i, vp, vp, i]
        lib.ref_get_ll.restype = None
        lib.ref_fill_global.argtypes = [vp, vp, vp, vp, vp, i, i, vp, i]
        lib.ref_fill_global.restype = None
        self._lib = lib

    def get_ll(self, *args):
        (d_h, h_h, A, E, Ad, Ed, Ap, Ep, df, si, M, nb, di, ni, L), _ = wrapper(*args)
        keep = args  # keep arrays alive during the call
        self._lib.ref_get_ll(d_h, h_h, A, E, Ad, Ed, Ap, Ep, float(df), si,
                             int(M), int(nb), di, ni, int(L))
        del keep

    def fill_global(self, *args):
        (Ag, Eg, A, E, si, M, nb, gi, L), _ = wrapper(*args)
        keep = args
        self._lib.ref_fill_global(Ag, Eg, A, E, si, int(M), int(nb), gi, int(L))
        del keep


_BACKEND = None


class ParallelModuleBase:
    def __init__(self, force_backend=None):
        global _BACKEND
        if _BACKEND is None:
            _BACKEND = _RefBackend()
        self.backend = _BACKEND

    @property
    def xp(self):
        return np

    @classmethod
    def GPU_RECOMMENDED(cls):
        return ["cpu"]
