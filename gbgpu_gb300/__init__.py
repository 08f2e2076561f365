"""gbgpu_gb300: the FastGB hot path of GBGPU on one NVIDIA GB300 (sm_103a).

Same class API as the reference package (``GBGPU``, ``GBGPUThirdBody``,
utility functions), with the waveform, likelihood and global-template fill
running as hand-written CUDA kernels behind the C ABI in
include/gbgpu_gb300.h.
"""

from . import constants, utility
from .constants import *  # noqa: F401,F403
from .orbits import EqualArmlengthOrbits, Orbits, TabulatedOrbits
from .utility import (AET, get_N, get_fGW, get_amplitude, get_fdot, get_chirp_mass,
                      get_eta, get_chirp_mass_from_f_fdot, cuda_set_device)

__version__ = "0.1.0"


def __getattr__(name):
    # the GPU-facing classes import torch and load the CUDA library lazily
    if name in ("GBGPU", "GBGPUBase", "plan_tiles", "WavePlan"):
        from . import gbgpu as _g
        return getattr(_g, name)
    if name == "GBGPUThirdBody":
        from .thirdbody import GBGPUThirdBody
        return GBGPUThirdBody
    if name in ("get_backend", "has_backend"):
        from . import backend as _b
        return getattr(_b, name)
    raise AttributeError(name)
