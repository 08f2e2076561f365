"""Minimal stand-in for ``gpubackendtools`` (test infrastructure only).

The reference's FastGB classes only need a base class that exposes ``xp``
(the array module) and ``backend`` (an object carrying ``get_ll``,
``fill_global`` and ``name``), see gbgpu/gbgpu.py:29-84 and
gbgpu/utils/parallelbase.py:8-11.  Here ``xp`` is NumPy and the backend
methods call the reference's own ``get_ll_wrap`` / ``fill_global_wrap``
compiled as C++ from gbgpu/cutils/gbgpu_utils.cu (oracle/_ref).
"""

from .parallelbase import ParallelModuleBase, wrapper  # noqa: F401
