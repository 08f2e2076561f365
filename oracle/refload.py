"""Import the reference's own FastGB Python in this container.

TEST INFRASTRUCTURE ONLY: used by tests/golden/make_golden.py and by CPU
tests that run only where the reference tree is mounted.  It puts the stub
``lisatools`` / ``gpubackendtools`` packages (oracle/stubs) on ``sys.path``
and registers ``gbgpu`` as a namespace over the reference's source directory
so that ``gbgpu/__init__.py`` (which needs the real backend manager) is not
executed; ``gbgpu.gbgpu``, ``gbgpu.thirdbody`` and ``gbgpu.utils.utility``
are then the unmodified reference modules.  The native calls they make go to
oracle/_ref/libgbgpu_ref.so (reference C++ built by oracle/Makefile).
"""

import os
import sys
import types

_HERE = os.path.dirname(os.path.abspath(__file__))
# the reference project checked out beside this repository (../reference),
# or wherever GBGPU_REFERENCE_ROOT points
REF_ROOT = os.environ.get("GBGPU_REFERENCE_ROOT",
                          os.path.join(os.path.dirname(os.path.dirname(_HERE)), "reference"))


def reference_available():
    return os.path.isfile(os.path.join(REF_ROOT, "src", "gbgpu", "gbgpu.py")) and \
        os.path.isfile(os.path.join(_HERE, "_ref", "libgbgpu_ref.so"))


def load_reference():
    """Return (gbgpu_module, thirdbody_module, utility_module, stub_lisatools)."""
    if not reference_available():
        raise RuntimeError("reference tree or oracle/_ref build not available")
    stubs = os.path.join(_HERE, "stubs")
    if stubs not in sys.path:
        sys.path.insert(0, stubs)
    if "gbgpu" not in sys.modules:
        pkg = types.ModuleType("gbgpu")
        pkg.__path__ = [os.path.join(REF_ROOT, "src", "gbgpu")]
        sys.modules["gbgpu"] = pkg
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        import gbgpu.gbgpu as ref_gbgpu
        import gbgpu.thirdbody as ref_third
        import gbgpu.utils.utility as ref_utility
    import lisatools
    import lisatools.detector
    import lisatools.sensitivity
    import lisatools.utils.constants
    return ref_gbgpu, ref_third, ref_utility, lisatools
