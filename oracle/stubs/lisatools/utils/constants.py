"""Stand-in for ``lisatools.utils.constants`` (lisaanalysistools >= 1.0.17).

TEST INFRASTRUCTURE ONLY.  This module exists so that the reference's own
Python (``gbgpu/gbgpu.py``, ``gbgpu/thirdbody.py``, ``gbgpu/utils/utility.py``)
can be imported in a container where ``lisatools`` is not installed.  The
values are the ones ``lisatools`` takes from ``lisaconstants``; G_SI, MSUN_SI
and PC_SI are pinned by the reference tutorial notebook outputs
(``get_amplitude(0.2, 0.1, 0.1, 6 kpc) = 6.37562267e-23`` and
``get_fdot(1e-3, m1=0.2, m2=0.1) = 1.73157515e-19``,
examples/GBGPU_tutorial.ipynb cells 30 and 32).
"""

import numpy as np

C_SI = 299792458.0
PI = np.pi
YRSID_SI = 31558149.763545603  # sidereal year (365.256363004 d)
G_SI = 6.67408e-11
MSUN_SI = 1.98848e30
PC_SI = 3.0856775814913674e16
AU_SI = 149597870700.0
Mjup = 1.898e27
G = G_SI
L_SI = 2.5e9
fstar = C_SI / (2.0 * np.pi * L_SI)

__all__ = ["C_SI", "PI", "YRSID_SI", "G_SI", "MSUN_SI", "PC_SI", "AU_SI",
           "Mjup", "G", "L_SI", "fstar"]
