"""Physical constants used on the FastGB path.

The names and values are those the reference imports from
``lisatools.utils.constants`` (gbgpu/gbgpu.py:9, gbgpu/utils/utility.py:5).
G_SI, MSUN_SI and PC_SI reproduce the reference tutorial's outputs
``get_amplitude(0.2, 0.1, 0.1, 6 kpc) = 6.37562267e-23`` and
``get_fdot(1e-3, m1=0.2, m2=0.1) = 1.73157515e-19``.
"""

import math

C_SI = 299792458.0
PI = math.pi
YRSID_SI = 31558149.763545603   # sidereal year, s
G_SI = 6.67408e-11
MSUN_SI = 1.98848e30
PC_SI = 3.0856775814913674e16
AU_SI = 149597870700.0
Mjup = 1.898e27
G = G_SI
L_SI = 2.5e9                     # LISA arm length, m
fstar = C_SI / (2.0 * math.pi * L_SI)

__all__ = ["C_SI", "PI", "YRSID_SI", "G_SI", "MSUN_SI", "PC_SI", "AU_SI", "Mjup", "G",
           "L_SI", "fstar"]
