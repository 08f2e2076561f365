"""Spacecraft orbits consumed by the waveform.

The reference takes any ``lisatools.detector.Orbits`` object and uses only
``get_pos(t, sc)``, ``armlength``, ``t_base`` and ``configure`` (gbgpu/gbgpu.py:
87-101, 181, 243, 390-397).  The same duck-typed interface is accepted here;
``EqualArmlengthOrbits`` is the analytic default (``lisatools``' file-based
orbits are not available here).  Positions are evaluated on the host
once per (N, T) and turned into a device table by ``gbx_orbit_table``.
"""

import numpy as np

from .constants import AU_SI, YRSID_SI


class Orbits:
    """Interface: get_pos(t, sc) -> (len(t), 3) metres; armlength; t_base."""

    armlength = 2.5e9
    t_base = np.array([0.0])

    def configure(self, *args, **kwargs):
        return None

    def get_pos(self, t, sc):
        raise NotImplementedError


class EqualArmlengthOrbits(Orbits):
    """Analytic LISA constellation to first order in eccentricity.

    Cornish & Rubbo, Phys. Rev. D 67, 022001 (2003), eqs. (56)-(58):
    alpha = 2 pi t / yr, beta_i = 2 pi (i - 1)/3, R = 1 AU, e = L/(2 sqrt(3) R),
      x_i = R cos a + (e R/2)(cos(2a - b_i) - 3 cos b_i)
      y_i = R sin a + (e R/2)(sin(2a - b_i) - 3 sin b_i)
      z_i = -sqrt(3) e R cos(a - b_i)
    """

    def __init__(self, armlength=2.5e9, duration=10.0 * YRSID_SI, **kwargs):
        self.armlength = float(armlength)
        self.t_base = np.linspace(0.0, float(duration), 1001)
        self._R = AU_SI
        self._ecc = self.armlength / (2.0 * np.sqrt(3.0) * AU_SI)
        self._fm = 1.0 / YRSID_SI

    def get_pos(self, t, sc):
        t = np.asarray(t, dtype=np.float64)
        sc = np.asarray(sc)
        alpha = 2.0 * np.pi * self._fm * t
        beta = 2.0 * np.pi * (sc - 1) / 3.0
        R = self._R
        eR = self._ecc * R
        x = R * np.cos(alpha) + 0.5 * eR * (np.cos(2.0 * alpha - beta) - 3.0 * np.cos(beta))
        y = R * np.sin(alpha) + 0.5 * eR * (np.sin(2.0 * alpha - beta) - 3.0 * np.sin(beta))
        z = -np.sqrt(3.0) * eR * np.cos(alpha - beta)
        return np.stack([x, y, z], axis=-1)
