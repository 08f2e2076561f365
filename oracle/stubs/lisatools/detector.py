"""Stand-in for ``lisatools.detector`` (test infrastructure only).

The reference consumes an orbit object through ``get_pos(t, sc)``,
``armlength``, ``t_base`` and ``configure(linear_interp_setup=True)``
(gbgpu/gbgpu.py:87-101, 181, 243, 394-396).  The real ``lisatools`` class
interpolates a numerical orbit file that is not available here; this stand-in
evaluates the analytic first-order-eccentricity constellation of
Cornish & Rubbo, Phys. Rev. D 67, 022001 (2003), eqs. (56)-(58):

    alpha = 2 pi f_m t + kappa,  beta_i = 2 pi (i - 1) / 3 + lambda
    x_i = R cos(alpha) + (e R / 2) (cos(2 alpha - beta_i) - 3 cos(beta_i))
    y_i = R sin(alpha) + (e R / 2) (sin(2 alpha - beta_i) - 3 sin(beta_i))
    z_i = -sqrt(3) e R cos(alpha - beta_i)

with R = 1 AU, e = L / (2 sqrt(3) R), f_m = 1 / yr and kappa = lambda = 0.
"""

import numpy as np

from .utils.constants import AU_SI, YRSID_SI


class Orbits:
    """Base class so that ``isinstance(orbits, Orbits)`` checks pass."""

    def configure(self, *args, **kwargs):
        return None


class EqualArmlengthOrbits(Orbits):
    def __init__(self, *args, armlength=2.5e9, use_gpu=False, **kwargs):
        self.armlength = float(armlength)
        self.t_base = np.linspace(0.0, 10.0 * YRSID_SI, 1001)
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
