"""Spacecraft orbits consumed by the waveform.

The reference takes any ``lisatools.detector.Orbits`` object and uses only
``get_pos(t, sc)``, ``armlength``, ``t_base`` and ``configure`` (gbgpu/gbgpu.py:
87-101, 181, 243, 390-397).  The same duck-typed interface is accepted here;
``EqualArmlengthOrbits`` is the analytic default and ``TabulatedOrbits``
takes numerically integrated positions on a time grid (arrays or an ``.npz``
file), as the file-based orbits of ``lisatools`` do.  Positions are
evaluated on the host once per (N, T) and turned into a device table by
``gbx_orbit_table``.
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


class TabulatedOrbits(Orbits):
    """Spacecraft positions tabulated on a time grid, interpolated per
    coordinate by a not-a-knot cubic spline (scipy.interpolate.CubicSpline).

    ``t``: (T,) increasing times [s]; ``pos``: (3, T, 3) positions [m] of
    spacecraft 1, 2, 3; ``armlength`` [m] (the nominal arm length the
    transfer frequency uses).  Times outside the grid raise ValueError (the
    waveform also checks T against ``t_base``).  The spline's error on a
    heliocentric orbit sampled every h seconds is about (5/384) (2 pi h / yr)^4
    R: ~400 m (1.3e-6 s of light travel time) for daily samples, ~2 m for
    6-hourly ones.
    """

    def __init__(self, t, pos, armlength=2.5e9):
        from scipy.interpolate import CubicSpline
        t = np.asarray(t, dtype=np.float64)
        pos = np.asarray(pos, dtype=np.float64)
        if t.ndim != 1 or t.size < 4 or np.any(np.diff(t) <= 0):
            raise ValueError("t must be increasing with at least 4 samples")
        if pos.shape != (3, t.size, 3):
            raise ValueError(f"pos must have shape (3, {t.size}, 3), got {pos.shape}")
        self.armlength = float(armlength)
        self.t_base = t
        self._splines = [CubicSpline(t, pos[s], axis=0) for s in range(3)]

    @classmethod
    def from_file(cls, path):
        """Load ``t``, ``pos`` and ``armlength`` from an ``.npz`` file."""
        with np.load(path) as f:
            return cls(f["t"], f["pos"], float(f["armlength"]) if "armlength" in f else 2.5e9)

    def get_pos(self, t, sc):
        t = np.asarray(t, dtype=np.float64)
        if t.size and (t.min() < self.t_base[0] or t.max() > self.t_base[-1]):
            raise ValueError("time outside the tabulated orbit")
        sc = np.broadcast_to(np.asarray(sc), t.shape)
        out = np.empty(t.shape + (3,))
        for s in (1, 2, 3):
            m = sc == s
            if np.any(m):
                out[m] = self._splines[s - 1](t[m])
        return out
