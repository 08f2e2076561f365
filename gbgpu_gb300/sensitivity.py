"""Analytic TDI 1.5 noise PSDs (fractional-frequency units).

Used where the reference calls ``lisatools.sensitivity`` -- the SNR bump in
``get_N`` (gbgpu/utils/utility.py:246-259) and the default PSD of
``information_matrix`` (gbgpu/gbgpu.py:1022-1028) -- and to make synthetic
data.  Single-link budget S_oms = (15e-12)^2 (1 + (2e-3/f)^4) m^2/Hz and
S_acc = (3e-15)^2 (1 + (4e-4/f)^2)(1 + (f/8e-3)^4) m^2 s^-4/Hz, with
x = 2 pi f L/c, S_op = S_oms (2 pi f/c)^2, S_pm = S_acc/(2 pi f c)^2:

    S_X = 16 sin^2 x [S_op + 2 (1 + cos^2 x) S_pm]
    S_A = S_E = 8 sin^2 x [(2 + cos x) S_op + 2 (3 + 2 cos x + cos 2x) S_pm]

(Babak, Hewitson & Petiteau, arXiv:2108.01167, sec. 2).
"""

import numpy as np

from .constants import C_SI, L_SI


def _budget(f):
    f = np.asarray(f, dtype=np.float64)
    s_oms = (15e-12) ** 2 * (1.0 + (2e-3 / f) ** 4)
    s_acc = (3e-15) ** 2 * (1.0 + (4e-4 / f) ** 2) * (1.0 + (f / 8e-3) ** 4)
    s_op = s_oms * (2.0 * np.pi * f / C_SI) ** 2
    s_pm = s_acc / (2.0 * np.pi * f * C_SI) ** 2
    x = 2.0 * np.pi * f * L_SI / C_SI
    return s_op, s_pm, x


class X1TDISens:
    """TDI 1.5 X-channel PSD (the S_X formula above)."""

    @staticmethod
    def get_Sn(f, **kwargs):
        """S_X(f) in fractional-frequency units; extra keywords are ignored."""
        s_op, s_pm, x = _budget(f)
        return 16.0 * np.sin(x) ** 2 * (s_op + 2.0 * (1.0 + np.cos(x) ** 2) * s_pm)


class A1TDISens:
    """TDI 1.5 A/E-channel PSD (the S_A formula above)."""

    @staticmethod
    def get_Sn(f, **kwargs):
        """S_A(f) = S_E(f) in fractional-frequency units; extra keywords are ignored."""
        s_op, s_pm, x = _budget(f)
        return 8.0 * np.sin(x) ** 2 * (
            (2.0 + np.cos(x)) * s_op
            + 2.0 * (3.0 + 2.0 * np.cos(x) + np.cos(2.0 * x)) * s_pm
        )


E1TDISens = A1TDISens
