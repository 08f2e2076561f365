"""GBGPUThirdBody: Galactic binaries with an eccentric third body.

Mirrors gbgpu/thirdbody.py:22-428.  On the GPU the line-of-sight Doppler
shift of the frequency and the trapezoid-integrated phase are evaluated inside
the waveform kernel (Kepler solve per sample and spacecraft, in-CTA prefix
sum); the methods below keep the reference's host-side hooks and helpers with
the same names and semantics.
"""

import numpy as np

from .constants import C_SI, PI, YRSID_SI
from .gbgpu import GBGPUBase
from .utility import get_fGW, get_N


class GBGPUThirdBody(GBGPUBase):
    NPARAMS = 14

    @property
    def citation(self):
        return super().citation

    def prepare_additional_args(self, A2, varpi, e2, P2, T2):
        """(A2, varpi, e2, P2 [yr], T2 [yr]); the kernel forms n2 = 2 pi/(P2 yr)
        and T2 yr itself (thirdbody.py:39-80)."""
        A2 = np.atleast_1d(A2) if not hasattr(A2, "device") else A2
        varpi = np.atleast_1d(varpi) if not hasattr(varpi, "device") else varpi
        e2 = np.atleast_1d(e2) if not hasattr(e2, "device") else e2
        P2 = np.atleast_1d(P2) if not hasattr(P2, "device") else P2
        T2 = np.atleast_1d(T2) if not hasattr(T2, "device") else T2
        self.P2 = P2
        return (A2, varpi, e2, P2, T2)

    def special_get_N(self, amp, f0, T, A2, varpi, e2, P2, T2, oversample=1):
        """Doubles N until the third-body orbit is resolved (thirdbody.py:82-153)."""
        amp = np.atleast_1d(amp)
        f0 = np.atleast_1d(f0)
        P2 = np.atleast_1d(P2)
        assert len(amp) == len(f0)
        assert len(P2) == len(f0)
        N = get_N(amp, f0, T, oversample=oversample)
        freq_N = 1 / ((T / YRSID_SI) / N)
        if np.any(freq_N < (2.0 / P2)):
            while np.any(freq_N < (2.0 / P2)):
                inds_fix = freq_N < (2.0 / P2)
                N = 2 * N * (inds_fix) + N * (~inds_fix)
                freq_N = 1 / ((T / YRSID_SI) / N)
            N = N * oversample
        return N.astype(int)

    # ---- host-side hooks (the CUDA kernel has its own fused versions) ----
    def shift_frequency(self, fi, xi, A2, varpi, e2, n2, T2):
        fi *= 1 + self.get_vLOS(xi, A2, varpi, e2, n2, T2) / C_SI
        return fi

    def add_to_argS(self, argS, f0, fdot, fddot, xi, A2, varpi, e2, n2, T2):
        term = np.zeros_like(xi)
        term[:, :, 1:] = np.cumsum(
            self.parab_step_ET(f0, fdot, fddot, A2, varpi, e2, n2, T2, xi[:, :, 1:], xi[:, :, :-1]),
            axis=-1)
        argS += term
        return argS

    def get_u(self, l, e):
        """Eccentric anomaly: Mikkola start + one 4th-order Newton step."""
        l = np.array(l, dtype=np.float64, copy=True)
        e = np.broadcast_to(np.asarray(e, dtype=np.float64), l.shape)
        neg = l < 0
        l = np.abs(l)
        over2pi = l > 2 * np.pi
        mult = np.where(over2pi, np.floor(l / (2 * np.pi)), 0.0)
        l = np.where(over2pi, l - mult * 2.0 * np.pi, l)
        overpi = l > np.pi
        l = np.where(overpi, 2.0 * np.pi - l, l)
        alpha = (1.0 - e) / (4.0 * e + 0.5)
        beta = 0.5 * l / (4.0 * e + 0.5)
        z = np.sqrt(beta * beta + alpha * alpha * alpha)
        z = np.where(neg, beta - z, beta + z)
        cz = np.abs(z) ** (1 / 3)
        z = np.where(z < 0, -cz, cz)
        s = z - alpha / z
        w = s - 0.078 * s ** 5 / (1.0 + e)
        u0 = l + e * (3.0 * w - 4.0 * w ** 3)
        f = u0 - e * np.sin(u0) - l
        f1 = 1.0 - e * np.cos(u0)
        f2 = (u0 - f - l) * 0.5
        f3 = (1.0 - f1) * 0.166666666666667
        f4 = -(u0 - f - l) * 0.0416666666666667
        u1 = -f / f1
        u2 = -f / (f1 + f2 * u1)
        u3 = -f / (f1 + f2 * u2 + f3 * u2 * u2)
        u4 = -f / (f1 + f2 * u3 + f3 * u3 * u3 + f4 * u3 * u3 * u3)
        u = u0 + u4
        u = np.where(overpi, 2.0 * np.pi - u, u)
        u = np.where(over2pi, 2.0 * np.pi * mult + u, u)
        return np.where(neg, -u, u)

    def get_phi(self, t, T, e, n):
        u = self.get_u(n[:, None, None] * (t - T[:, None, None]),
                       np.broadcast_to(e[:, None, None], t.shape))
        ee = np.broadcast_to(e[:, None, None], t.shape)
        adjust = ee > 1e-6
        safe = np.where(adjust, ee, 1.0)
        beta = (1.0 - np.sqrt(1.0 - safe * safe)) / safe
        return np.where(adjust, u + 2.0 * np.arctan2(beta * np.sin(u), 1.0 - beta * np.cos(u)), u)

    def get_vLOS(self, t, A2, varpi, e2, n2, T2):
        phi2 = self.get_phi(t, T2, e2, n2)
        return A2[:, None, None] * (np.sin(phi2 + varpi[:, None, None])
                                    + e2[:, None, None] * np.sin(varpi[:, None, None]))

    def parab_step_ET(self, f0, fdot, fddot, A2, varpi, e2, n2, T2, t0, t0_old):
        dtt = t0 - t0_old
        g1 = self.get_vLOS(t0_old, A2, varpi, e2, n2, T2) * get_fGW(f0, fdot, fddot, t0_old)
        g3 = self.get_vLOS(t0, A2, varpi, e2, n2, T2) * get_fGW(f0, fdot, fddot, t0)
        return dtt * (g1 + g3) / 2.0 * PI * 2 / C_SI
