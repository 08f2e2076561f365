"""GBGPUThirdBody: Galactic binaries with an eccentric third body.

Mirrors gbgpu/thirdbody.py:22-428.  On the GPU the line-of-sight Doppler
shift of the frequency and the trapezoid-integrated phase are evaluated inside
the waveform kernel (Kepler solve per sample and spacecraft, in-CTA prefix
sum); the methods below keep the reference's host-side hooks and helpers with
the same names and semantics.
"""

import numpy as np

from .constants import C_SI, G, MSUN_SI, Mjup, PI, YRSID_SI
from .gbgpu import GBGPUBase
from .utility import get_fGW, get_N


class GBGPUThirdBody(GBGPUBase):
    """GBGPU with a third body on an eccentric orbit around the binary
    (thirdbody.py:22-428): five more parameters, A2, varpi, e2, P2 [yr] and
    T2 [yr]."""

    NPARAMS = 14

    @property
    def citation(self):
        """References to cite (thirdbody.py:34-37)."""
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
        """fi (1 + v_LOS(xi)/c) (thirdbody.py:155-180)."""
        fi *= 1 + self.get_vLOS(xi, A2, varpi, e2, n2, T2) / C_SI
        return fi

    def add_to_argS(self, argS, f0, fdot, fddot, xi, A2, varpi, e2, n2, T2):
        """argS plus the trapezoid-integrated Doppler phase along the samples (thirdbody.py:182-226)."""
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
        """True anomaly at times t from the Kepler solution (thirdbody.py:322-350)."""
        u = self.get_u(n[:, None, None] * (t - T[:, None, None]),
                       np.broadcast_to(e[:, None, None], t.shape))
        ee = np.broadcast_to(e[:, None, None], t.shape)
        adjust = ee > 1e-6
        safe = np.where(adjust, ee, 1.0)
        beta = (1.0 - np.sqrt(1.0 - safe * safe)) / safe
        return np.where(adjust, u + 2.0 * np.arctan2(beta * np.sin(u), 1.0 - beta * np.cos(u)), u)

    def get_vLOS(self, t, A2, varpi, e2, n2, T2):
        """Line-of-sight velocity A2 (sin(phi + varpi) + e2 sin varpi) (thirdbody.py:352-380)."""
        phi2 = self.get_phi(t, T2, e2, n2)
        return A2[:, None, None] * (np.sin(phi2 + varpi[:, None, None])
                                    + e2[:, None, None] * np.sin(varpi[:, None, None]))

    def get_aLOS(self, A2, varpi, e2, P2, T2, t, eps=1e-9):
        """Line-of-sight acceleration by a central difference of v_LOS with
        step ``eps`` [s] at times ``t`` (B, ..., ...) [s]; P2 in years, T2 in
        seconds (thirdbody.py:430-461).  The reference passes v_LOS's
        arguments in another order than its signature; here they are passed
        as that signature defines them."""
        A2, varpi, e2, T2 = (np.atleast_1d(np.asarray(x, dtype=np.float64))
                             for x in (A2, varpi, e2, T2))
        n2 = 2 * np.pi / (np.atleast_1d(np.asarray(P2, dtype=np.float64)) * YRSID_SI)
        t = np.asarray(t, dtype=np.float64)
        up = self.get_vLOS(t + eps, A2, varpi, e2, n2, T2)
        down = self.get_vLOS(t - eps, A2, varpi, e2, n2, T2)
        return (up - down) / (2 * eps)

    def get_f_derivatives(self, f0, fdot, fddot, A2, varpi, e2, P2, T2, t=None, eps=5e4):
        """Instantaneous frequency f (1 + v_LOS/c) and its first and second
        time derivatives by central differences (thirdbody.py:463-535).

        ``t`` is (B, n, 3): per binary and evaluation point the times
        ``[t_d - eps, t_d, t_d + eps]``; by default one point per binary at
        t_d = 0.  P2 in years, T2 in seconds.  Returns (f, fdot, fddot), each
        (B, n).  The reference differences along the binary axis and passes
        v_LOS's arguments out of order; the differences here run along the
        last (time) axis, as its docstring describes."""
        A2, varpi, e2, T2, f0, fdot, fddot = (np.atleast_1d(np.asarray(x, dtype=np.float64))
                                              for x in (A2, varpi, e2, T2, f0, fdot, fddot))
        n2 = 2 * np.pi / (np.atleast_1d(np.asarray(P2, dtype=np.float64)) * YRSID_SI)
        if t is None:
            t = np.tile(np.array([-eps, 0.0, eps]), (len(A2), 1, 1))
        elif not isinstance(t, (list, np.ndarray)):
            raise ValueError("t must be a list or an np.ndarray")
        t = np.asarray(t, dtype=np.float64)
        assert t.ndim == 3 and t.shape[-1] == 3 and t.shape[0] == len(A2)
        h = (t[..., 2] - t[..., 0]) / 2.0
        ft = f0[:, None, None] + fdot[:, None, None] * t + 0.5 * fddot[:, None, None] * t * t
        ft = ft * (1.0 + self.get_vLOS(t, A2, varpi, e2, n2, T2) / C_SI)
        return (ft[..., 1], (ft[..., 2] - ft[..., 0]) / (2 * h),
                (ft[..., 2] - 2 * ft[..., 1] + ft[..., 0]) / (h * h))

    def parab_step_ET(self, f0, fdot, fddot, A2, varpi, e2, n2, T2, t0, t0_old):
        """One trapezoid step of the Doppler phase between t0_old and t0 (thirdbody.py:382-428)."""
        dtt = t0 - t0_old
        g1 = self.get_vLOS(t0_old, A2, varpi, e2, n2, T2) * get_fGW(f0, fdot, fddot, t0_old)
        g3 = self.get_vLOS(t0, A2, varpi, e2, n2, T2) * get_fGW(f0, fdot, fddot, t0)
        return dtt * (g1 + g3) / 2.0 * PI * 2 / C_SI


def get_T2(P2, e2, phi2, third_period_unit="yrs"):
    """Time of pericentre T2 [yr] from the orbital phase phi2 (thirdbody.py:
    648-684): u2 = 2 atan(sqrt((1-e2)/(1+e2)) tan(phi2/2)), T2 = (u2 - e2 sin u2)
    / n2, moved into [0, P2) when negative.  ``P2`` in years ("yrs") or
    seconds ("sec"); the caller's arrays are not modified."""
    P2 = np.array(P2, dtype=np.float64, copy=True)
    if third_period_unit == "yrs":
        P2 *= YRSID_SI
    elif third_period_unit != "sec":
        raise NotImplementedError
    u2 = 2.0 * np.arctan(np.sqrt((1 - e2) / (1 + e2)) * np.tan(phi2 / 2.0))
    n2 = 2 * np.pi / P2
    temp_T2 = (u2 - e2 * np.sin(u2)) / n2
    return (temp_T2 / YRSID_SI) * (temp_T2 >= 0.0) + \
        ((P2 - np.abs(temp_T2)) / YRSID_SI) * (temp_T2 < 0.0)


def third_body_factors(M, mc, P2, e2, iota, Omega2, omega2, phi2, lam, beta,
                       third_mass_unit="Mjup", third_period_unit="yrs"):
    """(A2, varpi, T2) from the physical parameters of the third body
    (thirdbody.py:538-645; Robson et al. 2018, arXiv:1806.00500): inner-binary
    mass M [Msun], third-body mass mc ("Mjup" or "MSUN"), period P2 ("yrs" or
    "sec"), eccentricity e2, orbital Euler angles iota, Omega2, omega2,
    orbital phase phi2, sky position lam, beta.  Same formulas as the
    reference (semi-major axis from the inner mass M, as there); the caller's
    arrays are not modified (the reference scales M, mc and P2 in place)."""
    M = np.array(M, dtype=np.float64, copy=True) * MSUN_SI
    if third_mass_unit == "Mjup":
        factor = Mjup
    elif third_mass_unit == "MSUN":
        factor = MSUN_SI
    else:
        raise NotImplementedError
    mc = np.array(mc, dtype=np.float64, copy=True) * factor
    P2 = np.array(P2, dtype=np.float64, copy=True)
    if third_period_unit == "yrs":
        P2 *= YRSID_SI
    elif third_period_unit != "sec":
        raise NotImplementedError
    m2 = M + mc
    theta = np.pi / 2 - beta
    phi = lam
    for x in (M, m2, iota, Omega2, omega2, phi2, theta, phi):
        assert np.shape(x) == P2.shape
    a2 = (G * M * P2 ** 2 / (4 * np.pi ** 2)) ** (1 / 3)
    p2 = a2 * (1 - e2 ** 2)
    C = np.cos(theta) * np.sin(iota) + np.sin(theta) * np.cos(iota) * np.sin(phi - Omega2)
    S = np.sin(theta) * np.cos(phi - Omega2)
    A_bar = np.sqrt(C ** 2 + S ** 2)
    phi_bar = np.arctan(C / (-S))
    omega_bar = (omega2 + phi_bar) % (2 * np.pi)
    amp2 = (mc / m2) * np.sqrt(G * m2 / p2) * A_bar
    T2 = get_T2(P2, e2, phi2, third_period_unit="sec")
    return amp2, omega_bar, T2
