"""Host-side helpers with the reference's names and semantics.

Mirrors gbgpu/utils/utility.py: ``AET`` (:24-38), ``get_fGW`` (:41-81),
``get_chirp_mass`` / ``get_eta`` / ``get_amplitude`` / ``get_fdot`` /
``get_chirp_mass_from_f_fdot`` (:84-194), ``get_N`` (:197-273) and
``cuda_set_device`` (:276-286).  They work on NumPy arrays (and, where noted,
on torch tensors).
"""

import numpy as np

from .constants import C_SI, G_SI, MSUN_SI, PC_SI, YRSID_SI, fstar
from . import sensitivity as tdi

tdi_available = True


def AET(X, Y, Z):
    """(A, E, T) = ((Z - X)/sqrt2, (X - 2Y + Z)/sqrt6, (X + Y + Z)/sqrt3)
    (gbgpu/utils/utility.py:24-38)."""
    return (
        (Z - X) / np.sqrt(2.0),
        (X - 2.0 * Y + Z) / np.sqrt(6.0),
        (X + Y + Z) / np.sqrt(3.0),
    )


def get_fGW(f0, fdot, fddot, t, xp=None):
    """f(t) = f0 + fdot t + fddot t^2 / 2, broadcasting binaries along axis 0
    (gbgpu/utils/utility.py:41-81)."""
    if xp is None:
        xp = np
    tdim = t.ndim
    dim_diff = tdim - 1
    if dim_diff > 0:
        assert (t.shape[0] == len(f0)) or (t.shape[0] == 1)
        dims = tuple(range(1, dim_diff + 1))
        f0 = xp.expand_dims(f0, dims)
        fdot = xp.expand_dims(fdot, dims)
        fddot = xp.expand_dims(fddot, dims)
    return f0 + fdot * t + 0.5 * fddot * t * t


def get_chirp_mass(m1, m2):
    """(m1 m2)^(3/5) / (m1 + m2)^(1/5) (gbgpu/utils/utility.py:84-96)."""
    return (m1 * m2) ** (3 / 5) / (m1 + m2) ** (1 / 5)


def get_eta(m1, m2):
    """Symmetric mass ratio m1 m2 / (m1 + m2)^2 (gbgpu/utils/utility.py:99-111)."""
    return (m1 * m2) / (m1 + m2) ** 2


def get_amplitude(m1, m2, f, d):
    """Strain amplitude; masses in solar masses, f in Hz, d in kpc
    (gbgpu/utils/utility.py:114-130)."""
    Mc = get_chirp_mass(m1, m2) * MSUN_SI
    d = d * 1e3 * PC_SI
    return 2 * (G_SI * Mc) ** (5.0 / 3.0) / (C_SI ** 4 * d) * (np.pi * f) ** (2.0 / 3.0)


def get_fdot(f, m1=None, m2=None, Mc=None):
    """Quadrupole frequency derivative from component masses or the chirp
    mass (solar masses) (gbgpu/utils/utility.py:133-169)."""
    if m1 is None and m2 is None and Mc is None:
        raise ValueError("Must provide either m1 & m2 or Mc.")
    elif m1 is not None or m2 is not None:
        assert m1 is not None and m2 is not None
        Mc = get_chirp_mass(m1, m2) * MSUN_SI
    elif Mc is not None:
        Mc = Mc * MSUN_SI
    return (96.0 / 5.0) * np.pi ** (8 / 3) * (G_SI * Mc / C_SI ** 3) ** (5 / 3) * f ** (11 / 3)


def get_chirp_mass_from_f_fdot(f, fdot):
    """Chirp mass (solar masses) from f and fdot, the inverse of get_fdot
    (gbgpu/utils/utility.py:172-194)."""
    Mc_SI = (5.0 / 96.0 * np.pi ** (-8 / 3) * (G_SI / C_SI ** 3) ** (-5 / 3)
             * f ** (-11 / 3) * fdot) ** (3 / 5)
    return Mc_SI / MSUN_SI


def get_N(amp, f0, Tobs, oversample=1):
    """Slow-part sample count per binary (gbgpu/utils/utility.py:197-273).

    Band table x observation-time multiplier, raised by the SNR estimate from
    the X-channel sensitivity, capped at 8192, times ``oversample``.  The
    reference's update ``M = M*(M>N) + N*(M<N)`` yields 0 when M == N; that
    behaviour is kept so N agrees with the reference for every input.
    """
    amp = np.atleast_1d(amp)
    f0 = np.atleast_1d(f0)
    mult = 8
    if (Tobs / YRSID_SI) <= 1.0:
        mult = 1
    elif (Tobs / YRSID_SI) <= 2.0:
        mult = 2
    elif (Tobs / YRSID_SI) <= 4.0:
        mult = 4
    elif (Tobs / YRSID_SI) <= 8.0:
        mult = 8
    mult = np.full_like(f0, mult, dtype=np.int32)
    N = 32 * mult
    N[f0 >= 0.1] = 1024 * mult[f0 >= 0.1]
    N[(f0 >= 0.03) & (f0 < 0.1)] = 512 * mult[(f0 >= 0.03) & (f0 < 0.1)]
    N[(f0 >= 0.01) & (f0 < 0.3)] = 256 * mult[(f0 >= 0.01) & (f0 < 0.3)]
    N[(f0 >= 0.001) & (f0 < 0.01)] = 64 * mult[(f0 >= 0.001) & (f0 < 0.01)]
    fonfs = f0 / fstar
    SnX = np.sqrt(tdi.X1TDISens.get_Sn(f0))
    Sm = SnX / (4.0 * np.sin(fonfs) * np.sin(fonfs))
    Acut = amp * np.sqrt(Tobs / Sm)
    M = (2.0 ** (np.log(Acut) / np.log(2.0) + 1.0)).astype(int)
    M = M * (M > N) + N * (M < N)
    N = M * (M > N) + N * (M < N)
    M[M > 8192] = 8192
    N = M
    return (N * oversample).astype(int)


def flops_per_binary(N, tdi2=False, third_body=False, likelihood=False):
    """Algorithmic floating-point operations of one binary: the single count
    every FLOP figure of this package is quoted with.

    Per time sample of the slow part (gbgpu.py:348-540): k.P 9, delayed times
    3, instantaneous frequencies 12, carrier phase 24, six link transfer
    functions 6 x 20, three arm projections 3 x 30, TDI X/Y/Z 40, the
    frequency factors f(t), omL, fctr, fctr2 and their products 32 (330 in
    all), plus 15 transcendental evaluations counted as one each; then three
    N-point FFTs at 5 N log2 N each.  TDI-2 adds its factor (20 per sample);
    the third body adds v_LOS (Kepler solve), f_GW and the trapezoid
    increment at three spacecraft (3 x 56) plus 9 transcendentals per sample
    (thirdbody.py:155-380); the likelihood adds conj(d) h / S and |h|^2 / S on
    A and E (24 per bin).  ``N`` may be an array (one N per binary).
    """
    N = np.asarray(N, dtype=np.float64)
    per_sample = 330.0 + 15.0
    if tdi2:
        per_sample += 20.0
    if third_body:
        per_sample += 3 * 56.0 + 9.0
    f = per_sample * N + 3 * 5.0 * N * np.log2(N)
    if likelihood:
        f = f + 24.0 * N
    return f


def cuda_set_device(dev):
    """Select the CUDA device used by subsequent calls (gbgpu/utils/utility.py:276)."""
    import torch
    torch.cuda.set_device(dev)
