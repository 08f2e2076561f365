"""Host-side third-body helpers of gbgpu_gb300.thirdbody (no GPU needed).

third_body_factors and get_T2 against the reference's own outputs
(tests/golden/third_converters.npz, made by tests/golden/make_golden.py);
get_aLOS and get_f_derivatives against the analytic time derivatives of the
line-of-sight velocity (the reference's versions pass get_vLOS's arguments
out of order, so they give no usable numbers to compare with).
"""

import numpy as np

from conftest import load_golden
from gbgpu_gb300.constants import C_SI, YRSID_SI
from gbgpu_gb300.thirdbody import GBGPUThirdBody, get_T2, third_body_factors


def _host_only():
    # the helpers are host NumPy: no device state is needed
    return object.__new__(GBGPUThirdBody)


def test_third_body_factors_match_reference():
    g = load_golden("third_converters")
    args = [g[k] for k in ("M", "mc", "P2", "e2", "iota", "Omega2", "omega2", "phi2", "lam", "beta")]
    keep = [a.copy() for a in args]
    A2, varpi, T2 = third_body_factors(*args)
    np.testing.assert_allclose(A2, g["A2"], rtol=1e-13)
    np.testing.assert_allclose(varpi, g["varpi"], rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(T2, g["T2"], rtol=1e-12)
    for a, b in zip(args, keep):                   # the caller's arrays are untouched
        np.testing.assert_array_equal(a, b)
    M, mc, P2 = g["M"], g["mc"] * 1e-3, g["P2"] * YRSID_SI
    A2s, varpis, T2s = third_body_factors(M, mc, P2, *args[3:], third_mass_unit="MSUN",
                                          third_period_unit="sec")
    np.testing.assert_allclose(A2s, g["A2_msun"], rtol=1e-13)
    np.testing.assert_allclose(varpis, g["varpi_msun"], rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(T2s, g["T2_msun"], rtol=1e-12)
    np.testing.assert_allclose(get_T2(g["P2"], g["e2"], g["phi2"]), g["T2_yrs"], rtol=1e-12)


def _vlos_and_derivative(t, A2, varpi, e2, P2, T2):
    """v_LOS and dv/dt from the Kepler solution: dphi/dt = n2 sqrt(1-e^2)/(1-e cos u)^2."""
    tb = _host_only()
    n2 = 2 * np.pi / (P2 * YRSID_SI)
    u = tb.get_u(n2[:, None, None] * (t - T2[:, None, None]),
                 np.broadcast_to(e2[:, None, None], t.shape))
    phi = tb.get_phi(t, T2, e2, n2)
    e = e2[:, None, None]
    dphi = n2[:, None, None] * np.sqrt(1 - e * e) / (1 - e * np.cos(u)) ** 2
    v = A2[:, None, None] * (np.sin(phi + varpi[:, None, None]) + e * np.sin(varpi[:, None, None]))
    return v, A2[:, None, None] * np.cos(phi + varpi[:, None, None]) * dphi


def _draw(B=5, seed=4):
    rng = np.random.default_rng(seed)
    A2 = 10 ** rng.uniform(0, 3, B)
    varpi = rng.uniform(0, 2 * np.pi, B)
    e2 = rng.uniform(0.05, 0.8, B)
    P2 = 10 ** rng.uniform(0, 1, B)
    T2 = rng.uniform(0, 1, B) * P2 * YRSID_SI
    return A2, varpi, e2, P2, T2, rng


def test_get_aLOS_is_the_time_derivative_of_vLOS():
    A2, varpi, e2, P2, T2, rng = _draw()
    t = rng.uniform(0, 1.2e8, (len(A2), 2, 7))
    a = _host_only().get_aLOS(A2, varpi, e2, P2, T2, t, eps=1.0)
    _, dv = _vlos_and_derivative(t, A2, varpi, e2, P2, T2)
    np.testing.assert_allclose(a, dv, rtol=1e-6, atol=1e-9 * np.abs(dv).max())


def test_get_f_derivatives():
    A2, varpi, e2, P2, T2, rng = _draw(seed=6)
    B = len(A2)
    f0 = rng.uniform(1e-3, 5e-3, B)
    fdot = 10 ** rng.uniform(-17, -15, B)
    fddot = 11 / 3 * fdot ** 2 / f0
    td = rng.uniform(0, 1e8, (B, 3))
    eps = 5e3
    t = np.stack([td - eps, td, td + eps], axis=-1)
    tb = _host_only()
    # no third body: the polynomial's own values and derivatives
    z = np.zeros(B)
    f, fd, fdd = tb.get_f_derivatives(f0, fdot, fddot, z, varpi, e2, P2, T2, t=t)
    np.testing.assert_allclose(f, f0[:, None] + fdot[:, None] * td + 0.5 * fddot[:, None] * td ** 2,
                               rtol=1e-15)
    np.testing.assert_allclose(fd, fdot[:, None] + fddot[:, None] * td, rtol=1e-6)
    # with the third body: f (1 + v/c) and its derivative
    f, fd, _ = tb.get_f_derivatives(f0, fdot, fddot, A2, varpi, e2, P2, T2, t=t)
    v, dv = _vlos_and_derivative(td[..., None], A2, varpi, e2, P2, T2)
    v, dv = v[..., 0], dv[..., 0]
    fp = f0[:, None] + fdot[:, None] * td + 0.5 * fddot[:, None] * td ** 2
    np.testing.assert_allclose(f, fp * (1 + v / C_SI), rtol=1e-15)
    ref = (fdot[:, None] + fddot[:, None] * td) * (1 + v / C_SI) + fp * dv / C_SI
    np.testing.assert_allclose(fd, ref, rtol=1e-4, atol=1e-6 * np.abs(ref).max())
    # default: one point per binary at t = 0
    f1, _, _ = tb.get_f_derivatives(f0, fdot, fddot, A2, varpi, e2, P2, T2)
    assert f1.shape == (B, 1)
