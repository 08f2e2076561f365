"""Minimal stand-in for the ``lisatools`` package (test infrastructure only).

Provides exactly the names the reference's FastGB path imports:
``lisatools.utils.constants``, ``lisatools.detector.{Orbits,
EqualArmlengthOrbits}`` and ``lisatools.sensitivity.{A1TDISens, X1TDISens}``.
The orbit is an analytic first-order-in-eccentricity constellation and the
sensitivities are analytic TDI 1.5 expressions; fidelity to the real
``lisatools`` orbit files and noise curves is not claimed.
"""
