"""Schwarzschild deflection table on the host build of the same code: the
outcome switches at b_crit = 3 sqrt(3) M, the closest approach is the
analytic turning radius, and the swept angle matches Darwin's integral
2 int du / sqrt(1/b^2 - u^2 + Rs u^3) to the FP32 RK4 accuracy."""
import math

import numpy as np
import pytest

from nullpath_gb300 import schwarzschild


def test_outcome_switches_at_critical_b(built):
    M = 1.0
    bc = 3 * math.sqrt(3) * M
    b = np.array([0.5, 0.9, 0.98, 1.03, 1.2, 3.0, 10.0]) * bc
    d, r, s = schwarzschild.deflection(M, b, device=False)
    assert list(s[:3]) == [1, 1, 1] and list(s[3:]) == [0, 0, 0, 0]


def test_turning_radius_and_deflection(built):
    integrate = pytest.importorskip("scipy.integrate")
    M, Rs, r0 = 1.0, 2.0, 1000.0
    b = np.array([6.0, 8.0, 12.0, 30.0, 100.0])
    d, rmin, s = schwarzschild.deflection(M, b, r_start=r0, device=False)
    for bi, di, ri in zip(b, d, rmin):
        # closest approach: largest root of r^3 - b^2 r + b^2 Rs = 0
        roots = np.roots([1.0, 0.0, -bi * bi, bi * bi * Rs])
        want = max(x.real for x in roots if abs(x.imag) < 1e-9)
        assert abs(ri - want) <= 2e-6 * want
        # swept angle from r0 in to r_min and out to r0 + 1 (substitution u = u_m (1 - t^2))
        um = 1.0 / want
        f = lambda u: 1.0 / math.sqrt(1.0 / bi ** 2 - u * u + Rs * u ** 3)
        g = lambda t, ua: 2 * um * t * f(um * (1 - t * t))
        part = lambda ua: integrate.quad(g, 0.0, math.sqrt(1 - ua / um), args=(ua,), epsabs=1e-13, epsrel=1e-12)[0]
        exact = part(1 / r0) + part(1 / (r0 + 1.0))
        assert abs(di - exact) <= 5e-4 * exact + 2e-5, (bi, di, exact)


def test_strong_deflection_limit(built):
    """Near b_crit the bending follows Bozza's strong-deflection limit
    alpha = -ln(b/b_c - 1) + b_bar, b_bar = ln(216 (7 - 4 sqrt 3)) - pi
    (V. Bozza, Phys. Rev. D 66, 103001, 2002), up to its O(b - b_c) term;
    the rays start and end at r0 = 1000 M, which adds -2 asin(b / r0)."""
    bc = 3 * math.sqrt(3)
    bbar = math.log(216 * (7 - 4 * math.sqrt(3))) - math.pi
    eps = np.array([1e-3, 3e-3, 1e-2])
    b = (bc * (1 + eps)).astype(np.float32)
    d, _, s = schwarzschild.deflection(1.0, b, r_start=1000.0, device=False)
    assert (s == 0).all()
    e_true = b.astype(np.float64) / bc - 1            # the float32 b actually traced
    alpha = d - math.pi + 2 * np.arcsin(b.astype(np.float64) / 1000.0)
    bozza = -np.log(e_true) + bbar
    assert (np.abs(alpha - bozza) < 3.0 * e_true + 2e-3).all(), (alpha, bozza)
