"""Equatorial crossings by Jacobi amplitude (csrc/equator_cf.cuh, host build
of np_geokerr_disk_crossings): against a 40-digit quadrature truth on
near-critical and ordinary rays (tests/golden/geokerr_crossings_truth.npz,
written by tests/golden/make_geokerr_crossings_truth.py), against the
Taylor-solver restatement (oracle.geokerr_crossings) on a camera grid, and
the window, vortical and outside-the-closed-forms cases."""
import math
import os

import numpy as np
import pytest

import oracle
from nullpath_gb300 import geokerr as gk

HERE = os.path.dirname(os.path.abspath(__file__))


def _truth():
    return np.load(os.path.join(HERE, "golden", "geokerr_crossings_truth.npz"))


# Per crossing order: a near-critical ray's later crossings follow half
# orbits near the photon orbit, each of which multiplies a perturbation of
# the ray by about 20.  The roots of U are polished against its exact
# (double-double) coefficients, so u carries no such growth (2e-14 at the
# sixth crossing, against 2.5e-9 with the double coefficients' roots and
# 3e-9 for the Taylor restatement); phi, summed from the pole terms, keeps
# some (2e-11 at the sixth).
BAR_U = (5e-14, 5e-14, 5e-14, 5e-14, 1e-13, 1e-13)
BAR_PHI = (5e-14, 2e-13, 5e-12, 3e-11, 3e-11, 1e-10)


def test_crossings_match_quadrature_truth():
    """Status, count, u (relative) and azimuth (rad) of the first six
    crossings of 36 rays, near-critical (l within 1e-10 .. 1e-3 of the
    critical curve) and ordinary, ingoing and outgoing, at a = 0.9, 0.998,
    0.5 and -0.7, against the 40-digit truth, per crossing order."""
    t = _truth()
    assert len(t["a"]) >= 30 and (t["status"] == 1).sum() >= 5 and (t["status"] == 0).sum() >= 5
    for i in range(len(t["a"])):
        h = gk.disk_crossings(float(t["a"][i]), t["u0"], t["mu0"], t["l"][i:i + 1], t["q2"][i:i + 1],
                              t["su"][i], t["sm"][i], float(t["u_far"]), K=6)
        n = int(t["n"][i])
        assert int(h["status"][0]) == int(t["status"][i]) and int(h["nx"][0]) == n, i
        if n == 0:
            continue
        du = np.abs(h["xu"][0, :n] - t["xu"][i, :n]) / t["xu"][i, :n]
        dphi = np.abs(h["xphi"][0, :n] - t["xphi"][i, :n])
        assert (du <= np.array(BAR_U[:n])).all() and (dphi <= np.array(BAR_PHI[:n])).all(), (i, du, dphi)


def test_unresolved_pairs_are_left_to_the_integrators():
    """Rays within 1e-15 .. 1e-11 (relative, in l) of the critical curve:
    the pair of radial roots near the photon orbit is then closer than the
    root iteration resolves, and such a ray must come back with status -1
    (integrated by the renderer, Taylor-solved by GEOKERR) rather than with
    wrong crossings.  Rays it does solve keep the Taylor restatement's
    first two crossings (before any winding) to 1e-10."""
    rng = np.random.default_rng(3)
    mu0 = math.cos(math.radians(80.0))
    left = solved = 0
    for a in (0.9, 0.998, 0.5):
        r_pro = 2 * (1 + math.cos(2 / 3 * math.acos(-a)))
        r_ret = 2 * (1 + math.cos(2 / 3 * math.acos(a)))
        for _ in range(40):
            r = rng.uniform(r_pro, r_ret)
            l = -(r ** 3 - 3 * r * r + a * a * r + a * a) / (a * (r - 1))
            q2 = r ** 3 * (4 * a * a - r * (r - 3) ** 2) / (a * a * (r - 1) ** 2)
            l *= 1 + 10.0 ** rng.uniform(-15, -11) * rng.choice([-1, 1])
            if q2 <= 0 or q2 + (a * a - l * l - q2) * mu0 * mu0 - a * a * mu0 ** 4 < 0:
                continue
            sm = float(rng.choice([-1.0, 1.0]))
            h = gk.disk_crossings(a, 0.02, mu0, np.array([l]), np.array([q2]), 1.0, sm, 1e-3, K=2)
            if h["status"][0] < 0:
                left += 1
                continue
            n, xu, _ = oracle.geokerr_crossings(0.02, mu0, a, l, q2, 1.0, sm, 1e-3, 2)
            assert h["nx"][0] == n
            assert np.max(np.abs(h["xu"][0, :n] - xu[:n]) / xu[:n]) <= 1e-10
            solved += 1
    assert left > 10 and solved > 10, (left, solved)


@pytest.mark.parametrize("a", [0.9, 0.998, 0.5])
def test_grid_crossings_match_taylor(a):
    """A 24 x 24 camera grid from r = 50 M (every q2 > 0 ray, ingoing): the
    same crossing count as the Taylor restatement up to u_far, u within
    1e-9 relative and phi within 1e-9 rad (both solvers are FP64; the rays
    nearest the critical curve set the bar)."""
    mu0, u0, u_far = math.cos(math.radians(80.0)), 0.02, 1e-3
    g = oracle.geokerr_camera_grid(a, mu0, 24, 24, -8.0, 8.0, -8.0, 8.0)
    sel = np.flatnonzero(g["q2"] > 0)
    h = gk.disk_crossings(a, u0, mu0, g["l"][sel], g["q2"][sel], 1.0, g["sm"][sel], u_far, K=6)
    assert (h["status"] >= 0).all()
    checked = 0
    for j, i in enumerate(sel):
        n, xu, xphi = oracle.geokerr_crossings(u0, mu0, a, g["l"][i], g["q2"][i], 1.0, g["sm"][i], u_far, 6)
        assert h["nx"][j] == n, (int(i), int(h["nx"][j]), n)
        if n > 0:
            assert np.max(np.abs(h["xu"][j, :n] - xu[:n]) / xu[:n]) <= 1e-9, int(i)
            assert np.max(np.abs(h["xphi"][j, :n] - xphi[:n])) <= 1e-9, int(i)
            checked += 1
    assert checked > 200


def test_window_selects_crossings_in_order():
    """A window [u_lo, u_hi] keeps exactly the crossings of the full list that
    fall inside it, in order, at most K (the renderer's disk annulus and its
    crossing-order cap)."""
    a, mu0, u0, u_far = 0.9, math.cos(math.radians(80.0)), 0.02, 1e-3
    rng = np.random.default_rng(4)
    l, q2 = rng.uniform(-7, 7, 400), rng.uniform(0.5, 40, 400)
    sm = np.where(rng.uniform(size=400) < 0.5, -1.0, 1.0)
    full = gk.disk_crossings(a, u0, mu0, l, q2, 1.0, sm, u_far, K=16, phi=False)
    u_lo, u_hi = 1.0 / 20.0, 1.0 / 2.5
    for K in (1, 3):
        w = gk.disk_crossings(a, u0, mu0, l, q2, 1.0, sm, u_far, u_lo, u_hi, K=K, phi=False)
        for i in range(400):
            xs = full["xu"][i, :full["nx"][i]]
            keep = xs[(xs >= u_lo) & (xs <= u_hi)][:K]
            assert w["nx"][i] == len(keep) and np.array_equal(w["xu"][i, :len(keep)], keep), i
            assert w["status"][i] == full["status"][i]


def test_vortical_and_outside_cases():
    """q2 < 0 rays never cross the equator (ingoing: captured); a = 0, q2 = 0
    and a start beyond u_far are outside the closed forms (status -1, the
    renderer integrates them)."""
    mu0, u0, u_far = 0.6, 0.02, 1e-3
    v = gk.disk_crossings(0.9, u0, mu0, np.array([0.3, -0.2]), np.array([-0.05, -0.1]), 1.0, 1.0, u_far)
    assert (v["nx"] == 0).all() and (v["status"] == 1).all()
    o = gk.disk_crossings(0.0, u0, mu0, np.array([3.0]), np.array([20.0]), 1.0, 1.0, u_far)
    assert o["status"][0] == -1 and o["nx"][0] == 0
    o = gk.disk_crossings(0.9, u0, 0.0, np.array([3.0]), np.array([0.0]), 1.0, 1.0, u_far)
    assert o["status"][0] == -1
    o = gk.disk_crossings(0.9, u0, mu0, np.array([3.0]), np.array([20.0]), 1.0, 1.0, 0.05)
    assert o["status"][0] == -1


def test_outgoing_start_matches_taylor():
    """Rays that start outward (su = -1) from inside the photon region's
    exterior cross the equator until u_far, as the Taylor restatement."""
    a, mu0, u0, u_far = 0.7, 0.3, 0.2, 1e-3
    rng = np.random.default_rng(5)
    for _ in range(40):
        l, q2 = rng.uniform(-4, 4), rng.uniform(0.5, 30)
        sm = float(rng.choice([-1.0, 1.0]))
        h = gk.disk_crossings(a, u0, mu0, np.array([l]), np.array([q2]), -1.0, sm, u_far, K=6)
        if h["status"][0] < 0:
            continue
        n, xu, xphi = oracle.geokerr_crossings(u0, mu0, a, l, q2, -1.0, sm, u_far, 6)
        assert h["nx"][0] == n and h["status"][0] == 0
        if n:
            assert np.max(np.abs(h["xu"][0, :n] - xu[:n]) / xu[:n]) <= 1e-10
            assert np.max(np.abs(h["xphi"][0, :n] - xphi[:n])) <= 1e-10
