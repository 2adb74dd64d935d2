"""Closed-form GEOKERR points (csrc/geokerr_cf.cuh, host build of the device
code) against a 40-digit truth (tests/golden/geokerr_cf_truth.npz, written by
oracle/geokerr_cf_mp.py) and against the Taylor-solver restatement
(oracle/geokerr_oracle.cpp): grids at four spins, outgoing rays, the sampling
options, and the rays left to the Taylor solver."""
import math
import os

import numpy as np
import pytest

import oracle
from nullpath_gb300 import geokerr as gk

HERE = os.path.dirname(os.path.abspath(__file__))
KEYS = ("u", "mu", "dt", "dphi", "lam")


def _rel(x, y):
    """Normwise relative difference max|x - y| / max|y| (mu and phi cross zero)."""
    return float(np.max(np.abs(np.asarray(x) - np.asarray(y))) / max(np.max(np.abs(y)), 1e-300))


def _truth():
    return np.load(os.path.join(HERE, "golden", "geokerr_cf_truth.npz"))


def test_truth_fixture_reproduces():
    """Two fixture rays recomputed by the 40-digit restatement."""
    mp = pytest.importorskip("mpmath")
    del mp
    from oracle import geokerr_cf_mp as cfmp
    t = _truth()
    for j in (0, len(t["a"]) - 1):
        a = float(t["a"][j])
        uplus = 1.0 / (1.0 + math.sqrt(1.0 - a * a))
        out = cfmp.points(1e-6, uplus, 0.5, a, t["l"][j], t["q2"][j], t["su"][j], t["sm"][j], 1, 32, 0.5)
        for k, key in enumerate(KEYS):
            assert _rel([float(x) for x in out[key]], t["pts"][j, k]) < 1e-15, (j, key)


def test_closed_form_matches_truth():
    """Near-polar, near-double-root (shadow edge) and random rays at
    a = 0.9, 0.5, 0.998, 0.1: every sampled quantity within 2e-12 of the
    truth, turning counts exact."""
    t = _truth()
    n = len(t["a"])
    assert n >= 40
    for j in range(n):
        a = float(t["a"][j])
        uplus = 1.0 / (1.0 + math.sqrt(1.0 - a * a))
        h = gk.points_host(a, 1e-6, uplus, 0.5, t["l"][j:j + 1], t["q2"][j:j + 1], t["su"][j:j + 1],
                           t["sm"][j:j + 1], 1, 32, 0.5)
        assert h["n"][0] == 32 and h["method"][0] in (1, 2), j
        for k, key in enumerate(KEYS):
            assert _rel(h[key][0], t["pts"][j, k]) < 2e-12, (j, a, key, _rel(h[key][0], t["pts"][j, k]))
        assert np.array_equal(h["tpm"][0], t["tpm"][j]) and np.array_equal(h["tpr"][0], t["tpr"][j]), j


def test_vortical_closed_form_matches_quadrature_truth():
    """q2 < 0 rays (two real radial roots below the motion, or two complex
    pairs; dn-form polar motion) against a 40-digit truth built by
    quadrature, independent of the Legendre reductions
    (tests/golden/geokerr_cf_truth_vortical.npz): 5e-14."""
    t = np.load(os.path.join(HERE, "golden", "geokerr_cf_truth_vortical.npz"))
    seen = set()
    for j in range(len(t["a"])):
        a = float(t["a"][j])
        uplus = 1.0 / (1.0 + math.sqrt(1.0 - a * a))
        h = gk.points_host(a, 1e-6, uplus, 0.5, t["l"][j:j + 1], t["q2"][j:j + 1], t["su"][j:j + 1],
                           t["sm"][j:j + 1], 1, 32, 0.5)
        seen.add(int(h["method"][0]))
        for k, key in enumerate(KEYS):
            assert _rel(h[key][0], t["pts"][j, k]) < 5e-14, (j, key)
        assert np.array_equal(h["tpm"][0], t["tpm"][j])
    assert seen == {3, 4}


def test_taylor_oracle_matches_truth():
    """The Taylor restatement on the same rays: 3e-11, its phi losing
    digits on near-polar orbits (the potential's coefficients carry 1 - mu+^2
    with the absolute accuracy of mu+^2)."""
    t = _truth()
    worst = 0.0
    for j in range(len(t["a"])):
        a = float(t["a"][j])
        uplus = 1.0 / (1.0 + math.sqrt(1.0 - a * a))
        ref = oracle.geokerr_points(1e-6, uplus, 0.5, a, t["l"][j], t["q2"][j], t["su"][j], t["sm"][j], 1, 32, 0.5)
        for k, key in enumerate(KEYS):
            worst = max(worst, _rel(ref[key], t["pts"][j, k]))
    assert worst < 3e-11


@pytest.mark.parametrize("a", [0.9, 0.5, 0.998, 0.1])
def test_grid_closed_form_vs_taylor(a):
    """32 x 32 standard grid: same point counts and turning counts as the
    Taylor restatement; t and the affine parameter to 2e-14, mu and phi
    to 3e-11 (the Taylor side's near-polar error, see above)."""
    mu0, u0 = 0.5, 1e-6
    uplus = 1.0 / (1.0 + math.sqrt(1.0 - a * a))
    g = oracle.geokerr_camera_grid(a, mu0, 32, 32)
    h = gk.points_host(a, u0, uplus, mu0, g["l"], g["q2"], g["su"], g["sm"], 1, 32, 0.5)
    assert (h["method"] > 0).mean() > 0.98
    for i in range(g["l"].size):
        ref = oracle.geokerr_points(u0, uplus, mu0, a, g["l"][i], g["q2"][i], g["su"][i], g["sm"][i], 1, 32, 0.5)
        k = ref["n"]
        assert h["n"][i] == k, i
        if k == 0:
            continue
        assert np.array_equal(h["tpm"][i, :k], ref["tpm"][:k]) and np.array_equal(h["tpr"][i, :k], ref["tpr"][:k]), i
        for key in ("u", "dt", "lam"):
            assert _rel(h[key][i, :k], ref[key][:k]) < 2e-14, (i, key)
        for key in ("mu", "dphi"):
            assert _rel(h[key][i, :k], ref[key][:k]) < 3e-11, (i, key)


@pytest.mark.parametrize("method", [3, 4])
def test_vortical_rays_closed_form(method):
    """q2 < 0 (vortical) rays of the 128 x 128 grid run in closed form
    (mu = s0 mu+ dn, Byrd & Friedman 218.00): with two real roots below the
    motion (method 3, B&F 260.00) or none (method 4, two complex pairs, the
    rotated form of B&F 267.00).  They agree with the Taylor restatement to
    3e-14, turning counts included."""
    a, mu0, u0 = 0.9, 0.5, 1e-6
    uplus = 1.0 / (1.0 + math.sqrt(1.0 - a * a))
    g = oracle.geokerr_camera_grid(a, mu0, 128, 128)
    sel = np.flatnonzero(g["q2"] < 0)
    h = gk.points_host(a, u0, uplus, mu0, g["l"][sel], g["q2"][sel], g["su"][sel], g["sm"][sel], 1, 32, 0.5)
    assert (h["method"] > 0).all()
    assert (h["method"] == method).sum() >= 8
    for j, i in enumerate(sel):
        if h["method"][j] != method:
            continue
        ref = oracle.geokerr_points(u0, uplus, mu0, a, g["l"][i], g["q2"][i], g["su"][i], g["sm"][i], 1, 32, 0.5)
        k = ref["n"]
        assert h["n"][j] == k == 32
        assert np.array_equal(h["tpm"][j], ref["tpm"]) and np.array_equal(h["tpr"][j], ref["tpr"])
        for key in KEYS:
            assert _rel(h[key][j], ref[key]) < 3e-14, (int(i), key)


def test_taylor_fallback_is_the_restatement():
    """Rays outside the closed forms (q2 = 0 equatorial orbits, a = 0) run
    the Taylor solver, bit for bit the restatement's."""
    u0 = 1e-6
    for a, l, q2, mu0, sm in ((0.9, 2.5, 0.0, 0.0, 1.0), (0.9, -3.0, 0.0, 0.0, -1.0),
                              (0.0, 4.0, 10.0, 0.3, 1.0), (0.0, -2.0, 25.0, -0.2, -1.0)):
        uplus = 1.0 / (1.0 + math.sqrt(1.0 - a * a))
        h = gk.points_host(a, u0, uplus, mu0, np.array([l]), np.array([q2]), np.array([1.0]), np.array([sm]),
                           1, 32, 0.5)
        assert h["method"][0] == 0
        ref = oracle.geokerr_points(u0, uplus, mu0, a, l, q2, 1.0, sm, 1, 32, 0.5)
        k = ref["n"]
        assert h["n"][0] == k and k > 0
        for key in KEYS:
            assert np.array_equal(h[key][0, :k], ref[key][:k]), (a, l, key)


def test_outgoing_rays_and_sampling_options():
    """Rays leaving from inside (su = -1, out to u = 0), one-way sampling
    (tpr = 0), other offsets and point counts: the same points as the Taylor
    restatement.  Ingoing rays sample to 0.9 u+ (a target on the horizon
    itself, where t and phi diverge, is reached by neither solver in a
    meaningful way)."""
    rng = np.random.default_rng(3)
    a = 0.7
    n = 60
    l = rng.uniform(-6, 6, n)
    q2 = rng.uniform(0.5, 30, n)
    u0 = rng.uniform(0.05, 0.3, n)
    mu0 = rng.uniform(-0.8, 0.8, n)
    uplus = 1.0 / (1.0 + math.sqrt(1.0 - a * a))
    for su, tpr, nup, off in ((-1.0, 1, 16, 0.5), (1.0, 0, 24, 0.0), (1.0, 1, 40, 0.25)):
        sm = np.where(rng.uniform(size=n) < 0.5, -1.0, 1.0)
        uf = np.where(su > 0, 0.9 * uplus, 1e-4) + 0.0 * l
        h = gk.points_host(a, u0, uf, mu0, l, q2, np.full(n, su), sm, tpr, nup, off)
        checked = 0
        for i in range(n):
            ref = oracle.geokerr_points(u0[i], uf[i], mu0[i], a, l[i], q2[i], su, sm[i], tpr, nup, off)
            k = ref["n"]
            assert h["n"][i] == k, (su, tpr, i)
            if k == 0:
                continue
            checked += h["method"][i] > 0
            assert np.array_equal(h["tpm"][i, :k], ref["tpm"][:k]) and np.array_equal(h["tpr"][i, :k], ref["tpr"][:k])
            for key in KEYS:
                assert _rel(h[key][i, :k], ref[key][:k]) < 3e-11, (su, tpr, i, key, _rel(h[key][i, :k], ref[key][:k]))
        assert checked >= n // 3
