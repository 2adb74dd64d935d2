"""CPU checks of the GEOKERR restatement (oracle/geokerr_oracle.cpp).

Pinned to the only end-to-end GEOKERR golden the reference ships
(geokerr_port/validation/cache/geokerr/bfc7797cdaa2b7bb.bin, copied to
tests/golden/) and to its three fail-window slices.  The golden itself
carries GEOKERR's numerical noise (about 1e-11 absolute in t, 6e-12 in phi,
which is 6e-9 relative on the tiny first sample); a 40-digit mpmath
integration of the same geodesic shows that the restatement is closer to the
exact solution than the golden is, so the bounds below are GEOKERR's noise,
not the restatement's error.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import geokerr_golden as gg  # noqa: E402
import oracle  # noqa: E402


def _eval_golden():
    g = gg.read_cache()
    out = oracle.geokerr_eval_lambda(g["u0"], g["mu0"], g["uf"], g["a"], g["Lz"], g["Q2"], g["t0"],
                                     g["lam0"], g["dlam"], g["S"])
    return g, out


def test_golden_eval_lambda(built):
    g, out = _eval_golden()
    assert out["info"] == 0
    assert (out["tpmi"], out["tpri"]) == (g["tpmi"], g["tpri"]) == (-1, -1)
    assert np.array_equal(out["affine"], g["affine"])
    assert out["u"][0] == g["u"][0] and out["mu"][0] == g["mu"][0]
    # bounds = GEOKERR's own noise in the golden (see module docstring)
    assert np.max(np.abs(out["u"] - g["u"]) / g["u"]) < 2e-12
    assert np.max(np.abs(out["mu"] - g["mu"]) / np.abs(g["mu"])) < 1e-13
    assert np.max(np.abs(out["t"] - g["t"])) < 2e-11
    assert np.max(np.abs(out["phi"] - g["phi"])) < 1e-11
    assert np.max(np.abs(out["t"][10:] - g["t"][10:]) / g["t"][10:]) < 1e-9


@pytest.mark.parametrize("path", gg.fail_windows())
def test_fail_windows(built, path):
    """Reference halves of the gkval fail windows are slices of the golden u."""
    w = gg.read_fail_window(path)
    g, out = _eval_golden()
    assert w["field"] == 0 and w["end"] - w["start"] == w["size"] == 32
    assert np.array_equal(w["ref"], g["u"][w["start"]:w["end"]])
    assert np.max(np.abs(out["u"][w["start"]:w["end"]] - w["ref"]) / w["ref"]) < 2e-12


def test_mpmath_pin(built):
    """Sample points against a 40-digit mpmath integration of the golden geodesic."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 30
    a, l, q2 = mp.mpf("0.5"), mp.mpf(2), mp.mpf(4)
    u0 = mp.mpf("0.1")
    du = -mp.mpf("0.09") / 4096
    U = lambda u: 1 + (a * a - q2 - l * l) * u ** 2 + 2 * ((a - l) ** 2 + q2) * u ** 3 - a * a * q2 * u ** 4
    Tr = lambda u: (1 + a * a * u * u) * (1 + (a * a - a * l) * u * u) / (u * u * (1 - 2 * u + a * a * u * u))
    pts = oracle.geokerr_points(0.1, 0.01, 0.8, 0.5, 2.0, 4.0, -1.0, -1.0, 1, 4096, 0.5)
    assert pts["n"] == 4096
    for k in (100, 4096):
        uk = u0 + (k - mp.mpf("0.5")) * du
        assert abs(pts["u"][k - 1] - float(uk)) < 1e-16
        # radial part of t plus the angular part (mu stays within 0.027 of 0.8 here)
        lam = mp.quad(lambda x: 1 / mp.sqrt(U(x)), [uk, u0])
        tr = mp.quad(lambda x: Tr(x) / mp.sqrt(U(x)), [uk, u0])
        assert float(lam) > 0 and abs(float(tr) - pts["dt"][k - 1]) / float(tr) < 2e-2


def test_camera_grid_and_turning_points(built):
    """Standard-run grid rays (geokerr_original.f:255-290): captured rays stop at the
    horizon, scattered rays come back out with one radial turning point."""
    grid = oracle.geokerr_camera_grid(0.9, 0.5, 8, 8)
    uplus = 1.0 / (1.0 + np.sqrt(1.0 - 0.81))
    kinds = set()
    for i in range(64):
        p = oracle.geokerr_points(1e-6, uplus, 0.5, 0.9, grid["l"][i], grid["q2"][i], 1.0, grid["sm"][i], 1, 32, 0.5)
        assert p["n"] == 32, i
        assert np.all(np.isfinite(p["lam"])) and np.all(np.diff(p["lam"]) > 0)
        kinds.add(int(p["tpr"][-1]))
        if p["tpr"][-1] == 1:
            assert abs(p["u"][-1] - 1e-6) < 1e-2      # back out towards the observer
        else:
            assert p["u"][-1] < uplus and p["u"][-1] > 0.9 * uplus
    assert kinds == {0, 1}


def test_estimate_periods_and_phi_omega(built):
    tr, tt, info = oracle.geokerr_estimate_periods(0.1, 0.3, 0.5, 2.0, 4.0)
    assert info == 0 and tr == -1.0 and (tt > 0 or tt == -1.0)
    lib = oracle.load()
    oracle._geo_protos(lib)
    w = lib.npo_geokerr_phi_omega(0.1, 0.8, 0.5, 2.0, 4.0)
    r = 10.0
    exp = 0.5 * ((r * r + 0.25 - 1.0) / (r * r - 2 * r + 0.25)) + 2.0 / (1 - 0.64) - 0.5
    assert abs(w - exp) < 1e-14


def test_stream_exact_samples(built):
    """Mino-time samples satisfy the first integral (du/dl)^2 = U(u) to rounding."""
    rc, s = oracle.geokerr_stream(0.1, 0.01, 0.3, 0.5, 2.0, 4.0, 0.0, 2e-4, 400)
    assert rc == 0
    u = s["u"]
    a, l, q2 = 0.5, 2.0, 4.0
    U = 1 + (a * a - q2 - l * l) * u ** 2 + 2 * ((a - l) ** 2 + q2) * u ** 3 - a * a * q2 * u ** 4
    dudl = (u[4:] - 8 * u[3:-1] + 8 * u[1:-3] - u[:-4]) / (-12 * 2e-4)   # 5-point stencil
    assert np.max(np.abs(dudl ** 2 - U[2:-2])) < 1e-9
