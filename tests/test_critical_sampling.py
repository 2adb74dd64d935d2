"""Critical-curve importance sampling (NP_JITTER_CRITICAL): the library's
critical-curve table equals the oracle's, matches the Schwarzschild shadow in
closed form, and separates captured from escaping rays."""
import ctypes as C
import math

import numpy as np

import nullpath_gb300 as npx
import oracle


def _table(sc):
    rho = np.zeros(256, dtype=np.float32)
    assert npx.load().np_critical_curve(C.byref(sc), rho.ctypes.data) == 0
    return rho


def test_table_matches_oracle(built):
    for spin, th, units in ((0.0, 80.0, npx.NP_UNITS_M), (0.9, 60.0, npx.NP_UNITS_M), (0.998, 80.0, npx.NP_UNITS_M),
                            (0.5, 75.0, npx.NP_UNITS_RS)):
        sc = npx.benchmark_scene(width=320, height=180, spp=4, spin=spin).replace(theta_deg=th, units=units,
                                                                                 jitter=npx.NP_JITTER_CRITICAL)
        assert np.array_equal(_table(sc), oracle.critical_curve(sc))


def test_schwarzschild_shadow_in_closed_form(built):
    # static observer at r: sin(alpha) = b_crit sqrt(1 - 2M/r) / r, b_crit = 3 sqrt(3) M
    sc = npx.benchmark_scene(width=64, height=64, spp=4, spin=0.0)
    r = sc.r_cam
    s = 3.0 * math.sqrt(3.0) * math.sqrt(1.0 - 2.0 / r) / r
    want = math.tan(math.asin(s))
    rho = _table(sc)
    assert np.allclose(rho, want, rtol=2e-7)


def test_table_separates_capture_from_escape(built):
    sc = npx.benchmark_scene(width=64, height=64, spp=1, spin=0.9).replace(theta_deg=70.0)
    rho = _table(sc).astype(np.float64)
    psi = -math.pi + 2 * math.pi * np.arange(256) / 256
    W, H = sc.width, sc.height
    th = math.tan(math.radians(sc.fov_y_deg) / 2)
    px, py = [], []
    for f in (0.995, 1.005):
        cx, cy = f * rho * np.cos(psi), f * rho * np.sin(psi)
        px.append((cx / th + 1.0) / 2.0 * W)
        py.append((1.0 - cy / th) / 2.0 * H)
    ref = oracle.trace_rays(sc, np.concatenate(px), np.concatenate(py))
    status = ref["status"] % 16
    inside, outside = status[:256], status[256:]
    assert (inside == 1).mean() > 0.97 and (outside != 1).mean() > 0.97
