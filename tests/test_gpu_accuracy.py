"""Disk-crossing accuracy of the mixed 7(8) path (compensated FP32 under
error control, Henon crossings, FP64 islands) against the Mino-time solver
on the 1280x720x4, a = 0.9 benchmark frame, through the C ABI.

Bar: the first disk crossing radius within 1e-5 M of the solver's at the
99th percentile.  The oracle is the CPU Mino-time solver (GEOR with mu_f =
0), restated in oracle/geokerr_oracle.cpp, fed the CPU camera's momenta of
the same rays.
"""
import numpy as np
import pytest

import nullpath_gb300 as npx
import oracle

pytestmark = pytest.mark.gpu

BAR_M = 1e-5


def _first_disk(xr, rin, rout):
    """First crossing radius inside [rin, rout] along the last axis (0 if none)."""
    inside = (xr >= rin) & (xr <= rout)
    idx = np.argmax(inside, axis=-1)
    first = np.take_along_axis(xr, idx[..., None], axis=-1)[..., 0]
    return np.where(inside.any(axis=-1), first, 0.0)


def test_frame_rows_first_crossing_meets_bar(cuda):
    """Every 45th row of the full frame (16 rows x 1280 pixels, sample 0 of
    each pixel, the sample np_render_device reports in rcross)."""
    import torch
    sc = npx.accurate_scene(npx.benchmark_scene()).replace(islands=npx.NP_ISLANDS_ALL)
    rgb, rc = npx.render(sc, "mixed")
    torch.cuda.synchronize()
    rc = rc.cpu().numpy().astype(np.float64)
    assert np.isfinite(rgb.cpu().numpy()).all()
    rows = list(range(0, sc.height, 45))
    errs, cls = [], []
    for y in rows:
        truth = _first_disk(oracle.frame_crossings(sc, y, y + 1)[0], sc.disk_rin, sc.disk_rout)
        got = rc[y]
        cls.append(((got > 0) == (truth > 0)).mean())
        both = (got > 0) & (truth > 0)
        errs.append(np.abs(got[both] - truth[both]))
    err = np.concatenate(errs)
    assert err.size > 1000, err.size
    assert np.mean(cls) > 0.999, np.mean(cls)
    p99 = np.quantile(err, 0.99)
    assert p99 <= BAR_M, (p99, err.max())


def test_random_rays_order1_meets_bar(cuda):
    """50,000 random image positions of the frame through np_trace_rays_device
    (the render's integrator): first crossing inside the disk, p99 <= 1e-5 M;
    second order p99 <= 1e-4 M (its rays pass the photon region once more)."""
    from nullpath_gb300 import accuracy
    sc = npx.accurate_scene(npx.benchmark_scene()).replace(islands=npx.NP_ISLANDS_ALL)
    res = accuracy.crossing_error(sc, n=50000, precision="mixed", seed=21)
    o1, o2 = res["order1"], res["order2"]
    assert o1["crossings"] > 3000 and o1["disagree"] <= 2, o1
    assert o1["r_err_p99"] <= BAR_M, o1
    assert o2["r_err_p99"] <= 1e-4, o2


def test_crossing_modes_and_islands(cuda):
    """Henon crossings beat the Hermite interpolant over the same 7(8) steps,
    and the islands (FP64 7(8) steps) do not worsen the bar."""
    from nullpath_gb300 import accuracy
    base = npx.accurate_scene(npx.benchmark_scene())
    henon = accuracy.crossing_error(base.replace(islands=0), n=20000, precision="mixed", seed=5)["order1"]
    herm = accuracy.crossing_error(base.replace(islands=0, crossing=npx.NP_CROSS_HERMITE), n=20000,
                                   precision="mixed", seed=5)["order1"]
    isl = accuracy.crossing_error(base.replace(islands=npx.NP_ISLANDS_ALL), n=20000, precision="mixed",
                                  seed=5)["order1"]
    assert henon["r_err_p99"] < herm["r_err_p99"], (henon, herm)
    assert henon["r_err_p99"] <= BAR_M and isl["r_err_p99"] <= BAR_M, (henon, isl)


def test_mixed78_matches_oracle_render(cuda):
    """Small frame of the benchmark camera: colours and first-crossing radii of
    the mixed 7(8) path against the FP64 oracle render in research mode
    (7(8) at rtol 1e-12, root-found crossings)."""
    import torch
    sc = npx.benchmark_scene(width=64, height=36, spp=1)
    ref = sc.replace(integrator=npx.NP_INTEG_RKF78, crossing=npx.NP_CROSS_ROOT, rtol=1e-12, atol=1e-14)
    ref_rgb, ref_rc = oracle.render(ref)
    rgb, rc = npx.render(npx.accurate_scene(sc), "mixed")
    torch.cuda.synchronize()
    rgb, rc = rgb.cpu().numpy(), rc.cpu().numpy()
    both = (rc > 0) & (ref_rc > 0)
    assert ((rc > 0) == (ref_rc > 0)).mean() > 0.995
    err = np.abs(rc[both].astype(np.float64) - ref_rc[both])
    # float32 radii: p99 within 1e-5 M; colours within 1e-3 relative on >= 99 % of pixels
    assert np.quantile(err, 0.99) <= 1e-5, np.quantile(err, 0.99)
    close = np.isclose(rgb, ref_rgb, rtol=1e-3, atol=1e-6).all(axis=0).mean()
    assert close > 0.99, close


def test_double_float_islands_match_fp64_islands(cuda):
    """Island steps and near-critical rays of the 7(8) path in double-float
    arithmetic (NP_ISLAND_ARITH_DF) against native FP64: the same crossings
    to 5e-6 M (p99; both integrate to rtol 1e-8 and take different step
    sequences, so they differ at the FP32 rounding floor of the path), and
    the bar against the Mino-time solver holds for both."""
    from nullpath_gb300 import accuracy
    sc = npx.accurate_scene(npx.benchmark_scene()).replace(islands=npx.NP_ISLANDS_ALL,
                                                           critical_solver=npx.NP_CRITICAL_INTEGRATE)
    rng = np.random.default_rng(9)
    px, py = rng.uniform(0, sc.width, 6000), rng.uniform(0, sc.height, 6000)
    a = npx.trace_rays(sc, px, py, "mixed")["cross"].cpu().numpy()[:, 0, 0]
    b = npx.trace_rays(sc.replace(island_arith=npx.NP_ISLAND_ARITH_DF), px, py, "mixed")["cross"].cpu().numpy()[:, 0, 0]
    both = (a >= sc.disk_rin) & (a <= sc.disk_rout) & (b >= sc.disk_rin) & (b <= sc.disk_rout)
    assert both.sum() > 300
    assert np.quantile(np.abs(a[both] - b[both]), 0.99) <= 5e-6
    r = accuracy.crossing_error(sc.replace(island_arith=npx.NP_ISLAND_ARITH_DF), n=20000, precision="mixed", seed=5)
    assert r["order1"]["r_err_p99"] <= BAR_M, r["order1"]
