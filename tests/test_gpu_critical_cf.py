"""Near-critical rays of the mixed path in closed form (crit_cf_solve on the
tracer's FP64 warps, np_scene_t.critical_solver = NP_CRITICAL_CLOSED_FORM)
and the crossings
entry point np_geokerr_disk_crossings_* on the GPU: the same bits as the
host build, the renderer's near-critical crossings against the Mino-time
(Taylor) solver, and frames against the same frames with the near-critical
rays integrated in FP64."""
import math

import numpy as np
import pytest

import nullpath_gb300 as npx
import oracle
from nullpath_gb300 import accuracy
from nullpath_gb300 import geokerr as gk

pytestmark = pytest.mark.gpu


def _all_but_a_few(st):
    """Every near-critical ray solved in closed form but a few per 10,000: a
    ray within ~1e-9 (relative) of the critical curve can have radial roots
    that the root iteration does not resolve, and is then integrated."""
    return st.deferred_rays - st.closed_form_rays <= 2 + st.deferred_rays // 10000


@pytest.fixture(scope="module")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_device_crossings_equal_host(cuda):
    """geokerr.cu is built without multiply-add contraction: the device
    crossings are the host build's bits (u, phi, count, status)."""
    rng = np.random.default_rng(11)
    n = 3000
    l, q2 = rng.uniform(-8, 8, n), rng.uniform(-2, 50, n)
    sm = np.where(rng.uniform(size=n) < 0.5, -1.0, 1.0)
    su = np.where(rng.uniform(size=n) < 0.8, 1.0, -1.0)
    mu0, u0 = math.cos(math.radians(80.0)), 0.02
    for a in (0.9, 0.998):
        h = gk.disk_crossings(a, u0, mu0, l, q2, su, sm, 1e-3, K=6)
        d = gk.disk_crossings(a, u0, mu0, l, q2, su, sm, 1e-3, K=6, device=True)
        cuda.cuda.synchronize()
        for k in ("xu", "xphi", "nx", "status"):
            assert np.array_equal(d[k].cpu().numpy(), h[k], equal_nan=True), (a, k)
        assert (h["status"] >= 0).mean() > 0.95


def _near_critical(sc, px, py):
    """Rays whose report changes when their near-critical handling does."""
    a = npx.trace_rays(sc, px, py, "mixed")
    b = npx.trace_rays(sc.replace(critical_solver=npx.NP_CRITICAL_INTEGRATE), px, py, "mixed")
    xa, xb = a["cross"].cpu().numpy(), b["cross"].cpu().numpy()
    return a, (np.abs(xa - xb).max(axis=(1, 2)) > 0)


@pytest.mark.parametrize("spin", [0.9, 0.998])
def test_trace_rays_near_critical_match_mino_solver(cuda, spin):
    """Critical-curve samples of the 1280x720 benchmark camera on the 7(8)
    mixed path: the near-critical rays' first four crossings (closed form)
    against the Mino-time solver's (np_geokerr_equator_crossings, FP64
    Taylor) to 1e-8 relative in r and 1e-8 rad in phi, counts equal."""
    sc = npx.accurate_scene(npx.benchmark_scene(spin=spin))
    px, py = accuracy.critical_positions(sc, 4000, seed=3)
    out, sel = _near_critical(sc, px, py)
    assert sel.sum() >= 20, sel.sum()
    consts = out["consts"].cpu().numpy()[sel]
    cross = out["cross"].cpu().numpy()[sel]
    u0, mu0, l, q2, su, sm = gk.render_ray_constants(consts, sc)
    xu, xphi, nx = gk.equator_crossings(sc.spin, u0, mu0, l, q2, su, sm, 1.0 / sc.escape_r, 4)
    xu, xphi, nx = xu.cpu().numpy(), xphi.cpu().numpy(), nx.cpu().numpy()
    ncf = (out["status"].cpu().numpy()[sel] >> 4)
    assert np.array_equal(np.minimum(ncf, 4), np.minimum(nx, 4))
    for i in range(sel.sum()):
        k = min(int(nx[i]), 4)
        if k == 0:
            continue
        r_ref = 1.0 / xu[i, :k]
        assert np.max(np.abs(cross[i, :k, 0] - r_ref) / r_ref) <= 1e-8, i
        assert np.max(np.abs(cross[i, :k, 1] - xphi[i, :k])) <= 1e-8, i


@pytest.mark.parametrize("spin", [0.9, 0.998])
def test_render_closed_form_against_integrated(cuda, spin):
    """A critical-sampled 320x180x4 frame on the 7(8) mixed path: every
    near-critical ray is solved in closed form, and the frame matches the
    same frame with those rays integrated in FP64 7(8) (rtol 1e-8): the
    same capture/disk class on >= 99.9 % of pixels, first-crossing radius
    within 1e-5 M on >= 99.9 % of the disk pixels."""
    sc = npx.accurate_scene(npx.benchmark_scene(width=320, height=180, spp=4, spin=spin)).replace(
        jitter=npx.NP_JITTER_CRITICAL)
    rgb, rc, st = npx.render(sc, "mixed", stats=True)
    rgb2, rc2, st2 = npx.render(sc.replace(critical_solver=npx.NP_CRITICAL_INTEGRATE), "mixed", stats=True)
    assert st.deferred_rays > 100 and _all_but_a_few(st), (st.deferred_rays, st.closed_form_rays)
    assert st2.closed_form_rays == 0 and st2.deferred_rays == st.deferred_rays
    assert st.rays == st2.rays == 320 * 180 * 4
    rc, rc2 = rc.cpu().numpy(), rc2.cpu().numpy()
    assert ((rc > 0) == (rc2 > 0)).mean() >= 0.999
    both = (rc > 0) & (rc2 > 0)
    assert (np.abs(rc[both] - rc2[both]) <= 1e-5).mean() >= 0.999
    assert np.isclose(rgb.cpu().numpy(), rgb2.cpu().numpy(), rtol=1e-3, atol=1e-6).all(axis=0).mean() >= 0.999


def test_render_many_near_critical_rays(cuda):
    """A 2048x1024x8 critical-sampled frame at a = 0.998 (about 190k
    near-critical rays, more than the tracer's warps take in one round):
    every ray is traced and every near-critical ray solved, and the frame
    matches the one with the near-critical rays integrated."""
    sc = npx.accurate_scene(npx.benchmark_scene(width=2048, height=1024, spp=8, spin=0.998)).replace(
        jitter=npx.NP_JITTER_CRITICAL)
    rgb, rc, st = npx.render(sc, "mixed", stats=True)
    assert st.rays == 2048 * 1024 * 8
    assert st.deferred_rays > 120000 and _all_but_a_few(st), (st.deferred_rays, st.closed_form_rays)
    # at a = 0.998 the prograde photon orbit lies inside the horizon band:
    # rays that wind there are solved whole in closed form too
    assert st.band_rays > 1000
    rgb2, rc2, st2 = npx.render(sc.replace(critical_solver=npx.NP_CRITICAL_INTEGRATE), "mixed", stats=True)
    assert st2.rays == st.rays and st2.band_rays == 0
    rc, rc2 = rc.cpu().numpy(), rc2.cpu().numpy()
    assert ((rc > 0) == (rc2 > 0)).mean() >= 0.999
    assert np.isclose(rgb.cpu().numpy(), rgb2.cpu().numpy(), rtol=1e-3, atol=1e-6).all(axis=0).mean() >= 0.999


@pytest.mark.parametrize("spin", [0.998])
def test_trace_rays_band_rays_match_mino_solver(cuda, spin):
    """Rays of the 7(8) mixed path that enter the horizon band (critical-curve
    samples at a = 0.998, where the band holds the prograde photon orbit):
    their crossings, from the
    closed form, against the Mino-time solver to 1e-8 relative, and the
    order-1 crossing error of the whole sample within 1e-5 M (p99)."""
    sc = npx.accurate_scene(npx.benchmark_scene(spin=spin))
    px, py = accuracy.critical_positions(sc, 4000, seed=5)
    a = npx.trace_rays(sc, px, py, "mixed")
    b = npx.trace_rays(sc.replace(critical_solver=npx.NP_CRITICAL_INTEGRATE), px, py, "mixed")
    sel = np.abs(a["cross"].cpu().numpy() - b["cross"].cpu().numpy()).max(axis=(1, 2)) > 0
    assert sel.sum() >= 20
    cross = a["cross"].cpu().numpy()[sel]
    u0, mu0, l, q2, su, sm = gk.render_ray_constants(a["consts"].cpu().numpy()[sel], sc)
    xu, xphi, nx = gk.equator_crossings(sc.spin, u0, mu0, l, q2, su, sm, 1.0 / sc.escape_r, 4)
    xu, nx = xu.cpu().numpy(), nx.cpu().numpy()
    for i in range(sel.sum()):
        k = min(int(nx[i]), 4)
        if k:
            r_ref = 1.0 / xu[i, :k]
            assert np.max(np.abs(cross[i, :k, 0] - r_ref) / r_ref) <= 1e-8, i
    r = accuracy.crossing_error(sc, n=8000, precision="mixed", seed=7, critical=True)
    assert r["order1"]["r_err_p99"] <= 1e-5 and r["order1"]["disagree"] == 0, r["order1"]


def test_render_outside_closed_forms_falls_back(cuda):
    """At a = 0 the closed forms do not apply (the radial potential is a
    cubic): the near-critical rays are integrated, as before."""
    sc = npx.accurate_scene(npx.benchmark_scene(width=160, height=90, spp=2, spin=0.0)).replace(
        jitter=npx.NP_JITTER_CRITICAL)
    rgb, rc, st = npx.render(sc, "mixed", stats=True)
    rgb2, rc2, st2 = npx.render(sc.replace(critical_solver=npx.NP_CRITICAL_INTEGRATE), "mixed", stats=True)
    assert st.deferred_rays > 0 and st.closed_form_rays == 0
    assert cuda.equal(rc, rc2) and cuda.equal(rgb, rgb2)


def test_render_rk4_family_closed_form(cuda):
    """The RK4 mixed path (reference step law) hands its near-critical rays
    to the closed form too: against the oracle's FP64 render of the same
    scene, the crossing radii of those rays can differ by the reference
    step law's own truncation error, so the bar is agreement in class on
    99 % of the pixels and radius within 1e-3 M on 99 % of the disk."""
    sc = npx.benchmark_scene(width=48, height=27, spp=1)
    ref_rgb, ref_rc = oracle.render(sc)
    rgb, rc, st = npx.render(sc, "mixed", stats=True)
    rc = rc.cpu().numpy()
    assert _all_but_a_few(st)
    assert ((ref_rc > 0) == (rc > 0)).mean() > 0.99
    both = (ref_rc > 0) & (rc > 0)
    assert (np.abs(rc[both] - ref_rc[both]) < 1e-3).mean() > 0.99
