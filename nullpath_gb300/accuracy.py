"""Error of the renderer's disk crossings against the FP64 GEOKERR-equivalent
Mino-time solver (GEOR with muf = 0) on the same rays.

For seeded random image positions the renderer traces each ray
(np_trace_rays_device, the same integrator as the render kernels) and
reports its first four equatorial crossings; the Mino-time solver takes the
ray's camera constants (l = L/E, q2 = Q/E^2, initial signs) and returns the
exact crossings.  Reported per crossing order: radius error (M), phi error
(rad) and disk-intensity error (relative, j ~ r^-q g^3 with the Keplerian
redshift g), over crossings inside the disk in both.
"""
import math

import numpy as np


def doppler_g(r, E, L, M, a):
    """Redshift of a prograde Keplerian emitter at radius r (bh_kerr.h:833-862)."""
    x = np.maximum(1.0, r / M)
    Om = 1.0 / ((a / M + x * np.sqrt(x)) * M)
    gtt = -(1.0 - 2.0 * M / r)
    gtp = -2.0 * M * a / r
    gpp = r * r + a * a + 2.0 * M * a * a / r
    den = -(gtt + Om * (2.0 * gtp + gpp * Om))
    ut = 1.0 / np.sqrt(np.maximum(den, 1e-24))
    return np.maximum(E / np.maximum(ut * (E - Om * L), 1e-18), 0.0)


def critical_positions(scene, n, seed=0, band=0.02):
    """n image positions, uniform over the frame, of which every second one
    is moved along its position angle to within +-band of the critical curve
    (the sampling of NP_JITTER_CRITICAL, from the library's critical-curve
    table)."""
    import ctypes as C
    from ._lib import load, check
    rho_c = np.zeros(256, dtype=np.float32)
    check(load().np_critical_curve(C.byref(scene), rho_c.ctypes.data))
    rng = np.random.default_rng(seed)
    W, H = scene.width, scene.height
    th = math.tan(math.radians(scene.fov_y_deg) / 2)
    asp = W / H
    px = rng.uniform(0.0, W, n)
    py = rng.uniform(0.0, H, n)
    cx = (px / W * 2 - 1) * asp * th
    cy = -(py / H * 2 - 1) * th
    psi = np.arctan2(cy, cx)
    t = (psi + math.pi) * (256 / (2 * math.pi))
    i0 = np.floor(t).astype(int)
    fr = t - i0
    i0 %= 256
    rc = (1 - fr) * rho_c[i0] + fr * rho_c[(i0 + 1) % 256]
    rho = rc * (1 + band * rng.uniform(-1, 1, n))
    sel = np.arange(n) % 2 == 1
    cx = np.where(sel, rho * np.cos(psi), cx)
    cy = np.where(sel, rho * np.sin(psi), cy)
    return (cx / (asp * th) + 1) / 2 * W, (1 - cy / th) / 2 * H


def crossing_error(scene, n=20000, precision="mixed", seed=0, orders=2, critical=False, cache=None):
    """Crossing radius, crossing azimuth and intensity of the first `orders`
    disk crossings of n rays, traced by the renderer, against the Mino-time
    solver's equatorial crossings of the same rays.  critical=True samples
    half the rays within +-2 % of the critical curve.  `cache` (a dict) keeps
    the solver's crossings between calls on the same rays (same camera, n,
    seed, sampling), whatever the precision or integrator."""
    import torch
    from .render import trace_rays
    from . import geokerr as gk

    if critical:
        px, py = critical_positions(scene, n, seed)
    else:
        rng = np.random.default_rng(seed)
        px = rng.uniform(0.0, scene.width, n)
        py = rng.uniform(0.0, scene.height, n)
    out = trace_rays(scene, px, py, precision)
    torch.cuda.synchronize()
    consts = out["consts"].cpu().numpy()
    cross = out["cross"].cpu().numpy()
    M = scene.mass
    lunit = M if scene.units == 1 else 2.0 * M
    a = scene.spin * M
    key = (n, seed, bool(critical), scene.width, scene.height, scene.spin, scene.theta_deg, scene.r_cam, scene.mass)
    if cache is not None and key in cache and np.array_equal(cache[key][0], consts):
        xr_ref, xphi_ref, cross_check = cache[key][1], cache[key][2], cache[key][3]
    else:
        u0, mu0, l, q2, su, sm = gk.render_ray_constants(consts, scene)
        r_far = scene.escape_r if scene.escape_r > 0 else (scene.r_cam + 20.0) * lunit
        xu, xphi, nx = gk.equator_crossings(scene.spin, u0, mu0, l, q2, su, sm, M / r_far, 4)
        xr_ref = np.where(xu.cpu().numpy() > 0, M / np.maximum(xu.cpu().numpy(), 1e-300), 0.0)
        xphi_ref = xphi.cpu().numpy()
        # the same crossings in closed form (Jacobi polar motion, inverted
        # Carlson radial integral): an independent check of the solver
        from .carlson import equator_crossings_cf
        cf_u, cf_n = equator_crossings_cf(scene.spin, u0, mu0, l, q2, su, sm, M / r_far, 4, device=True)
        tx, tn = xu.cpu().numpy(), nx.cpu().numpy()
        same = cf_n == tn
        both = same[:, None] & (np.arange(4)[None, :] < np.maximum(tn, 0)[:, None]) & (tx > 0)
        cross_check = {"count_agreement": float(same.mean()),
                       "max_rel_u_diff": float((np.abs(cf_u[both] - tx[both]) / tx[both]).max()) if both.any() else 0.0}
        if cache is not None:
            cache[key] = (consts.copy(), xr_ref, xphi_ref, cross_check)
    E = -consts[:, 0]
    L = consts[:, 1]
    rin = scene.disk_rin if scene.disk_rin > 0 else 3.0 * 2.0 * M
    rout = scene.disk_rout if scene.disk_rout > 0 else 20.0 * 2.0 * M
    q = scene.emissivity_q
    res = {"rays": n, "precision": precision, "solver_vs_closed_form": cross_check}
    for k in range(orders):
        r = cross[:, k, 0]
        rr = xr_ref[:, k]
        both = (r >= rin) & (r <= rout) & (rr >= rin) & (rr <= rout)
        either = ((r >= rin) & (r <= rout)) | ((rr >= rin) & (rr <= rout))
        if not both.any():
            res["order%d" % (k + 1)] = {"crossings": 0}
            continue
        dr = np.abs(r[both] - rr[both])
        dphi = np.abs(cross[both, k, 1] - xphi_ref[both, k])
        Ia = rr[both] ** (-q) * doppler_g(rr[both], E[both], L[both], M, a) ** 3
        Ib = r[both] ** (-q) * doppler_g(r[both], E[both], L[both], M, a) ** 3
        dI = np.abs(Ib - Ia) / Ia
        res["order%d" % (k + 1)] = {
            "crossings": int(both.sum()), "disagree": int((either & ~both).sum()),
            "r_err_max": float(dr.max()), "r_err_p99": float(np.quantile(dr, 0.99)),
            "r_err_p50": float(np.median(dr)),
            "phi_err_max": float(dphi.max()), "phi_err_p99": float(np.quantile(dphi, 0.99)),
            "I_relerr_max": float(dI.max()), "I_relerr_p99": float(np.quantile(dI, 0.99)),
            "frac_r_err_le_1e-5": float((dr <= 1e-5).mean()),
        }
    return res
