"""Research mode of the FP64 path: Fehlberg's embedded 7(8) integrator,
root-found disk crossings and invariant-gated acceptance (the research-mode
accuracy plan of the reference, docs/PLAN.md:35-66), on the CPU oracle:
the tableau's order, crossing radii against the Mino-time GEOKERR solver,
and the drift of the Hamiltonian and of Carter's constant."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import oracle
import nullpath_gb300 as npx
from nullpath_gb300 import geokerr as gk
from nullpath_gb300._abi import (benchmark_scene, NP_INTEG_RKF78, NP_CROSS_ROOT, NP_CROSS_HERMITE,
                                 NP_PREC_FP64, NP_PREC_MIXED, NP_ERR_INVALID)

N = 200


@pytest.fixture(scope="module")
def rays(built):
    rng = np.random.default_rng(0)
    return rng.uniform(0, 64, N), rng.uniform(0, 36, N)


def _scene(**kw):
    return benchmark_scene(width=64, height=36, spp=1).replace(**kw)


RESEARCH = dict(integrator=NP_INTEG_RKF78, crossing=NP_CROSS_ROOT, rtol=1e-12, atol=1e-14, inv_gate=1e-12)


def _geokerr_radii(consts, sc):
    u0, mu0, l, q2, su, sm = gk.render_ray_constants(consts, sc)
    out = np.zeros((len(u0), 4))
    for i in range(len(u0)):
        k, xu, _ = oracle.geokerr_crossings(u0[i], mu0[i], sc.spin, l[i], q2[i], su[i], sm[i], 1.0 / sc.escape_r, 4)
        out[i, :k] = np.where(xu[:k] > 0, 1.0 / np.maximum(xu[:k], 1e-300), 0.0)
    return out


def _crossing_relerr(sc, px, py):
    o = oracle.trace_rays(sc, px, py)
    ref = _geokerr_radii(o["consts"], sc)
    r = o["cross"][:, :, 0]
    m = (r > 0) & (ref > 0) & (r < 30) & (ref < 30)
    return np.abs(r[m] - ref[m]) / ref[m], o


def test_tableau_order(built):
    """Quadrature conditions: the 8th-order weights and the embedded
    7th-order weights (b + e) integrate c^k exactly for k <= 7 (the two
    differ in the non-quadrature order conditions, checked by convergence
    below); the error weights sum to zero."""
    A, b, e = oracle.rkf78_tableau()
    c = A.sum(axis=1)
    assert np.allclose(c, [0, 2 / 27, 1 / 9, 1 / 6, 5 / 12, 1 / 2, 5 / 6, 1 / 6, 2 / 3, 1 / 3, 1, 0, 1], atol=1e-15)
    for k in range(8):
        assert abs(b @ c ** k - 1.0 / (k + 1)) < 1e-14, k
    b7 = b + e
    for k in range(8):
        assert abs(b7 @ c ** k - 1.0 / (k + 1)) < 1e-14, k
    assert abs(e.sum()) < 1e-16
    assert np.allclose(np.triu(A), 0.0)


def test_tableau_convergence_orders(built):
    """Global error on a Kepler orbit (eccentricity 0.5) falls as h^8 for the
    propagated solution and as h^7 for the embedded one."""
    A, b, e = oracle.rkf78_tableau()

    def f(y):
        r3 = (y[0] ** 2 + y[1] ** 2) ** 1.5
        return np.array([y[2], y[3], -y[0] / r3, -y[1] / r3])

    def integrate(h, n, w):
        y = np.array([0.5, 0.0, 0.0, np.sqrt(3.0)])     # periapsis of e = 0.5, a = 1
        for _ in range(n):
            k = np.zeros((13, 4))
            for j in range(13):
                k[j] = f(y + h * (A[j, :j] @ k[:j]))
            y = y + h * (w @ k)
        return y

    T = 2 * np.pi                                        # one period
    exact = np.array([0.5, 0.0, 0.0, np.sqrt(3.0)])
    for w, order in ((b, 8), (b + e, 7)):
        errs = [np.abs(integrate(T / n, n, w) - exact).max() for n in (128, 256)]
        rate = np.log2(errs[0] / errs[1])
        assert order - 0.4 < rate < order + 0.6, (order, rate, errs)


def test_research_crossings_match_geokerr(rays):
    """Order-1..4 crossing radii of the 7(8) integrator with root-found
    crossings agree with the Mino-time solver to 1e-10 (relative); the
    reference's RK4 with Hermite crossings is at the 1e-7 level."""
    px, py = rays
    err, o = _crossing_relerr(_scene(**RESEARCH), px, py)
    assert err.size >= 30 and err.max() < 1e-10, err.max()
    err4, o4 = _crossing_relerr(_scene(crossing=NP_CROSS_HERMITE), px, py)
    assert np.quantile(err4, 0.99) > 1e-8
    assert o["steps"].mean() < 0.2 * o4["steps"].mean()


def test_root_crossings_tighten_rk4(rays):
    px, py = rays
    e_h, _ = _crossing_relerr(_scene(crossing=NP_CROSS_HERMITE), px, py)
    e_r, _ = _crossing_relerr(_scene(crossing=NP_CROSS_ROOT), px, py)
    assert np.quantile(e_r, 0.99) < 0.5 * np.quantile(e_h, 0.99)


def test_invariant_drift_and_gate(rays):
    """Research settings keep |H| / (sum of its terms) and |dQ| / Q-scale
    at the 1e-11 level over every accepted step.  At rtol 1e-10 a gate of
    1e-12 on each step's change of H and Q cuts the Carter drift more than
    tenfold for a few percent more steps."""
    px, py = rays
    d, steps = oracle.trace_invariants(_scene(**RESEARCH), px, py)
    assert d[:, 0].max() < 1e-10 and d[:, 1].max() < 1e-10
    assert np.quantile(d[:, 1], 0.99) < 1e-11
    loose = dict(RESEARCH, rtol=1e-10, atol=1e-12, inv_gate=0.0)
    d0, s0 = oracle.trace_invariants(_scene(**loose), px, py)
    d1, s1 = oracle.trace_invariants(_scene(**dict(loose, inv_gate=1e-12)), px, py)
    assert np.quantile(d1[:, 1], 0.99) < 0.1 * np.quantile(d0[:, 1], 0.99)
    assert s0.mean() < s1.mean() < 1.1 * s0.mean()     # gated steps are rejected and retaken smaller
    # the reference's fixed-step RK4 loses the constraint near the horizon
    d4, _ = oracle.trace_invariants(_scene(), px, py)
    assert d4[:, 0].max() > 1e-3


def test_scene_validation_and_path_checks(built):
    lib = npx.load()
    s = _scene(**RESEARCH)
    assert lib.np_scene_validate(C.byref(s)) == 0
    for bad in (dict(integrator=3), dict(crossing=3), dict(inv_gate=-1.0), dict(inv_gate=float("nan")),
                dict(inv_gate=1.0)):
        t = s.replace(**bad)
        assert lib.np_scene_validate(C.byref(t)) == NP_ERR_INVALID, bad
    for bad in (dict(rtol_fp64=float("nan")), dict(rtol_fp64=1.0)):
        t = s.replace(**bad)
        assert lib.np_scene_validate(C.byref(t)) == NP_ERR_INVALID, bad
    rgb = (C.c_float * (3 * 64 * 36))()
    # root crossings on the mixed path are Henon steps of the 7(8) integrator:
    # with RK4 or step doubling the mixed path refuses them before looking for
    # a device
    for kw in (dict(crossing=NP_CROSS_ROOT), dict(crossing=NP_CROSS_ROOT, integrator=1)):
        t = _scene(**kw)
        assert lib.np_render_host(C.byref(t), NP_PREC_MIXED, rgb, None, None, None) == NP_ERR_INVALID
        assert b"rkf78" in lib.np_last_error()


def test_cli_research_mode_refuses_mixed(built):
    cli = os.path.join(os.path.dirname(npx.lib_path()), "render")
    p = subprocess.run([cli, "--mode", "research", "--precision", "mixed", "--w", "8", "--h", "8"],
                       capture_output=True, text=True, timeout=60)
    assert p.returncode == 1 and "precision fp64" in p.stderr


def test_research_in_reference_units_and_zamo(built):
    """Research mode on a reference-default scene (lengths in Rs, M = 10,
    static camera) and on the ZAMO camera of research_scene(): crossing radii
    against the Mino-time solver.  The reference's camera builds the ray
    direction in FP32 (render.cu:137-159), so its momentum is null only to
    ~1e-7 and the Mino-time constants describe a slightly different ray:
    there the bar is 1e-6; in units of M (FP64 camera) it is 1e-10."""
    from nullpath_gb300._abi import reference_defaults, research_scene
    rng = np.random.default_rng(5)
    for sc in (reference_defaults().replace(width=32, height=18, spp=1, spin=0.9, theta_deg=80.0, fov_y_deg=55.0,
                                            integrator=NP_INTEG_RKF78, crossing=NP_CROSS_ROOT, rtol=1e-12,
                                            atol=1e-14, inv_gate=1e-12),
               research_scene(benchmark_scene(width=32, height=18, spp=1))):
        px, py = rng.uniform(0, sc.width, 120), rng.uniform(0, sc.height, 120)
        o = oracle.trace_rays(sc, px, py)
        M = sc.mass
        csc = sc
        if sc.units == 0:
            # reference scenes set the camera and the spin up in float
            # (render.cu:137-139, 161-170): theta = fl(fl(theta) fl(pi)) / 180,
            # a = fl(fl(a/M) M)
            th = np.float32(np.float32(sc.theta_deg) * np.float32(np.pi)) / np.float32(180.0)
            af = np.float32(np.float32(sc.spin) * np.float32(M))
            csc = sc.replace(theta_deg=float(th) * 180.0 / np.pi, spin=float(af) / M)
        u0, mu0, l, q2, su, sm = gk.render_ray_constants(o["consts"], csc)
        lunit = M if sc.units == 1 else 2.0 * M
        r_far = sc.escape_r if sc.escape_r > 0 else (sc.r_cam + 10.0) * lunit
        errs = []
        for i in range(len(px)):
            k, xu, _ = oracle.geokerr_crossings(u0[i], mu0[i], csc.spin, l[i], q2[i], su[i], sm[i], M / r_far, 4)
            n = min(k, int(o["status"][i]) >> 4, 4)
            for j in range(n):
                r_ref = M / xu[j]
                errs.append(abs(o["cross"][i, j, 0] - r_ref) / r_ref)
        bar = 1e-6 if sc.units == 0 else 1e-10
        assert len(errs) > 20 and max(errs) < bar, (sc.units, len(errs), max(errs))


def test_cli_mixed_root_needs_rkf78(built):
    cli = os.path.join(os.path.dirname(npx.lib_path()), "render")
    p = subprocess.run([cli, "--precision", "mixed", "--crossing", "root", "--w", "8", "--h", "8"],
                       capture_output=True, text=True, timeout=60)
    assert p.returncode == 1 and "--integrator rkf78" in p.stderr
    p = subprocess.run([cli, "--precision", "mixed", "--inv-gate", "1e-12", "--w", "8", "--h", "8"],
                       capture_output=True, text=True, timeout=60)
    assert p.returncode == 1 and "precision fp64" in p.stderr
