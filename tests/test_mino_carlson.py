"""Semi-analytic Mino times with Carlson's R_F (csrc/mino_carlson.cuh, host
build) against adaptive quadrature and against the Mino-time Taylor solver's
samples of the same geodesics (oracle/geokerr_oracle.cpp)."""
import math

import numpy as np
import pytest

from nullpath_gb300 import carlson
import oracle


def _U(u, a, l, q2):
    B, K = a * a - l * l - q2, (l - a) ** 2 + q2
    return 1 + B * u * u + 2 * K * u ** 3 - a * a * q2 * u ** 4


def _M(mu, a, l, q2):
    B = a * a - l * l - q2
    return q2 + B * mu * mu - a * a * mu ** 4


def test_against_quadrature(built):
    integrate = pytest.importorskip("scipy.integrate")
    rng = np.random.default_rng(2)
    checked = 0
    for _ in range(300):
        a = rng.uniform(0.0, 0.99)
        l = rng.uniform(-8, 8)
        q2 = rng.uniform(0.1, 40)
        # a radial segment from large r inwards that stays where U > 0
        u1 = rng.uniform(0.005, 0.2)
        us = np.linspace(0.001, u1, 200)
        if (_U(us, a, l, q2) <= 0).any():
            continue
        lu, lm = carlson.mino_times(a, 0.001, u1, 0.0, 0.3, l, q2, device=False)
        assert np.isfinite(lu), (a, l, q2)     # real roots or one complex pair: both in closed form
        ref = integrate.quad(lambda u: 1 / math.sqrt(_U(u, a, l, q2)), 0.001, u1, epsabs=1e-14, epsrel=1e-13)[0]
        # a small a q2 makes the quartic nearly cubic (a far root): 1e-9
        assert abs(lu - ref) <= 1e-9 * ref, (a, l, q2, lu, ref)
        if _M(0.3, a, l, q2) > 0 and all(_M(m, a, l, q2) > 0 for m in np.linspace(0, 0.3, 50)):
            refm = integrate.quad(lambda m: 1 / math.sqrt(_M(m, a, l, q2)), 0.0, 0.3, epsabs=1e-14, epsrel=1e-13)[0]
            assert abs(lm - refm) <= 1e-11 * refm
        checked += 1
    assert checked > 50


def test_against_taylor_solver_samples(built):
    """Along exact Mino-time samples of a geodesic (the Taylor solver of the
    GEOKERR path), the Carlson Mino time from the start to each sample before
    the first turning point equals the sample's lambda."""
    rng = np.random.default_rng(4)
    done = 0
    for _ in range(60):
        a = rng.uniform(0.1, 0.95)
        l = rng.uniform(-4, 4)
        q2 = rng.uniform(1, 30)
        u0, mu0 = 0.01, rng.uniform(-0.6, 0.6)
        rc, s = oracle.geokerr_stream(u0, 0.5, mu0, a, l, q2, 0.0, 0.02, 40)
        if rc != 0:
            continue
        u, mu, lam = s["u"], s["mu"], s["affine"]
        du, dmu = np.diff(u), np.diff(mu)
        # the monotonic prefix of both motions
        k = 1
        while k < len(u) and du[k - 1] > 0 and np.sign(dmu[k - 1]) == np.sign(dmu[0]):
            k += 1
        k -= 1          # a turning point can fall inside the last interval
        if k < 4:
            continue
        lu, lm = carlson.mino_times(a, np.full(k, u0), u[:k], np.full(k, mu0), mu[:k], l, q2, device=False)
        assert np.isfinite(lu).all()
        assert np.allclose(lu, lam[:k], rtol=1e-10, atol=1e-12), (a, l, q2)
        assert np.allclose(lm, lam[:k], rtol=1e-10, atol=1e-12), (a, l, q2)
        done += 1
    assert done >= 30


def test_jacobi_against_scipy(built):
    sp = pytest.importorskip("scipy.special")
    rng = np.random.default_rng(6)
    u = rng.uniform(-20, 20, 3000)
    m = np.concatenate([rng.uniform(0, 1, 2990), [0.0, 1e-17, 1.0, 1 - 1e-17, 0.5, 0.999999, 1e-9, 0.3, 0.7, 0.9]])
    sn, cn, dn = carlson.jacobi(u, m)
    rs, rc, rd, _ = sp.ellipj(u, m)
    assert np.allclose(sn, rs, atol=2e-13) and np.allclose(cn, rc, atol=2e-13) and np.allclose(dn, rd, atol=2e-13)


def test_polar_motion_against_taylor_solver(built):
    """mu(lambda) in closed form (Jacobi cn, Carlson R_F) against the Taylor
    solver's exact Mino-time samples, through several polar turning points."""
    rng = np.random.default_rng(8)
    done = 0
    for _ in range(150):
        a = rng.uniform(0.0, 0.99)
        l = rng.uniform(-5, 5)
        q2 = rng.uniform(0.5, 30)
        mu0 = rng.uniform(-0.5, 0.5)
        sm = rng.choice([-1.0, 1.0])
        B = a * a - l * l - q2
        mp2 = 2 * q2 / (math.sqrt(B * B + 4 * a * a * q2) - B)
        if mu0 * mu0 >= mp2:
            continue
        # in Mino time the polar motion does not depend on the radial one
        rc, s = oracle.geokerr_stream(1e-3, 0.5, mu0, a, l, q2, 0.0, 0.02, 200)
        if rc != 0:
            continue
        # keep the samples before the ray reaches the horizon (u stops moving)
        live = np.ones(len(s["u"]), bool)
        stop = np.flatnonzero(np.diff(s["u"]) == 0.0)
        if len(stop):
            live[stop[0] + 1:] = False
        if live.sum() < 15:
            continue
        # geokerr_stream's dmu/dlambda starts negative for mu0 > 0
        sm_stream = -1.0 if mu0 > 0 else 1.0
        mu = carlson.mu_of_lambda(a, l, q2, mu0, sm_stream, s["affine"][live], device=False)
        assert np.allclose(mu, s["mu"][live], atol=1e-10), (a, l, q2, mu0, np.abs(mu - s["mu"][live]).max())
        done += 1
    assert done >= 20


@pytest.mark.parametrize("spin,theta", [(0.9, 80.0), (0.998, 60.0), (0.3, 20.0)])
def test_closed_form_crossings_match_taylor_solver(built, spin, theta):
    """Equatorial crossings in closed form (polar Jacobi motion + inverted
    radial Carlson integral) against the Mino-time Taylor solver on the
    renderer's own camera rays: same crossing counts, u within 1e-11."""
    import nullpath_gb300 as npx
    from nullpath_gb300 import geokerr as gk
    sc = npx.benchmark_scene(width=64, height=36, spp=1, spin=spin).replace(theta_deg=theta)
    rng = np.random.default_rng(3)
    px, py = rng.uniform(0, 64, 200), rng.uniform(0, 36, 200)
    ref = oracle.trace_rays(sc, px, py)
    u0, mu0, l, q2, su, sm = gk.render_ray_constants(ref["consts"], sc)
    u_end = 1.0 / sc.escape_r
    xu, nx = carlson.equator_crossings_cf(spin, u0, mu0, l, q2, su, sm, u_end, 4)
    agree = 0
    for i in range(len(px)):
        n, tx, _ = oracle.geokerr_crossings(u0[i], mu0[i], spin, l[i], q2[i], su[i], sm[i], u_end, 4)
        if n == nx[i]:
            agree += 1
            k = max(n, 0)
            assert np.allclose(xu[i][:k], tx[:k], rtol=1e-11, atol=0), (i, xu[i][:k], tx[:k])
    assert agree >= 0.99 * len(px)
