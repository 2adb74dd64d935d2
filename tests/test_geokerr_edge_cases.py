"""The GEOKERR restatement on the edge-case families of the reference's
GEOKERR test generator (geokerr_port/tests/comprehensive_test_suite.py:
118-196): near-extremal spins a = 0.999..0.99999 over impact parameters
0.01..10, starts just outside the horizon, impact parameters around the
critical value, weak-field (b up to 1000) and strong-field rays, all
equatorial (q2 = 0, mu = 0).  Every sample before the radial turning point
is checked against an independent adaptive quadrature of the equatorial
Mino-time integrals: affine lambda = int du / (u^2 sqrt(U)), t and phi the
same with dt/dlambda, dphi/dlambda (M = E = 1).  The generator ships no
expected outputs, so these are the reference's inputs with the physics as
the answer."""
import math

import numpy as np
import pytest

import oracle

quad = pytest.importorskip("scipy.integrate").quad


def edge_cases():
    """(family, a, b, r0, su): the generator's families, restated."""
    out = []
    for a in (0.999, 0.9999, 0.99999):                      # :123-133
        for b in np.logspace(-2, 1, 10):
            out.append(("near_extremal", a, float(b), 1000.0, 1))
    for a in (0.0, 0.5, 0.9):                               # :135-146, started outward
        rp = 1.0 + math.sqrt(1.0 - a * a)
        for f in (1.001, 1.01, 1.1):
            out.append(("near_horizon", a, 4.0, rp * f, -1))
    for a in (0.0, 0.3, 0.6, 0.9):                          # :148-159
        bc = 3.0 * math.sqrt(3.0) / 2.0 if a == 0 else 2.6 - 0.4 * a
        for f in (0.99, 1.0, 1.01):
            out.append(("critical", a, bc * f, 100.0, 1))
    for b in (50.0, 100.0, 500.0, 1000.0):                  # :174-183
        out.append(("weak_field", 0.9, b, 1000.0, 1))
    for b in (0.1, 0.5, 1.0):                               # :185-194
        out.append(("strong_field", 0.8, b, 100.0, 1))
    return out


def _integrals(a, l, u0, u):
    U = lambda x: 1.0 + (a * a - l * l) * x * x + 2.0 * (a - l) ** 2 * x ** 3
    Del = lambda x: 1.0 / (x * x) - 2.0 / x + a * a
    dt = lambda x: ((1.0 / (x * x) + a * a) * (1.0 / (x * x) + a * a - a * l) / Del(x) + a * l - a * a) / math.sqrt(U(x))
    dph = lambda x: (a * (1.0 / (x * x) + a * a - a * l) / Del(x) + l - a) / math.sqrt(U(x))
    lam = lambda x: 1.0 / (x * x * math.sqrt(U(x)))
    kw = dict(epsabs=0.0, epsrel=1e-13, limit=200)
    # dlambda_Mino = |du| / sqrt(U) along the ray, whichever way u runs
    lo, hi = (u0, u) if u > u0 else (u, u0)
    return [quad(f, lo, hi, **kw)[0] for f in (lam, dt, dph)]


@pytest.mark.parametrize("case", edge_cases(), ids=lambda c: "%s-a%g-b%.4g-r%.4g" % c[:4])
def test_equatorial_edge_case(built, case):
    fam, a, b, r0, su = case
    u0 = 1.0 / r0
    rp = 1.0 + math.sqrt(1.0 - a * a)
    uf = 1.0 / rp if su > 0 else 1e-4
    pts = oracle.geokerr_points(u0, uf, 0.0, a, b, 0.0, su, 1.0, tpr=1, nup=64, offset=0.5)
    n = pts["n"]
    if fam == "near_horizon" and a == 0.9 and n <= 0:
        # r0 = 1.1 r_+ at a = 0.9 with b = 4 lies where U(u) < 0: no null
        # geodesic starts there, and the sampler reports none
        U0 = 1.0 + (a * a - b * b) * u0 * u0 + 2.0 * (a - b) ** 2 * u0 ** 3
        assert U0 < 0.0
        return
    assert n == 64
    assert np.all(np.isfinite(pts["u"][:n]))
    pre = np.nonzero(pts["tpr"][:n] == 0)[0]
    assert pre.size >= 32
    # samples within a few steps of the turning point sit on the square-root
    # singularity of the quadrature; compare the ones before it
    du = abs(pts["u"][1] - pts["u"][0])
    turn = pts["tpr"][:n].max() > 0
    for k in pre[::4]:
        uk = pts["u"][k]
        if turn and abs(uk - pts["u"][pre[-1]]) < 3.0 * du:
            continue
        lam, dt, dph = _integrals(a, b, u0, uk)
        assert abs(pts["lam"][k] - lam) <= 1e-9 * abs(lam) + 1e-12, (k, pts["lam"][k], lam)
        assert abs(pts["dt"][k] - dt) <= 1e-8 * abs(dt) + 1e-10, (k, pts["dt"][k], dt)
        assert abs(pts["dphi"][k] - dph) <= 1e-8 * abs(dph) + 1e-10, (k, pts["dphi"][k], dph)


@pytest.mark.parametrize("a,b,r0,su", [(0.9, 50.0, 1000.0, 1), (0.5, 4.0, 20.0, -1), (0.998, 3.0, 100.0, 1),
                                        (0.0, 8.0, 50.0, 1)])
def test_final_state_matches_quadrature(built, a, b, r0, su):
    """The restatement's state at a given Mino time (the solver behind
    geokerr_cuda_batch): for an equatorial ray, the Mino time from u0 to the
    returned u, and t and phi there, agree with adaptive quadrature."""
    u0 = 1.0 / r0
    # outgoing rays reach u = 0 at Mino time ~u0, ingoing ones turn or fall in after ~1/b
    lam_total = 0.8 * u0 if su < 0 else 0.5 / b
    for frac in (0.25, 0.5, 1.0):
        lam = frac * lam_total
        ok, out = oracle.geokerr_final(u0, 0.0, a, b, 0.0, float(su), 1.0, lam)
        assert ok == 1 and abs(out[1]) < 1e-15
        U = lambda x: 1.0 + (a * a - b * b) * x * x + 2.0 * (a - b) ** 2 * x ** 3
        lo, hi = sorted((u0, out[0]))
        mino = quad(lambda x: 1.0 / math.sqrt(U(x)), lo, hi, epsabs=0.0, epsrel=1e-13, limit=200)[0]
        assert abs(mino - lam) <= 1e-10 * lam, (mino, lam)
        lam_aff, dt, dph = _integrals(a, b, u0, out[0])
        assert abs(out[2] - dt) <= 1e-8 * abs(dt) + 1e-10 and abs(out[3] - dph) <= 1e-8 * abs(dph) + 1e-10


def test_mino_time_round_trip(built):
    """The restatement of compute_mino_time_batch_cuda: the Mino time to
    uf, directly and after the radial turning point, brings the state at that
    time back to uf; the direct time matches quadrature of 1/sqrt(U)."""
    a, l, q2, u0, uf, mu0 = 0.7, 6.0, 12.0, 0.01, 0.05, 0.3
    ok0, lam0 = oracle.geokerr_mino_time(u0, uf, mu0, a, l, q2, 1.0, 1.0, False)
    ok1, lam1 = oracle.geokerr_mino_time(u0, uf, mu0, a, l, q2, 1.0, 1.0, True)
    assert ok0 == 1 and ok1 == 1 and lam1 > lam0 > 0.0
    for lam in (lam0, lam1):
        ok, out = oracle.geokerr_final(u0, mu0, a, l, q2, 1.0, 1.0, lam)
        assert ok == 1 and abs(out[0] - uf) <= 1e-12 * uf, (lam, out)
    U = lambda x: 1.0 + (a * a - q2 - l * l) * x * x + 2.0 * ((a - l) ** 2 + q2) * x ** 3 - a * a * q2 * x ** 4
    direct = quad(lambda x: 1.0 / math.sqrt(U(x)), u0, uf, epsabs=0.0, epsrel=1e-13)[0]
    assert abs(direct - lam0) <= 1e-11 * lam0
    # a ray that turns before uf never gets there directly; after the turn it escapes
    ok, _ = oracle.geokerr_mino_time(u0, 0.5, mu0, a, l, q2, 1.0, 1.0, False)
    assert ok == 0
