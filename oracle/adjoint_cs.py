"""Complex-step derivative of one sample of the differentiable render (test
infrastructure only: the GPU adjoint is checked against it; nothing in the
product imports this file).

The sample map is the FP64 path of the differentiable render restated in
plain Python: camera direction (stratified or wanghash jitter, render.cu:
145-154), static-observer or ZAMO camera momentum (bh_kerr.h:781-826,
910-967), Carter-form Kerr Hamiltonian right-hand side, RK4 with the step law
h = h0 clamp(r/M, 1, 100) (render.cu:185,207) times the polar-axis factor
sin(theta) / (sin(theta) + 0.05) of the differentiable render, equator crossings located on
the cubic Hermite interpolant of the step, and the disk colour sum
sum_k r_k^-q g_k^3 with the Keplerian redshift g (bh_kerr.h:833-862) over the
first `disk_max_orders` crossings inside [rin, rout] (render.cu:229-231).

Evaluating the map with one parameter moved by i*1e-30 carries the exact
derivative of the discrete map in the imaginary part (Squire & Trapp 1998,
"Using complex variables to estimate derivatives of real functions"): no
cancellation, so it holds where the map changes too fast in the parameter
for a finite difference (rays with L near 0 that pass close to the pole).
Pure-Python loops: a ray of ~1000 steps takes about a second.
"""
import cmath
import math

_M32 = 0xFFFFFFFF

# Width of the polar-axis factor sin(theta) / (sin(theta) + sigma) of the
# differentiable render's step law (csrc/adjoint.cu).
POLE_SIGMA = 0.05

def _mix32(x):
    x &= _M32
    x ^= x >> 16
    x = (x * 0x7FEB352D) & _M32
    x ^= x >> 15
    x = (x * 0x846CA68B) & _M32
    x ^= x >> 16
    return x


def _strat_unit(seed, pix, sample, dim):
    h = _mix32(_mix32(_mix32((seed + 0x9E3779B9 * (dim + 1)) & _M32) ^ pix) ^ ((sample * 0x85EBCA6B) & _M32))
    return (h >> 8) * (1.0 / 16777216.0)


def _wang_unit(v):
    v &= _M32
    v = (v ^ 61) ^ (v >> 16)
    v = (v * 9) & _M32
    v ^= v >> 4
    v = (v * 0x27D4EB2D) & _M32
    v ^= v >> 15
    import numpy as np
    return float(np.float32(v & 0x00FFFFFF) * np.float32(1.0 / 16777216.0))


def _re(x):
    return x.real if isinstance(x, complex) else x


def _sqrt(x):
    return cmath.sqrt(x) if isinstance(x, complex) else math.sqrt(x)


def _sin(x):
    return cmath.sin(x) if isinstance(x, complex) else math.sin(x)


def _cos(x):
    return cmath.cos(x) if isinstance(x, complex) else math.cos(x)


def direction(sc, x, y, sl):
    """Local camera direction (n_r, n_theta, n_phi) of sample `sl` of pixel
    (x, y), in double as the lengths-in-M path computes it."""
    W, H = sc["width"], sc["height"]
    sample = sc["sample_offset"] + sl
    if sc["jitter"] == 0:
        import numpy as np
        jx = float(np.float32(_wang_unit(x * 73856093 ^ y * 19349663 ^ sample * 83492791)) - np.float32(0.5))
        jy = float(np.float32(_wang_unit(x * 83492791 ^ y * 2654435761 ^ sample * 19349663)) - np.float32(0.5))
        px, py = x + 0.5 + jx, y + 0.5 + jy
    else:
        m = max(1, int(math.floor(math.sqrt(max(1, sc["spp"])))))
        pix = y * W + x
        c = sample % (m * m)
        px = x + ((c % m) + _strat_unit(sc["seed"], pix, sample, 0)) / m
        py = y + ((c // m) + _strat_unit(sc["seed"], pix, sample, 1)) / m
    th = math.tan(0.5 * sc["fov_y_deg"] * math.pi / 180.0)
    ndc_x = px / W * 2.0 - 1.0
    ndc_y = py / H * 2.0 - 1.0
    cx = ndc_x * (W / H) * th
    cy = -ndc_y * th
    nrm = 1.0 / math.sqrt(cx * cx + cy * cy + 1.0)
    return -nrm, cy * nrm, cx * nrm


def camera(M, a, r, th, nr, nth, nph, zamo):
    """Covariant photon momentum (p_t, p_r, p_theta, p_phi) at the camera."""
    sn, cs = _sin(th), _cos(th)
    s2, r2, a2 = sn * sn, r * r, a * a
    Sig = r2 + a2 * cs * cs
    Del = r2 - 2 * M * r + a2
    A = (r2 + a2) ** 2 - a2 * Del * s2
    gtt = -(1 - 2 * M * r / Sig)
    gtp = -(2 * M * a * r * s2 / Sig)
    gpp = A * s2 / Sig
    grr = Sig / Del
    ghh = Sig
    if not zamo:
        ut = 1 / _sqrt(-gtt)
        er, eh = 1 / _sqrt(grr), 1 / _sqrt(ghh)
        if abs(_re(gtp)) > 1e-12:
            beta = -gtt / gtp
            n2 = gtt + 2 * gtp * beta + gpp * beta * beta
            inv = 1 / _sqrt(-n2 if _re(n2) < 0 else n2)
            ept, epp = inv, beta * inv
        else:
            ept, epp = 0.0, 1 / _sqrt(gpp)
        Pt, Pr, Ph, Pp = ut + nph * ept, nr * er, nth * eh, nph * epp
    else:
        alpha = _sqrt(Del * Sig / A)
        omega = 2 * M * a * r / A
        Pt = 1 / alpha
        Pp = omega / alpha + nph * _sqrt(Sig / A) / (-sn if _re(sn) < 0 else sn)
        Pr = nr * _sqrt(Del / Sig)
        Ph = nth / _sqrt(Sig)
    return gtt * Pt + gtp * Pp, grr * Pr, ghh * Ph, gtp * Pt + gpp * Pp


def rhs(y, E, L, a, M):
    """d(r, theta, p_r, p_theta)/dlambda of 2 Sigma H = Delta p_r^2 + p_theta^2
    - P^2/Delta + L^2/sin^2 - 2 a E L + a^2 E^2 sin^2, P = (r^2+a^2)E - aL."""
    r, t, pr, pth = y
    sn, cs = _sin(t), _cos(t)
    s2 = sn * sn
    is2 = 1 / s2
    A = a * a
    Sig = r * r + A * cs * cs
    iS = 1 / Sig
    Del = r * r - 2 * M * r + A
    P = (r * r + A) * E - a * L
    PiD = P * (1 / Del)
    Wt = L * L * is2 + A * E * E * s2 - 2 * a * E * L
    F = Del * pr * pr + pth * pth - P * PiD + Wt
    Fr = 2 * (r - M) * (pr * pr + PiD * PiD) - 4 * r * E * PiD
    sc2 = 2 * sn * cs
    Ft = sc2 * (A * E * E - L * L * is2 * is2)
    return (Del * pr * iS, pth * iS, -0.5 * iS * (Fr - 2 * r * iS * F), -0.5 * iS * (Ft + A * sc2 * iS * F))


def _axpy(y, h, k):
    return tuple(y[i] + h * k[i] for i in range(4))


def _rk4(y, E, L, a, M, h):
    k1 = rhs(y, E, L, a, M)
    k2 = rhs(_axpy(y, 0.5 * h, k1), E, L, a, M)
    k3 = rhs(_axpy(y, 0.5 * h, k2), E, L, a, M)
    k4 = rhs(_axpy(y, h, k3), E, L, a, M)
    h6 = h / 6
    return tuple(y[i] + h6 * (k1[i] + 2 * (k2[i] + k3[i]) + k4[i]) for i in range(4))


def _herm_root(d0, d1, m0, m1):
    s = abs(_re(d0)) / (abs(_re(d0)) + abs(_re(d1)) + 1e-30)
    lo, hi = 0.0, 1.0
    for _ in range(30):
        s2 = s * s
        s3 = s2 * s
        p = (2 * s3 - 3 * s2 + 1) * d0 + (s3 - 2 * s2 + s) * m0 + (3 * s2 - 2 * s3) * d1 + (s3 - s2) * m1
        dp = (6 * s2 - 6 * s) * (d0 - d1) + (3 * s2 - 4 * s + 1) * m0 + (3 * s2 - 2 * s) * m1
        if (_re(p) > 0) == (_re(d0) > 0):
            lo = _re(s)
        else:
            hi = _re(s)
        sn = s - p / dp if _re(dp) != 0 else 0.5 * (lo + hi)
        if not (lo < _re(sn) < hi):
            sn = 0.5 * (lo + hi)
        done = abs(_re(sn) - _re(s)) < 1e-15
        s = sn
        if done:
            break
    return s


def _doppler(r, E, L, a, M):
    x = r / M
    Om = 1 / ((a / M + x * _sqrt(x)) * M)
    ir = 1 / r
    gtt = -(1 - 2 * M * ir)
    gtp = -2 * M * a * ir
    gpp = r * r + a * a + 2 * M * a * a * ir
    den = -(gtt + 2 * gtp * Om + gpp * Om * Om)
    return E * _sqrt(den) / (E - Om * L)


def trace(sc, a, th_cam, q, x, y, sl):
    """One sample: (status, orders, steps, disk_sum) with status 0 escaped,
    1 captured, 2 step budget spent; any of a, th_cam, q may be complex."""
    M = sc["mass"]
    r_cam = sc["r_cam"] * M
    rin = sc["disk_rin"] if sc["disk_rin"] > 0 else 6.0 * M
    rout = sc["disk_rout"] if sc["disk_rout"] > 0 else 40.0 * M
    r_far = sc["escape_r"] if sc["escape_r"] > 0 else r_cam + 20.0 * M
    h0 = sc["step_scale"]
    max_orders = max(1, sc["disk_max_orders"])
    gtt0 = -(1.0 - 2.0 * M * r_cam / (r_cam ** 2 + _re(a) ** 2 * math.cos(_re(th_cam)) ** 2))
    zamo = sc["camera"] == 1 or not (gtt0 < 0.0)
    nr, nth, nph = direction(sc, x, y, sl)
    pt, pr, pth, pph = camera(M, a, r_cam, th_cam, nr, nth, nph, zamo)
    E, L = -pt, pph
    yv = (r_cam, th_cam, pr, pth)
    f0 = rhs(yv, E, L, a, M)
    rp = M + math.sqrt(max(0.0, M * M - _re(a) ** 2))
    hp = math.pi / 2
    orders, disk = 0, 0.0
    for n in range(sc["max_steps"]):
        xr = yv[0] / M
        h = h0 if _re(xr) <= 1 else (h0 * 100 if _re(xr) >= 100 else h0 * xr)
        sn = _sin(yv[1])
        h = h * sn / (sn + POLE_SIGMA)          # the polar-axis factor of the differentiable step law
        y1 = _rk4(yv, E, L, a, M, h)
        if not (_re(y1[0]) > rp * 1.000001 and _re(y1[1]) > 1e-7 and _re(y1[1]) < 3.1415925):
            return 1, orders, n + 1, disk
        f1 = rhs(y1, E, L, a, M)
        d0, d1 = yv[1] - hp, y1[1] - hp
        if (_re(d0) > 0 > _re(d1)) or (_re(d0) < 0 < _re(d1)):
            u = _herm_root(d0, d1, h * f0[1], h * f1[1])
            u2 = u * u
            u3 = u2 * u
            rc = ((2 * u3 - 3 * u2 + 1) * yv[0] + (u3 - 2 * u2 + u) * h * f0[0] + (3 * u2 - 2 * u3) * y1[0]
                  + (u3 - u2) * h * f1[0])
            if orders < max_orders and rin <= _re(rc) <= rout:
                g = _doppler(rc, E, L, a, M)
                disk = disk + rc ** (-q) * g ** 3
                orders += 1
        yv, f0 = y1, f1
        if _re(yv[0]) > r_far and n + 1 > 11:
            return 0, orders, n + 1, disk
    return 2, orders, sc["max_steps"], disk


def sample_gradient(sc, index, weight=2.2):
    """Per-sample gradient of the loss with dLoss/dimage = 1 in every channel:
    weight = 1 + 0.75 + 0.45 (the disk colour's channel sum).  Returns
    (sig, [d/dspin, d/dtheta_cam, d/dgain, d/dq]) with sig = status + 4 orders,
    matching the per-sample output of the GPU adjoint."""
    W, H = sc["width"], sc["height"]
    sl, pix = divmod(index, W * H)
    y, x = divmod(pix, W)
    M = sc["mass"]
    a0 = sc["spin"] * M
    th0 = sc["theta_deg"] * math.pi / 180.0
    q0 = sc["emissivity_q"]
    status, orders, _, disk = trace(sc, a0, th0, q0, x, y, sl)
    sig = status + 4 * orders
    if status == 1 or orders == 0 or not sc["disk_on"]:
        return sig, [0.0, 0.0, 0.0, 0.0]
    eps = 1e-30
    B = weight / sc["spp"]
    gain = sc["disk_gain"]
    da = trace(sc, complex(a0, eps), th0, q0, x, y, sl)[3].imag / eps
    dth = trace(sc, a0, complex(th0, eps), q0, x, y, sl)[3].imag / eps
    dq = trace(sc, a0, th0, complex(q0, eps), x, y, sl)[3].imag / eps
    return sig, [gain * B * da * M, gain * B * dth, B * disk, gain * B * dq]


def scene_dict(scene):
    """Field dict of an np_scene_t ctypes structure."""
    return {f[0]: getattr(scene, f[0]) for f in scene._fields_}
