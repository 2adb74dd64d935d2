"""High-precision restatement of GEOKERR's sampled points in closed form
(test infrastructure: generates truth vectors for tests/golden; never
imported by the library).

The reference computes t and phi along a geodesic semi-analytically with
Carlson's integrals (GEOPHITIME, geokerr_port/reference/geokerr_original.f:
1648-2360, with GEOR/GEOMU for u and mu, :771-1187, 2672-3136).  This module
evaluates the same integrals independently, in mpmath at 40 digits, by
Legendre reduction:

* radial motion in [u1, u2] between real roots of U(u) = 1 + B u^2 + 2 K u^3
  - a^2 q2 u^4; with four real roots the Legendre variable
  S = (u3 - u1)(u2 - u) / ((u2 - u1)(u3 - u)) (Byrd & Friedman 256.00 from
  u2), with two real roots and a complex pair the half argument of Byrd &
  Friedman 259.00's cn-substitution;
* polar motion mu = mu+ cn(omega lambda - s_mu F0 | k) (q2 > 0);
* t, phi and the affine parameter from the partial fractions of their
  right-hand sides (1, 1/u, 1/u^2, 1/(1 - r+- u), mu^2, 1/(1 - mu^2)),
  each a combination of F, E, Pi(n) and the integral of 1/(1 - n sin^2)^2
  (DLMF 19.25), with mpmath's elliprf / elliprd / elliprj / elliprc;
* the GEOKERR sampling rules (geokerr_original.f:357-605): nup points
  uniform in u from u0 to the radial turning point and back.

Rays with q2 <= 0, a = 0 or other root structures are not covered (None).
"""
import mpmath as mp

mp.mp.dps = 40


def _rc(x, y):
    """R_C with the principal value for y < 0 (DLMF 19.6.16 / 19.2.20)."""
    if y > 0:
        return mp.re(mp.elliprc(x, y))
    return mp.re(mp.sqrt(x / (x - y)) * mp.elliprc(x - y, -y))


def _rj(x, y, z, p):
    """R_J, principal value for p < 0 (DLMF 19.20.14)."""
    if p > 0:
        return mp.elliprj(x, y, z, p)
    q = y + (z - y) * (y - x) / (y - p)
    return ((q - y) * mp.elliprj(x, y, z, q) - 3 * mp.elliprf(x, y, z) +
            3 * mp.sqrt(x * y * z / (x * z + p * q)) * _rc(x * z + p * q, p * q)) / (y - p)


class Amp:
    """Legendre integrals at amplitude phi, S = sin^2 phi, C = cos^2 phi."""

    def __init__(self, S, C, m):
        self.S, self.C, self.m = S, C, m
        self.s = mp.sqrt(S)
        self.D2 = 1 - m * S
        self.F = self.s * mp.elliprf(C, self.D2, 1) if S > 0 else mp.mpf(0)
        self.Sd = self.s ** 3 / 3 * mp.elliprd(C, self.D2, 1) if S > 0 else mp.mpf(0)

    def Pi(self, n):
        """int_0^phi dtheta / ((1 - n sin^2) Delta); principal value past a pole."""
        S, C, m, s = self.S, self.C, self.m, self.s
        if S == 0:
            return mp.mpf(0)
        p = 1 - n * S
        if p > 0:
            return self.F + n * s ** 3 / 3 * _rj(C, self.D2, 1, p)
        nn = m / n      # DLMF 19.7.8
        pim = self.F + nn * s ** 3 / 3 * _rj(C, self.D2, 1, 1 - nn * S)
        return self.F + s * _rc(C * self.D2, p * (1 - nn * S)) - pim

    def Pi2(self, n):
        """int_0^phi dtheta / ((1 - n sin^2)^2 Delta), from d/dphi of
        s c d / (1 - n s^2)."""
        S, C, m, s = self.S, self.C, self.m, self.s
        if S == 0:
            return mp.mpf(0)
        V = s * mp.sqrt(C) * mp.sqrt(self.D2) / (1 - n * S)
        al = 2 * (n - 1) * (n - m) / n ** 2
        be = (2 + 2 * m - n - 3 * m / n) / n
        return (V - be * self.Pi(n) - m / n ** 2 * self.F + m / n * self.Sd) / al


class _R4:
    """Four real roots; S = 0 at u2; integrals from u to u2."""

    def __init__(self, c4, u1, u2, u3, u4):
        self.u1, self.u2, self.u3 = u1, u2, u3
        self.m = (u2 - u1) * (u4 - u3) / ((u3 - u1) * (u4 - u2))
        self.g = 2 / mp.sqrt(abs(c4) * (u3 - u1) * (u4 - u2))

    def G(self, u, poles):
        """Integrals increasing in u: minus int_u^{u2} f du / sqrt(U) for
        f = 1, 1/u^2 and 1/(u - p)."""
        u1, u2, u3 = self.u1, self.u2, self.u3
        den = (u2 - u1) * (u3 - u)
        A = Amp((u3 - u1) * (u2 - u) / den, (u - u1) * (u3 - u2) / den, self.m)
        out = [-self.g * A.F]
        for p in poles:
            # 1/(u - p) = 1/(u3 - p) + C_p / (1 - n_p S)
            n = (u3 - p) * (u2 - u1) / ((u2 - p) * (u3 - u1))
            Cp = (u3 - u2) / ((u3 - p) * (u2 - p))
            out.append(-self.g * (A.F / (u3 - p) + Cp * A.Pi(n)))
        n = u3 * (u2 - u1) / (u2 * (u3 - u1))
        a_, b_ = 1 / u3, (u3 - u2) / (u3 * u2)
        out.insert(1, -self.g * (a_ * a_ * A.F + 2 * a_ * b_ * A.Pi(n) + b_ * b_ * A.Pi2(n)))
        return out


class _R2C:
    """Two real roots and a complex pair; S = sn^2(w/2) with cn w = X(u)."""

    def __init__(self, c4, u1, u2, rho, sig):
        self.u1, self.u2 = u1, u2
        self.A = mp.sqrt((u2 - rho) ** 2 + sig ** 2)
        self.B = mp.sqrt((u1 - rho) ** 2 + sig ** 2)
        self.m = ((u2 - u1) ** 2 - (self.A - self.B) ** 2) / (4 * self.A * self.B)
        self.g = 2 / mp.sqrt(abs(c4) * self.A * self.B)

    def _pf(self, p):
        """1/(u - p) = cinf + sum_j al_j / (1 - n_j S)."""
        u1, u2, A, B, m = self.u1, self.u2, self.A, self.B, self.m
        a0, a1, a2 = (u1 - p) * A, -(A * (u1 - p) - B * (u2 - p)), -m * B * (u2 - p)
        disc = mp.sqrt(a1 * a1 - 4 * a0 * a2)
        n1, n2 = (-a1 + disc) / (2 * a0), (-a1 - disc) / (2 * a0)
        D = lambda S: A - (A - B) * S - m * B * S * S
        al1 = D(1 / n1) / (a0 * (1 - n2 / n1))
        al2 = D(1 / n2) / (a0 * (1 - n1 / n2))
        return 1 / (u2 - p), (n1, al1), (n2, al2)

    def G(self, u, poles):
        """int_{u1}^u f du / sqrt(U) for f = 1, 1/u^2, 1/(u - p)."""
        u1, u2, A, B, m = self.u1, self.u2, self.A, self.B, self.m
        den = (u2 - u) * B + (u - u1) * A
        X = ((u2 - u) * B - (u - u1) * A) / den
        dnw = mp.sqrt(1 - m + m * X * X)
        Am = Amp((1 - X) / (1 + dnw), (X + dnw) / (1 + dnw), m)
        out = [self.g * Am.F]
        for p in poles:
            cinf, (n1, al1), (n2, al2) = self._pf(p)
            out.append(self.g * (cinf * Am.F + al1 * Am.Pi(n1) + al2 * Am.Pi(n2)))
        cinf, (n1, al1), (n2, al2) = self._pf(mp.mpf(0))
        t1, t2 = Am.Pi(n1), Am.Pi(n2)
        sq = (cinf ** 2 * Am.F + 2 * cinf * (al1 * t1 + al2 * t2) + 2 * al1 * al2 * (n1 * t1 - n2 * t2) / (n1 - n2) +
              al1 ** 2 * Am.Pi2(n1) + al2 ** 2 * Am.Pi2(n2))
        out.insert(1, self.g * sq)
        return out


def _polar_roots(a, l, q2, mu0):
    """GEOKERR's polar roots in mu^2 with its moved-root rule
    (geokerr_original.f:1121-1170)."""
    a2 = a * a
    b = a2 - (q2 + l * l)
    yy = -(b + (1 if b >= 0 else -1) * mp.sqrt(b * b + 4 * q2 * a2)) / 2
    if b < 0:
        a2mneg, mpos = -yy, q2 / yy
    else:
        a2mneg, mpos = a2 * q2 / yy, -yy / a2
    mpos = min(mpos, mp.mpf(1))
    if a2mneg < 0 or a2 == 0:
        if mp.sqrt(mpos) < mu0:
            mpos = mu0 * mu0
    else:
        if a2mneg > a2 * mu0 * mu0:
            a2mneg = a2 * mu0 * mu0
        if mu0 * mu0 > mpos:
            mpos = mu0 * mu0
    return mpos, a2mneg


def points(u0, uf, mu0, a, l, q2, su, sm, tpr=1, nup=32, offset=0.5):
    """GEOKERR points of one ray (floats in, mpf lists out) or None when the
    ray is outside the closed forms."""
    a, l, q2, u0, uf, mu0 = (mp.mpf(x) for x in (a, l, q2, u0, uf, mu0))
    if not (q2 > 0) or a == 0:
        return None
    Bc, Kc = a * a - l * l - q2, (l - a) ** 2 + q2
    c = [mp.mpf(1), mp.mpf(0), Bc, 2 * Kc, -a * a * q2]
    roots = mp.polyroots(c[::-1], maxsteps=400, extraprec=400)
    real = sorted(mp.re(r) for r in roots if abs(mp.im(r)) < mp.mpf(10) ** -30)
    cplx = [r for r in roots if mp.im(r) > mp.mpf(10) ** -30]
    sq = mp.sqrt(1 - a * a)
    rp, rm = 1 + sq, a * a / (1 + sq)
    uplus = 1 / rp
    poles = [mp.mpf(0), 1 / rp, 1 / rm]
    if len(real) == 4:
        u1, u2 = real[0], real[1]
        rad, top = _R4(c[4], *real), None
    elif len(real) == 2 and len(cplx) == 1:
        u1, u2 = real
        rad = _R2C(c[4], u1, u2, mp.re(cplx[0]), mp.im(cplx[0]))
        top = rad.G(u2, poles)
    else:
        return None
    if not (u1 < u0 <= u2):
        return None
    mpos, a2mneg = _polar_roots(a, l, q2, mu0)
    if not (a2mneg < 0):
        return None
    if su > 0 and u2 < uplus:
        ub, tp = u2, tpr
    else:
        ub, tp = (uplus if su > 0 else mp.mpf(0)), 0
    if top is None:
        top = [mp.mpf(0)] * 5
    UF = uf
    if tp == 1 and ((su > 0 and UF > ub) or (su < 0 and UF < ub)):
        UF = ub
    if tp == 1 and UF == ub:
        UF = u0
    du = (1 if ub - u0 >= 0 else -1) * su * ((ub - u0) + (2 * tp - 1) * (ub - UF)) / nup
    kmax = 0 if du == 0 else min(int(mp.floor((ub - u0) / du + offset)), nup)
    last = max(0, nup if tp == 1 else min(kmax, nup))
    if last > 0:
        kk = min(last, kmax)
        if (su > 0 and kk >= 1 and not (u0 + (kk - offset) * du < uplus)) or \
                (su < 0 and not (u0 + (last - offset) * du > 0)):
            last = 0
    # polar: mu = mu+ cn(omega lambda + w0)
    mp_ = mp.sqrt(mpos)
    om = mp.sqrt(a * a * mpos - a2mneg)
    mth = a * a * mpos / (om * om)
    Kth = mp.ellipk(mth)
    c0 = max(mp.mpf(-1), min(mp.mpf(1), mu0 / mp_))
    F0 = mp.ellipf(mp.acos(c0), mth)
    w0 = -(1 if sm >= 0 else -1) * F0
    nth = -mpos / (1 - mpos)

    Acomp = Amp(mp.mpf(1), mp.mpf(0), mth)

    def Phi(w):
        """(int_0^w mu^2 dw', int_0^w dw' / (1 - mu^2)), mu = mu+ cn w'."""
        j = mp.floor(w / (2 * Kth) + mp.mpf(1) / 2)
        r = w - 2 * j * Kth
        sn, cn = mp.ellipfun('sn', abs(r), m=mth), mp.ellipfun('cn', abs(r), m=mth)
        A = Amp(sn * sn, cn * cn, mth)
        sg = 1 if r >= 0 else -1
        mu2 = 2 * j * mpos * (Acomp.F - Acomp.Sd) + sg * mpos * (A.F - A.Sd)
        inv = 2 * j * Acomp.Pi(nth) / (1 - mpos) + sg * A.Pi(nth) / (1 - mpos)
        return mu2, inv
    Ph0 = Phi(w0)
    G0 = rad.G(u0, poles)
    cp = 2 * (2 * rp - a * l) / (rp - rm)
    cm = 2 * (2 * rm - a * l) / (rm - rp)
    dp = a * (2 * rp - a * l) / (rp * (rp - rm))
    dm = a * (2 * rm - a * l) / (rm * (rm - rp))
    out = {k: [] for k in ("u", "mu", "dt", "dphi", "lam", "tpm", "tpr")}
    for k in range(1, last + 1):
        branch2 = k > kmax
        ut = 2 * ub - (u0 + (k - offset) * du) if branch2 else u0 + (k - offset) * du
        Gk = rad.G(ut, poles)
        if su > 0:
            I = [2 * t - g0 - gk if branch2 else gk - g0 for t, g0, gk in zip(top, G0, Gk)]
        else:
            I = [g0 - gk for g0, gk in zip(G0, Gk)]
        lam = I[0]
        w = om * lam + w0
        mu2, inv = Phi(w)
        Imu2, Iinv = (mu2 - Ph0[0]) / om, (inv - Ph0[1]) / om
        Ip, Im = -I[3] / rp, -I[4] / rm
        out["u"].append(ut)
        out["mu"].append(mp_ * mp.ellipfun('cn', w, m=mth))
        out["dt"].append(I[1] + 2 * I[2] + cp * Ip + cm * Im + a * a * Imu2)
        out["dphi"].append(dp * Ip + dm * Im - l * lam + l * Iinv)
        out["lam"].append(I[1] + a * a * Imu2)
        out["tpm"].append(int(mp.floor(w / (2 * Kth)) - mp.floor(w0 / (2 * Kth))))
        out["tpr"].append(1 if branch2 else 0)
    return out


def points_vortical(u0, uf, mu0, a, l, q2, su, sm, tpr=1, nup=32, offset=0.5):
    """Truth for q2 < 0 (vortical) rays, independent of any Legendre
    reduction: the polar motion mu = s0 mu+ dn(a mu+ lambda + w0 | k) with
    mpmath's Jacobi functions (Byrd & Friedman 218.00), the polar integrals
    by quadrature in w, and the radial integrals by quadrature in u (these
    rays meet no radial turning point: U > 0 from u0 to the horizon).
    Returns None outside that case."""
    a, l, q2, u0, uf, mu0 = (mp.mpf(x) for x in (a, l, q2, u0, uf, mu0))
    if not (q2 < 0) or a == 0 or mu0 == 0:
        return None
    Bc, Kc = a * a - l * l - q2, (l - a) ** 2 + q2
    c = [mp.mpf(1), mp.mpf(0), Bc, 2 * Kc, -a * a * q2]
    U = lambda u: c[0] + c[2] * u ** 2 + c[3] * u ** 3 + c[4] * u ** 4
    roots = mp.polyroots(c[::-1], maxsteps=400, extraprec=400)
    if any(abs(mp.im(r)) < mp.mpf(10) ** -30 and mp.re(r) > 0 for r in roots):
        return None                      # a positive real root: not this case
    sq = mp.sqrt(1 - a * a)
    rp, rm = 1 + sq, a * a / (1 + sq)
    uplus = 1 / rp
    if su > 0:
        ub, tp = uplus, 0
    else:
        ub, tp = mp.mpf(0), 0
    du = (1 if ub - u0 >= 0 else -1) * su * ((ub - u0) - (ub - uf)) / nup
    kmax = 0 if du == 0 else min(int(mp.floor((ub - u0) / du + offset)), nup)
    last = max(0, min(kmax, nup))
    if last > 0 and ((su > 0 and not (u0 + (last - offset) * du < uplus)) or
                     (su < 0 and not (u0 + (last - offset) * du > 0))):
        last = 0
    mpos, a2mneg = _polar_roots(a, l, q2, mu0)
    if not (a2mneg > 0):
        return None
    mp_ = mp.sqrt(mpos)
    om = a * mp_
    mth = (a * a * mpos - a2mneg) / (a * a * mpos)
    s0 = 1 if mu0 > 0 else -1
    # dn(w0) = |mu0| / mu+; d mu / d lambda = -s0 mu+ k^2 sn cn omega
    S0 = (a * a * mpos - a * a * mu0 * mu0) / (a * a * mpos - a2mneg)
    F0 = mp.ellipf(mp.asin(mp.sqrt(max(mp.mpf(0), min(mp.mpf(1), S0)))), mth)
    w0 = F0 if sm * s0 < 0 else -F0
    Kth = mp.ellipk(mth)
    dn = lambda w: mp.ellipfun('dn', w, m=mth)

    def wquad(f, wa, wb):
        pts = [wa] + [mp.mpf(k) * Kth for k in range(int(mp.floor(min(wa, wb) / Kth)) + 1,
                                                     int(mp.floor(max(wa, wb) / Kth)) + 1)] + [wb]
        pts = sorted(set(pts))
        v = mp.quad(f, pts)
        return v if wb >= wa else -v

    def uquad(f, ua, ub_):
        lo, hi = min(ua, ub_), max(ua, ub_)
        pts = [lo]
        x = lo
        while x * 10 < hi:
            x = x * 10
            pts.append(x)
        pts.append(hi)
        return mp.quad(lambda x: f(x) / mp.sqrt(U(x)), pts)

    cp = 2 * (2 * rp - a * l) / (rp - rm)
    cm = 2 * (2 * rm - a * l) / (rm - rp)
    dp = a * (2 * rp - a * l) / (rp * (rp - rm))
    dm = a * (2 * rm - a * l) / (rm * (rm - rp))
    out = {k: [] for k in ("u", "mu", "dt", "dphi", "lam", "tpm", "tpr")}
    for k in range(1, last + 1):
        ut = u0 + (k - offset) * du
        lam = uquad(lambda x: 1, u0, ut)
        i2 = uquad(lambda x: 1 / (x * x), u0, ut)
        i1 = uquad(lambda x: 1 / x, u0, ut)
        ip = uquad(lambda x: 1 / (1 - rp * x), u0, ut)
        im = uquad(lambda x: 1 / (1 - rm * x), u0, ut)
        w = om * lam + w0
        mu2 = wquad(lambda v: mpos * dn(v) ** 2, w0, w) / om
        inv = wquad(lambda v: 1 / (1 - mpos * dn(v) ** 2), w0, w) / om
        out["u"].append(ut)
        out["mu"].append(s0 * mp_ * dn(w))
        out["dt"].append(i2 + 2 * i1 + cp * ip + cm * im + a * a * mu2)
        out["dphi"].append(dp * ip + dm * im - l * lam + l * inv)
        out["lam"].append(i2 + a * a * mu2)
        out["tpm"].append(int(mp.floor(w / Kth) - mp.floor(w0 / Kth)))
        out["tpr"].append(0)
    return out


def crossings(u0, mu0, a, l, q2, su, sm, u_far, K=6, guess=None):
    """Truth for the equatorial crossings of a q2 > 0 ray, independent of the
    Legendre reductions: the Mino times lambda_j = ((2j + 1) K(k) - w0) /
    omega of mu = mu+ cn(omega lambda + w0 | k) with mpmath's elliptic
    functions; the radial Mino time lambda(u) = int du / sqrt(U) by
    quadrature (u = u2 - t^2 near the turning point u2, breakpoints
    geometric towards it), inverted at each lambda_j by Newton steps
    (dlambda/du = 1/sqrt(U)) from `guess` (a list of u, one per crossing)
    or from bisection; the azimuth change
    dphi = d+ Ip + d- Im - l lambda + l int dw / (1 - mu^2) / omega by the same
    quadratures.  The ray ends at the horizon (ingoing, no turning point
    outside it) or at u_far after its turning point.  Returns
    (status, [u_j], [dphi_j]) for the first K crossings (status 0: leaves,
    1: captured), or None outside this case."""
    a, l, q2, u0, mu0, u_far = (mp.mpf(x) for x in (a, l, q2, u0, mu0, u_far))
    if not (q2 > 0) or a == 0:
        return None
    Bc, Kc = a * a - l * l - q2, (l - a) ** 2 + q2
    c = [mp.mpf(1), mp.mpf(0), Bc, 2 * Kc, -a * a * q2]
    U = lambda u: c[0] + c[2] * u ** 2 + c[3] * u ** 3 + c[4] * u ** 4
    roots = mp.polyroots(c[::-1], maxsteps=400, extraprec=400)
    real = sorted(mp.re(r) for r in roots if abs(mp.im(r)) < mp.mpf(10) ** -30)
    above = [r for r in real if r >= u0]
    below = [r for r in real if r < u0]
    if not below:
        return None
    u2 = above[0] if above else mp.inf
    sq = mp.sqrt(1 - a * a)
    rp, rm = 1 + sq, a * a / (1 + sq)
    uplus = 1 / rp
    turns = su > 0 and u2 < uplus
    # the nearest complex root or the second real root bounds the peak of
    # 1/sqrt(U) at u2: breakpoints geometric in the distance to u2
    near = [abs(r - u2) for r in roots if abs(r - u2) > mp.mpf(10) ** -30] if turns else []
    width = min(near) if near else mp.mpf(1)
    # U(u) = (u - u2) Q(u), Q by synthetic division
    b3 = c[4]
    b2 = c[3] + u2 * b3 if turns else 0
    b1 = c[2] + u2 * b2 if turns else 0
    b0 = c[1] + u2 * b1 if turns else 0
    Q = lambda u: ((b3 * u + b2) * u + b1) * u + b0

    cplx = [r for r in roots if mp.im(r) > mp.mpf(10) ** -30]

    def open_int(f, ua, ub):
        """int_ua^ub f(u) du / sqrt(U) away from real roots: breakpoints
        geometric towards the real part of a complex pair inside the range
        (1/sqrt(U) peaks there with width of its imaginary part)."""
        pts = [ua, ub]
        for z in cplx:
            rho, sig = mp.re(z), mp.im(z)
            if ua < rho < ub:
                pts.append(rho)
                s = sig / 4
                while rho - s > ua or rho + s < ub:
                    for x in (rho - s, rho + s):
                        if ua < x < ub:
                            pts.append(x)
                    s *= 4
        return mp.quad(lambda x: f(x) / mp.sqrt(U(x)), sorted(set(pts)))

    def lam_int(f, ua, ub):
        """int_ua^ub f(u) du / sqrt(U), ua <= ub <= u2."""
        if ub <= ua:
            return mp.mpf(0)
        if not turns:
            return open_int(f, ua, ub)
        # u = u2 - t^2 removes the square-root zero of U = (u - u2) Q(u) at u2
        ta, tb = mp.sqrt(u2 - ub), mp.sqrt(u2 - ua)
        g = lambda t: 2 * f(u2 - t * t) / mp.sqrt(-Q(u2 - t * t))
        pts = [ta]
        s = mp.sqrt(width) / 4
        while s < tb:
            if s > ta:
                pts.append(s)
            s *= 4
        pts.append(tb)
        return mp.quad(g, pts)

    one = lambda x: mp.mpf(1)
    fp = lambda x: 1 / (1 - rp * x)
    fm = lambda x: 1 / (1 - rm * x)
    if su > 0:
        if turns:
            lam_t = lam_int(one, u0, u2)
            lam_end = lam_t + lam_int(one, u_far, u2)
            status = 0
        else:
            lam_t = None
            lam_end = open_int(one, u0, uplus)
            status = 1
    else:
        lam_t, status = None, 0
        lam_end = open_int(one, u_far, u0)
    # polar motion
    mpos, a2mneg = _polar_roots(a, l, q2, mu0)
    mp_ = mp.sqrt(mpos)
    om = mp.sqrt(a * a * mpos - a2mneg)
    mth = a * a * mpos / (om * om)
    Kth = mp.ellipk(mth)
    c0 = max(mp.mpf(-1), min(mp.mpf(1), mu0 / mp_))
    w0 = -(1 if sm >= 0 else -1) * mp.ellipf(mp.acos(c0), mth)
    cn = lambda w: mp.ellipfun('cn', w, m=mth)

    def lam_of(u, out):
        """Mino time at u on the branch before (out = False) or after the
        turning point, and its derivative in u."""
        if su > 0 and not out:
            return lam_int(one, u0, u)
        if su > 0:
            return lam_t + lam_int(one, u, u2)
        return open_int(one, u, u0)

    xs, phis = [], []
    j = -2
    while len(xs) < K and j < 256:
        lam = ((2 * j + 1) * Kth - w0) / om
        j += 1
        if not (lam > 0):
            continue
        if not (lam < lam_end):
            break
        out = turns and lam > lam_t
        lo, hi = ((u0, u2) if not out else (u_far, u2)) if su > 0 and turns else \
            ((u0, uplus) if su > 0 else (u_far, u0))
        sgn = 1 if (su > 0 and not out) else -1          # dlambda/du sign
        u = mp.mpf(guess[len(xs)]) if guess is not None and len(xs) < len(guess) else (lo + hi) / 2
        for _ in range(60):
            f = lam_of(u, out) - lam
            if (f > 0) == (sgn > 0):
                hi = u
            else:
                lo = u
            un = u - sgn * f * mp.sqrt(U(u))
            if not (lo < un < hi):
                un = (lo + hi) / 2
            done = abs(un - u) < mp.mpf(10) ** -32 * abs(u)
            u = un
            if done:
                break
        xs.append(u)
        # azimuth: radial parts by quadrature along the path, polar by quadrature in w
        if su > 0 and not out and turns:
            ip, im = lam_int(fp, u0, u), lam_int(fm, u0, u)
        elif su > 0 and not out:
            ip, im = open_int(fp, u0, u), open_int(fm, u0, u)
        elif su > 0:
            ip = lam_int(fp, u0, u2) + lam_int(fp, u, u2)
            im = lam_int(fm, u0, u2) + lam_int(fm, u, u2)
        else:
            ip, im = open_int(fp, u, u0), open_int(fm, u, u0)
        w = om * lam + w0
        pts = sorted(set([w0] + [k * Kth for k in range(int(mp.floor(w0 / Kth)) + 1, int(mp.floor(w / Kth)) + 1)] +
                         [w]))
        inv = mp.quad(lambda v: 1 / (1 - mpos * cn(v) ** 2), pts) / om
        dp = a * (2 * rp - a * l) / (rp * (rp - rm))
        dm = a * (2 * rm - a * l) / (rm * (rm - rp))
        phis.append(dp * ip + dm * im - l * lam + l * inv)
    return status, xs, phis
