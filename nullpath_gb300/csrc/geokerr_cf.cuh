// geokerr_cf.cuh -- GEOKERR's sampled geodesic points in closed form: every
// (ray, sample) pair is evaluated on its own (the role of GEOR / GEOMU /
// GEOPHITIME, geokerr_original.f:771-1187, 1648-2360, 2672-3136), for host
// and device.
//
// With E = M = 1, u = 1/r, mu = cos(theta) and Mino time lambda, the motion
// separates (du/dlambda)^2 = U(u), (dmu/dlambda)^2 = M(mu), and
//   dt/dlambda     = 1/u^2 + 2/u + c+/(1 - r+ u) + c-/(1 - r- u) + a^2 mu^2
//   dphi/dlambda   = d+/(1 - r+ u) + d-/(1 - r- u) - l + l/(1 - mu^2)
//   daffine/dlambda = 1/u^2 + a^2 mu^2
// with r+- = 1 +- sqrt(1 - a^2), c+- = 2 (2 r+- - a l)/(r+- - r-+) and
// d+- = a (2 r+- - a l)/(r+- (r+- - r-+)): the partial fractions of the
// right-hand sides of the Taylor solver in geokerr.cu (the constant terms
// a^2 - a l of the t equation cancel).  Every radial term is then an integral
// of 1, 1/(u - p) or 1/u^2 against du/sqrt(U), and every polar term one of
// mu^2 or 1/(1 - mu^2) against dmu/sqrt(M).
//
// Radial, four real roots u1 < u2 < u3 < u4, motion in [u1, u2] (U has the
// sign of -a^2 q2 at infinity): the Legendre variable
//   S = sin^2(phi) = (u3 - u1)(u2 - u) / ((u2 - u1)(u3 - u)),  S = 0 at u2,
//   m = (u2 - u1)(u4 - u3) / ((u3 - u1)(u4 - u2)),
//   int_u^{u2} du / sqrt(U) = g F(phi | m),  g = 2 / sqrt(|c4| (u3 - u1)(u4 - u2))
// (the reduction of Byrd & Friedman 256.00 written from u2), and
//   1/(u - p) = 1/(u2 - p) + K_p S / (1 - n_p S),
//   n_p = (u3 - p)(u2 - u1) / ((u2 - p)(u3 - u1)),
//   K_p = (u3 - u2)(u2 - u1) / ((u2 - p)^2 (u3 - u1)),
//   1 - n_p S = (u - p)(u3 - u2) / ((u2 - p)(u3 - u))   (no cancellation).
// Radial, two real roots u1 < u2 and a complex pair rho +- i sigma: Byrd &
// Friedman 259.00 give cn(w) = X(u) with int_{u1}^u du/sqrt(U) = w /
// sqrt(|c4| A B); its half argument S = sn^2(w/2) = (1 - X)/(1 + dn w) is a
// monotone Legendre variable over all of [u1, u2], u is a ratio of quadratics
// in S, and 1/(u - p) splits into two terms 1/(1 - n_j S) with real n_j.
//
// Legendre integrals of the amplitude (S = sin^2 phi, C = cos^2 phi,
// Delta^2 = 1 - m S), all with Carlson's R-functions (DLMF 19.25):
//   F  = s R_F(C, Delta^2, 1),           Sd = int sin^2/Delta = s^3/3 R_D(C, Delta^2, 1)
//   J(n)  = int sin^2 / ((1 - n sin^2) Delta) = s^3/3 R_J(C, Delta^2, 1, 1 - n S)
//   Pi(n) = F + n J(n); for n < -1 from the R_J transformation DLMF 19.21.12
//           (p and q = y - (x - y)(z - y)/(p - y)), which keeps Pi accurate as
//           n -> -inf; past the pole (n > 1, 1 - n S < 0) the principal value
//           from Pi(n) + Pi(m/n) = F + s R_C(C Delta^2, (1 - n S)(1 - m S/n))
//           (DLMF 19.7.8)
//   Pi2(n) = int 1/((1 - n sin^2)^2 Delta), by differentiating
//           s c d / (1 - n S) and eliminating Pi in favour of J (no 1/n terms).
// Radial, q2 < 0: two real roots below the motion and a complex pair (Byrd &
// Friedman 260.00, the same half-argument algebra), or two complex pairs (a
// rotated form of B&F 267.00: u = rho1 + sigma1 tan(theta' + theta0), whose
// pole terms add odd parts integrated in closed form with R_C).
// Polar: mu = mu+ cn(omega lambda - s_mu F0 | k) for q2 > 0, and
// mu = s0 mu+ dn(omega lambda + w0 | k) for q2 < 0 (B&F 213.00, 218.00); the
// integrals over whole half periods are complete values, so each sample
// needs the amplitude of one reduced argument.
//
// Only +, -, *, / and sqrt enter (the Jacobi functions come from a Newton
// solve of F(s) = w, not from trigonometric functions), so with contraction
// off the host and device builds give the same bits.
#pragma once

#include <cmath>
#include <cstdint>

#include "carlson.cuh"
#include "mino_carlson.cuh"

namespace np {
namespace gkcf {

namespace cr = ::np::carlson;

#define GKCF_HD NP_CARLSON_HD

// ---------------------------------------------------------------------------
// Legendre integrals of one amplitude
// m and its complement mc = 1 - m are both carried (mc from its own
// cancellation-free expression: near m = 1, 1 - m would keep only the
// absolute accuracy of m).
struct Amp {
    double S, C, m, mc, s, D2, F, Sd;
};

GKCF_HD Amp amp_make(double S, double C, double m, double mc) {
    Amp A;
    A.S = S; A.C = C; A.m = m; A.mc = mc;
    A.s = std::sqrt(S);
    A.D2 = C + mc * S;      // 1 - m S
    if (S > 0.0) {
        A.F = A.s * cr::rf(C, A.D2, 1.0);
        A.Sd = A.s * S / 3.0 * cr::rd(C, A.D2, 1.0);
    } else {
        A.F = 0.0; A.Sd = 0.0;
    }
    return A;
}

// p = 1 - n S, formed by the caller without cancellation where it can be small
GKCF_HD double amp_pi(const Amp& A, double n, double p) {
    if (A.S == 0.0) return 0.0;
    const double m = A.m, mc = A.mc, s = A.s, S = A.S, C = A.C, D2 = A.D2;
    if (n < -1.0) {
        const double q = D2 - mc * m * S / (m - n);
        return s * cr::rf(C, D2, 1.0) * m / (m - n) - n * s / (m - n) * cr::rc(C / D2, p * q / D2) +
               n * mc * m * s * S * cr::rj(C, D2, 1.0, q) / (3.0 * (m - n) * (m - n));
    }
    if (p > 0.0) return A.F + n * s * S / 3.0 * cr::rj(C, D2, 1.0, p);
    const double nn = m / n;
    const double pim = A.F + nn * s * S / 3.0 * cr::rj(C, D2, 1.0, 1.0 - nn * S);
    return A.F + s * cr::rc(C * D2, p * (1.0 - nn * S)) - pim;
}

GKCF_HD double amp_j(const Amp& A, double n, double p) {
    if (A.S == 0.0) return 0.0;
    if (p > 0.0) return A.s * A.S / 3.0 * cr::rj(A.C, A.D2, 1.0, p);
    return (amp_pi(A, n, p) - A.F) / n;
}

// e = n - 1 is passed exactly: the denominator (n - 1)(n - m) = e (e + mc)
// vanishes as n -> 1 together with mc -> 0 (a near-double radial root)
// J = amp_j(A, n, p), computed once by the caller and shared with Pi = F + n J
GKCF_HD double amp_pi2(const Amp& A, double n, double e, double p, double J) {
    if (A.S == 0.0) return 0.0;
    const double m = A.m;
    const double V = A.s * std::sqrt(A.C) * std::sqrt(A.D2) / p;
    const double num = n * n * V - (2.0 * n + 2.0 * m * n - n * n - 2.0 * m) * A.F -
                       n * (2.0 * n + 2.0 * m * n - n * n - 3.0 * m) * J + m * n * A.Sd;
    return num / (2.0 * e * (e + A.mc));
}

// sn, cn, dn of w in [0, K(m)]: for w <= K/2 the amplitude's sine s solves
// s R_F(1 - s^2, 1 - m s^2, 1) = w by Newton steps (a bisection bracket
// guards them) from a starting value that is already close: sn, cn and dn
// of w / 2^n <= 1/16 from their Maclaurin series to the seventh power
// (A&S 16.22) and n duplications
//   sn(2v) = 2 s c d / (1 - m s^4), cn(2v) = (c^2 - s^2 d^2) / (1 - m s^4),
//   dn(2v) = (d^2 - m s^2 c^2) / (1 - m s^4)
// (A&S 16.18), which take only +, -, * and /.  From there one or two Newton
// steps reach the root (from s = min(w, sn(K/2)) it took 20-30 steps as
// m -> 1).  Beyond K/2 the complementary argument K - w is solved and
// sn(w) = cd(K - w), cn(w) = k' sd(K - w), dn(w) = k' nd(K - w).  S2 = sn^2
// and C2 = cn^2 are returned without forming 1 - sn^2.
GKCF_HD double sn_start(double x, double m) {
    double v = x;
    int n = 0;
    while (v > 0.0625 && n < 64) { v *= 0.5; ++n; }
    const double v2 = v * v;
    double s = v * (1.0 - v2 * ((1.0 + m) / 6.0 - v2 * ((1.0 + m * (14.0 + m)) / 120.0 -
                                                        v2 * ((1.0 + m * (135.0 + m * (135.0 + m))) / 5040.0))));
    double c = 1.0 - v2 * (0.5 - v2 * ((1.0 + 4.0 * m) / 24.0 - v2 * ((1.0 + m * (44.0 + 16.0 * m)) / 720.0)));
    double d = 1.0 - v2 * (0.5 * m - v2 * (m * (4.0 + m) / 24.0 - v2 * (m * (16.0 + m * (44.0 + m)) / 720.0)));
    for (int k = 0; k < n; ++k) {
        const double s2 = s * s, den = 1.0 - m * s2 * s2;
        const double sn = 2.0 * s * c * d / den;
        const double cn = (c * c - s2 * d * d) / den;
        const double dn = (d * d - m * s2 * c * c) / den;
        s = sn; c = cn; d = dn;
    }
    return s;
}

GKCF_HD void jacobi(double w, double m, double mc, double K, double& S2, double& C2, double& D2) {
    const bool comp = w > 0.5 * K;
    const double x = comp ? K - w : w;
    double s = 0.0;
    if (x > 0.0) {
        double hi = 1.0 / std::sqrt(1.0 + std::sqrt(mc)), lo = 0.0;
        s = sn_start(x, m);
        if (!(s > lo && s < hi)) s = std::fmin(x, hi);
        for (int it = 0; it < 64; ++it) {
            const double c2 = (1.0 - s) * (1.0 + s), d2 = c2 + mc * s * s;
            const double f = s * cr::rf(c2, d2, 1.0) - x;
            if (f == 0.0) break;
            if (f > 0.0) hi = s; else lo = s;
            double sn = s - f * std::sqrt(c2 * d2);
            if (sn == s) break;                              // converged to the last bit
            const bool newton = sn >= lo && sn <= hi;
            if (!newton) sn = 0.5 * (lo + hi);
            // quadratic convergence: a Newton step below 1e-11 s leaves an
            // error far below the last bit (the curvature factor is at most
            // ~1e6 here)
            const bool done = newton && std::fabs(sn - s) <= 1e-11 * s;
            s = sn;
            if (done) break;
        }
    }
    const double ss = s * s, cc = (1.0 - s) * (1.0 + s), dd = cc + mc * ss;
    if (!comp) { S2 = ss; C2 = cc; D2 = dd; return; }
    S2 = cc / dd; C2 = mc * ss / dd; D2 = mc / dd;
}

// ---------------------------------------------------------------------------
// Per-ray constants
// kR2O: two real roots r1 < r2 below the motion and a complex pair (q2 < 0),
// motion in u > r2; it shares the kR2C code with (u1, u2, A, B) -> (r2, r1, B, -A).
// kC4: two complex pairs (q2 < 0), every u allowed.
enum { kFallback = 0, kR4 = 1, kR2C = 2, kR2O = 3, kC4 = 4 };

struct CfRay {
    int32_t kind, tpr, kmax, last;
    double a, l, u0, ub, du, offset, su;
    double r[4];            // R4: u1..u4; R2C: u1, u2, A, B; C4: rho1, sigma1, cos th0, sin th0
    double m, mc, g;        // radial parameter, 1 - m; scale (R4: g, R2C: 2 / sqrt(|c4| A B))
    double pole[3];         // 0, 1/r+, 1/r- (R4: n_p)
    double pc[3][6];        // R2C: e1, e2 (e_j = n_j - 1), al1, al2, cinf, a0 per pole;
                            // C4: Dc, Ds, a, e-coefficient, kappa, u/(u - p) constant
    double pn[3][2];        // R2C: n1, n2; C4: n, n - 1 per pole
    double comp[6];         // C4: complete F, J(n_p) x 3, Pi(n_0), Pi2(n_0)
    double rp, rm, cp, cm, dp, dm;
    // polar
    // pkind 0: mu = mu+ cn (q2 > 0); 1: mu = s0 mu+ dn (q2 < 0, vortical)
    int32_t pkind, pad;
    double mpos, omp, mp, om, mth, mcth, Kth, nth, pq, s0, w0, mu2K, invK, Ph0mu2, Ph0inv;
    double G0[7], Gtop[7];  // 1, 1/u^2, 1/u, 1/(u - 1/r+), 1/(u - 1/r-), u/(u - 1/r+), u/(u - 1/r-) integrals
};

// atanh(z) = z R_C(1, 1 - z^2), |z| < 1, with 1 - z^2 supplied exactly
GKCF_HD double atanh_rc(double z, double one_minus_z2) { return z * cr::rc(1.0, one_minus_z2); }

// W(S) = 1/2 int_0^S ds / ((1 - n s) sqrt(1 - m s)), n >= 1 > m, q = 1 - n S
// exact (principal value past s = 1/n).  With y = sqrt(1 - m s) and
// c = (n - m)/n it is (1/(2 n sqrt c)) [2 ln((y_S + sqrt c)/(1 + sqrt c)) - ln|q|];
// both logarithms as atanh through R_C (no log call, no cancellation as m -> 0).
GKCF_HD double w_odd(double S, double n, double m, double q) {
    if (S == 0.0) return 0.0;
    const double sc = std::sqrt((n - m) / n);
    const double y = std::sqrt(1.0 - m * S);
    const double x = m * S / ((1.0 + y) * (1.0 + sc));       // 1 - (y + sc)/(1 + sc)
    const double t1 = -4.0 * atanh_rc(x / (2.0 - x), 4.0 * (1.0 - x) / ((2.0 - x) * (2.0 - x)));
    const double aq = std::fabs(q);
    const double t2 = -2.0 * atanh_rc((aq - 1.0) / (aq + 1.0), 4.0 * aq / ((aq + 1.0) * (aq + 1.0)));
    return (t1 + t2) / (2.0 * n * sc);
}

// W2(S) = 1/2 int_0^S ds / ((1 - n s)^2 sqrt(1 - m s)), from
// d/ds [y / (1 - n s)] = (m/2) / ((1 - n s) y) + (n - m) / ((1 - n s)^2 y).
GKCF_HD double w2_odd(double S, double n, double m, double q, double w) {
    const double y = std::sqrt(1.0 - m * S);
    const double top = (n * S - m * S / (1.0 + y)) / q;      // y/(1 - n S) - 1
    return (top - m * w) / (2.0 * (n - m));
}

// An odd, quasi-periodic Legendre integral at amplitude theta' in (-pi, pi)
// from its value on [0, pi/2] and its complete value.
GKCF_HD double quadrant(double base, double complete, double cp, double sp) {
    const double b = cp >= 0.0 ? base : 2.0 * complete - base;
    return sp >= 0.0 ? b : -b;
}

// C4 (two complex pairs, Byrd & Friedman 267.00 in rotated form): with
// u = rho1 + sigma1 tan(theta), U du^2 = c4 (alpha cos^2 + 2 beta sin cos +
// gamma sin^2) dtheta^2 / cos^4 ..., and the rotation theta = theta' + theta0
// onto the eigenvectors of [[alpha, beta], [beta, gamma]] (alpha = (rho1 -
// rho2)^2 + sigma2^2, beta = (rho1 - rho2) sigma1, gamma = sigma1^2), so
// that int du / sqrt(U) = F(theta' | m) / sqrt(c4 l1), m = 1 - l2/l1.  A
// pole term is 1/(u - p) = a + e S/(1 - n S) + kappa sin cos/(1 - n S) with
// n = 1 + Ds^2/Dc^2: an even part (F, J) and an odd part (W).
GKCF_HD void c4_angle(const CfRay& R, double u, double& ct, double& cp, double& sp) {
    const double t = u - R.r[0];
    const double h = std::sqrt(t * t + R.r[1] * R.r[1]);
    ct = R.r[1] / h;
    const double st = t / h;
    cp = ct * R.r[2] + st * R.r[3];
    sp = st * R.r[2] - ct * R.r[3];
}

// Radial Legendre amplitude of u (and, for R2C, D(S) = the Moebius denominator)
GKCF_HD Amp radial_amp(const CfRay& R, double u, double& Dfac) {
    const double m = R.m, mc = R.mc;
    if (R.kind == kC4) {
        double ct, cp, sp;
        c4_angle(R, u, ct, cp, sp);
        Dfac = 0.0;
        return amp_make(sp * sp, cp * cp, m, mc);
    }
    if (R.kind == kR4) {
        const double u1 = R.r[0], u2 = R.r[1], u3 = R.r[2];
        const double den = (u2 - u1) * (u3 - u);
        Dfac = 0.0;
        return amp_make((u3 - u1) * (u2 - u) / den, (u - u1) * (u3 - u2) / den, m, mc);
    }
    const double u1 = R.r[0], u2 = R.r[1], A = R.r[2], B = R.r[3];
    const double den = (u2 - u) * B + (u - u1) * A;
    const double omx = 2.0 * (u - u1) * A / den;       // 1 - X
    const double opx = 2.0 * (u2 - u) * B / den;       // 1 + X
    const double X = 0.5 * (opx - omx);
    const double dnw = std::sqrt(mc + m * X * X);
    const double S = omx / (1.0 + dnw);
    const double C = X > 0.0 ? (X + dnw) / (1.0 + dnw) : mc * omx * opx / ((dnw - X) * (1.0 + dnw));
    Dfac = A * B * (u2 - u1) * (C * (1.0 + S) + mc * S * S) / den;   // A B (u2 - u1)(1 - m S^2) / den
    return amp_make(S, C, m, mc);
}

// R2C: the two pole factors 1 - n_j S at u, the one near zero from their product
GKCF_HD void r2c_factors(const CfRay& R, int ip, const Amp& A, double u, double Dfac, double& f1, double& f2) {
    const double* c = R.pc[ip];
    f1 = A.C - c[0] * A.S;      // 1 - n S = (1 - S) - e S
    f2 = A.C - c[1] * A.S;
    const double prod = (u - R.pole[ip]) * Dfac / c[5];
    if (std::fabs(f1) < std::fabs(f2)) f1 = prod / f2;
    else f2 = prod / f1;
}

// G(u): the seven radial integrals against du/sqrt(U), increasing in u
// (R4: minus the integral from u to u2; R2C: the integral from u1 to u).
// u/(u - p) = 1 + p/(u - p) is integrated with the constant written as the
// anchor's value (u2/(u2 - p), u3/(u3 - p), u1/(u1 - p)): the radial phi rate
// d+ r+ u/(1 - r+ u) + d- r- u/(1 - r- u) is then free of the cancellation
// between the O(l) terms of its partial fractions at small u.
GKCF_HD void radial_G(const CfRay& R, double u, double* G) {
    double Dfac;
    const Amp A = radial_amp(R, u, Dfac);
    if (R.kind == kC4) {
        double ct, cp, sp;
        c4_angle(R, u, ct, cp, sp);
        const double g = R.g, m = R.m, S = A.S;
        const double F = quadrant(A.F, R.comp[0], cp, sp);
        G[0] = g * F;
        for (int ip = 0; ip < 3; ++ip) {
            const double* c = R.pc[ip];
            const double p = R.pole[ip], Dc = c[0], Ds = c[1], n = R.pn[ip][0];
            // 1 - n S = (u - p) cos(theta) (Dc cos theta' - Ds sin theta') / Dc^2
            const double q = (u - p) * ct * (Dc * cp - Ds * sp) / (Dc * Dc);
            const double Jb = amp_j(A, n, q);
            const double J = quadrant(Jb, R.comp[1 + ip], cp, sp);
            const double w = w_odd(S, n, m, q);
            G[2 + ip] = g * (c[2] * F + c[3] * J + c[4] * w);
            if (ip > 0) G[4 + ip] = g * (c[5] * F + p * (c[3] * J + c[4] * w));
            if (ip == 0) {
                // (a + e S/(1 - nS) + kappa sc/(1 - nS))^2: even part with
                // int S/(1 - nS)^2 = (Pi2 - Pi)/n, int S^2/(1 - nS)^2 = (Pi2 - 2 Pi + F)/n^2,
                // odd part 2 kappa (a W + e (W2 - W)/n)
                const double Pi = quadrant(A.F + n * Jb, R.comp[4], cp, sp);      // n >= 1
                const double P2 = quadrant(amp_pi2(A, n, R.pn[0][1], q, Jb), R.comp[5], cp, sp);
                const double Q1 = (P2 - Pi) / n, Q2 = (P2 - 2.0 * Pi + F) / (n * n);
                const double w2 = w2_odd(S, n, m, q, w);
                const double a0 = c[2], e0 = c[3], k0 = c[4];
                G[1] = g * (a0 * a0 * F + 2.0 * a0 * e0 * J + e0 * e0 * Q2 + k0 * k0 * (Q1 - Q2) +
                            2.0 * k0 * (a0 * w + e0 * (w2 - w) / n));
            }
        }
        return;
    }
    if (R.kind == kR4) {
        const double u1 = R.r[0], u2 = R.r[1], u3 = R.r[2], g = R.g;
        G[0] = -g * A.F;
        for (int ip = 0; ip < 3; ++ip) {
            const double p = R.pole[ip], n = (u3 - p) * (u2 - u1) / ((u2 - p) * (u3 - u1));
            const double e = (u3 - u2) * (p - u1) / ((u2 - p) * (u3 - u1));      // n - 1
            const double f = (u - p) * (u3 - u2) / ((u2 - p) * (u3 - u));
            double h, x, T;
            if (n < -1.0) {
                const double Cp = (u3 - u2) / ((u3 - p) * (u2 - p));
                T = amp_pi(A, n, f);
                h = A.F / (u3 - p) + Cp * T;
                x = u3 / (u3 - p) * A.F + p * Cp * T;
            } else {
                const double Kp = (u3 - u2) * (u2 - u1) / ((u2 - p) * (u2 - p) * (u3 - u1));
                T = amp_j(A, n, f);
                h = A.F / (u2 - p) + Kp * T;
                x = u2 / (u2 - p) * A.F + p * Kp * T;
            }
            G[2 + ip] = -g * h;
            if (ip > 0) G[4 + ip] = -g * x;
            if (ip == 0) {
                // (1/u2 + K0 S/(1 - n S))^2, with int S^2/(1 - n S)^2 = (Pi2 - 2 Pi + F)/n^2;
                // n > 1 here (the pole u = 0 lies inside [u1, u2]), so T = J and Pi = F + n J
                const double K0 = (u3 - u2) * (u2 - u1) / (u2 * u2 * (u3 - u1));
                const double Q = (amp_pi2(A, n, e, f, T) - 2.0 * (A.F + n * T) + A.F) / (n * n);
                G[1] = -g * (A.F / (u2 * u2) + 2.0 * K0 / u2 * T + K0 * K0 * Q);
            }
        }
        return;
    }
    const double g = R.g;
    G[0] = g * A.F;
    for (int ip = 0; ip < 3; ++ip) {
        const double* c = R.pc[ip];
        double f1, f2;
        r2c_factors(R, ip, A, u, Dfac, f1, f2);
        const double n1 = R.pn[ip][0], n2 = R.pn[ip][1];
        // int dv / (1 - n S) = F + n J, or Pi for n < -1
        const bool pi1 = n1 < -1.0, pi2 = n2 < -1.0;
        const double j1 = pi1 ? 0.0 : amp_j(A, n1, f1), j2 = pi2 ? 0.0 : amp_j(A, n2, f2);
        const double t1 = pi1 ? amp_pi(A, n1, f1) : A.F + n1 * j1;
        const double t2 = pi2 ? amp_pi(A, n2, f2) : A.F + n2 * j2;
        G[2 + ip] = g * (c[4] * A.F + c[2] * t1 + c[3] * t2);
        if (ip > 0) {
            // u/(u - p): constant u1/(u1 - p) less p al_j of the Pi-form terms
            const double p = R.pole[ip];
            double k0 = R.r[0] / (R.r[0] - p), x = 0.0;
            if (pi1) { k0 -= p * c[2]; x += p * c[2] * t1; } else x += p * c[2] * n1 * j1;
            if (pi2) { k0 -= p * c[3]; x += p * c[3] * t2; } else x += p * c[3] * n2 * j2;
            G[4 + ip] = g * (k0 * A.F + x);
        }
        if (ip == 0) {
            const double cross = 2.0 * c[2] * c[3] / (c[0] - c[1]);
            const double jj1 = pi1 ? amp_j(A, n1, f1) : j1, jj2 = pi2 ? amp_j(A, n2, f2) : j2;
            G[1] = g * (c[4] * c[4] * A.F + 2.0 * c[4] * (c[2] * t1 + c[3] * t2) + cross * (n1 * t1 - n2 * t2) +
                        c[2] * c[2] * amp_pi2(A, n1, c[0], f1, jj1) + c[3] * c[3] * amp_pi2(A, n2, c[1], f2, jj2));
        }
    }
}

// Polar integrals Phi(w) = (int_0^w mu^2 dw', int_0^w dw'/(1 - mu^2)) with
// mu = mu+ cn w'; also cn w and the half-period index j of w.
GKCF_HD void polar_Phi(const CfRay& R, double w, double& mu2, double& inv, double& cn, double& jj) {
    const double K = R.Kth, m = R.mth;
    const double j = std::floor(w / (2.0 * K) + 0.5);
    const double r = w - 2.0 * j * K;
    double S2, C2, D2;
    jacobi(std::fabs(r), m, R.mcth, K, S2, C2, D2);
    const Amp A = amp_make(S2, C2, m, R.mcth);
    const double sg = r >= 0.0 ? 1.0 : -1.0;
    // mu^2 = mu+^2 cn^2 = mu+^2 (1 - S), or mu+^2 dn^2 = mu+^2 (1 - m S)
    mu2 = 2.0 * j * R.mu2K + sg * R.mpos * (A.F - (R.pkind ? m : 1.0) * A.Sd);
    inv = 0.0;
    // 1 - mu^2 = (1 - mu+^2)(1 - nth S), 1 - nth S = (1 - mu+^2 + pq S) / (1 - mu+^2)
    if (R.l != 0.0) inv = 2.0 * j * R.invK + sg * amp_pi(A, R.nth, (R.omp + R.pq * S2) / R.omp) / R.omp;
    if (R.pkind) {
        cn = R.s0 * std::sqrt(D2);                 // mu / mu+ = s0 dn, even with period 2K
    } else {
        const double par = j - 2.0 * std::floor(0.5 * j);
        cn = (par != 0.0 ? -1.0 : 1.0) * std::sqrt(C2);
    }
    jj = j;
}

// Complex-pair poles: 1/(u - p) = D(S) / N_p(S) with the Moebius denominator
// D(S) = (1 - S)(A + B S) + B mc S^2 and N_p(S) = a0 (1 - n1 S)(1 - n2 S);
// e = n - 1 solves a0 e^2 + ((u1 - p) A + (u2 - p) B) e + (u2 - p) B mc = 0
// (exact coefficients), and the residues are
//   al_j = D(1/n_j) n_j / (a0 (n_j - n_k)) = (e_j (A n_j + B) + B mc) / (n_j a0 (e_j - e_k)).
// Each root is taken from the form in which it has no cancellation: n from
// a0 n^2 + a1 n + a2 = 0 where |n - 1| >= 1/2, else n = 1 + e.
GKCF_HD void complex_poles(CfRay& R) {
    const double u1 = R.r[0], u2 = R.r[1], A = R.r[2], Bq = R.r[3];
    for (int ip = 0; ip < 3; ++ip) {
        const double p = R.pole[ip];
        const double a0 = (u1 - p) * A, b1 = (u1 - p) * A + (u2 - p) * Bq, c0 = (u2 - p) * Bq * R.mc;
        const double a1 = (u2 - p) * Bq - (u1 - p) * A, a2 = -R.m * Bq * (u2 - p);
        const double dn = std::sqrt(a1 * a1 - 4.0 * a0 * a2);
        const double qn = -0.5 * (a1 + (a1 >= 0.0 ? dn : -dn));
        double n1 = qn / a0, n2 = a2 / qn;
        if (std::fabs(n2) > std::fabs(n1)) { const double t = n1; n1 = n2; n2 = t; }
        const double de = std::sqrt(b1 * b1 - 4.0 * a0 * c0);
        const double qe = -0.5 * (b1 + (b1 >= 0.0 ? de : -de));
        const double ea = qe / a0, eb = c0 / qe;
        double e1 = n1 - 1.0, e2 = n2 - 1.0;
        const double ec1 = std::fabs(ea - e1) < std::fabs(eb - e1) ? ea : eb;
        const double ec2 = std::fabs(ea - e2) < std::fabs(eb - e2) ? ea : eb;
        if (std::fabs(ec1) < 0.5) { e1 = ec1; n1 = 1.0 + ec1; }
        if (std::fabs(ec2) < 0.5) { e2 = ec2; n2 = 1.0 + ec2; }
        double* pc = R.pc[ip];
        pc[0] = e1; pc[1] = e2;
        pc[2] = (e1 * (A * n1 + Bq) + Bq * R.mc) / (n1 * a0 * (e1 - e2));
        pc[3] = (e2 * (A * n2 + Bq) + Bq * R.mc) / (n2 * a0 * (e2 - e1));
        pc[4] = 1.0 / (u2 - p);
        pc[5] = a0;
        R.pn[ip][0] = n1; R.pn[ip][1] = n2;
    }
}

// Roots of U polished against its exact coefficients.  U(u) = 1 + c2 u^2 +
// c3 u^3 + c4 u^4 with c2 = a^2 - l^2 - q2, c3 = 2 ((l - a)^2 + q2) and
// c4 = -a^2 q2 is formed in double-double arithmetic from the double inputs
// (Dekker's exact product by fma, Knuth's two-sum) and evaluated by a
// compensated Horner scheme; Newton steps on that value move each root to
// the root of the exact polynomial.  The double coefficients alone are
// rounded by ~1e-16 relative, which moves a pair of nearly double roots
// (a ray near the critical curve) by ~1e-16 / (U'' (u3 - u2)): 1e-13 at
// u3 - u2 = 5e-5, and the crossings past the photon orbit inherit it times
// the orbit's growth factor.  A step larger than a quarter of the distance
// to the nearest other root is not taken.
struct DD { double hi, lo; };
GKCF_HD DD dd_fast(double a, double b) { const double s = a + b; return DD{s, b - (s - a)}; }
GKCF_HD DD dd_two_sum(double a, double b) {
    const double s = a + b, bb = s - a;
    return DD{s, (a - (s - bb)) + (b - bb)};
}
GKCF_HD DD dd_two_prod(double a, double b) { const double p = a * b; return DD{p, std::fma(a, b, -p)}; }
GKCF_HD DD dd_add(DD x, DD y) { const DD t = dd_two_sum(x.hi, y.hi); return dd_fast(t.hi, t.lo + x.lo + y.lo); }
GKCF_HD DD dd_mul(DD x, double y) { const DD p = dd_two_prod(x.hi, y); return dd_fast(p.hi, p.lo + x.lo * y); }

struct UExact { DD c2, c3, c4; };
GKCF_HD UExact u_exact(double a, double l, double q2) {
    UExact c;
    const DD a2 = dd_two_prod(a, a), l2 = dd_two_prod(l, l);
    c.c2 = dd_add(dd_add(a2, DD{-l2.hi, -l2.lo}), DD{-q2, 0.0});
    const DD d = dd_two_sum(l, -a);
    const DD d2 = dd_two_prod(d.hi, d.hi);
    const DD k = dd_add(dd_fast(d2.hi, d2.lo + 2.0 * d.hi * d.lo), DD{q2, 0.0});
    c.c3 = DD{2.0 * k.hi, 2.0 * k.lo};
    c.c4 = dd_mul(a2, -q2);
    return c;
}

// Returns false when the root is not resolved: a step would move it by more
// than a quarter of the distance to its neighbour (the iteration that found
// the roots could not separate a nearly double pair), or the steps do not
// settle to the last bits.
GKCF_HD bool polish_real(const UExact& c, double& x, double gap) {
    for (int it = 0; it < 3; ++it) {
        DD t = dd_add(dd_mul(c.c4, x), c.c3);
        t = dd_add(dd_mul(t, x), c.c2);
        t = dd_mul(dd_mul(t, x), x);
        t = dd_add(t, DD{1.0, 0.0});
        const double d = x * (2.0 * c.c2.hi + x * (3.0 * c.c3.hi + 4.0 * x * c.c4.hi));
        if (!(d != 0.0)) return false;
        const double dx = (t.hi + t.lo) / d;
        if (!(std::fabs(dx) <= 0.25 * gap)) return false;
        x -= dx;
        if (std::fabs(dx) <= 4e-16 * std::fabs(x)) return true;   // the next step is below the last bit
    }
    return false;
}

// the complex root rho + i sigma (sigma > 0), by complex Newton steps;
// false as for polish_real (the conjugate is 2 sigma away)
GKCF_HD bool polish_pair(const UExact& c, double& rho, double& sigma) {
    double x = rho, y = sigma;
    for (int it = 0; it < 3; ++it) {
        // U(z) by Horner in double-double complex arithmetic
        DD re = c.c4, im = DD{0.0, 0.0};
        for (int k = 0; k < 4; ++k) {
            const DD nre = dd_add(dd_mul(re, x), dd_mul(im, -y));
            const DD nim = dd_add(dd_mul(re, y), dd_mul(im, x));
            re = nre; im = nim;
            if (k == 0) re = dd_add(re, c.c3);
            else if (k == 1) re = dd_add(re, c.c2);
            else if (k == 3) re = dd_add(re, DD{1.0, 0.0});
        }
        // U'(z) = z (2 c2 + z (3 c3 + 4 c4 z)) in double
        const double c2 = c.c2.hi, c3 = c.c3.hi, c4 = c.c4.hi;
        double pr = 3.0 * c3 + 4.0 * c4 * x, pi = 4.0 * c4 * y;
        double qr = 2.0 * c2 + (pr * x - pi * y), qi = pr * y + pi * x;
        const double dr = qr * x - qi * y, di = qr * y + qi * x;
        const double den = dr * dr + di * di;
        if (!(den > 0.0)) return false;
        const double ur = re.hi + re.lo, ui = im.hi + im.lo;
        const double sr = (ur * dr + ui * di) / den, si = (ui * dr - ur * di) / den;
        if (!(std::fabs(sr) + std::fabs(si) <= 0.25 * y)) return false;
        x -= sr; y -= si;
        if (std::fabs(sr) + std::fabs(si) <= 4e-16 * (std::fabs(x) + y)) {
            rho = x; sigma = y;
            return true;
        }
    }
    return false;
}

// Polishes the roots of a q2 > 0 potential as found (nr real roots sorted,
// a complex pair when nr = 2).  false when a root is not resolved: such a
// ray (within ~1e-9 relative of the critical curve, where the pair's
// separation is below what the root iteration resolves) is left to the
// integrators.
GKCF_HD bool polish_roots(double a, double l, double q2, int nr, double* rr, double& rho, double& sigma) {
    const UExact c = u_exact(a, l, q2);
    double out[4];
    bool ok = true;
    for (int i = 0; i < nr; ++i) {
        double gap = nr == 2 ? std::fabs(rr[1] - rr[0]) : INFINITY;
        for (int j = 0; j < nr; ++j)
            if (j != i) gap = std::fmin(gap, std::fabs(rr[j] - rr[i]));
        if (nr == 2 && sigma > 0.0) {
            const double dz = std::sqrt((rr[i] - rho) * (rr[i] - rho) + sigma * sigma);
            gap = std::fmin(gap, dz);
        }
        out[i] = rr[i];
        ok = polish_real(c, out[i], gap) && ok;
    }
    for (int i = 0; i < nr; ++i) rr[i] = out[i];
    if (nr == 2 && sigma > 0.0) ok = polish_pair(c, rho, sigma) && ok;
    return ok;
}

// Radial reductions of q2 > 0 (c4 = -a^2 q2 < 0), motion in [u1, u2] holding
// u0 with the turning point u2 ahead of an ingoing ray: kind, roots, m, mc
// and g of R; false when u0 is outside that interval.
// Four real roots u1 < u2 < u3 < u4:
GKCF_HD bool reduce_r4(const double* rr, double c4, double u0, CfRay& R) {
    const double u1 = rr[0], u2 = rr[1], u3 = rr[2], u4 = rr[3];
    if (!(u1 < u0 && u0 <= u2) || !(u2 < u3)) return false;
    R.kind = kR4;
    for (int i = 0; i < 4; ++i) R.r[i] = rr[i];
    R.m = (u2 - u1) * (u4 - u3) / ((u3 - u1) * (u4 - u2));
    R.mc = (u3 - u2) * (u4 - u1) / ((u3 - u1) * (u4 - u2));
    R.g = 2.0 / std::sqrt(-c4 * (u3 - u1) * (u4 - u2));
    return true;
}

// two real roots u1 < u2 and the complex pair rho +- i sigma:
GKCF_HD bool reduce_r2c(const double* rr, double rho, double sigma, double c4, double u0, CfRay& R) {
    const double u1 = rr[0], u2 = rr[1];
    if (!(u1 < u0 && u0 <= u2)) return false;
    R.kind = kR2C;
    const double A = std::sqrt((u2 - rho) * (u2 - rho) + sigma * sigma);
    const double Bq = std::sqrt((u1 - rho) * (u1 - rho) + sigma * sigma);
    R.r[0] = u1; R.r[1] = u2; R.r[2] = A; R.r[3] = Bq;
    const double mdirect = ((u2 - u1) * (u2 - u1) - (A - Bq) * (A - Bq)) / (4.0 * A * Bq);
    // 1 - m = (A + B - (u2 - u1))(A + B + u2 - u1) / (4 A B), with
    // A - |u2 - rho| = sigma^2 / (A + |u2 - rho|) (likewise B)
    // (|u2 - rho| + |rho - u1| - (u2 - u1) is 0 for rho in [u1, u2], and
    // twice the distance to the interval outside it: set, not rounded)
    const double d2 = std::fabs(u2 - rho), d1 = std::fabs(rho - u1);
    const double outside = rho < u1 ? 2.0 * (u1 - rho) : (rho > u2 ? 2.0 * (rho - u2) : 0.0);
    const double gap = sigma * sigma / (A + d2) + sigma * sigma / (Bq + d1) + outside;
    R.mc = gap * (A + Bq + (u2 - u1)) / (4.0 * A * Bq);
    R.m = R.mc < 0.5 ? 1.0 - R.mc : mdirect;
    R.g = 2.0 / std::sqrt(-c4 * A * Bq);
    return true;
}

// Roots of GEOKERR's polar potential M(mu) = q2 + (a^2 - l^2 - q2) mu^2 -
// a^2 mu^4 in mu^2, by the stable quadratic formula: mpos = mu+^2 and a2mneg
// = a^2 mu-^2 (carried with its factor a^2 so that a = 0 needs no special
// case); a root that the start violates by rounding moves to mu0^2.
GKCF_HD void polar_roots(double a, double l, double q2, double mu0, double& mpos, double& a2mneg) {
    const double a2 = a * a, b = a2 - (q2 + l * l);
    const double yy = -0.5 * (b + (b >= 0.0 ? 1.0 : -1.0) * std::sqrt(b * b + 4.0 * q2 * a2));
    if (b < 0.0) { a2mneg = -yy; mpos = q2 / yy; }
    else { a2mneg = a2 * q2 / yy; mpos = -yy / a2; }
    if (mpos > 1.0) mpos = 1.0;
    if (a2mneg < 0.0 || a2 == 0.0) {
        if (std::sqrt(mpos) < mu0) mpos = mu0 * mu0;
    } else {
        if (a2mneg > a2 * mu0 * mu0) a2mneg = a2 * mu0 * mu0;
        if (mu0 * mu0 > mpos) mpos = mu0 * mu0;
    }
}

// Per-ray setup; kind = kFallback when the ray is outside the closed forms
// (q2 = 0, a = 0, a motion between the middle roots of four real ones, a
// double root, a polar orbit through the pole with l != 0).
GKCF_HD void setup(double a, double l, double q2, double u0, double uf, double mu0, double su, double sm, int tpr_in,
                   int nup, double offset, double mpos, double a2mneg, CfRay& R) {
    R.kind = kFallback;
    R.tpr = 0; R.kmax = 0; R.last = 0;
    R.a = a; R.l = l; R.u0 = u0; R.offset = offset; R.su = su;
    if (q2 == 0.0 || a == 0.0 || a2mneg == 0.0 || !(mpos > 0.0) || nup <= 0) return;
    if (!(1.0 - mpos > 1e-15) && l != 0.0) return;
    const double B = a * a - l * l - q2, Kc = (l - a) * (l - a) + q2;
    const double c[5] = {1.0, 0.0, B, 2.0 * Kc, -a * a * q2};
    double rr[4], rho = 0.0, sigma = 0.0;
    const int nr = ::np::mino::real_roots(c, 4, rr, &rho, &sigma);
    if (c[4] < 0.0 && (nr == 4 || (nr == 2 && sigma > 0.0)) && !polish_roots(a, l, q2, nr, rr, rho, sigma)) return;
    const double sq = std::sqrt(1.0 - a * a);
    R.rp = 1.0 + sq;
    R.rm = a * a / R.rp;
    R.pole[0] = 0.0; R.pole[1] = 1.0 / R.rp; R.pole[2] = 1.0 / R.rm;
    const double uplus = 1.0 / R.rp;
    double uturn = INFINITY;      // radial turning point ahead of an ingoing ray
    if (nr == 4 && c[4] < 0.0) {
        if (!reduce_r4(rr, c[4], u0, R)) return;
        uturn = R.r[1];
    } else if (nr == 2 && sigma > 0.0 && c[4] < 0.0) {
        if (!reduce_r2c(rr, rho, sigma, c[4], u0, R)) return;
        complex_poles(R);
        uturn = R.r[1];
    } else if (nr == 2 && sigma > 0.0 && c[4] > 0.0) {
        // Motion above both real roots (Byrd & Friedman 260.00):
        // cn w = ((u - r1) A - (u - r2) B) / ((u - r1) A + (u - r2) B),
        // int_{r2}^u du / sqrt(U) = w / sqrt(c4 A B), m = ((A + B)^2 - (r2 - r1)^2) / (4 A B);
        // the same half-argument algebra as kR2C with (u1, u2, A, B) = (r2, r1, B, -A).
        const double r1 = rr[0], r2 = rr[1];
        if (!(r2 < u0)) return;
        R.kind = kR2O;
        const double A = std::sqrt((r2 - rho) * (r2 - rho) + sigma * sigma);
        const double Bq = std::sqrt((r1 - rho) * (r1 - rho) + sigma * sigma);
        R.r[0] = r2; R.r[1] = r1; R.r[2] = Bq; R.r[3] = -A;
        // 1 - m = ((r2 - r1) - |A - B|)((r2 - r1) + |A - B|) / (4 A B); for rho
        // outside [r1, r2], (r2 - r1) - |A - B| = sigma^2 (1/(A' + d') - 1/(B' + d''))
        // with the nearer root first (no cancellation)
        const double d2 = std::fabs(rho - r2), d1 = std::fabs(rho - r1), w = r2 - r1;
        double gap;
        if (rho >= r2) gap = sigma * sigma / (A + d2) - sigma * sigma / (Bq + d1);
        else if (rho <= r1) gap = sigma * sigma / (Bq + d1) - sigma * sigma / (A + d2);
        else gap = w - std::fabs(A - Bq);
        R.mc = gap * (w + std::fabs(A - Bq)) / (4.0 * A * Bq);
        R.m = R.mc < 0.5 ? 1.0 - R.mc : ((A + Bq) * (A + Bq) - w * w) / (4.0 * A * Bq);
        R.g = 2.0 / std::sqrt(c[4] * A * Bq);
        complex_poles(R);
    } else if (nr == 0 && c[4] > 0.0) {
        ::np::mino::Cx z[4];
        double r0[4], rh, sg;
        if (::np::mino::real_roots(c, 4, r0, &rh, &sg, z) != 0) return;
        // the two roots in the upper half plane; the wider pair is the tan centre
        int i1 = -1, i2 = -1;
        for (int k = 0; k < 4; ++k)
            if (z[k].im > 0.0) { if (i1 < 0) i1 = k; else i2 = k; }
        if (i1 < 0 || i2 < 0) return;
        if (z[i2].im > z[i1].im) { const int t = i1; i1 = i2; i2 = t; }
        const double rho1 = z[i1].re, s1 = z[i1].im, rho2 = z[i2].re, s2 = z[i2].im;
        const double d = rho1 - rho2;
        const double al = d * d + s2 * s2, be = d * s1, ga = s1 * s1, hd = 0.5 * (al - ga);
        const double l1 = 0.5 * (al + ga) + std::sqrt(hd * hd + be * be);
        const double l2 = s1 * s1 * s2 * s2 / l1;                 // det / l1
        // unit eigenvector of l1, from the better-conditioned of two forms
        double vx = be, vy = l1 - al;
        const double wx = l1 - ga, wy = be;
        if (wx * wx + wy * wy > vx * vx + vy * vy) { vx = wx; vy = wy; }
        const double nv = std::sqrt(vx * vx + vy * vy);
        double c0 = vx / nv, s0 = vy / nv;
        if (c0 < 0.0) { c0 = -c0; s0 = -s0; }
        R.kind = kC4;
        R.r[0] = rho1; R.r[1] = s1; R.r[2] = c0; R.r[3] = s0;
        R.m = (l1 - l2) / l1;
        R.mc = l2 / l1;
        R.g = 1.0 / std::sqrt(c[4] * l1);
        const Amp AK = amp_make(1.0, 0.0, R.m, R.mc);
        R.comp[0] = AK.F;
        for (int ip = 0; ip < 3; ++ip) {
            const double p = R.pole[ip], t1 = rho1 - p;
            const double Dc = t1 * c0 + s1 * s0, Ds = s1 * c0 - t1 * s0;
            const double e = Ds * Ds / (Dc * Dc), n = 1.0 + e;
            if (!(std::fabs(Dc) > 0.0) || !(e > 1e-12)) { R.kind = kFallback; return; }
            double* pc = R.pc[ip];
            pc[0] = Dc; pc[1] = Ds;
            pc[2] = c0 / Dc;
            pc[3] = Ds * (c0 * Ds + s0 * Dc) / (Dc * Dc * Dc);
            pc[4] = -(c0 * Ds + s0 * Dc) / (Dc * Dc);
            pc[5] = (rho1 * c0 + s1 * s0) / Dc;                    // 1 + p a
            R.pn[ip][0] = n; R.pn[ip][1] = e;
            R.comp[1 + ip] = amp_j(AK, n, -e);                     // 1 - n = -e
            if (ip == 0) {
                R.comp[4] = AK.F + n * R.comp[1];
                R.comp[5] = amp_pi2(AK, n, e, -e, R.comp[1]);
            }
        }
    } else {
        return;
    }
    // coefficients of the partial fractions
    R.cp = 2.0 * (2.0 * R.rp - a * l) / (R.rp - R.rm);
    R.cm = 2.0 * (2.0 * R.rm - a * l) / (R.rm - R.rp);
    R.dp = a * (2.0 * R.rp - a * l) / (R.rp * (R.rp - R.rm));
    R.dm = a * (2.0 * R.rm - a * l) / (R.rm * (R.rm - R.rp));
    // sampling, as the Taylor sampler: NUP points uniform in u from U0 to the
    // turning point UB and back (geokerr_original.f:357-605)
    double ub;
    int tpr = 0;
    if (su > 0.0 && uturn < uplus) { ub = uturn; tpr = tpr_in; }
    else ub = su > 0.0 ? uplus : 0.0;
    double UF = uf;
    if (tpr == 1 && ((su > 0.0 && UF > ub) || (su < 0.0 && UF < ub))) UF = ub;
    if (tpr == 1 && UF == ub) UF = u0;
    const double du = ((ub - u0) >= 0.0 ? 1.0 : -1.0) * su * ((ub - u0) + (2.0 * tpr - 1.0) * (ub - UF)) / (double)nup;
    int kmax = (du == 0.0) ? 0 : (int)((ub - u0) / du + offset);
    if (kmax > nup) kmax = nup;
    R.ub = ub; R.tpr = tpr; R.du = du; R.kmax = kmax;
    R.last = tpr == 1 ? nup : (kmax < nup ? kmax : nup);
    if (R.last < 0) R.last = 0;
    // A target the ray never reaches (at or inside the horizon before a
    // turning point, at or beyond u = 0 on the way out) leaves the ray
    // without points, as in the Taylor sampler.
    if (R.last > 0) {
        if (su > 0.0) {
            const int kk = R.last < kmax ? R.last : kmax;
            if (kk >= 1 && !(u0 + (kk - offset) * du < uplus)) R.last = 0;
        } else if (!(u0 + (R.last - offset) * du > 0.0)) {
            R.last = 0;
        }
    }
    // polar constants
    R.mpos = mpos;
    // 1 - mu+^2 is the small root of a^2 y^2 - (a^2 + l^2 + q2) y + l^2 = 0,
    // taken without the cancellation of 1 - mpos unless GEOKERR's rules
    // moved the root (to mu0^2, or to 1 by clamping)
    {
        const double a2 = a * a, bb = a2 - (q2 + l * l);
        const double yy = -0.5 * (bb + (bb >= 0.0 ? 1.0 : -1.0) * std::sqrt(bb * bb + 4.0 * q2 * a2));
        const double m0 = bb < 0.0 ? q2 / yy : -yy / a2;
        const double E = a2 + l * l + q2;
        R.omp = (m0 == mpos) ? 2.0 * l * l / (E + std::sqrt((E - 2.0 * a * l) * (E + 2.0 * a * l))) : 1.0 - mpos;
    }
    R.mp = std::sqrt(mpos);
    double F0;
    if (a2mneg < 0.0) {
        // mu = mu+ cn(omega lambda + w0 | k), omega^2 = a^2 mu+^2 - a^2 mneg,
        // k^2 = a^2 mu+^2 / omega^2
        R.pkind = 0;
        const double w2 = a * a * mpos - a2mneg;
        R.om = std::sqrt(w2);
        R.mth = a * a * mpos / w2;
        R.mcth = -a2mneg / w2;
        R.pq = mpos;
        R.s0 = 1.0;
        double c0 = mu0 / R.mp;
        c0 = c0 > 1.0 ? 1.0 : (c0 < -1.0 ? -1.0 : c0);
        R.Kth = cr::rf(0.0, R.mcth, 1.0);
        const Amp A0 = amp_make((1.0 - c0) * (1.0 + c0), c0 * c0, R.mth, R.mcth);
        F0 = c0 >= 0.0 ? A0.F : 2.0 * R.Kth - A0.F;
        R.w0 = -(sm < 0.0 ? -1.0 : 1.0) * F0;
    } else {
        // vortical (q2 < 0): mu^2 between mneg and mu+^2 (Byrd & Friedman 218.00),
        // mu = s0 mu+ dn(omega lambda + w0 | k), omega = a mu+,
        // k^2 = (mu+^2 - mneg) / mu+^2; dn(w0) = |mu0| / mu+
        R.pkind = 1;
        const double a2mp = a * a * mpos, diff = a2mp - a2mneg;     // a^2 (mu+^2 - mneg)
        if (!(diff > 0.0) || mu0 == 0.0) { R.kind = kFallback; return; }
        R.om = std::sqrt(a2mp);
        R.mth = diff / a2mp;
        R.mcth = a2mneg / a2mp;
        R.pq = diff / (a * a);
        R.s0 = mu0 > 0.0 ? 1.0 : -1.0;
        R.Kth = cr::rf(0.0, R.mcth, 1.0);
        const double am0 = a * a * mu0 * mu0;
        double S0 = (a2mp - am0) / diff, C0 = (am0 - a2mneg) / diff;
        S0 = S0 < 0.0 ? 0.0 : (S0 > 1.0 ? 1.0 : S0);
        C0 = C0 < 0.0 ? 0.0 : (C0 > 1.0 ? 1.0 : C0);
        F0 = amp_make(S0, C0, R.mth, R.mcth).F;
        // d mu / d lambda = -s0 mu+ k^2 sn cn omega: negative times s0 on (0, K)
        R.w0 = (sm * R.s0 < 0.0) ? F0 : -F0;
    }
    R.nth = -R.pq / R.omp;
    const Amp Ac = amp_make(1.0, 0.0, R.mth, R.mcth);
    R.mu2K = mpos * (R.Kth - (R.pkind ? R.mth : 1.0) * Ac.Sd);
    R.invK = l != 0.0 ? amp_pi(Ac, R.nth, 1.0 - R.nth) / R.omp : 0.0;
    double cn0, j0;
    polar_Phi(R, R.w0, R.Ph0mu2, R.Ph0inv, cn0, j0);
    // radial integrals at the start and at the turning point
    radial_G(R, u0, R.G0);
    if (tpr == 1 && R.kind == kR2C) radial_G(R, uturn, R.Gtop);
    else for (int i = 0; i < 7; ++i) R.Gtop[i] = 0.0;
    bool ok = true;
    for (int i = 0; i < 7; ++i) ok = ok && std::isfinite(R.G0[i]) && std::isfinite(R.Gtop[i]);
    ok = ok && std::isfinite(R.Ph0mu2) && std::isfinite(R.Ph0inv) && std::isfinite(R.om) && R.om > 0.0;
    if (!ok) R.kind = kFallback;
}

struct Point {
    double u, mu, dt, dphi, lam;
    int32_t tpm, tpr;
};

// The point at u = ut of a ray set up above, before (branch2 = false) or
// after its radial turning point.
GKCF_HD Point point_at(const CfRay& R, double ut, bool branch2) {
    Point P;
    double Gk[7], I[7];
    radial_G(R, ut, Gk);
    for (int i = 0; i < 7; ++i) {
        if (R.su > 0.0) I[i] = branch2 ? 2.0 * R.Gtop[i] - R.G0[i] - Gk[i] : Gk[i] - R.G0[i];
        else I[i] = R.G0[i] - Gk[i];
    }
    const double lam = I[0];
    const double w = R.om * lam + R.w0;
    double mu2, inv, cn, j;
    polar_Phi(R, w, mu2, inv, cn, j);
    const double Imu2 = (mu2 - R.Ph0mu2) / R.om, Iinv = (inv - R.Ph0inv) / R.om;
    const double Ip = -I[3] / R.rp, Im = -I[4] / R.rm;
    const double a2 = R.a * R.a;
    P.u = ut;
    P.mu = R.mp * cn;
    P.dt = I[1] + 2.0 * I[2] + R.cp * Ip + R.cm * Im + a2 * Imu2;
    // d+ + d- = l: phi' = d+ (1/(1 - r+ u) - 1) + d- (1/(1 - r- u) - 1) + l/(1 - mu^2),
    // with 1/(1 - r u) - 1 = -u/(u - 1/r)
    P.dphi = -R.dp * I[5] - R.dm * I[6] + R.l * Iinv;
    P.lam = I[1] + a2 * Imu2;
    // turning points of mu: cn = +-1 at multiples of 2K; dn at multiples of K
    const double Kt = R.pkind ? R.Kth : 2.0 * R.Kth;
    P.tpm = (int32_t)(std::floor(w / Kt) - std::floor(R.w0 / Kt));
    P.tpr = branch2 ? 1 : 0;
    return P;
}

// Sample k (1-based, k <= R.last) of a ray set up above.
GKCF_HD Point sample(const CfRay& R, int k) {
    const bool branch2 = k > R.kmax;
    const double ut = branch2 ? 2.0 * R.ub - (R.u0 + (k - R.offset) * R.du) : R.u0 + (k - R.offset) * R.du;
    return point_at(R, ut, branch2);
}

}  // namespace gkcf
}  // namespace np
