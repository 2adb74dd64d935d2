// mino_carlson.cuh -- Mino-time integrals of Kerr null geodesics in closed
// form with Carlson's R_F, for host and device (the semi-analytic route of
// GEOMU / GEOR, geokerr_original.f:771-1187, 2672-3136, for the cases below).
//
// With E = 1, l = L/E, q2 = Q/E^2 and u = 1/r, mu = cos(theta):
//   radial potential  U(u)  = 1 + B u^2 + 2 K u^3 - a^2 q2 u^4,
//   polar potential   M(mu) = q2 + B mu^2 - a^2 mu^4,
//   B = a^2 - l^2 - q2,  K = (l - a)^2 + q2,
// and Mino time is lambda = int du / sqrt(U) = int dmu / sqrt(M) along the ray.
//
// Polar (q2 > 0): M = a^2 (mu_+^2 - mu^2)(mu^2 + mu_-^2), so
//   int_0^mu dmu / sqrt(M) = (mu / sqrt(q2)) R_F(1, 1 - mu^2/mu_+^2, 1 + mu^2/mu_-^2)
// (DLMF 19.29.4 with two quadratic factors of the form 1 + c t^2), written
// with 1/mu_-^2 = 2 a^2 / (sqrt(D) - B), mu_+^2 = 2 q2 / (sqrt(D) - B),
// D = B^2 + 4 a^2 q2, which stay finite as a -> 0.
//
// Radial: on an interval between consecutive real roots r_j < u < r_j+1
// where U > 0, U = |c| prod_i (a_i + b_i u) with positive linear factors, and
//   int_y^x du / sqrt(U) = 2 R_F(U12^2, U13^2, U14^2) / sqrt(|c|),
//   U_ij = (X_i X_j Y_k Y_l + Y_i Y_j X_k X_l) / (x - y),
//   X_i = sqrt(a_i + b_i x), Y_i = sqrt(a_i + b_i y)
// (B. C. Carlson, "A table of elliptic integrals of the first kind", Math.
// Comp. 49 (1987) 595-606, eq. 2.1; DLMF 19.29.4-19.29.7).  A cubic U
// (a q2 = 0) uses a constant fourth factor.  The roots come from the
// Aberth-Ehrlich simultaneous iteration on the complex plane, polished by
// Newton steps.  With one complex root pair the segment integral is an
// incomplete F(phi | m) in the forms of Byrd & Friedman 259.00 (quartic) and
// 239.00 (cubic), evaluated with R_F.
#pragma once

#include <cmath>

#include "carlson.cuh"

namespace np {
namespace mino {

struct Cx { double re, im; };
NP_CARLSON_HD Cx cadd(Cx a, Cx b) { return Cx{a.re + b.re, a.im + b.im}; }
NP_CARLSON_HD Cx csub(Cx a, Cx b) { return Cx{a.re - b.re, a.im - b.im}; }
NP_CARLSON_HD Cx cmul(Cx a, Cx b) { return Cx{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
NP_CARLSON_HD Cx cdiv(Cx a, Cx b) {
    const double d = b.re * b.re + b.im * b.im;
    return Cx{(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
}

// Roots of sum_{k<=n} c[k] x^k (c[n] != 0, n <= 4) by Aberth-Ehrlich.
// Returns the number of roots found real (stored sorted in r) or -1 when the
// iteration did not converge; a complex pair is returned in (rho, sigma)
// (rho +- i sigma, sigma > 0) when there is one; `all` (optional) receives
// every root as found.
NP_CARLSON_HD int real_roots(const double* c, int n, double* r, double* rho = nullptr, double* sigma = nullptr,
                             Cx* all = nullptr) {
    Cx z[4];
    double R = 0.0;
    for (int k = 0; k < n; ++k) R = std::fmax(R, std::fabs(c[k] / c[n]));
    R = 1.0 + R;
    // starting points on the circle of radius R at the angles 0.4 + 2 pi k / n,
    // as literals (identical in host and device builds)
    const double c4[4][2] = {{0.9210609940028851, 0.3894183423086505}, {-0.38941834230865036, 0.9210609940028851},
                             {-0.9210609940028852, -0.3894183423086503}, {0.38941834230865063, -0.921060994002885}};
    const double c3[3][2] = {{0.9210609940028851, 0.3894183423086505}, {-0.7977766741403581, 0.60295304808712},
                             {-0.12328431986252686, -0.9923713903957702}};
    for (int k = 0; k < n; ++k) {
        const double* d = n == 4 ? c4[k] : (n == 3 ? c3[k] : c4[2 * k]);
        z[k] = Cx{R * d[0], R * d[1]};
    }
    // Converged when every correction is below 1e-15 relative, or when the
    // largest has stalled below 1e-11 (roots of a close pair, real or
    // complex, are only determined to the coefficients' rounding over their
    // separation, and the corrections then stay at that noise level).
    bool conv = false;
    double last = INFINITY;
    for (int it = 0; it < 200 && !conv; ++it) {
        conv = true;
        double worst = 0.0;
        for (int k = 0; k < n; ++k) {
            Cx p{c[n], 0.0}, dp{0.0, 0.0};
            for (int j = n - 1; j >= 0; --j) {
                dp = cadd(cmul(dp, z[k]), p);
                p = cadd(cmul(p, z[k]), Cx{c[j], 0.0});
            }
            if (p.re == 0.0 && p.im == 0.0) continue;
            const Cx w = cdiv(p, dp);
            Cx s{0.0, 0.0};
            for (int j = 0; j < n; ++j)
                if (j != k) s = cadd(s, cdiv(Cx{1.0, 0.0}, csub(z[k], z[j])));
            const Cx step = cdiv(w, csub(Cx{1.0, 0.0}, cmul(w, s)));
            z[k] = csub(z[k], step);
            const double rel = (std::fabs(step.re) + std::fabs(step.im)) /
                               (1.0 + std::fabs(z[k].re) + std::fabs(z[k].im));
            worst = std::fmax(worst, rel);
            if (rel > 1e-15) conv = false;
        }
        if (!conv && it >= 16 && worst < 1e-11 && worst > 0.25 * last) conv = true;
        last = worst;
    }
    if (!conv) return -1;
    if (all)
        for (int k = 0; k < n; ++k) all[k] = z[k];
    int m = 0;
    for (int k = 0; k < n; ++k) {
        if (std::fabs(z[k].im) > 1e-7 * (1.0 + std::fabs(z[k].re))) {
            if (rho && sigma && z[k].im > 0.0) { *rho = z[k].re; *sigma = z[k].im; }
            continue;
        }
        double x = z[k].re;
        for (int it = 0; it < 3; ++it) {       // Newton polish on the real polynomial
            double p = c[n], dp = 0.0;
            for (int j = n - 1; j >= 0; --j) { dp = dp * x + p; p = p * x + c[j]; }
            if (dp == 0.0) break;
            x -= p / dp;
        }
        r[m++] = x;
    }
    for (int i = 1; i < m; ++i)
        for (int j = i; j > 0 && r[j - 1] > r[j]; --j) { double t = r[j]; r[j] = r[j - 1]; r[j - 1] = t; }
    return m;
}

// Incomplete elliptic integral of the first kind F(phi | m) for phi in
// [0, pi] with Carlson's R_F (beyond pi/2, F = 2K - F(pi - phi)).
NP_CARLSON_HD double ell_f(double phi, double m) {
    const double s = std::sin(phi), c = std::cos(phi);
    const double f = s * carlson::rf(c * c, 1.0 - m * s * s, 1.0);
    return c >= 0.0 ? f : 2.0 * carlson::rf(0.0, 1.0 - m, 1.0) - f;
}

// int_{r1}^{u} du / sqrt((u - r1)(r2 - u)((u - rho)^2 + sigma^2)) for
// r1 <= u <= r2 (P. F. Byrd & M. D. Friedman, Handbook of Elliptic Integrals
// for Engineers and Scientists, 1971, 259.00): F(acos X | m) / sqrt(A B),
// A^2 = (r2 - rho)^2 + sigma^2, B^2 = (r1 - rho)^2 + sigma^2,
// X = ((r2 - u) B - (u - r1) A) / ((r2 - u) B + (u - r1) A),
// m = ((r2 - r1)^2 - (A - B)^2) / (4 A B).
NP_CARLSON_HD double quartic_pair_prim(double r1, double r2, double rho, double sigma, double u) {
    const double A = std::sqrt((r2 - rho) * (r2 - rho) + sigma * sigma);
    const double B = std::sqrt((r1 - rho) * (r1 - rho) + sigma * sigma);
    const double m = std::fmin(1.0, std::fmax(0.0, ((r2 - r1) * (r2 - r1) - (A - B) * (A - B)) / (4.0 * A * B)));
    const double p = (r2 - u) * B, q = (u - r1) * A;
    const double X = std::fmax(-1.0, std::fmin(1.0, (p - q) / (p + q)));
    return ell_f(std::acos(X), m) / std::sqrt(A * B);
}

// int_{r1}^{u} du / sqrt((u - r1)((u - rho)^2 + sigma^2)) for u >= r1
// (Byrd & Friedman 239.00): F(acos X | m) / sqrt(A), A^2 = (rho - r1)^2 +
// sigma^2, X = (A - (u - r1)) / (A + (u - r1)), m = (A + rho - r1) / (2 A).
NP_CARLSON_HD double cubic_pair_prim(double r1, double rho, double sigma, double u) {
    const double A = std::sqrt((rho - r1) * (rho - r1) + sigma * sigma);
    const double m = std::fmin(1.0, std::fmax(0.0, (A + rho - r1) / (2.0 * A)));
    const double d = u - r1;
    const double X = std::fmax(-1.0, std::fmin(1.0, (A - d) / (A + d)));
    return ell_f(std::acos(X), m) / std::sqrt(A);
}

// int_{u_a}^{u_b} du / sqrt(U(u)) for u_a, u_b in one interval of U > 0
// bounded by real roots (the Mino time of a monotonic radial segment).
NP_CARLSON_HD double mino_u(double a, double l, double q2, double u_a, double u_b) {
    const double B = a * a - l * l - q2, K = (l - a) * (l - a) + q2;
    double c[5] = {1.0, 0.0, B, 2.0 * K, -a * a * q2};
    int n = c[4] != 0.0 ? 4 : (c[3] != 0.0 ? 3 : 0);
    if (n == 0) return carlson::nan_();
    double r[4], rho = 0.0, sigma = 0.0;
    const int m = real_roots(c, n, r, &rho, &sigma);
    if (m < 0) return carlson::nan_();
    if (m == n - 2 && sigma > 0.0) {
        // one complex pair: two real roots bracketing u (quartic, c4 < 0) or
        // one real root below u (cubic, c3 > 0)
        const double ya = std::fmin(u_a, u_b), xb = std::fmax(u_a, u_b);
        if (n == 4) {
            if (!(c[4] < 0.0) || ya < r[0] - 1e-12 || xb > r[1] + 1e-12) return carlson::nan_();
            const double lo = r[0], hi = r[1];
            const double ga = quartic_pair_prim(lo, hi, rho, sigma, std::fmin(hi, std::fmax(lo, ya)));
            const double gb = quartic_pair_prim(lo, hi, rho, sigma, std::fmin(hi, std::fmax(lo, xb)));
            return std::fabs(gb - ga) / std::sqrt(-c[4]);
        }
        if (!(c[3] > 0.0) || ya < r[0] - 1e-12) return carlson::nan_();
        const double ga = cubic_pair_prim(r[0], rho, sigma, std::fmax(r[0], ya));
        const double gb = cubic_pair_prim(r[0], rho, sigma, std::fmax(r[0], xb));
        return std::fabs(gb - ga) / std::sqrt(c[3]);
    }
    if (m != n) return carlson::nan_();
    double y = std::fmin(u_a, u_b), x = std::fmax(u_a, u_b);
    if (x == y) return 0.0;
    // the interval (r_j, r_j+1) containing both endpoints (roots may be touched)
    const double tol = 1e-12 * (1.0 + std::fabs(x));
    double lo = -INFINITY, hi = INFINITY;
    for (int i = 0; i < m; ++i) {
        if (r[i] <= y + tol) lo = r[i];
        if (r[i] >= x - tol && hi == INFINITY) hi = r[i];
    }
    for (int i = 0; i < m; ++i)
        if (r[i] > lo && r[i] < hi) return carlson::nan_();      // a root inside the segment
    x = std::fmin(x, hi);
    y = std::fmax(y, lo);
    double ai[4], bi[4];
    int above = 0;
    for (int i = 0; i < m; ++i) {
        if (r[i] <= lo) { ai[i] = -r[i]; bi[i] = 1.0; }
        else { ai[i] = r[i]; bi[i] = -1.0; ++above; }
    }
    if (m == 3) { ai[3] = 1.0; bi[3] = 0.0; }
    // U = c_n prod (u - r_i) = c_n (-1)^above prod (a_i + b_i u) must be positive
    const double lead = c[n] * ((above & 1) ? -1.0 : 1.0);
    if (!(lead > 0.0)) return carlson::nan_();
    double X[4], Y[4];
    for (int i = 0; i < 4; ++i) {
        X[i] = std::sqrt(std::fmax(0.0, ai[i] + bi[i] * x));
        Y[i] = std::sqrt(std::fmax(0.0, ai[i] + bi[i] * y));
    }
    const double d = x - y;
    const double U12 = (X[0] * X[1] * Y[2] * Y[3] + Y[0] * Y[1] * X[2] * X[3]) / d;
    const double U13 = (X[0] * X[2] * Y[1] * Y[3] + Y[0] * Y[2] * X[1] * X[3]) / d;
    const double U14 = (X[0] * X[3] * Y[1] * Y[2] + Y[0] * Y[3] * X[1] * X[2]) / d;
    return 2.0 * carlson::rf(U12 * U12, U13 * U13, U14 * U14) / std::sqrt(lead);
}

// int_0^mu dmu / sqrt(M(mu)), q2 > 0 and |mu| <= mu_+ (odd in mu).
NP_CARLSON_HD double mino_mu_prim(double a, double l, double q2, double mu) {
    if (!(q2 > 0.0)) return carlson::nan_();
    const double B = a * a - l * l - q2;
    const double sD = std::sqrt(B * B + 4.0 * a * a * q2);
    const double den = sD - B;                          // > 0 for q2 > 0
    const double inv_mp2 = den / (2.0 * q2), inv_mm2 = 2.0 * a * a / den;
    const double m2 = mu * mu;
    const double t = 1.0 - m2 * inv_mp2;
    if (t < -1e-12) return carlson::nan_();
    return mu / std::sqrt(q2) * carlson::rf(1.0, std::fmax(0.0, t), 1.0 + m2 * inv_mm2);
}

// Mino time between mu_a and mu_b on one monotonic polar branch.
NP_CARLSON_HD double mino_mu(double a, double l, double q2, double mu_a, double mu_b) {
    return std::fabs(mino_mu_prim(a, l, q2, mu_b) - mino_mu_prim(a, l, q2, mu_a));
}

// Jacobi elliptic functions sn, cn, dn of argument u and parameter m = k^2
// (0 <= m <= 1) by the arithmetic-geometric mean and descending Landen
// transformation (Abramowitz & Stegun 16.4).
NP_CARLSON_HD void jacobi_sncndn(double u, double m, double& sn, double& cn, double& dn) {
    if (m < 1e-16) { sn = std::sin(u); cn = std::cos(u); dn = 1.0; return; }
    if (m > 1.0 - 1e-16) {
        const double t = std::tanh(u), c = 1.0 / std::cosh(u);
        sn = t; cn = c; dn = c;
        return;
    }
    double a[16], c[16];
    a[0] = 1.0;
    double b = std::sqrt(1.0 - m);
    c[0] = std::sqrt(m);
    int n = 0;
    while (n < 15 && std::fabs(c[n]) > 1e-16 * a[n]) {
        a[n + 1] = 0.5 * (a[n] + b);
        c[n + 1] = 0.5 * (a[n] - b);
        b = std::sqrt(a[n] * b);
        ++n;
    }
    double phi = std::ldexp(1.0, n) * a[n] * u;
    double phi_prev = phi;
    for (int j = n; j > 0; --j) {
        phi_prev = phi;
        phi = 0.5 * (phi + std::asin(c[j] / a[j] * std::sin(phi)));
    }
    sn = std::sin(phi);
    cn = std::cos(phi);
    dn = n > 0 ? cn / std::cos(phi_prev - phi) : std::sqrt(1.0 - m * sn * sn);
}

// Polar motion in closed form (the role of GEOMU's Jacobi inversion,
// geokerr_original.f:1147-1178, for q2 > 0):
//   mu(lambda) = mu_+ cn(omega lambda - sm F, k),
//   omega^2 = a^2 (mu_+^2 + mu_-^2),  k^2 = mu_+^2 / (mu_+^2 + mu_-^2),
//   F = F(acos(mu0 / mu_+), k) = sin(phi) R_F(cos^2 phi, 1 - k^2 sin^2 phi, 1),
// which solves (dmu/dlambda)^2 = M(mu) through its turning points; sm is the
// sign of dmu/dlambda at lambda = 0 (mu = cos(theta)).
NP_CARLSON_HD double mu_of_lambda(double a, double l, double q2, double mu0, double sm, double lam) {
    if (!(q2 > 0.0)) return carlson::nan_();
    const double B = a * a - l * l - q2;
    const double sD = std::sqrt(B * B + 4.0 * a * a * q2);
    const double den = sD - B;
    const double mp2 = 2.0 * q2 / den;                 // mu_+^2
    const double a2mp2 = a * a * mp2, a2mm2 = 0.5 * den;   // a^2 mu_+^2, a^2 mu_-^2
    const double w2 = a2mp2 + a2mm2;
    const double omega = std::sqrt(w2), m = a2mp2 / w2;
    const double mp = std::sqrt(mp2);
    const double c0 = std::fmax(-1.0, std::fmin(1.0, mu0 / mp));
    const double phi = std::acos(c0);
    const double s = std::sin(phi), c = std::cos(phi);
    // F(phi) for phi in [0, pi]: beyond pi/2, F = 2K - F(pi - phi)
    const double Fh = s * carlson::rf(c * c, 1.0 - m * s * s, 1.0);
    const double F = c0 >= 0.0 ? Fh : 2.0 * carlson::rf(0.0, 1.0 - m, 1.0) - Fh;
    double sn, cn, dn;
    jacobi_sncndn(omega * lam - (sm < 0.0 ? -1.0 : 1.0) * F, m, sn, cn, dn);
    return mp * cn;
}

// ---------------------------------------------------------------------------
// Equatorial crossings in closed form (GEOR with mu_f = 0,
// geokerr_original.f:2672-3136): the polar motion gives the Mino times of
// the crossings, lambda_j = ((2j + 1) K(k) + s_mu F) / omega; the radial
// motion is unfolded into G(u) = int_lo^u du / sqrt(U) on the interval of U > 0
// holding u0 (turning point at its upper end) and inverted at each lambda_j by
// safeguarded Newton steps (dG/du = 1/sqrt(U)).

struct RadialCF {
    double a, l, q2, c[5];
    int n;                      // degree of U
    double lo, hi;              // interval of U > 0 containing u0 (hi may be +inf)
    double r[4], rho, sigma;    // real roots, complex pair
    int nreal;
};

NP_CARLSON_HD double U_of(const RadialCF& R, double u) {
    double p = R.c[R.n];
    for (int j = R.n - 1; j >= 0; --j) p = p * u + R.c[j];
    return p;
}

NP_CARLSON_HD bool radial_setup(double a, double l, double q2, double u0, RadialCF& R) {
    const double B = a * a - l * l - q2, K = (l - a) * (l - a) + q2;
    R.a = a; R.l = l; R.q2 = q2;
    R.c[0] = 1.0; R.c[1] = 0.0; R.c[2] = B; R.c[3] = 2.0 * K; R.c[4] = -a * a * q2;
    R.n = R.c[4] != 0.0 ? 4 : (R.c[3] != 0.0 ? 3 : 0);
    if (R.n == 0) return false;
    R.rho = 0.0; R.sigma = 0.0;
    R.nreal = real_roots(R.c, R.n, R.r, &R.rho, &R.sigma);
    if (R.nreal < 0) return false;
    R.lo = -INFINITY; R.hi = INFINITY;
    for (int i = 0; i < R.nreal; ++i) {
        if (R.r[i] <= u0) R.lo = R.r[i];
        else if (R.hi == INFINITY) R.hi = R.r[i];
    }
    return R.lo > -INFINITY && U_of(R, u0) >= 0.0;
}

// G(u) = int_lo^u du / sqrt(U), lo <= u <= hi.
NP_CARLSON_HD double radial_G(const RadialCF& R, double u) {
    if (R.nreal == R.n - 2 && R.sigma > 0.0) {
        if (R.n == 4) return quartic_pair_prim(R.r[0], R.r[1], R.rho, R.sigma, u) / std::sqrt(-R.c[4]);
        return cubic_pair_prim(R.r[0], R.rho, R.sigma, u) / std::sqrt(R.c[3]);
    }
    return mino_u(R.a, R.l, R.q2, R.lo, u);
}

// u in [lo, min(hi, u_cap)] with G(u) = g (G increasing), by Newton steps
// kept inside a bisection bracket.
NP_CARLSON_HD double radial_invert(const RadialCF& R, double g, double u_cap) {
    double lo = R.lo, hi = std::fmin(R.hi, u_cap);
    double u = 0.5 * (lo + hi);
    for (int it = 0; it < 100; ++it) {
        const double f = radial_G(R, u) - g;
        if (f > 0.0) hi = u; else lo = u;
        const double Uu = U_of(R, u);
        double un = Uu > 0.0 ? u - f * std::sqrt(Uu) : 0.5 * (lo + hi);
        if (!(un > lo && un < hi)) un = 0.5 * (lo + hi);
        if (std::fabs(un - u) <= 1e-15 * (1.0 + std::fabs(u))) { u = un; break; }
        u = un;
    }
    return u;
}

// Crossing u values of a ray leaving (u0, mu0) with signs su (du/dlambda) and
// sm (dmu/dlambda): up to K crossings in xu, their count returned; the ray
// ends at the horizon u_h or when it has climbed out to u <= u_end.
// Returns -1 when the potentials are outside the closed forms (q2 <= 0).
NP_CARLSON_HD int equator_crossings_cf(double a, double u0, double mu0, double l, double q2, double su, double sm,
                                       double u_end, int K, double* xu) {
    if (!(q2 > 0.0)) return -1;
    RadialCF R;
    if (!radial_setup(a, l, q2, u0, R)) return -1;
    const double rp = 1.0 + std::sqrt(std::fmax(0.0, 1.0 - a * a));
    const double u_h = 1.0 / rp;
    // polar: mu = mu_+ cn(omega lambda - sm F, k)
    const double B = a * a - l * l - q2;
    const double sD = std::sqrt(B * B + 4.0 * a * a * q2);
    const double den = sD - B;
    const double mp2 = 2.0 * q2 / den;
    const double w2 = a * a * mp2 + 0.5 * den;
    const double omega = std::sqrt(w2), m = a * a * mp2 / w2;
    const double mp = std::sqrt(mp2);
    const double F = ell_f(std::acos(std::fmax(-1.0, std::fmin(1.0, mu0 / mp))), m);
    const double Kc = carlson::rf(0.0, 1.0 - m, 1.0);
    const double sgn = sm < 0.0 ? -1.0 : 1.0;
    // radial unfolding: s = G(u0) + su lambda on the way in, mirrored at hi
    const double G0 = radial_G(R, u0);
    const double Gmax = R.hi < INFINITY ? radial_G(R, R.hi) : INFINITY;
    const double Gh = u_h < R.hi ? radial_G(R, u_h) : INFINITY;      // horizon before the turning point
    const double Gend = radial_G(R, std::fmax(R.lo, u_end));
    int nx = 0;
    for (int j = -2; nx < K && j < 64; ++j) {
        const double lam = ((2.0 * j + 1.0) * Kc + sgn * F) / omega;
        if (lam < 0.0) continue;
        double sU = G0 + (su >= 0.0 ? 1.0 : -1.0) * lam;    // unfolded radial coordinate
        double g;
        if (su >= 0.0) {
            if (sU >= Gh) break;                             // fell through the horizon first
            g = sU <= Gmax ? sU : 2.0 * Gmax - sU;           // past the turning point: outward
            if (sU > Gmax && g <= Gend) break;               // escaped
        } else {
            g = sU;
            if (g <= Gend) break;
        }
        xu[nx++] = radial_invert(R, g, u_h);
    }
    return nx;
}

}  // namespace mino
}  // namespace np
