// equator_cf.cuh -- equatorial crossings of one photon in closed form, for
// host and device: the near-critical rays of the mixed renderer, its ray
// reports, and np_geokerr_disk_crossings_*.
//
// With E = M = 1, constants l and q2, a start at u0 = 1/r and mu0 = cos(theta)
// with signs su = sign(du/dlambda) and sm = sign(dmu/dlambda):
//   polar   mu = mu+ cn(omega lambda + w0 | k) (q2 > 0) vanishes at the Mino
//           times lambda_j = ((2j + 1) K(k) - w0) / omega;
//   radial  in the Legendre variable S = sin^2(phi) of geokerr_cf.cuh (four
//           real roots: S = 0 at the turning point u2; two real roots and a
//           complex pair: S = sn^2 of the half argument, S = 1 at u2),
//           lambda = g |F(u) - F(u0)| up to the turning point u2 and
//           lambda_t + g |F(u2) - F(u)| after it,
// so each crossing is one Jacobi amplitude: F = F(u0) -+ lambda / g, S =
// sn^2(F | m), and u a ratio of linear (R4) or quadratic (R2C) terms in S.
// The ray ends at the horizon (an ingoing ray whose u2 lies at or inside
// it) or at u_far after its turning point (or at once, when it starts
// outward).  q2 < 0 rays keep the sign of mu and never cross the equator.
// The crossings are those of the Mino-time solver (GEOR with muf = 0,
// geokerr_original.f:2672-3136), taken by amplitude instead of by
// integration.
#pragma once

#include "geokerr_cf.cuh"

namespace np {
namespace gkcf {

struct EqX {
    int32_t status;     // 0: leaves through u_far, 1: falls into the horizon, -1: outside the closed forms
    int32_t n;          // crossings recorded
    double u_turn;      // radial turning point passed, 0 when none
};

// Legendre F of u (kinds kR4 and kR2C), the amplitude of radial_amp
GKCF_HD double radial_F(const CfRay& R, double u) {
    double S, C;
    if (R.kind == kR4) {
        const double u1 = R.r[0], u2 = R.r[1], u3 = R.r[2];
        const double den = (u2 - u1) * (u3 - u);
        S = (u3 - u1) * (u2 - u) / den;
        C = (u - u1) * (u3 - u2) / den;
    } else {
        const double u1 = R.r[0], u2 = R.r[1], A = R.r[2], B = R.r[3];
        const double den = (u2 - u) * B + (u - u1) * A;
        const double omx = 2.0 * (u - u1) * A / den, opx = 2.0 * (u2 - u) * B / den;
        const double X = 0.5 * (opx - omx);
        const double dnw = std::sqrt(R.mc + R.m * X * X);
        S = omx / (1.0 + dnw);
        C = X > 0.0 ? (X + dnw) / (1.0 + dnw) : R.mc * omx * opx / ((dnw - X) * (1.0 + dnw));
    }
    if (!(S > 0.0)) return 0.0;
    return std::sqrt(S) * cr::rf(C, C + R.mc * S, 1.0);
}

// u of the amplitude (S = sn^2, C = cn^2, D2 = dn^2): the inverse of the
// Legendre variable, each form free of cancellation where it is used (R4:
// from S near u2, from C near u1; R2C: (1 - X)/(1 + X) = S dn^2 / cn^2).
GKCF_HD double radial_u(const CfRay& R, double S, double C, double D2) {
    if (R.kind == kR4) {
        const double u1 = R.r[0], u2 = R.r[1], u3 = R.r[2];
        if (S <= 0.5) return (u2 * (u3 - u1) - S * u3 * (u2 - u1)) / ((u3 - u1) - S * (u2 - u1));
        return (u1 * (u3 - u2) + C * u3 * (u2 - u1)) / ((u3 - u2) + C * (u2 - u1));
    }
    const double u1 = R.r[0], u2 = R.r[1], A = R.r[2], B = R.r[3];
    const double t = B * S * D2;
    return (u2 * t + u1 * A * C) / (A * C + t);
}

// Crossings of the ray with u in [u_lo, u_hi], in order, at most kmax: u in
// xu, and (when non-null) the Mino time in xl and the branch in xb (0
// before the radial turning point, 1 after).  Crossings outside the window
// are passed over; the ray is followed until it ends.  a = 0, q2 = 0, a
// start inside the photon region or outside the escape radius, a ray so
// near the critical curve (~1e-9 relative) that its pair of roots is not
// resolved, and q2 < 0 radial motions other than those named above return
// status -1.
GKCF_HD EqX equator_crossings(double a, double l, double q2, double u0, double mu0, double su, double sm,
                              double u_far, double u_lo, double u_hi, int kmax, double* xu, double* xl,
                              int32_t* xb) {
    EqX o{-1, 0, 0.0};
    if (!(a != 0.0) || !(q2 != 0.0) || !(std::fabs(a) < 1.0) || !(u_far >= 0.0 && u_far < u0)) return o;
    const double uplus = 1.0 / (1.0 + std::sqrt(1.0 - a * a));
    const double B = a * a - l * l - q2, Kc = (l - a) * (l - a) + q2;
    const double c[5] = {1.0, 0.0, B, 2.0 * Kc, -a * a * q2};
    double rr[4], rho = 0.0, sigma = 0.0;
    const int nr = ::np::mino::real_roots(c, 4, rr, &rho, &sigma);
    if (q2 < 0.0) {
        // U > 0 at u = 0 and as u -> inf (c4 > 0): no real root, or two with
        // the start above both (ingoing: captured; outgoing: turns at r2 > 0
        // and is captured, else leaves) or below both (turns at r1, leaves)
        if (nr == 0) {
            o.status = su > 0.0 ? 1 : 0;
        } else if (nr == 2 && sigma > 0.0 && rr[1] < u0) {
            if (su > 0.0) o.status = 1;
            else if (rr[1] > u_far) { o.status = 1; o.u_turn = rr[1]; }
            else o.status = 0;
        } else if (nr == 2 && sigma > 0.0 && u0 < rr[0]) {
            o.status = 0;
            if (su > 0.0) o.u_turn = rr[0];
        }
        return o;
    }
    CfRay R;
    if (c[4] < 0.0 && (nr == 4 || (nr == 2 && sigma > 0.0)) && !polish_roots(a, l, q2, nr, rr, rho, sigma))
        return o;
    if (nr == 4 && c[4] < 0.0) {
        if (!reduce_r4(rr, c[4], u0, R)) return o;
    } else if (nr == 2 && sigma > 0.0 && c[4] < 0.0) {
        if (!reduce_r2c(rr, rho, sigma, c[4], u0, R)) return o;
    } else {
        return o;
    }
    const double u2 = R.r[1], g = R.g;
    const double Kr = cr::rf(0.0, R.mc, 1.0);
    const double F0 = radial_F(R, u0);
    const double Ft = R.kind == kR4 ? 0.0 : Kr;          // F at the turning point u2
    const double dir = R.kind == kR4 ? -1.0 : 1.0;       // sign of dF/du
    const bool turns = su > 0.0 && u2 < uplus;
    double lam_t = 0.0, lam_end;
    if (su > 0.0 && turns) {
        lam_t = g * std::fabs(Ft - F0);
        lam_end = lam_t + g * std::fabs(Ft - radial_F(R, u_far));
        o.status = 0;
        o.u_turn = u2;
    } else if (su > 0.0) {
        lam_end = g * std::fabs(radial_F(R, uplus) - F0);
        o.status = 1;
    } else {
        lam_end = g * std::fabs(F0 - radial_F(R, u_far));
        o.status = 0;
    }
    // polar motion (as setup(), q2 > 0): mu = mu+ cn(omega lambda + w0 | k)
    double mpos, a2mneg;
    polar_roots(a, l, q2, mu0, mpos, a2mneg);
    if (!(mpos > 0.0) || !(a2mneg < 0.0)) { o.status = -1; return o; }
    const double w2 = a * a * mpos - a2mneg;
    const double om = std::sqrt(w2), mth = a * a * mpos / w2, mcth = -a2mneg / w2;
    const double Kth = cr::rf(0.0, mcth, 1.0);
    double c0 = mu0 / std::sqrt(mpos);
    c0 = c0 > 1.0 ? 1.0 : (c0 < -1.0 ? -1.0 : c0);
    const Amp A0 = amp_make((1.0 - c0) * (1.0 + c0), c0 * c0, mth, mcth);
    const double F0p = c0 >= 0.0 ? A0.F : 2.0 * Kth - A0.F;
    const double w0 = -(sm < 0.0 ? -1.0 : 1.0) * F0p;
    if (!std::isfinite(lam_end) || !std::isfinite(om) || !(om > 0.0) || !std::isfinite(w0)) {
        o.status = -1;
        return o;
    }
    // zeros of cn: omega lambda + w0 = (2j + 1) K, w0 in [-2K, 2K]
    for (int j = -2; j < 256 && o.n < kmax; ++j) {
        const double lam = ((2.0 * j + 1.0) * Kth - w0) / om;
        if (!(lam > 0.0)) continue;
        if (!(lam < lam_end)) break;
        const bool out = turns && lam > lam_t;
        double F = out ? Ft - dir * (lam - lam_t) / g : F0 + (su > 0.0 ? dir : -dir) * lam / g;
        F = F < 0.0 ? 0.0 : (F > Kr ? Kr : F);
        double S, C, D2;
        jacobi(F, R.m, R.mc, Kr, S, C, D2);
        const double u = radial_u(R, S, C, D2);
        if (!(u >= u_lo && u <= u_hi)) continue;
        xu[o.n] = u;
        if (xl) xl[o.n] = lam;
        if (xb) xb[o.n] = out ? 1 : 0;
        o.n++;
    }
    return o;
}

// The azimuth change from the start at n crossings found above (xu, xb), from
// the closed-form points of geokerr_cf.cuh; NaN where the ray is outside
// them (a polar orbit through the pole with l != 0).
GKCF_HD void crossing_phi(double a, double l, double q2, double u0, double mu0, double su, double sm, double u_far,
                          int n, const double* xu, const int32_t* xb, double* xphi) {
    double mpos, a2mneg;
    polar_roots(a, l, q2, mu0, mpos, a2mneg);
    CfRay R;
    setup(a, l, q2, u0, u_far, mu0, su, sm, 1, 1, 0.5, mpos, a2mneg, R);
    const bool ok = R.kind == kR4 || R.kind == kR2C;
    for (int k = 0; k < n; ++k) xphi[k] = ok ? point_at(R, xu[k], xb[k] != 0).dphi : cr::nan_();
}

}  // namespace gkcf
}  // namespace np
