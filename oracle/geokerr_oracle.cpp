/*
 * geokerr_oracle.cpp -- CPU FP64 restatement of GEOKERR's geodesic sampler.
 *
 * TEST INFRASTRUCTURE ONLY (the checker of nullpath_gb300/csrc/geokerr.cu).
 *
 * GEOKERR (Dexter & Agol 2009; geokerr_port/reference/geokerr_original.f)
 * needs a Fortran compiler that this host does not have, so this file
 * restates its observable behaviour:
 *
 *   sampling        GEOKERR, geokerr_original.f:357-605 -- NUP points uniform in
 *                   u from UOUT, offset by OFFSET steps, in to the radial turning
 *                   point UB and back out (TPR = 1), MUFILL inactive (NPTS = 0);
 *   per point       mu, Delta t, Delta phi, affine lambda, mu/u turning counts
 *                   (GEOMU :771, GEOPHITIME :1648);
 *   C ABI           geokerr_eval_lambda, geokerr_estimate_periods,
 *                   geokerr_phi_omega (geokerr_eval_lambda.f90:57-306),
 *                   including its linear resampling onto a uniform lambda grid.
 *
 * The per-point values come from the Mino-time form of the Kerr null geodesic
 * (M = E = 1, l = L_z, q2 = Carter Q, u = 1/r, mu = cos theta):
 *   (du/dl)^2 = U(u) = 1 + (a^2 - q2 - l^2) u^2 + 2 ((a - l)^2 + q2) u^3 - a^2 q2 u^4
 *   (dmu/dl)^2 = M(mu) = q2 + (a^2 - q2 - l^2) mu^2 - a^2 mu^4
 *   dt/dl   = (r^2 + a^2)(r^2 + a^2 - a l)/Delta + a l - a^2 (1 - mu^2)
 *   dphi/dl = a (r^2 + a^2 - a l)/Delta + l/(1 - mu^2) - a
 *   dlambda_affine/dl = r^2 + a^2 mu^2
 * integrated in the second-order form u'' = U'(u)/2, mu'' = M'(mu)/2, which
 * has no singularity at turning points, by the Taylor-series method (order
 * 24, coefficients by automatic differentiation; Jorba & Zou, Experimental
 * Math. 14, 2005).  Each step is an exact power series, so sample points are
 * located by Newton iteration on the series and evaluated at full precision.
 * GEOKERR's case table (NCASE 1-8) is replaced by the physical rule it
 * encodes: UB is the first root of U met in the direction SU, else the
 * horizon u_+ (SU > 0) or 0 (SU < 0) with TPR = 0.
 *
 * Compile with -ffp-contract=off.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace geo {

constexpr int P = 24;          // series order
constexpr double TOL = 1e-17;  // per-step truncation target

struct Params {
    double a, l, q2;
    double A2, A3, A4;         // U(u) = 1 + A2 u^2 + A3 u^3 + A4 u^4
    double Q0, B2, B4;         // M(mu) = Q0 + B2 mu^2 + B4 mu^4 (Q0 = q2 for consistent inputs)
    double uplus;
};

// Constants of the motion and the polar potential GEOKERR integrates.  The
// roots mpos, mneg of M in mu^2 follow GEOMU's stable quadratic formula
// (geokerr_original.f:1121-1129); when mu0 lies outside them GEOMU moves the
// violated root to mu0^2 (:1134-1137 symmetric, :1163-1170 asymmetric), so
// the polar motion starts at a turning point of
//   M~(mu) = -a^2 (mu^2 - mpos)(mu^2 - mneg).
// a^2 mneg is carried instead of mneg so that a = 0 needs no special case.
static Params make_params(double a, double l, double q2, double mu0) {
    Params p;
    p.a = a; p.l = l; p.q2 = q2;
    p.A2 = a * a - q2 - l * l;
    p.A3 = 2.0 * ((a - l) * (a - l) + q2);
    p.A4 = -a * a * q2;
    p.uplus = 1.0 / (1.0 + std::sqrt(1.0 - a * a));
    const double a2 = a * a, ql2 = q2 + l * l, b = a2 - ql2;
    const double yy = -0.5 * (b + (b >= 0.0 ? 1.0 : -1.0) * std::sqrt(b * b + 4.0 * q2 * a2));
    double mpos, a2mneg;
    if (b < 0.0) { a2mneg = -yy; mpos = q2 / yy; }
    else { a2mneg = a2 * q2 / yy; mpos = -yy / a2; }
    if (mpos > 1.0) mpos = 1.0;
    if (a2mneg < 0.0 || a2 == 0.0) {               // symmetric: the orbit crosses the equator
        if (std::sqrt(mpos) < mu0) mpos = mu0 * mu0;
    } else {                                        // asymmetric (vortical)
        if (a2mneg > a2 * mu0 * mu0) a2mneg = a2 * mu0 * mu0;
        if (mu0 * mu0 > mpos) mpos = mu0 * mu0;
    }
    p.B4 = -a2;
    p.B2 = a2 * mpos + a2mneg;
    p.Q0 = -mpos * a2mneg;
    return p;
}

static inline double Ufun(const Params& p, double u) {
    return 1.0 + u * u * (p.A2 + u * (p.A3 + u * p.A4));
}
static inline double Mfun(const Params& p, double m) {
    double m2 = m * m;
    return p.Q0 + m2 * (p.B2 + m2 * p.B4);
}

// Potentials at the start, rounding below zero (a start on a turning point)
// clamped to zero; false when the start is forbidden.
static bool start_potentials(const Params& p, double u0, double mu0, double& U0, double& M0) {
    U0 = Ufun(p, u0);
    M0 = Mfun(p, mu0);
    const double m2 = mu0 * mu0, u2 = u0 * u0;
    const double su = 1.0 + u2 * (std::fabs(p.A2) + std::fabs(u0) * (std::fabs(p.A3) + std::fabs(u0) * std::fabs(p.A4)));
    const double sm = std::fabs(p.Q0) + m2 * (std::fabs(p.B2) + m2 * std::fabs(p.B4));
    if (!(U0 >= -1e-12 * su) || !(M0 >= -1e-12 * sm)) return false;
    U0 = std::max(U0, 0.0);
    M0 = std::max(M0, 0.0);
    return true;
}

// State at the start of a step.
// dpole = 1 - |mu| carried near the poles (pole form, see taylor); -1 when
// not carried.
struct State { double u, du, m, dm, t, ph, lam, dpole = -1.0; };

// Taylor coefficients of one step (value + derivatives / k!).
struct Series {
    double u[P + 1], m[P + 1], t[P + 1], ph[P + 1], lam[P + 1];
    double d[P + 1];     // d = 1 - s mu in the pole form
    bool pole = false;
};

static void taylor(const Params& p, const State& s, Series& c) {
    double U2[P + 1], U3[P + 1], M2[P + 1], M3[P + 1];
    double Du[P + 1], Nph[P + 1], phr[P + 1], Sm[P + 1], phm[P + 1];
    double U4[P + 1], Nt[P + 1], Dt[P + 1], tr[P + 1], iu2[P + 1];
    const double a = p.a, l = p.l, a2 = a * a;
    double W[P + 1];     // 1 - mu^2, from d in the pole form
    c.u[0] = s.u; c.u[1] = s.du;
    // pole form (|mu| >= 1/2): integrate d = 1 - s mu, d'' = -(B2 (1 - d) +
    // 2 B4 (1 - d)^3), so that 1 - mu^2 = d (2 - d) has d's relative accuracy
    c.pole = std::fabs(s.m) >= 0.5;
    const double sg = s.m >= 0.0 ? 1.0 : -1.0;
    double Pd[P + 1];    // 1 - d = s mu
    if (c.pole) {
        c.d[0] = s.dpole >= 0.0 ? s.dpole : 1.0 - std::fabs(s.m);
        c.d[1] = -sg * s.dm;
    } else {
        c.m[0] = s.m; c.m[1] = s.dm;
    }
    for (int k = 0; k <= P; ++k) {
        // series of u^2, u^3, mu^2, mu^3 up to order k (u_k, m_k known)
        double su2 = 0.0;
        for (int j = 0; j <= k; ++j) su2 += c.u[j] * c.u[k - j];
        U2[k] = su2;
        double su3 = 0.0;
        for (int j = 0; j <= k; ++j) su3 += U2[j] * c.u[k - j];
        U3[k] = su3;
        if (c.pole) {
            Pd[k] = (k == 0 ? 1.0 : 0.0) - c.d[k];
            c.m[k] = sg * Pd[k];
            double q2s = 0.0, dd = 0.0;
            for (int j = 0; j <= k; ++j) { q2s += Pd[j] * Pd[k - j]; dd += c.d[j] * c.d[k - j]; }
            M2[k] = q2s;
            W[k] = 2.0 * c.d[k] - dd;
            double q3s = 0.0;
            for (int j = 0; j <= k; ++j) q3s += M2[j] * Pd[k - j];
            M3[k] = q3s;                                // (1 - d)^3
        } else {
            double sm2 = 0.0;
            for (int j = 0; j <= k; ++j) sm2 += c.m[j] * c.m[k - j];
            M2[k] = sm2;
            double sm3 = 0.0;
            for (int j = 0; j <= k; ++j) sm3 += M2[j] * c.m[k - j];
            M3[k] = sm3;
            W[k] = (k == 0) ? (1.0 - c.m[0]) * (1.0 + c.m[0]) : -M2[k];
        }
        if (k + 2 <= P) {
            double fu = p.A2 * c.u[k] + 1.5 * p.A3 * U2[k] + 2.0 * p.A4 * U3[k];
            c.u[k + 2] = fu / ((k + 1.0) * (k + 2.0));
            if (c.pole) {
                double fd = -(p.B2 * Pd[k] + 2.0 * p.B4 * M3[k]);
                c.d[k + 2] = fd / ((k + 1.0) * (k + 2.0));
            } else {
                double fm = p.B2 * c.m[k] + 2.0 * p.B4 * M3[k];
                c.m[k + 2] = fm / ((k + 1.0) * (k + 2.0));
            }
        }
    }
    for (int k = 0; k <= P; ++k) {
        double s4 = 0.0;
        for (int j = 0; j <= k; ++j) s4 += U2[j] * U2[k - j];
        U4[k] = s4;
        Du[k] = (k == 0 ? 1.0 : 0.0) - 2.0 * c.u[k] + a2 * U2[k];             // Delta u^2
        Nph[k] = a * ((k == 0 ? 1.0 : 0.0) + (a2 - a * l) * U2[k]);
        Sm[k] = W[k];                                                         // 1 - mu^2
        Nt[k] = (k == 0 ? 1.0 : 0.0) + (2.0 * a2 - a * l) * U2[k] + a2 * (a2 - a * l) * U4[k];
        double sd = 0.0;
        for (int j = 0; j <= k; ++j) sd += U2[j] * Du[k - j];
        Dt[k] = sd;                                                            // u^2 * Delta u^2
    }
    // quotients by recursive series division
    for (int k = 0; k <= P; ++k) {
        double x = Nph[k], y = (k == 0 ? l : 0.0), z = Nt[k], w = (k == 0 ? 1.0 : 0.0);
        for (int j = 0; j < k; ++j) {
            x -= phr[j] * Du[k - j];
            y -= phm[j] * Sm[k - j];
            z -= tr[j] * Dt[k - j];
            w -= iu2[j] * U2[k - j];
        }
        phr[k] = x / Du[0];
        phm[k] = y / Sm[0];
        tr[k] = z / Dt[0];
        iu2[k] = w / U2[0];
    }
    c.t[0] = s.t; c.ph[0] = s.ph; c.lam[0] = s.lam;
    for (int k = 0; k < P; ++k) {
        double dt = tr[k] + (k == 0 ? a * l - a2 : 0.0) + a2 * M2[k];
        double dph = phr[k] + phm[k] - (k == 0 ? a : 0.0);
        double dl = iu2[k] + a2 * M2[k];
        c.t[k + 1] = dt / (k + 1.0);
        c.ph[k + 1] = dph / (k + 1.0);
        c.lam[k + 1] = dl / (k + 1.0);
    }
}

static inline double horner(const double* c, double h) {
    double v = c[P];
    for (int k = P - 1; k >= 0; --k) v = v * h + c[k];
    return v;
}
static inline double horner_d(const double* c, double h) {
    double v = P * c[P];
    for (int k = P - 1; k >= 1; --k) v = v * h + k * c[k];
    return v;
}


// Radius of convergence of a series estimated from coefficients eight
// orders apart (two estimates, so odd or even series are handled).
static double radius(const double* x) {
    double r = 1e300;
    for (int k = P - 1; k <= P; ++k)
        // the 8th root as three correctly rounded square roots, as the GPU solver
        if (x[k] != 0.0 && x[k - 8] != 0.0) r = std::min(r, std::sqrt(std::sqrt(std::sqrt(std::fabs(x[k - 8] / x[k])))));
    return r;
}

// Step size: a fixed fraction of the smallest radius of convergence, so the
// truncated term is ~0.2^24 ~ 1e-17 of the series scale (Jorba & Zou), and
// capped so that a step holds at most one radial and one polar turning point.
// `acc` includes the t, phi and lambda series (their poles sit at u = 0 and
// at the horizon).
static double step_size(const Params& p, const Series& c, const State& s, bool acc) {
    double R = std::min(radius(c.u), radius(c.m));
    if (acc) R = std::min(R, std::min(radius(c.t), std::min(radius(c.ph), radius(c.lam))));
    double h = 0.2 * R;
    double wu = std::sqrt(std::fabs(p.A2) + 3.0 * std::fabs(p.A3) * std::fabs(s.u) + 6.0 * std::fabs(p.A4) * s.u * s.u + 1e-30);
    double wm = std::sqrt(std::fabs(p.B2) + 6.0 * std::fabs(p.B4) * s.m * s.m + 1e-30);
    return std::min(h, 0.5 / std::max(wu, wm));
}

static State advance(const Series& c, double h) {
    State s;
    s.u = horner(c.u, h); s.du = horner_d(c.u, h);
    s.m = horner(c.m, h); s.dm = horner_d(c.m, h);
    s.dpole = c.pole ? horner(c.d, h) : -1.0;
    s.t = horner(c.t, h); s.ph = horner(c.ph, h); s.lam = horner(c.lam, h);
    return s;
}

// Root in [lo, hi] of g(s) = series(s) - target with g(lo), g(hi) of
// opposite sign (or zero); safeguarded Newton.
static double solve(const double* c, double target, double lo, double hi, bool deriv_series) {
    auto g = [&](double s) { return (deriv_series ? horner_d(c, s) : horner(c, s)) - target; };
    auto gp = [&](double s) {
        if (!deriv_series) return horner_d(c, s);
        double v = P * (P - 1.0) * c[P];
        for (int k = P - 1; k >= 2; --k) v = v * s + k * (k - 1.0) * c[k];
        return v;
    };
    double glo = g(lo);
    if (glo == 0.0) return lo;
    double x = 0.5 * (lo + hi);
    double ghi = g(hi);
    if (ghi != glo) x = lo + (hi - lo) * glo / (glo - ghi);
    for (int it = 0; it < 100; ++it) {
        double gx = g(x);
        if (gx == 0.0) return x;
        if ((gx > 0) == (glo > 0)) { lo = x; glo = gx; } else { hi = x; }
        double d = gp(x);
        double xn = (d != 0.0) ? x - gx / d : 0.5 * (lo + hi);
        if (!(xn > lo && xn < hi)) xn = 0.5 * (lo + hi);
        if (std::fabs(xn - x) <= 1e-16 * std::max(1.0, std::fabs(x)) || hi - lo <= 1e-300) { x = xn; break; }
        x = xn;
    }
    return x;
}

// GEOKERR output arrays.
struct Points {
    std::vector<double> u, mu, dt, dphi, lam;
    std::vector<int> tpm, tpr;
};

// GEOKERR (geokerr_original.f:357-605) with USEGEOR = .FALSE., PHIT = .TRUE.,
// NPTS = KEXT = 0 and UOUT = U0.  Returns the number of points written
// (NUP when the sample grid is regular, 0 otherwise).
static int geokerr(double u0, double uf, double mu0, double a, double l, double q2, double su, double sm,
                   int tpr_in, int nup, double offset, Points& out) {
    Params p = make_params(a, l, q2, mu0);
    out.u.assign(nup, 0.0); out.mu.assign(nup, 0.0); out.dt.assign(nup, 0.0);
    out.dphi.assign(nup, 0.0); out.lam.assign(nup, 0.0); out.tpm.assign(nup, 0); out.tpr.assign(nup, 0);
    double Uu0, Mm0;
    if (!start_potentials(p, u0, mu0, Uu0, Mm0)) return 0;
    State s0{u0, su * std::sqrt(Uu0), mu0, sm * std::sqrt(Mm0), 0.0, 0.0, 0.0};

    // Pass 1: find the radial turning point in the direction su before the
    // horizon (su > 0) or before u = 0 (su < 0).
    double ub;
    int tpr = tpr_in;
    {
        State s = s0;
        bool found = false;
        ub = su > 0 ? p.uplus : 0.0;
        for (int it = 0; it < 200000; ++it) {
            Series c;
            taylor(p, s, c);
            double h = step_size(p, c, s, false);
            State e = advance(c, h);
            bool past = su > 0 ? (e.u >= p.uplus) : (e.u <= 0.0);
            if ((e.du > 0) != (s.du > 0) && e.du != 0.0 && !past) {
                double st = solve(c.u, 0.0, 0.0, h, true);
                ub = horner(c.u, st);
                found = true;
                break;
            }
            if (past) break;
            s = e;
        }
        if (!found) tpr = 0;
    }
    // GEOMU stops UF at the turning point (geokerr_original.f:1077-1078, 1088-1089);
    // GEOKERR then traces back out to UOUT (:441-444).
    double UF = uf;
    if (tpr == 1 && ((su > 0 && UF > ub) || (su < 0 && UF < ub))) UF = ub;
    if (tpr == 1 && UF == ub) UF = u0;
    double du = ((ub - u0) >= 0 ? 1.0 : -1.0) * su * ((ub - u0) + (2.0 * tpr - 1.0) * (ub - UF));
    du /= (double)nup;
    int kmax = (du == 0.0) ? 0 : std::min((int)((ub - u0) / du + offset), nup);
    if (kmax <= 0 && tpr == 0) return 0;
    int last = tpr == 1 ? nup : std::min(kmax, nup);
    std::vector<double> targets(last);
    for (int k = 1; k <= last; ++k)
        targets[k - 1] = (k <= kmax) ? u0 + (k - offset) * du : 2.0 * ub - (u0 + (k - offset) * du);

    // Pass 2: walk the geodesic, emitting samples in path order.
    State s = s0;
    int next = 0, tp_mu = 0, tp_r = 0;
    for (int it = 0; it < 400000 && next < last; ++it) {
        Series c;
        taylor(p, s, c);
        double h = step_size(p, c, s, true);
        State e = advance(c, h);
        // turning points inside the step
        double s_r = -1.0, s_m = -1.0;
        if ((e.du > 0) != (s.du > 0) && e.du != 0.0 && s.du != 0.0) s_r = solve(c.u, 0.0, 0.0, h, true);
        if ((e.dm > 0) != (s.dm > 0) && e.dm != 0.0 && s.dm != 0.0) s_m = solve(c.m, 0.0, 0.0, h, true);
        // samples inside the step
        while (next < last) {
            const double ut = targets[next];
            const bool branch2 = next + 1 > kmax;
            double lo = 0.0, hi = h;
            if (s_r >= 0.0) {                  // the step holds the radial turning point
                if (branch2) lo = s_r; else hi = s_r;
            } else if (branch2 != (tp_r == 1)) {
                break;                         // sample lies beyond the turning point
            }
            double ga = horner(c.u, lo) - ut, gb = horner(c.u, hi) - ut;
            if ((ga > 0) == (gb > 0) && ga != 0.0 && gb != 0.0) break;   // not in this step
            double x = solve(c.u, ut, lo, hi, false);
            out.u[next] = ut;
            out.mu[next] = horner(c.m, x);
            out.dt[next] = horner(c.t, x);
            out.dphi[next] = horner(c.ph, x);
            out.lam[next] = horner(c.lam, x);
            out.tpm[next] = tp_mu + ((s_m >= 0.0 && x > s_m) ? 1 : 0);
            out.tpr[next] = branch2 ? 1 : 0;
            next++;
        }
        if (s_m >= 0.0) tp_mu++;
        if (s_r >= 0.0) tp_r = 1;
        bool past = su > 0 ? (e.u >= p.uplus) : (e.u <= 0.0);
        if (past) break;
        s = e;
    }
    return next == last ? last : 0;
}

}  // namespace geo

extern "C" {

// GEOKERR sampler: NUP points (u, mu, dt, dphi, lambda, tpm, tpr); returns
// the number of points written (0 on failure).
int npo_geokerr(double u0, double uf, double mu0, double a, double l, double q2, double su, double sm,
                int tpr, int nup, double offset, double* u, double* mu, double* dt, double* dphi,
                double* lam, int32_t* tpm, int32_t* tprv) {
    if (nup <= 0) return 0;
    geo::Points pts;
    int n = geo::geokerr(u0, uf, mu0, a, l, q2, su, sm, tpr, nup, offset, pts);
    for (int i = 0; i < n; ++i) {
        if (u) u[i] = pts.u[i];
        if (mu) mu[i] = pts.mu[i];
        if (dt) dt[i] = pts.dt[i];
        if (dphi) dphi[i] = pts.dphi[i];
        if (lam) lam[i] = pts.lam[i];
        if (tpm) tpm[i] = pts.tpm[i];
        if (tprv) tprv[i] = pts.tpr[i];
    }
    return n;
}

// geokerr_eval_lambda (geokerr_eval_lambda.f90:57-203).
void npo_geokerr_eval_lambda(double u0, double mu0, double uf, double a, double Lz, double Q2, double t0,
                             double lam0, double dlam, int S, double* u, double* mu, double* t, double* phi,
                             double* affine, int* tpmi, int* tpri, int* info) {
    *info = 0;
    if (S <= 0) { *info = 1; return; }
    const int nup = S;
    const double su = (uf - u0) >= 0.0 ? 1.0 : -1.0;
    const double sm = mu0 <= 0.0 ? 1.0 : -1.0;
    geo::Points pts;
    int n = geo::geokerr(u0, uf, mu0, a, Lz, Q2, su, sm, 1, nup, 0.5, pts);
    if (n != nup) {
        *info = 2;
        for (int i = 0; i < S; ++i) u[i] = mu[i] = t[i] = phi[i] = affine[i] = NAN;
        *tpmi = -1; *tpri = -1;
        return;
    }
    const std::vector<double>& L = pts.lam;
    const double base = L[0];
    int j = 0;   // 0-based counterpart of the f90 index j
    for (int i = 0; i < S; ++i) {
        double lamk = lam0 + dlam * (double)i;
        affine[i] = lamk;
        while (j < nup - 1 && (L[j + 1] - base) < lamk - 1.0e-30) j++;
        if (lamk <= L[0] - base) {
            u[i] = pts.u[0]; mu[i] = pts.mu[0]; t[i] = t0 + pts.dt[0]; phi[i] = pts.dphi[0];
        } else if (lamk >= L[nup - 1] - base) {
            u[i] = pts.u[nup - 1]; mu[i] = pts.mu[nup - 1]; t[i] = t0 + pts.dt[nup - 1]; phi[i] = pts.dphi[nup - 1];
        } else {
            double x0 = L[j] - base, x1 = L[j + 1] - base;
            double w = (x1 <= x0 + 1.0e-30) ? 0.0 : (lamk - x0) / (x1 - x0);
            u[i] = (1.0 - w) * pts.u[j] + w * pts.u[j + 1];
            mu[i] = (1.0 - w) * pts.mu[j] + w * pts.mu[j + 1];
            t[i] = t0 + ((1.0 - w) * pts.dt[j] + w * pts.dt[j + 1]);
            phi[i] = (1.0 - w) * pts.dphi[j] + w * pts.dphi[j + 1];
        }
        if (i == 0) { u[i] = u0; mu[i] = mu0; }
    }
    int tm = -1, tr = -1;
    for (int jj = 0; jj < nup; ++jj) {
        if (tm < 0 && pts.tpm[jj] > 0)
            for (int i = 0; i < S; ++i) if (affine[i] >= L[jj] - base) { tm = i; break; }
        if (tr < 0 && pts.tpr[jj] > 0)
            for (int i = 0; i < S; ++i) if (affine[i] >= L[jj] - base) { tr = i; break; }
        if (tm >= 0 && tr >= 0) break;
    }
    *tpmi = tm; *tpri = tr;
}

// geokerr_estimate_periods (geokerr_eval_lambda.f90:205-297).
void npo_geokerr_estimate_periods(double u0, double mu0, double a, double Lz, double Q2, double* Tr,
                                  double* Ttheta, int* info) {
    const int nup = 4096;
    const double sm = mu0 <= 0.0 ? 1.0 : -1.0;
    geo::Points pts;
    int n = geo::geokerr(u0, u0, mu0, a, Lz, Q2, 1.0, sm, 1, nup, 0.5, pts);
    *Tr = -1.0; *Ttheta = -1.0; *info = 0;
    if (n <= 0) return;
    const double base = pts.lam[0];
    int m1 = -1, m2 = -1, r1 = -1, r2 = -1, pm = 0, pr = 0;
    for (int j = 0; j < n; ++j) {
        if (m1 < 0 && pm < 1 && pts.tpm[j] >= 1) m1 = j;
        if (m2 < 0 && pm < 2 && pts.tpm[j] >= 2) m2 = j;
        if (r1 < 0 && pr < 1 && pts.tpr[j] >= 1) r1 = j;
        if (r2 < 0 && pr < 2 && pts.tpr[j] >= 2) r2 = j;
        pm = std::max(pm, (int)pts.tpm[j]); pr = std::max(pr, (int)pts.tpr[j]);
        if (m2 >= 0 && r2 >= 0) break;
    }
    if (r1 >= 0 && r2 >= 0) *Tr = 2.0 * std::max(1e-18, (pts.lam[r2] - base) - (pts.lam[r1] - base));
    if (m1 >= 0 && m2 >= 0) *Ttheta = 2.0 * std::max(1e-18, (pts.lam[m2] - base) - (pts.lam[m1] - base));
}

// Exact Mino-time samples lam0 + k dlam (geokerr_stream_cuda conventions:
// du/dlambda sign from uf - u0, dmu/dlambda sign -1 for mu0 > 0; samples
// past the horizon or u = 0 repeat the last state; sample 0 seeded exactly).
int npo_geokerr_stream(double u0, double uf, double mu0, double a, double L, double Q2, double lam0, double dlam,
                       int S, double* u, double* mu, double* t, double* phi, double* aff) {
    using namespace geo;
    if (S <= 0) return -1;
    const double su = (uf - u0) >= 0.0 ? 1.0 : -1.0;
    const double sm = mu0 <= 0.0 ? 1.0 : -1.0;
    Params p = make_params(a, L, Q2, mu0);
    double U0, M0;
    start_potentials(p, u0, mu0, U0, M0);
    State s{u0, su * std::sqrt(U0), mu0, sm * std::sqrt(M0), 0, 0, 0};
    double lam_a = 0.0;
    int k = 0;
    while (k < S && lam0 + k * dlam < 0.0) { u[k] = u0; mu[k] = mu0; t[k] = 0; phi[k] = 0; aff[k] = lam0 + k * dlam; ++k; }
    for (int it = 0; it < 400000 && k < S; ++it) {
        Series c;
        taylor(p, s, c);
        double h = step_size(p, c, s, true);
        while (k < S) {
            double lk = lam0 + k * dlam;
            if (lk > lam_a + h) break;
            double x = lk - lam_a;
            u[k] = horner(c.u, x); mu[k] = horner(c.m, x); t[k] = horner(c.t, x); phi[k] = horner(c.ph, x); aff[k] = lk;
            ++k;
        }
        State e = advance(c, h);
        if (e.u >= p.uplus || e.u <= 0.0 || !std::isfinite(e.t)) {
            double uu = k > 0 ? u[k - 1] : u0, mm = k > 0 ? mu[k - 1] : mu0;
            double tt = k > 0 ? t[k - 1] : 0.0, pp = k > 0 ? phi[k - 1] : 0.0;
            for (; k < S; ++k) { u[k] = uu; mu[k] = mm; t[k] = tt; phi[k] = pp; aff[k] = lam0 + k * dlam; }
            break;
        }
        s = e;
        lam_a += h;
    }
    u[0] = u0; mu[0] = mu0;
    return 0;
}

// First K equatorial crossings (mu = 0; GEOR with muf = 0) of a ray leaving
// (u0, mu0): u and phi of each, count returned (-1 when the start is
// forbidden).  The ray ends at the horizon, at u <= u_end or after K crossings.
int npo_geokerr_crossings(double u0, double mu0, double a, double l, double q2, double su, double sm, double u_end,
                          int K, double* xu, double* xphi) {
    using namespace geo;
    for (int k = 0; k < K; ++k) { xu[k] = 0.0; xphi[k] = 0.0; }
    Params p = make_params(a, l, q2, mu0);
    double U0, M0;
    if (!start_potentials(p, u0, mu0, U0, M0)) return -1;
    State s{u0, su * std::sqrt(U0), mu0, sm * std::sqrt(M0), 0, 0, 0};
    int found = 0;
    for (int it = 0; it < 200000 && found < K; ++it) {
        Series c;
        taylor(p, s, c);
        double h = step_size(p, c, s, true);
        State e = advance(c, h);
        if ((s.m > 0.0) != (e.m > 0.0) && s.m != 0.0) {
            double x = solve(c.m, 0.0, 0.0, h, false);
            double ux = horner(c.u, x);
            if (ux > u_end && ux < p.uplus) { xu[found] = ux; xphi[found] = horner(c.ph, x); ++found; }
        }
        if (e.u >= p.uplus || e.u <= u_end || !std::isfinite(e.ph)) break;
        s = e;
    }
    return found;
}

// State at Mino time lam of the ray leaving (u0, mu0) with signs su, sm:
// out = (u, mu, t, phi); returns 1, or 0 when the ray reached the horizon
// or u = 0 first (out = the last state before it) or the start is
// forbidden (out = NaN).  Restates np_geokerr_final_state_host.
int npo_geokerr_final(double u0, double mu0, double a, double l, double q2, double su, double sm, double lam,
                      double* out) {
    using namespace geo;
    const double nan_v = std::nan("");
    out[0] = out[1] = out[2] = out[3] = nan_v;
    if (!(std::fabs(a) < 1.0) || !(lam >= 0.0)) return 0;
    Params p = make_params(a, l, q2, mu0);
    double U0, M0;
    if (!start_potentials(p, u0, mu0, U0, M0)) return 0;
    State s{u0, (su >= 0.0 ? 1.0 : -1.0) * std::sqrt(U0), mu0, (sm >= 0.0 ? 1.0 : -1.0) * std::sqrt(M0), 0, 0, 0};
    double lam_a = 0.0;
    for (int it = 0; it < 400000; ++it) {
        Series c;
        taylor(p, s, c);
        double h = step_size(p, c, s, true);
        if (lam_a + h >= lam) {
            double x = lam - lam_a;
            out[0] = horner(c.u, x); out[1] = horner(c.m, x); out[2] = horner(c.t, x); out[3] = horner(c.ph, x);
            return 1;
        }
        State e = advance(c, h);
        if (e.u >= p.uplus || e.u <= 0.0 || !std::isfinite(e.t)) break;
        s = e;
        lam_a += h;
    }
    out[0] = s.u; out[1] = s.m; out[2] = s.t; out[3] = s.ph;
    return 0;
}

// Mino time from u0 to the first arrival at uf of the ray leaving with
// signs su, sm (after_tp != 0: the first arrival after the radial turning
// point); returns 1 with *lam, or 0 when uf is not reached that way.
// Restates compute_mino_time_batch_cuda / compute_geokerr_complete_cuda.
int npo_geokerr_mino_time(double u0, double uf, double mu0, double a, double l, double q2, double su, double sm,
                          int after_tp, double* lam) {
    using namespace geo;
    *lam = std::nan("");
    if (!(std::fabs(a) < 1.0)) return 0;
    Params p = make_params(a, l, q2, mu0);
    double U0, M0;
    if (!start_potentials(p, u0, mu0, U0, M0)) return 0;
    State s{u0, (su >= 0.0 ? 1.0 : -1.0) * std::sqrt(U0), mu0, (sm >= 0.0 ? 1.0 : -1.0) * std::sqrt(M0), 0, 0, 0};
    double lam_a = 0.0;
    bool passed = false;
    for (int it = 0; it < 400000; ++it) {
        Series c;
        taylor(p, s, c);
        double h = step_size(p, c, s, false);
        State e = advance(c, h);
        double s_r = -1.0;
        if ((e.du > 0) != (s.du > 0) && e.du != 0.0 && s.du != 0.0) s_r = solve(c.u, 0.0, 0.0, h, true);
        const double lo[2] = {0.0, s_r}, hi[2] = {s_r >= 0.0 ? s_r : h, h};
        for (int g = 0; g < (s_r >= 0.0 ? 2 : 1); ++g) {
            if (after_tp && !(passed || g == 1)) continue;
            double ga = horner(c.u, lo[g]) - uf, gb = horner(c.u, hi[g]) - uf;
            if (ga == 0.0 || gb == 0.0 || (ga > 0) != (gb > 0)) {
                *lam = lam_a + solve(c.u, uf, lo[g], hi[g], false);
                return 1;
            }
        }
        if (s_r >= 0.0) passed = true;
        if (e.u >= p.uplus || e.u <= 0.0) return 0;
        s = e;
        lam_a += h;
    }
    return 0;
}

// geokerr_phi_omega (geokerr_eval_lambda.f90:299-306): dphi/dlambda at u0.
double npo_geokerr_phi_omega(double u0, double mu0, double a, double Lz, double Q2) {
    (void)Q2;
    double r = std::max(1e-12, 1.0 / std::max(1e-12, u0));
    double Delta = std::max(1e-30, r * r - 2.0 * r + a * a);
    double sin2 = std::max(1e-30, 1.0 - mu0 * mu0);
    return a * (((r * r + a * a) - a * Lz) / Delta) + Lz / sin2 - a;
}

}  // extern "C"
