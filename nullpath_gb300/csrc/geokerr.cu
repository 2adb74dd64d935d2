// geokerr.cu -- GEOKERR-equivalent Mino-time geodesic solver on sm_103a, behind
// the C ABI of include/geokerr_c_api.h.
//
// One geodesic per thread, FP64 throughout (this is one of the FP64 islands
// of the design: the whole solver is short and must hold 1e-12).  The
// equations, in Mino time l with M = E = 1, u = 1/r, mu = cos(theta):
//   u''  = U'(u)/2,  U(u) = 1 + A2 u^2 + A3 u^3 + A4 u^4
//          A2 = a^2 - q2 - l^2, A3 = 2((a - l)^2 + q2), A4 = -a^2 q2
//   mu'' = M'(mu)/2, M(mu) = Q0 + B2 mu^2 + B4 mu^4 (GEOKERR's polar potential,
//          with its rule that a mu0 outside the polar roots becomes the
//          turning point, geokerr_original.f:1121-1170)
//   t'   = (r^2 + a^2)(r^2 + a^2 - a l)/Delta + a l - a^2 (1 - mu^2)
//   phi' = a (r^2 + a^2 - a l)/Delta + l/(1 - mu^2) - a
//   lambda_affine' = r^2 + a^2 mu^2
// are advanced by order-24 Taylor series whose coefficients come from the
// recurrences of the polynomial right-hand sides and of series division
// (Jorba & Zou 2005).  A step is a fixed fraction of the smallest radius of
// convergence, so every step is exact to rounding and sample points are found
// by Newton iteration on the step's series.  The sampling logic is GEOKERR's
// (geokerr_original.f:357-605): NUP points uniform in u from U0, offset by
// OFFSET steps, in to the radial turning point UB and back out.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <algorithm>
#include <vector>

#include <cuda_runtime.h>

#include "geokerr_c_api.h"
#include "geokerr_cf.cuh"
#include "equator_cf.cuh"
#include "np_render.h"

void np_record_error(const char* msg);

namespace {

thread_local std::string g_gk_error;

int gk_fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_gk_error = buf;
    np_record_error(buf);
    return code;
}

constexpr int P = 24;

struct Par {
    double a, l, A2, A3, A4, Q0, B2, B4, uplus;
    double mpos, a2mneg;   // polar roots in mu^2 (a^2 times the second)
};

// Constants of the motion and GEOKERR's polar potential (roots of M in mu^2
// by the stable quadratic formula; a violated root moves to mu0^2).  a^2 mneg
// is carried instead of mneg so that a = 0 needs no special case.
__host__ __device__ Par make_par(double a, double l, double q2, double mu0) {
    Par p;
    p.a = a; p.l = l;
    p.A2 = a * a - q2 - l * l;
    p.A3 = 2.0 * ((a - l) * (a - l) + q2);
    p.A4 = -a * a * q2;
    p.uplus = 1.0 / (1.0 + sqrt(1.0 - a * a));
    const double a2 = a * a;
    double mpos, a2mneg;
    np::gkcf::polar_roots(a, l, q2, mu0, mpos, a2mneg);
    p.mpos = mpos;
    p.a2mneg = a2mneg;
    p.B4 = -a2;
    p.B2 = a2 * mpos + a2mneg;
    p.Q0 = -mpos * a2mneg;
    return p;
}

__host__ __device__ __forceinline__ double Uof(const Par& p, double u) { return 1.0 + u * u * (p.A2 + u * (p.A3 + u * p.A4)); }
__host__ __device__ __forceinline__ double Mof(const Par& p, double m) { double m2 = m * m; return p.Q0 + m2 * (p.B2 + m2 * p.B4); }

// Potentials at the start point, with rounding below zero (a start on a
// turning point, as GEOMU's moved polar root makes it) clamped to zero;
// returns false when the start is genuinely forbidden.
__host__ __device__ __forceinline__ bool start_potentials(const Par& p, double u0, double mu0, double& U0, double& M0) {
    U0 = Uof(p, u0);
    M0 = Mof(p, mu0);
    const double m2 = mu0 * mu0, u2 = u0 * u0;
    const double su = 1.0 + u2 * (fabs(p.A2) + fabs(u0) * (fabs(p.A3) + fabs(u0) * fabs(p.A4)));
    const double sm = fabs(p.Q0) + m2 * (fabs(p.B2) + m2 * fabs(p.B4));
    if (!(U0 >= -1e-12 * su) || !(M0 >= -1e-12 * sm)) return false;
    U0 = fmax(U0, 0.0);
    M0 = fmax(M0, 0.0);
    return true;
}

// d = 1 - |mu| carried accurately near the poles (see taylor); -1 when not
// carried (it is then formed from mu where needed).
struct St { double u, du, m, dm, t, ph, lam, d = -1.0; };
// Series of one step plus the scratch series of the recurrences; one object
// per thread, owned by the kernel frame (no callee-local arrays).
struct Ser {
    double u[P + 1], m[P + 1], t[P + 1], ph[P + 1], lam[P + 1];
    double d[P + 1], P1[P + 1], Sd[P + 1];   // polar series of the pole form
    bool pole;
    double U2[P + 1], M2[P + 1], U3[P + 1], M3[P + 1];
    double Du[P + 1], Sm[P + 1], Dt[P + 1], phr[P + 1], phm[P + 1], tr[P + 1], iu2[P + 1];
    double U4[P + 1], Nph[P + 1], Nt[P + 1];
};

// Taylor coefficients of one step; `acc` adds the t, phi, lambda series.
//
// Pole form.  phi's polar rate is L / (1 - mu^2), and near a pole 1 - mu^2
// formed from mu keeps only the absolute accuracy of mu: for a ray that turns
// at 1 - mu_+ ~ 1e-5 that is a relative error of 1e-11 in the rate.  Where
// |mu| >= 1/2 the polar motion is therefore integrated in d = 1 - s mu (s =
// sign mu), whose equation d'' = -(B2 (1 - d) + 2 B4 (1 - d)^3) is again a
// polynomial, and 1 - mu^2 = d (2 - d) keeps d's relative accuracy.  The mu
// series is formed from d's, so every other use is unchanged.
__host__ __device__ __forceinline__ void taylor(const Par& p, const St& s, Ser& c, bool acc) {
    double* U2 = c.U2;
    double* M2 = c.M2;
    double* U3 = c.U3;
    double* M3 = c.M3;
    c.u[0] = s.u; c.u[1] = s.du;
    c.pole = fabs(s.m) >= 0.5;
    const double sg = s.m >= 0.0 ? 1.0 : -1.0;
    if (c.pole) {
        c.d[0] = s.d >= 0.0 ? s.d : 1.0 - fabs(s.m);      // exact for |mu| >= 1/2 (Sterbenz)
        c.d[1] = -sg * s.dm;
    } else {
        c.m[0] = s.m; c.m[1] = s.dm;
    }
    for (int k = 0; k <= P; ++k) {
        double su2 = 0.0;
        for (int j = 0; j <= k; ++j) su2 += c.u[j] * c.u[k - j];
        U2[k] = su2;
        double su3 = 0.0;
        for (int j = 0; j <= k; ++j) su3 += U2[j] * c.u[k - j];
        U3[k] = su3;
        if (c.pole) {
            c.P1[k] = (k == 0 ? 1.0 : 0.0) - c.d[k];         // 1 - d = s mu
            c.m[k] = sg * c.P1[k];
            double sm2 = 0.0, sd2 = 0.0;
            for (int j = 0; j <= k; ++j) { sm2 += c.P1[j] * c.P1[k - j]; sd2 += c.d[j] * c.d[k - j]; }
            M2[k] = sm2;
            c.Sd[k] = 2.0 * c.d[k] - sd2;                      // 1 - mu^2 = d (2 - d)
            double sm3 = 0.0;
            for (int j = 0; j <= k; ++j) sm3 += M2[j] * c.P1[k - j];
            M3[k] = sm3;                                       // (1 - d)^3
        } else {
            double sm2 = 0.0;
            for (int j = 0; j <= k; ++j) sm2 += c.m[j] * c.m[k - j];
            M2[k] = sm2;
            double sm3 = 0.0;
            for (int j = 0; j <= k; ++j) sm3 += M2[j] * c.m[k - j];
            M3[k] = sm3;
            c.Sd[k] = (k == 0) ? (1.0 - c.m[0]) * (1.0 + c.m[0]) : -M2[k];
        }
        if (k + 2 <= P) {
            const double fu = p.A2 * c.u[k] + 1.5 * p.A3 * U2[k] + 2.0 * p.A4 * U3[k];
            c.u[k + 2] = fu / ((k + 1.0) * (k + 2.0));
            if (c.pole) {
                const double fd = -(p.B2 * c.P1[k] + 2.0 * p.B4 * M3[k]);
                c.d[k + 2] = fd / ((k + 1.0) * (k + 2.0));
            } else {
                const double fm = p.B2 * c.m[k] + 2.0 * p.B4 * M3[k];
                c.m[k + 2] = fm / ((k + 1.0) * (k + 2.0));
            }
        }
    }

    if (!acc) return;
    const double a = p.a, l = p.l, a2 = a * a;
    double *Du = c.Du, *Sm = c.Sm, *Dt = c.Dt, *phr = c.phr, *phm = c.phm, *tr = c.tr, *iu2 = c.iu2;
    double* U4 = c.U4;
    double* Nph = c.Nph;
    double* Nt = c.Nt;
    for (int k = 0; k <= P; ++k) {
        double s4 = 0.0;
        for (int j = 0; j <= k; ++j) s4 += U2[j] * U2[k - j];
        U4[k] = s4;
        Du[k] = (k == 0 ? 1.0 : 0.0) - 2.0 * c.u[k] + a2 * U2[k];            // Delta u^2
        Nph[k] = a * ((k == 0 ? 1.0 : 0.0) + (a2 - a * l) * U2[k]);
        // 1 - mu^2: from d in the pole form (full relative accuracy), else
        // (1 - mu)(1 + mu) at order 0
        Sm[k] = c.Sd[k];
        Nt[k] = (k == 0 ? 1.0 : 0.0) + (2.0 * a2 - a * l) * U2[k] + a2 * (a2 - a * l) * U4[k];
        double sd = 0.0;
        for (int j = 0; j <= k; ++j) sd += U2[j] * Du[k - j];
        Dt[k] = sd;                                                           // u^2 Delta u^2
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
        const double dt = tr[k] + (k == 0 ? a * l - a2 : 0.0) + a2 * M2[k];
        const double dph = phr[k] + phm[k] - (k == 0 ? a : 0.0);
        const double dl = iu2[k] + a2 * M2[k];
        c.t[k + 1] = dt / (k + 1.0);
        c.ph[k + 1] = dph / (k + 1.0);
        c.lam[k + 1] = dl / (k + 1.0);
    }
}

__host__ __device__ __forceinline__ double hv(const double* c, double h) {
    double v = c[P];
    for (int k = P - 1; k >= 0; --k) v = v * h + c[k];
    return v;
}
__host__ __device__ __forceinline__ double hd(const double* c, double h) {
    double v = P * c[P];
    for (int k = P - 1; k >= 1; --k) v = v * h + k * c[k];
    return v;
}
__host__ __device__ __forceinline__ double hdd(const double* c, double h) {
    double v = P * (P - 1.0) * c[P];
    for (int k = P - 1; k >= 2; --k) v = v * h + k * (k - 1.0) * c[k];
    return v;
}

__host__ __device__ __forceinline__ double radius(const double* x) {
    double r = 1e300;
    for (int k = P - 1; k <= P; ++k)
        // the 8th root as three correctly rounded square roots (pow is not
        // correctly rounded, and its step sizes would differ between libms)
        if (x[k] != 0.0 && x[k - 8] != 0.0) r = fmin(r, sqrt(sqrt(sqrt(fabs(x[k - 8] / x[k])))));
    return r;
}

// 0.2 x the smallest radius of convergence (truncation ~0.2^24 of the series
// scale), capped so a step holds at most one radial and one polar turning point.
__host__ __device__ double step_size(const Par& p, const Ser& c, const St& s, bool acc) {
    double R = fmin(radius(c.u), radius(c.m));
    if (acc) R = fmin(R, fmin(radius(c.t), fmin(radius(c.ph), radius(c.lam))));
    double wu = sqrt(fabs(p.A2) + 3.0 * fabs(p.A3) * fabs(s.u) + 6.0 * fabs(p.A4) * s.u * s.u + 1e-30);
    double wm = sqrt(fabs(p.B2) + 6.0 * fabs(p.B4) * s.m * s.m + 1e-30);
    return fmin(0.2 * R, 0.5 / fmax(wu, wm));
}

__host__ __device__ St advance(const Ser& c, double h, bool acc) {
    St s;
    s.u = hv(c.u, h); s.du = hd(c.u, h);
    s.m = hv(c.m, h); s.dm = hd(c.m, h);
    s.d = c.pole ? hv(c.d, h) : -1.0;
    if (acc) { s.t = hv(c.t, h); s.ph = hv(c.ph, h); s.lam = hv(c.lam, h); }
    else { s.t = s.ph = s.lam = 0.0; }
    return s;
}

// Root in [lo, hi] of series(s) - target (or of its derivative when `deriv`),
// the end values bracketing it; safeguarded Newton, at most 100 iterations.
__host__ __device__ double solve(const double* c, double target, double lo, double hi, bool deriv) {
    double glo = (deriv ? hd(c, lo) : hv(c, lo)) - target;
    if (glo == 0.0) return lo;
    double ghi = (deriv ? hd(c, hi) : hv(c, hi)) - target;
    double x = (ghi != glo) ? lo + (hi - lo) * glo / (glo - ghi) : 0.5 * (lo + hi);
    for (int it = 0; it < 100; ++it) {
        double gx = (deriv ? hd(c, x) : hv(c, x)) - target;
        if (gx == 0.0) return x;
        if ((gx > 0) == (glo > 0)) { lo = x; glo = gx; } else { hi = x; }
        double d = deriv ? hdd(c, x) : hd(c, x);
        double xn = (d != 0.0) ? x - gx / d : 0.5 * (lo + hi);
        if (!(xn > lo && xn < hi)) xn = 0.5 * (lo + hi);
        if (fabs(xn - x) <= 1e-16 * fmax(1.0, fabs(x)) || hi - lo <= 1e-300) { x = xn; break; }
        x = xn;
    }
    return x;
}

constexpr int kMaxSteps = 200000;

// First radial turning point in the direction su before the horizon / u = 0.
__host__ __device__ bool find_turning(const Par& p, const St& s0, double su, double& ub) {
    St s = s0;
    ub = su > 0 ? p.uplus : 0.0;
    Ser c;
    for (int it = 0; it < kMaxSteps; ++it) {
        taylor(p, s, c, false);
        double h = step_size(p, c, s, false);
        St e = advance(c, h, false);
        bool past = su > 0 ? (e.u >= p.uplus) : (e.u <= 0.0);
        if ((e.du > 0) != (s.du > 0) && e.du != 0.0 && !past) {
            ub = hv(c.u, solve(c.u, 0.0, 0.0, h, true));
            return true;
        }
        if (past) return false;
        s = e;
    }
    return false;
}

struct PointOut {
    double *u, *mu, *dt, *dphi, *lam;
    int32_t *tpm, *tpr;
    long long stride;   // element offset of this ray's first point
};

// GEOKERR sampler; returns the number of points written (0 on failure).
__host__ __device__ int sample_points(const Par& p, double u0, double uf, double mu0, double su, double sm, int tpr_in,
                             int nup, double offset, const PointOut& o) {
    double Uu0, Mm0;
    if (nup <= 0 || !start_potentials(p, u0, mu0, Uu0, Mm0)) return 0;
    const St s0{u0, su * sqrt(Uu0), mu0, sm * sqrt(Mm0), 0.0, 0.0, 0.0};
    double ub;
    int tpr = tpr_in;
    if (!find_turning(p, s0, su, ub)) tpr = 0;
    double UF = uf;
    if (tpr == 1 && ((su > 0 && UF > ub) || (su < 0 && UF < ub))) UF = ub;
    if (tpr == 1 && UF == ub) UF = u0;
    double du = ((ub - u0) >= 0 ? 1.0 : -1.0) * su * ((ub - u0) + (2.0 * tpr - 1.0) * (ub - UF)) / (double)nup;
    int kmax = (du == 0.0) ? 0 : min((int)((ub - u0) / du + offset), nup);
    if (kmax <= 0 && tpr == 0) return 0;
    const int last = tpr == 1 ? nup : min(kmax, nup);
    St s = s0;
    int next = 0, tp_mu = 0, tp_r = 0;
    Ser c;
    for (int it = 0; it < 2 * kMaxSteps && next < last; ++it) {
        taylor(p, s, c, true);
        double h = step_size(p, c, s, true);
        St e = advance(c, h, true);
        double s_r = -1.0, s_m = -1.0;
        if ((e.du > 0) != (s.du > 0) && e.du != 0.0 && s.du != 0.0) s_r = solve(c.u, 0.0, 0.0, h, true);
        if ((e.dm > 0) != (s.dm > 0) && e.dm != 0.0 && s.dm != 0.0) s_m = solve(c.m, 0.0, 0.0, h, true);
        while (next < last) {
            const int k = next + 1;
            const bool branch2 = k > kmax;
            const double ut = branch2 ? 2.0 * ub - (u0 + (k - offset) * du) : u0 + (k - offset) * du;
            double lo = 0.0, hi = h;
            if (s_r >= 0.0) { if (branch2) lo = s_r; else hi = s_r; }
            else if (branch2 != (tp_r == 1)) break;
            double ga = hv(c.u, lo) - ut, gb = hv(c.u, hi) - ut;
            if ((ga > 0) == (gb > 0) && ga != 0.0 && gb != 0.0) break;
            double x = solve(c.u, ut, lo, hi, false);
            const long long i = o.stride + next;
            o.u[i] = ut;
            o.mu[i] = hv(c.m, x);
            o.dt[i] = hv(c.t, x);
            o.dphi[i] = hv(c.ph, x);
            o.lam[i] = hv(c.lam, x);
            o.tpm[i] = tp_mu + ((s_m >= 0.0 && x > s_m) ? 1 : 0);
            o.tpr[i] = branch2 ? 1 : 0;
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

__global__ void geokerr_points_kernel(int n, double a, const double* __restrict__ u0, const double* __restrict__ uf,
                                      const double* __restrict__ mu0, const double* __restrict__ l,
                                      const double* __restrict__ q2, const double* __restrict__ su,
                                      const double* __restrict__ sm, int tpr, int nup, double offset,
                                      double* u, double* mu, double* dt, double* dphi, double* lam,
                                      int32_t* tpm, int32_t* tprv, int32_t* npts) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Par p = make_par(a, l[i], q2[i], mu0[i]);
    PointOut o{u, mu, dt, dphi, lam, tpm, tprv, (long long)i * nup};
    int w = sample_points(p, u0[i], uf[i], mu0[i], su[i], sm[i], tpr, nup, offset, o);
    if (npts) npts[i] = w;
}

// Closed-form points (geokerr_cf.cuh): one thread per ray computes the
// ray's constants, one thread per (ray, sample) evaluates a point, and the
// rays outside the closed forms run the Taylor sampler above from a compacted
// list.  mode 0 takes su, sm and tpr from the caller; mode 1 uses
// geokerr_eval_lambda's conventions (su from uf - u0, sm = -1 for mu0 > 0,
// tpr = 1; geokerr_eval_lambda.f90:102-118).
__host__ __device__ inline void cf_signs(int mode, int i, const double* u0, const double* uf, const double* mu0,
                                         const double* su, const double* sm, int tpr, double& sui, double& smi,
                                         int& tpri) {
    if (mode == 0) { sui = su[i]; smi = sm[i]; tpri = tpr; return; }
    sui = (uf[i] - u0[i]) >= 0.0 ? 1.0 : -1.0;
    smi = mu0[i] <= 0.0 ? 1.0 : -1.0;
    tpri = 1;
}

// Returns false when the start is forbidden (no points, as sample_points).
__host__ __device__ inline bool cf_ray(int mode, int i, double a, const double* u0, const double* uf,
                                       const double* mu0, const double* l, const double* q2, const double* su,
                                       const double* sm, int tpr, int nup, double offset, np::gkcf::CfRay& R) {
    double sui, smi, U0, M0;
    int tpri;
    cf_signs(mode, i, u0, uf, mu0, su, sm, tpr, sui, smi, tpri);
    const Par p = make_par(a, l[i], q2[i], mu0[i]);
    if (!start_potentials(p, u0[i], mu0[i], U0, M0)) return false;
    np::gkcf::setup(a, l[i], q2[i], u0[i], uf[i], mu0[i], sui, smi, tpri, nup, offset, p.mpos, p.a2mneg, R);
    return true;
}

__global__ void cf_setup_kernel(int n, int mode, double a, const double* __restrict__ u0,
                                const double* __restrict__ uf, const double* __restrict__ mu0,
                                const double* __restrict__ l, const double* __restrict__ q2,
                                const double* __restrict__ su, const double* __restrict__ sm, int tpr, int nup,
                                double offset, np::gkcf::CfRay* rays, int32_t* npts, int32_t* fb, int32_t* nfb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    np::gkcf::CfRay R;
    if (!cf_ray(mode, i, a, u0, uf, mu0, l, q2, su, sm, tpr, nup, offset, R)) {
        R.kind = -1;
        R.last = 0;
    }
    rays[i] = R;
    if (R.kind == np::gkcf::kFallback) fb[atomicAdd(nfb, 1)] = i;
    else if (npts) npts[i] = R.last;
}

__global__ void cf_points_kernel(int n, int nup, const np::gkcf::CfRay* __restrict__ rays, double* u, double* mu,
                                 double* dt, double* dphi, double* lam, int32_t* tpm, int32_t* tprv) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int i = (int)(t / nup), k = (int)(t % nup) + 1;
    if (i >= n) return;
    const np::gkcf::CfRay& R = rays[i];
    if (R.kind <= np::gkcf::kFallback || k > R.last) return;
    const np::gkcf::Point P = np::gkcf::sample(R, k);
    const long long o = (long long)i * nup + (k - 1);
    u[o] = P.u; mu[o] = P.mu; dt[o] = P.dt; dphi[o] = P.dphi; lam[o] = P.lam; tpm[o] = P.tpm; tprv[o] = P.tpr;
}

__global__ void cf_fallback_kernel(const int32_t* __restrict__ fb, const int32_t* __restrict__ nfb, int mode,
                                   double a, const double* __restrict__ u0, const double* __restrict__ uf,
                                   const double* __restrict__ mu0, const double* __restrict__ l,
                                   const double* __restrict__ q2, const double* __restrict__ su,
                                   const double* __restrict__ sm, int tpr, int nup, double offset, double* u,
                                   double* mu, double* dt, double* dphi, double* lam, int32_t* tpm, int32_t* tprv,
                                   int32_t* npts) {
    const int count = *nfb;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < count; idx += gridDim.x * blockDim.x) {
        const int i = fb[idx];
        double sui, smi;
        int tpri;
        cf_signs(mode, i, u0, uf, mu0, su, sm, tpr, sui, smi, tpri);
        const Par p = make_par(a, l[i], q2[i], mu0[i]);
        PointOut o{u, mu, dt, dphi, lam, tpm, tprv, (long long)i * nup};
        const int w = sample_points(p, u0[i], uf[i], mu0[i], sui, smi, tpri, nup, offset, o);
        if (npts) npts[i] = w;
    }
}

// eval_lambda, step 2: linear resampling onto lam0 + k dlam
// (geokerr_eval_lambda.f90:125-199).
__global__ void eval_resample_kernel(int n, int S, const double* __restrict__ u0, const double* __restrict__ mu0,
                                     const double* __restrict__ t0, const double* __restrict__ lam0,
                                     const double* __restrict__ dlam, const double* w_u, const double* w_mu,
                                     const double* w_dt, const double* w_dphi, const double* w_lam,
                                     const int32_t* w_tpm, const int32_t* w_tpr, const int32_t* w_n,
                                     double* u, double* mu, double* t, double* phi, double* affine,
                                     int32_t* tpmi, int32_t* tpri, int32_t* info) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const long long b = (long long)r * S;
    if (w_n[r] != S) {
        for (int i = 0; i < S; ++i) {
            u[b + i] = mu[b + i] = t[b + i] = phi[b + i] = affine[b + i] = nan("");
        }
        tpmi[r] = -1; tpri[r] = -1; info[r] = 2;
        return;
    }
    const double* L = w_lam + b;
    const double base = L[0];
    int j = 0;
    for (int i = 0; i < S; ++i) {
        const double lamk = lam0[r] + dlam[r] * (double)i;
        affine[b + i] = lamk;
        while (j < S - 1 && (L[j + 1] - base) < lamk - 1.0e-30) j++;
        double uu, mm, tt, pp;
        if (lamk <= L[0] - base) {
            uu = w_u[b]; mm = w_mu[b]; tt = t0[r] + w_dt[b]; pp = w_dphi[b];
        } else if (lamk >= L[S - 1] - base) {
            uu = w_u[b + S - 1]; mm = w_mu[b + S - 1]; tt = t0[r] + w_dt[b + S - 1]; pp = w_dphi[b + S - 1];
        } else {
            const double x0 = L[j] - base, x1 = L[j + 1] - base;
            const double w = (x1 <= x0 + 1.0e-30) ? 0.0 : (lamk - x0) / (x1 - x0);
            uu = (1.0 - w) * w_u[b + j] + w * w_u[b + j + 1];
            mm = (1.0 - w) * w_mu[b + j] + w * w_mu[b + j + 1];
            tt = t0[r] + ((1.0 - w) * w_dt[b + j] + w * w_dt[b + j + 1]);
            pp = (1.0 - w) * w_dphi[b + j] + w * w_dphi[b + j + 1];
        }
        if (i == 0) { uu = u0[r]; mm = mu0[r]; }
        u[b + i] = uu; mu[b + i] = mm; t[b + i] = tt; phi[b + i] = pp;
    }
    int tm = -1, tr = -1;
    for (int jj = 0; jj < S && (tm < 0 || tr < 0); ++jj) {
        if (tm < 0 && w_tpm[b + jj] > 0)
            for (int i = 0; i < S; ++i) if (affine[b + i] >= L[jj] - base) { tm = i; break; }
        if (tr < 0 && w_tpr[b + jj] > 0)
            for (int i = 0; i < S; ++i) if (affine[b + i] >= L[jj] - base) { tr = i; break; }
    }
    tpmi[r] = tm; tpri[r] = tr; info[r] = 0;
}

// Exact samples at uniform Mino time (geokerr_stream_cuda).  Samples past
// the horizon or past u = 0 repeat the last state reached.
__global__ void stream_kernel(double u0, double uf, double mu0, double a, double L, double Q2, double lam0,
                              double dlam, int S, double* u, double* mu, double* t, double* phi, double* aff) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const double su = (uf - u0) >= 0.0 ? 1.0 : -1.0;
    const double sm = mu0 <= 0.0 ? 1.0 : -1.0;
    Par p = make_par(a, L, Q2, mu0);
    double U0, M0;
    start_potentials(p, u0, mu0, U0, M0);
    St s{u0, su * sqrt(U0), mu0, sm * sqrt(M0), 0.0, 0.0, 0.0};
    double lam_a = 0.0;
    int k = 0;
    Ser c;
    while (k < S && lam0 + k * dlam < 0.0) {   // before the start: the start state
        u[k] = u0; mu[k] = mu0; t[k] = 0.0; phi[k] = 0.0; aff[k] = lam0 + k * dlam; ++k;
    }
    for (int it = 0; it < 2 * kMaxSteps && k < S; ++it) {
        taylor(p, s, c, true);
        double h = step_size(p, c, s, true);
        while (k < S) {
            double lk = lam0 + k * dlam;
            if (lk > lam_a + h) break;
            double x = lk - lam_a;
            u[k] = hv(c.u, x); mu[k] = hv(c.m, x); t[k] = hv(c.t, x); phi[k] = hv(c.ph, x); aff[k] = lk;
            ++k;
        }
        St e = advance(c, h, true);
        if (e.u >= p.uplus || e.u <= 0.0 || !isfinite(e.t)) {
            double uu = k > 0 ? u[k - 1] : u0, mm = k > 0 ? mu[k - 1] : mu0;
            double tt = k > 0 ? t[k - 1] : 0.0, pp = k > 0 ? phi[k - 1] : 0.0;
            for (; k < S; ++k) { u[k] = uu; mu[k] = mm; t[k] = tt; phi[k] = pp; aff[k] = lam0 + k * dlam; }
            break;
        }
        s = e;
        lam_a += h;
    }
    if (S > 0) { u[0] = u0; mu[0] = mu0; }   // exact seeding of sample 0 (geokerr_stream.cu:86-89)
}

// Mino time from u0 to the first arrival at uf and mu there; ncase 1 when
// uf is reached before a radial turning point, 2 after it, 3 when the ray
// has no turning point (it falls in or escapes).
// With after_tp (may be null) and after_tp[i] != 0, arrivals before the
// radial turning point are skipped: the arrival on the way back out.
__global__ void complete_kernel(int n, const double* __restrict__ u0, const double* __restrict__ uf,
                                const double* __restrict__ mu0, const double* __restrict__ a,
                                const double* __restrict__ l, const double* __restrict__ q2,
                                const int* __restrict__ su_in, const int* __restrict__ sm_in,
                                const int* __restrict__ after_tp,
                                double* lam_out, double* muf_out, int* ncase, char* valid) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    lam_out[i] = nan(""); muf_out[i] = nan(""); ncase[i] = 0; valid[i] = 0;
    if (!(fabs(a[i]) < 1.0)) return;
    const double su = su_in[i] >= 0 ? 1.0 : -1.0, sm = sm_in[i] >= 0 ? 1.0 : -1.0;
    Par p = make_par(a[i], l[i], q2[i], mu0[i]);
    double U0, M0;
    if (!start_potentials(p, u0[i], mu0[i], U0, M0)) return;
    St s{u0[i], su * sqrt(U0), mu0[i], sm * sqrt(M0), 0.0, 0.0, 0.0};
    double ub;
    const bool has_tp = find_turning(p, s, su, ub);
    const double target = uf[i];
    const bool need_tp = after_tp && after_tp[i] != 0;
    double lam_a = 0.0;
    bool passed = false;
    Ser c;
    for (int it = 0; it < kMaxSteps; ++it) {
        taylor(p, s, c, false);
        double h = step_size(p, c, s, false);
        St e = advance(c, h, false);
        double s_r = -1.0;
        if ((e.du > 0) != (s.du > 0) && e.du != 0.0 && s.du != 0.0) s_r = solve(c.u, 0.0, 0.0, h, true);
        double seg_lo[2] = {0.0, s_r}, seg_hi[2] = {s_r >= 0.0 ? s_r : h, h};
        for (int g = 0; g < (s_r >= 0.0 ? 2 : 1); ++g) {
            if (need_tp && !(passed || g == 1)) continue;
            double ga = hv(c.u, seg_lo[g]) - target, gb = hv(c.u, seg_hi[g]) - target;
            if (ga == 0.0 || gb == 0.0 || (ga > 0) != (gb > 0)) {
                double x = solve(c.u, target, seg_lo[g], seg_hi[g], false);
                lam_out[i] = lam_a + x;
                muf_out[i] = hv(c.m, x);
                ncase[i] = has_tp ? ((passed || g == 1) ? 2 : 1) : 3;
                valid[i] = 1;
                return;
            }
        }
        if (s_r >= 0.0) passed = true;
        if (e.u >= p.uplus || e.u <= 0.0) return;
        s = e;
        lam_a += h;
    }
}

// Equatorial crossings (mu = 0, GEOR with muf = 0) of rays leaving u0:
// for each ray the first K crossings' u and phi, and their count.  A ray
// ends at the horizon, at u <= u_end (escape) or after K crossings.
__global__ void crossings_kernel(int n, double a, const double* __restrict__ u0, const double* __restrict__ mu0,
                                 const double* __restrict__ l, const double* __restrict__ q2,
                                 const double* __restrict__ su, const double* __restrict__ sm, double u_end, int K,
                                 double* xu, double* xphi, int32_t* nx) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int k = 0; k < K; ++k) { xu[(long long)i * K + k] = 0.0; xphi[(long long)i * K + k] = 0.0; }
    nx[i] = 0;
    Par p = make_par(a, l[i], q2[i], mu0[i]);
    double U0, M0;
    if (!start_potentials(p, u0[i], mu0[i], U0, M0)) { nx[i] = -1; return; }
    St s{u0[i], su[i] * sqrt(U0), mu0[i], sm[i] * sqrt(M0), 0.0, 0.0, 0.0};
    int found = 0;
    Ser c;
    for (int it = 0; it < kMaxSteps && found < K; ++it) {
        taylor(p, s, c, true);
        double h = step_size(p, c, s, true);
        St e = advance(c, h, true);
        // mu = 0 crossings inside the step (at most one: the step holds at most
        // one polar turning point and |mu| < mu_+ keeps the sign changes apart)
        if ((s.m > 0.0) != (e.m > 0.0) && s.m != 0.0) {
            double x = solve(c.m, 0.0, 0.0, h, false);
            double ux = hv(c.u, x);
            if (ux > u_end && ux < p.uplus) {
                xu[(long long)i * K + found] = ux;
                xphi[(long long)i * K + found] = hv(c.ph, x);
                ++found;
            }
        }
        if (e.u >= p.uplus || e.u <= u_end || !isfinite(e.ph)) break;
        s = e;
    }
    nx[i] = found;
}

// State at Mino time lam[i] of ray i (spin a[i]) leaving (u0[i], mu0[i])
// with signs su[i], sm[i] of du/dlambda and dmu/dlambda: u, mu, t and phi
// (t and phi from 0 at the start).  A ray that reaches the horizon or u = 0
// first keeps the last state before it and is flagged 0 in valid; a
// forbidden start gives NaN.
__global__ void final_state_kernel(int n, const double* __restrict__ a, const double* __restrict__ u0,
                                   const double* __restrict__ mu0, const double* __restrict__ l,
                                   const double* __restrict__ q2, const double* __restrict__ su,
                                   const double* __restrict__ sm, const double* __restrict__ lam, double* uo,
                                   double* muo, double* to, double* pho, char* valid) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double nan_v = nan("");
    uo[i] = nan_v; muo[i] = nan_v; to[i] = nan_v; pho[i] = nan_v; valid[i] = 0;
    if (!(fabs(a[i]) < 1.0) || !(lam[i] >= 0.0)) return;
    Par p = make_par(a[i], l[i], q2[i], mu0[i]);
    double U0, M0;
    if (!start_potentials(p, u0[i], mu0[i], U0, M0)) return;
    St s{u0[i], (su[i] >= 0.0 ? 1.0 : -1.0) * sqrt(U0), mu0[i], (sm[i] >= 0.0 ? 1.0 : -1.0) * sqrt(M0), 0.0, 0.0, 0.0};
    const double target = lam[i];
    double lam_a = 0.0;
    Ser c;
    for (int it = 0; it < kMaxSteps; ++it) {
        taylor(p, s, c, true);
        double h = step_size(p, c, s, true);
        if (lam_a + h >= target) {
            double x = target - lam_a;
            uo[i] = hv(c.u, x); muo[i] = hv(c.m, x); to[i] = hv(c.t, x); pho[i] = hv(c.ph, x);
            valid[i] = 1;
            return;
        }
        St e = advance(c, h, true);
        if (e.u >= p.uplus || e.u <= 0.0 || !isfinite(e.t)) break;
        s = e;
        lam_a += h;
    }
    uo[i] = s.u; muo[i] = s.m; to[i] = s.t; pho[i] = s.ph;
}

int grid(int n, int b) { return (n + b - 1) / b; }

// The closed-form pipeline on a stream: setup, points, Taylor fallback.  Its
// per-ray workspace (n CfRay records and the fallback list) is taken from the
// stream-ordered pool and released on the stream.
int points_cf_launch(int n, int mode, double a, const double* u0, const double* uf, const double* mu0,
                     const double* l, const double* q2, const double* su, const double* sm, int tpr, int nup,
                     double offset, double* u, double* mu, double* dt, double* dphi, double* lam, int32_t* tpm,
                     int32_t* tprv, int32_t* npts, cudaStream_t st) {
    if ((long long)n * nup > (1ll << 31) - 1) return gk_fail(NP_ERR_INVALID, "n * nup exceeds 2^31 - 1");
    const size_t bytes = (size_t)n * sizeof(np::gkcf::CfRay) + ((size_t)n + 1) * sizeof(int32_t);
    void* w = nullptr;
    if (cudaMallocAsync(&w, bytes, st) != cudaSuccess) {
        cudaGetLastError();
        return gk_fail(NP_ERR_ALLOC, "cudaMallocAsync of %zu bytes failed", bytes);
    }
    np::gkcf::CfRay* rays = (np::gkcf::CfRay*)w;
    int32_t* fb = (int32_t*)(rays + n);
    int32_t* nfb = fb + n;
    cudaMemsetAsync(nfb, 0, sizeof(int32_t), st);
    // one ray per thread; warp-sized blocks spread a grid of a few thousand
    // rays over every SM (the kernel is FP64-bound once resident)
    cf_setup_kernel<<<grid(n, 32), 32, 0, st>>>(n, mode, a, u0, uf, mu0, l, q2, su, sm, tpr, nup, offset, rays, npts,
                                                fb, nfb);
    // The Taylor rays (a few serial integrations) run on a side stream
    // beside the per-point kernel; the caller's stream waits for both.
    cudaStream_t side = nullptr;
    cudaEvent_t ev_setup = nullptr, ev_fb = nullptr;
    const bool overlap = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking) == cudaSuccess &&
                         cudaEventCreateWithFlags(&ev_setup, cudaEventDisableTiming) == cudaSuccess &&
                         cudaEventCreateWithFlags(&ev_fb, cudaEventDisableTiming) == cudaSuccess;
    cudaStream_t fb_stream = st;
    if (overlap) {
        cudaEventRecord(ev_setup, st);
        cudaStreamWaitEvent(side, ev_setup, 0);
        fb_stream = side;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 1;
    const int fb_blocks = std::min(grid(n, 32), 4 * sms);
    cf_fallback_kernel<<<fb_blocks, 32, 0, fb_stream>>>(fb, nfb, mode, a, u0, uf, mu0, l, q2, su, sm, tpr, nup, offset,
                                                        u, mu, dt, dphi, lam, tpm, tprv, npts);
    const long long total = (long long)n * nup;
    cf_points_kernel<<<(unsigned)((total + 127) / 128), 128, 0, st>>>(n, nup, rays, u, mu, dt, dphi, lam, tpm, tprv);
    if (overlap) {
        cudaEventRecord(ev_fb, side);
        cudaStreamWaitEvent(st, ev_fb, 0);
    }
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(w, st);
    if (ev_setup) cudaEventDestroy(ev_setup);
    if (ev_fb) cudaEventDestroy(ev_fb);
    if (side) cudaStreamDestroy(side);
    return e == cudaSuccess ? NP_OK : gk_fail(NP_ERR_KERNEL, "%s", cudaGetErrorString(e));
}

// Host arrays in, final states out (geokerr_cuda_batch and friends): copies
// n rays' inputs to the device, runs final_state_kernel, copies back.
// Returns false when the device work failed.
bool final_states_host(int n, const double* a, const double* u0, const double* mu0, const double* l,
                       const double* q2, const double* su, const double* sm, const double* lam, double* uo,
                       double* muo, double* to, double* pho, char* valid) {
    const size_t m = (size_t)n;
    char* d = nullptr;
    if (cudaMalloc(&d, m * (12 * sizeof(double) + 1)) != cudaSuccess) return false;
    double* dd = (double*)d;
    const double* ins[8] = {a, u0, mu0, l, q2, su, sm, lam};
    bool ok = true;
    for (int k = 0; k < 8 && ok; ++k)
        ok = cudaMemcpy(dd + k * m, ins[k], m * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess;
    char* dv = (char*)(dd + 12 * m);
    if (ok) {
        final_state_kernel<<<grid(n, 64), 64>>>(n, dd, dd + m, dd + 2 * m, dd + 3 * m, dd + 4 * m, dd + 5 * m,
                                                dd + 6 * m, dd + 7 * m, dd + 8 * m, dd + 9 * m, dd + 10 * m,
                                                dd + 11 * m, dv);
        ok = cudaDeviceSynchronize() == cudaSuccess;
    }
    double* outs[4] = {uo, muo, to, pho};
    for (int k = 0; k < 4 && ok; ++k)
        ok = cudaMemcpy(outs[k], dd + (8 + k) * m, m * sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess;
    if (ok) ok = cudaMemcpy(valid, dv, m, cudaMemcpyDeviceToHost) == cudaSuccess;
    cudaFree(d);
    return ok;
}

// geokerr_cuda_batch / geokerr_improved_batch: per ray, E, L, Q2 in any
// normalisation (l = L/E, q2 = Q2/E^2; the Mino time of the E = 1 problem
// is E lambda_max), outgoing in r and increasing in mu as the reference's
// wrappers integrate (geokerr_cuda.cu:259-264).
void batch_final(const double* a_vals, const double* r0_vals, const double* mu0_vals, const double* E_vals,
                 const double* L_vals, const double* Q2_vals, double* r_final, double* mu_final, double* phi_final,
                 double* t_final, int n, double lambda_max) {
    if (n <= 0 || !a_vals || !r0_vals || !mu0_vals || !E_vals || !L_vals || !Q2_vals || !r_final || !mu_final ||
        !phi_final || !t_final)
        return;
    std::vector<double> u0(n), l(n), q2(n), su(n, -1.0), sm(n, 1.0), lam(n), uo(n), mo(n), to(n), po(n);
    std::vector<char> valid(n);
    for (int i = 0; i < n; ++i) {
        const double E = E_vals[i];
        u0[i] = r0_vals[i] > 0.0 ? 1.0 / r0_vals[i] : nan("");
        l[i] = E > 0.0 ? L_vals[i] / E : nan("");
        q2[i] = E > 0.0 ? Q2_vals[i] / (E * E) : nan("");
        lam[i] = E > 0.0 ? E * lambda_max : nan("");
    }
    const double nan_v = nan("");
    if (!final_states_host(n, a_vals, u0.data(), mu0_vals, l.data(), q2.data(), su.data(), sm.data(), lam.data(),
                           uo.data(), mo.data(), to.data(), po.data(), valid.data())) {
        for (int i = 0; i < n; ++i) r_final[i] = mu_final[i] = phi_final[i] = t_final[i] = nan_v;
        return;
    }
    for (int i = 0; i < n; ++i) {
        r_final[i] = uo[i] > 0.0 ? 1.0 / uo[i] : nan_v;
        mu_final[i] = mo[i];
        phi_final[i] = po[i];
        t_final[i] = to[i];
    }
}

}  // namespace

extern "C" {

int np_geokerr_points_device(int n, double a, const double* u0, const double* uf, const double* mu0,
                             const double* l, const double* q2, const double* su, const double* sm,
                             int tpr, int nup, double offset, double* u, double* mu, double* dt, double* dphi,
                             double* lam, int32_t* tpm, int32_t* tprv, int32_t* npts, void* stream) {
    if (n < 0 || nup <= 0) return gk_fail(NP_ERR_INVALID, "bad sizes");
    if (n == 0) return NP_OK;
    if (!(fabs(a) < 1.0)) return gk_fail(NP_ERR_INVALID, "spin must satisfy |a| < 1");
    return points_cf_launch(n, 0, a, u0, uf, mu0, l, q2, su, sm, tpr, nup, offset, u, mu, dt, dphi, lam, tpm, tprv,
                            npts, (cudaStream_t)stream);
}

int np_geokerr_points_taylor_device(int n, double a, const double* u0, const double* uf, const double* mu0,
                                    const double* l, const double* q2, const double* su, const double* sm, int tpr,
                                    int nup, double offset, double* u, double* mu, double* dt, double* dphi,
                                    double* lam, int32_t* tpm, int32_t* tprv, int32_t* npts, void* stream) {
    if (n < 0 || nup <= 0) return gk_fail(NP_ERR_INVALID, "bad sizes");
    if (n == 0) return NP_OK;
    if (!(fabs(a) < 1.0)) return gk_fail(NP_ERR_INVALID, "spin must satisfy |a| < 1");
    geokerr_points_kernel<<<grid(n, 64), 64, 0, (cudaStream_t)stream>>>(n, a, u0, uf, mu0, l, q2, su, sm, tpr, nup,
                                                                        offset, u, mu, dt, dphi, lam, tpm, tprv, npts);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NP_OK : gk_fail(NP_ERR_KERNEL, "%s", cudaGetErrorString(e));
}

int np_geokerr_points_host(int n, double a, const double* u0, const double* uf, const double* mu0, const double* l,
                           const double* q2, const double* su, const double* sm, int tpr, int nup, double offset,
                           double* u, double* mu, double* dt, double* dphi, double* lam, int32_t* tpm, int32_t* tprv,
                           int32_t* npts, int32_t* method) {
    if (n < 0 || nup <= 0) return gk_fail(NP_ERR_INVALID, "bad sizes");
    if (!(fabs(a) < 1.0)) return gk_fail(NP_ERR_INVALID, "spin must satisfy |a| < 1");
    if (!u0 || !uf || !mu0 || !l || !q2 || !su || !sm || !u || !mu || !dt || !dphi || !lam || !tpm || !tprv)
        return gk_fail(NP_ERR_INVALID, "NULL argument");
    for (int i = 0; i < n; ++i) {
        np::gkcf::CfRay R;
        int w = 0, how = 0;
        if (cf_ray(0, i, a, u0, uf, mu0, l, q2, su, sm, tpr, nup, offset, R)) {
            if (R.kind == np::gkcf::kFallback) {
                const Par p = make_par(a, l[i], q2[i], mu0[i]);
                PointOut o{u, mu, dt, dphi, lam, tpm, tprv, (long long)i * nup};
                w = sample_points(p, u0[i], uf[i], mu0[i], su[i], sm[i], tpr, nup, offset, o);
            } else {
                how = R.kind;
                for (int k = 1; k <= R.last; ++k) {
                    const np::gkcf::Point P = np::gkcf::sample(R, k);
                    const long long o = (long long)i * nup + (k - 1);
                    u[o] = P.u; mu[o] = P.mu; dt[o] = P.dt; dphi[o] = P.dphi; lam[o] = P.lam;
                    tpm[o] = P.tpm; tprv[o] = P.tpr;
                }
                w = R.last;
            }
        }
        if (npts) npts[i] = w;
        if (method) method[i] = how;
    }
    return NP_OK;
}

int np_geokerr_equator_crossings_device(int n, double a, const double* u0, const double* mu0, const double* l,
                                        const double* q2, const double* su, const double* sm, double u_end, int K,
                                        double* xu, double* xphi, int32_t* nx, void* stream) {
    if (n < 0 || K <= 0) return gk_fail(NP_ERR_INVALID, "bad sizes");
    if (n == 0) return NP_OK;
    if (!(fabs(a) < 1.0)) return gk_fail(NP_ERR_INVALID, "spin must satisfy |a| < 1");
    crossings_kernel<<<grid(n, 64), 64, 0, (cudaStream_t)stream>>>(n, a, u0, mu0, l, q2, su, sm, u_end, K, xu, xphi,
                                                                   nx);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NP_OK : gk_fail(NP_ERR_KERNEL, "%s", cudaGetErrorString(e));
}

size_t np_geokerr_eval_lambda_work_bytes(int n, int S) {
    if (n <= 0 || S <= 0) return 0;
    return (size_t)n * S * (5 * sizeof(double) + 2 * sizeof(int32_t)) + (size_t)n * sizeof(int32_t) + 256;
}

int np_geokerr_eval_lambda_device(int n, double a, const double* u0, const double* mu0, const double* uf,
                                  const double* Lz, const double* Q2, const double* t0, const double* lam0,
                                  const double* dlam, int S, double* u, double* mu, double* t, double* phi,
                                  double* affine, int32_t* tpmi, int32_t* tpri, int32_t* info, void* work,
                                  void* stream) {
    if (n < 0 || S <= 0) return gk_fail(NP_ERR_INVALID, "bad sizes");
    if (n == 0) return NP_OK;
    if (!(fabs(a) < 1.0)) return gk_fail(NP_ERR_INVALID, "spin must satisfy |a| < 1");
    cudaStream_t st = (cudaStream_t)stream;
    void* w = work;
    bool own = false;
    if (!w) {
        if (cudaMalloc(&w, np_geokerr_eval_lambda_work_bytes(n, S)) != cudaSuccess)
            return gk_fail(NP_ERR_ALLOC, "cudaMalloc of %zu bytes failed", np_geokerr_eval_lambda_work_bytes(n, S));
        own = true;
    }
    const size_t m = (size_t)n * S;
    double* wd = (double*)w;
    double *w_u = wd, *w_mu = wd + m, *w_dt = wd + 2 * m, *w_dphi = wd + 3 * m, *w_lam = wd + 4 * m;
    int32_t* wi = (int32_t*)(wd + 5 * m);
    int32_t *w_tpm = wi, *w_tpr = wi + m, *w_n = wi + 2 * m;
    int rc = points_cf_launch(n, 1, a, u0, uf, mu0, Lz, Q2, nullptr, nullptr, 1, S, 0.5, w_u, w_mu, w_dt, w_dphi,
                              w_lam, w_tpm, w_tpr, w_n, st);
    if (rc != NP_OK) {
        if (own) { cudaStreamSynchronize(st); cudaFree(w); }
        return rc;
    }
    eval_resample_kernel<<<grid(n, 64), 64, 0, st>>>(n, S, u0, mu0, t0, lam0, dlam, w_u, w_mu, w_dt, w_dphi, w_lam,
                                                    w_tpm, w_tpr, w_n, u, mu, t, phi, affine, tpmi, tpri, info);
    cudaError_t e = cudaGetLastError();
    if (own) {
        cudaError_t e2 = cudaStreamSynchronize(st);
        cudaFree(w);
        if (e == cudaSuccess) e = e2;
    }
    return e == cudaSuccess ? NP_OK : gk_fail(NP_ERR_KERNEL, "%s", cudaGetErrorString(e));
}

void geokerr_eval_lambda(double u0, double mu0, double uf, double a, double Lz, double Q2, double t0,
                         double lam0, double dlam, int S, double* u, double* mu, double* t, double* phi,
                         double* affine, int* tpmi, int* tpri, int* info) {
    if (info) *info = 0;
    if (S <= 0) { if (info) *info = 1; return; }
    // one device block: 8 scalars in, 5 x S doubles + 3 ints out, work after
    const size_t outb = 5 * (size_t)S * sizeof(double) + 3 * sizeof(int32_t);
    const size_t inb = 8 * sizeof(double);
    const size_t wb = np_geokerr_eval_lambda_work_bytes(1, S);
    char* d = nullptr;
    if (cudaMalloc(&d, inb + outb + wb + 512) != cudaSuccess) { if (info) *info = 3; return; }
    double hin[8] = {u0, mu0, uf, Lz, Q2, t0, lam0, dlam};
    double* din = (double*)d;
    cudaMemcpy(din, hin, inb, cudaMemcpyHostToDevice);
    double* dout = (double*)(d + 256);
    int32_t* di = (int32_t*)(dout + 5 * (size_t)S);
    void* dw = (void*)(((uintptr_t)(di + 3) + 255) & ~(uintptr_t)255);
    int rc = np_geokerr_eval_lambda_device(1, a, din, din + 1, din + 2, din + 3, din + 4, din + 5, din + 6, din + 7,
                                           S, dout, dout + S, dout + 2 * S, dout + 3 * S, dout + 4 * S,
                                           di, di + 1, di + 2, dw, nullptr);
    int32_t hi[3] = {-1, -1, 3};
    if (rc == NP_OK && cudaDeviceSynchronize() == cudaSuccess) {
        cudaMemcpy(u, dout, S * sizeof(double), cudaMemcpyDeviceToHost);
        cudaMemcpy(mu, dout + S, S * sizeof(double), cudaMemcpyDeviceToHost);
        cudaMemcpy(t, dout + 2 * S, S * sizeof(double), cudaMemcpyDeviceToHost);
        cudaMemcpy(phi, dout + 3 * S, S * sizeof(double), cudaMemcpyDeviceToHost);
        cudaMemcpy(affine, dout + 4 * S, S * sizeof(double), cudaMemcpyDeviceToHost);
        cudaMemcpy(hi, di, 3 * sizeof(int32_t), cudaMemcpyDeviceToHost);
    }
    cudaFree(d);
    if (tpmi) *tpmi = hi[0];
    if (tpri) *tpri = hi[1];
    if (info) *info = hi[2];
}

void geokerr_estimate_periods(double u0, double mu0, double a, double Lz, double Q2, double* Tr, double* Ttheta,
                              int* info) {
    const int nup = 4096;
    if (Tr) *Tr = -1.0;
    if (Ttheta) *Ttheta = -1.0;
    if (info) *info = 0;
    const size_t m = nup;
    char* d = nullptr;
    const size_t bytes = 8 * sizeof(double) + m * (5 * sizeof(double) + 2 * sizeof(int32_t)) + 1024;
    if (cudaMalloc(&d, bytes) != cudaSuccess) { if (info) *info = 3; return; }
    const double sm = mu0 <= 0.0 ? 1.0 : -1.0;
    double hin[8] = {u0, u0, mu0, Lz, Q2, 1.0, sm, 0.0};
    double* din = (double*)d;
    cudaMemcpy(din, hin, sizeof(hin), cudaMemcpyHostToDevice);
    double* dp = din + 8;
    int32_t* di = (int32_t*)(dp + 5 * m);
    int rc = np_geokerr_points_device(1, a, din, din + 1, din + 2, din + 3, din + 4, din + 5, din + 6, 1, nup, 0.5,
                                      dp, dp + m, dp + 2 * m, dp + 3 * m, dp + 4 * m, di, di + m, di + 2 * m, nullptr);
    if (rc == NP_OK && cudaDeviceSynchronize() == cudaSuccess) {
        double* lam = new double[m];
        int32_t* tpm = new int32_t[m];
        int32_t* tpr = new int32_t[m];
        int32_t n = 0;
        cudaMemcpy(lam, dp + 4 * m, m * sizeof(double), cudaMemcpyDeviceToHost);
        cudaMemcpy(tpm, di, m * sizeof(int32_t), cudaMemcpyDeviceToHost);
        cudaMemcpy(tpr, di + m, m * sizeof(int32_t), cudaMemcpyDeviceToHost);
        cudaMemcpy(&n, di + 2 * m, sizeof(int32_t), cudaMemcpyDeviceToHost);
        if (n > 0) {
            const double base = lam[0];
            int m1 = -1, m2 = -1, r1 = -1, r2 = -1, pm = 0, pr = 0;
            for (int j = 0; j < n; ++j) {
                if (m1 < 0 && pm < 1 && tpm[j] >= 1) m1 = j;
                if (m2 < 0 && pm < 2 && tpm[j] >= 2) m2 = j;
                if (r1 < 0 && pr < 1 && tpr[j] >= 1) r1 = j;
                if (r2 < 0 && pr < 2 && tpr[j] >= 2) r2 = j;
                pm = std::max(pm, (int)tpm[j]); pr = std::max(pr, (int)tpr[j]);
                if (m2 >= 0 && r2 >= 0) break;
            }
            if (Tr && r1 >= 0 && r2 >= 0) *Tr = 2.0 * std::max(1e-18, (lam[r2] - base) - (lam[r1] - base));
            if (Ttheta && m1 >= 0 && m2 >= 0) *Ttheta = 2.0 * std::max(1e-18, (lam[m2] - base) - (lam[m1] - base));
        }
        delete[] lam; delete[] tpm; delete[] tpr;
    } else if (info) {
        *info = 3;
    }
    cudaFree(d);
}

double geokerr_phi_omega(double u0, double mu0, double a, double Lz, double Q2) {
    (void)Q2;
    double r = std::max(1e-12, 1.0 / std::max(1e-12, u0));
    double Delta = std::max(1e-30, r * r - 2.0 * r + a * a);
    double sin2 = std::max(1e-30, 1.0 - mu0 * mu0);
    return a * (((r * r + a * a) - a * Lz) / Delta) + Lz / sin2 - a;
}

int geokerr_stream_cuda(double u0, double uf, double mu0, double a, double L, double Q2, double lam0, double dlam,
                        int S, double* h_u, double* h_mu, double* h_t, double* h_phi, double* h_affine) {
    if (S <= 0 || !h_u || !h_mu || !h_t || !h_phi || !h_affine || !(fabs(a) < 1.0)) return -1;
    double* d = nullptr;
    if (cudaMalloc(&d, 5 * (size_t)S * sizeof(double)) != cudaSuccess) return -2;
    stream_kernel<<<1, 1>>>(u0, uf, mu0, a, L, Q2, lam0, dlam, S, d, d + S, d + 2 * S, d + 3 * S, d + 4 * S);
    if (cudaDeviceSynchronize() != cudaSuccess) { cudaFree(d); return -3; }
    cudaMemcpy(h_u, d, S * sizeof(double), cudaMemcpyDeviceToHost);
    cudaMemcpy(h_mu, d + S, S * sizeof(double), cudaMemcpyDeviceToHost);
    cudaMemcpy(h_t, d + 2 * S, S * sizeof(double), cudaMemcpyDeviceToHost);
    cudaMemcpy(h_phi, d + 3 * S, S * sizeof(double), cudaMemcpyDeviceToHost);
    cudaMemcpy(h_affine, d + 4 * S, S * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return 0;
}

int geokerr_complete_stream_cuda(double u0, double uf, double mu0, double a, double L, double Q2, double lam0,
                                 double dlam, int S, double* h_u, double* h_mu, double* h_t, double* h_phi,
                                 double* h_affine) {
    if (S <= 0 || !h_u || !h_mu || !h_t || !h_phi || !h_affine || !(fabs(a) < 1.0)) return -1;
    int tpmi = -1, tpri = -1, info = 0;
    geokerr_eval_lambda(u0, mu0, uf, a, L, Q2, 0.0, lam0, dlam, S, h_u, h_mu, h_t, h_phi, h_affine, &tpmi, &tpri,
                        &info);
    if (info == 3) return -2;
    return info == 0 ? 0 : -3;
}

void compute_geokerr_complete_cuda(const double* h_u0, const double* h_uf, const double* h_mu0, const double* h_a,
                                   const double* h_l, const double* h_q2, const int* h_su, const int* h_sm,
                                   double* h_lambda_results, double* h_muf_results, int* h_ncase_results,
                                   char* h_valid_results, int n_cases) {
    if (n_cases <= 0) return;
    const size_t n = n_cases;
    const size_t bytes = n * (8 * sizeof(double) + 3 * sizeof(int) + 1) + 1024;
    char* d = nullptr;
    if (cudaMalloc(&d, bytes) != cudaSuccess) {
        for (size_t i = 0; i < n; ++i) h_valid_results[i] = 0;
        return;
    }
    double* dd = (double*)d;
    double *du0 = dd, *duf = dd + n, *dmu0 = dd + 2 * n, *da = dd + 3 * n, *dl = dd + 4 * n, *dq2 = dd + 5 * n;
    double *dlam = dd + 6 * n, *dmuf = dd + 7 * n;
    int* di = (int*)(dd + 8 * n);
    int *dsu = di, *dsm = di + n, *dnc = di + 2 * n;
    char* dv = (char*)(di + 3 * n);
    cudaMemcpy(du0, h_u0, n * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(duf, h_uf, n * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(dmu0, h_mu0, n * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(da, h_a, n * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(dl, h_l, n * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(dq2, h_q2, n * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(dsu, h_su, n * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(dsm, h_sm, n * sizeof(int), cudaMemcpyHostToDevice);
    complete_kernel<<<grid(n_cases, 64), 64>>>(n_cases, du0, duf, dmu0, da, dl, dq2, dsu, dsm, nullptr, dlam, dmuf,
                                               dnc, dv);
    if (cudaDeviceSynchronize() == cudaSuccess) {
        cudaMemcpy(h_lambda_results, dlam, n * sizeof(double), cudaMemcpyDeviceToHost);
        cudaMemcpy(h_muf_results, dmuf, n * sizeof(double), cudaMemcpyDeviceToHost);
        cudaMemcpy(h_ncase_results, dnc, n * sizeof(int), cudaMemcpyDeviceToHost);
        cudaMemcpy(h_valid_results, dv, n, cudaMemcpyDeviceToHost);
    } else {
        for (size_t i = 0; i < n; ++i) h_valid_results[i] = 0;
    }
    cudaFree(d);
}

void geokerr_cuda_batch(const double* a_vals, const double* r0_vals, const double* mu0_vals, const double* E_vals,
                        const double* L_vals, const double* Q2_vals, double* r_final, double* mu_final,
                        double* phi_final, double* t_final, int n_geodesics, int n_steps, double lambda_max) {
    (void)n_steps;   // the Mino-time solver needs no step count
    batch_final(a_vals, r0_vals, mu0_vals, E_vals, L_vals, Q2_vals, r_final, mu_final, phi_final, t_final,
                n_geodesics, lambda_max);
}

void geokerr_improved_batch(const double* a_vals, const double* r0_vals, const double* mu0_vals,
                            const double* E_vals, const double* L_vals, const double* Q2_vals, double* r_final,
                            double* mu_final, double* phi_final, double* t_final, int n_geodesics, int n_steps,
                            double lambda_max) {
    (void)n_steps;
    batch_final(a_vals, r0_vals, mu0_vals, E_vals, L_vals, Q2_vals, r_final, mu_final, phi_final, t_final,
                n_geodesics, lambda_max);
}

int np_geokerr_final_state_host(int n, const double* a, const double* u0, const double* mu0, const double* l,
                                const double* q2, const double* su, const double* sm, const double* lam, double* u,
                                double* mu, double* t, double* phi, char* valid) {
    if (n < 0 || (n > 0 && (!a || !u0 || !mu0 || !l || !q2 || !su || !sm || !lam || !u || !mu || !t || !phi ||
                            !valid)))
        return gk_fail(NP_ERR_INVALID, "bad arguments");
    if (n == 0) return NP_OK;
    return final_states_host(n, a, u0, mu0, l, q2, su, sm, lam, u, mu, t, phi, valid)
               ? NP_OK : gk_fail(NP_ERR_KERNEL, "final-state kernel failed");
}

void compute_mino_time_batch_cuda(const double* h_u0, const double* h_uf, const double* h_mu0, const double* h_muf,
                                  const double* h_a, const double* h_l, const double* h_q2, const int* h_tpm,
                                  const int* h_tpr, const int* h_su, const int* h_sm, const int* h_ncase,
                                  double* h_lambda_results, char* h_valid_results, int n_cases) {
    (void)h_muf; (void)h_tpm; (void)h_ncase;
    if (n_cases <= 0 || !h_u0 || !h_uf || !h_mu0 || !h_a || !h_l || !h_q2 || !h_tpr || !h_su || !h_sm ||
        !h_lambda_results || !h_valid_results)
        return;
    const size_t n = n_cases;
    const size_t bytes = n * (8 * sizeof(double) + 4 * sizeof(int) + 1) + 1024;
    char* d = nullptr;
    if (cudaMalloc(&d, bytes) != cudaSuccess) {
        for (size_t i = 0; i < n; ++i) h_valid_results[i] = 0;
        return;
    }
    double* dd = (double*)d;
    double *du0 = dd, *duf = dd + n, *dmu0 = dd + 2 * n, *da = dd + 3 * n, *dl = dd + 4 * n, *dq2 = dd + 5 * n;
    double *dlam = dd + 6 * n, *dmuf = dd + 7 * n;
    int* di = (int*)(dd + 8 * n);
    int *dsu = di, *dsm = di + n, *dnc = di + 2 * n, *dtp = di + 3 * n;
    char* dv = (char*)(di + 4 * n);
    bool ok = cudaMemcpy(du0, h_u0, n * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(duf, h_uf, n * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(dmu0, h_mu0, n * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(da, h_a, n * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(dl, h_l, n * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(dq2, h_q2, n * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(dsu, h_su, n * sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(dsm, h_sm, n * sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(dtp, h_tpr, n * sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess;
    if (ok) {
        complete_kernel<<<grid(n_cases, 64), 64>>>(n_cases, du0, duf, dmu0, da, dl, dq2, dsu, dsm, dtp, dlam, dmuf,
                                                   dnc, dv);
        ok = cudaDeviceSynchronize() == cudaSuccess &&
             cudaMemcpy(h_lambda_results, dlam, n * sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess &&
             cudaMemcpy(h_valid_results, dv, n, cudaMemcpyDeviceToHost) == cudaSuccess;
    }
    if (!ok)
        for (size_t i = 0; i < n; ++i) h_valid_results[i] = 0;
    cudaFree(d);
}

void geokerr_single_case_(double* u0, double* uf, double* mu0, double* muf, double* a, double* l, double* q2,
                          int* su, int* sm, double* lambda, double* muf_out, int* ncase, int* valid) {
    (void)muf;
    if (!u0 || !uf || !mu0 || !a || !l || !q2 || !su || !sm || !lambda || !muf_out || !ncase || !valid) return;
    char v = 0;
    compute_geokerr_complete_cuda(u0, uf, mu0, a, l, q2, su, sm, lambda, muf_out, ncase, &v, 1);
    *valid = v ? 1 : 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// GEOKERR's standard camera grid (geokerr_original.f:183-220), one ray per
// thread on the device and the same function on the host.
namespace {
__host__ __device__ inline void camera_grid_one(double a, double mu0, int n_alpha, int n_beta, double a1, double a2,
                                                double b1, double b2, double lim, long long idx, double& al, double& be,
                                                double& l, double& q2, double& su, double& sm) {
    const int i = (int)(idx / n_beta), j = (int)(idx % n_beta);
    al = a1 + (a2 - a1) * (i + 0.5) / n_alpha;
    be = b1 + (b2 - b1) * (j + 0.5) / n_beta;
    const double as = fabs(a) < lim ? 0.0 : a;
    l = -al * sqrt(1.0 - mu0 * mu0);
    q2 = be * be - (as * as - al * al) * mu0 * mu0;
    if (fabs(q2) < lim * lim) q2 = 0.0;
    if (fabs(l) < lim) l = 0.0;
    su = 1.0;
    sm = (be > 0.0 && mu0 < 1.0) ? 1.0 : -1.0;
}

__global__ void camera_grid_kernel(double a, double mu0, int n_alpha, int n_beta, double a1, double a2, double b1,
                                   double b2, double lim, double* al, double* be, double* l, double* q2, double* su,
                                   double* sm) {
    const long long n = (long long)n_alpha * n_beta;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        camera_grid_one(a, mu0, n_alpha, n_beta, a1, a2, b1, b2, lim, k, al[k], be[k], l[k], q2[k], su[k], sm[k]);
}

int camera_grid_check(int n_alpha, int n_beta, double mu0, const void* p0, const void* p1, const void* p2,
                      const void* p3, const void* p4, const void* p5) {
    if (n_alpha <= 0 || n_beta <= 0 || (long long)n_alpha * n_beta > (1ll << 31) || !(fabs(mu0) <= 1.0) || !p0 ||
        !p1 || !p2 || !p3 || !p4 || !p5)
        return gk_fail(NP_ERR_INVALID, "camera grid: invalid sizes, mu0 or NULL output");
    return NP_OK;
}
}  // namespace

extern "C" int np_geokerr_camera_grid_device(double a, double mu0, int n_alpha, int n_beta, double a1, double a2,
                                             double b1, double b2, double input_limit, double* d_alpha,
                                             double* d_beta, double* d_l, double* d_q2, double* d_su, double* d_sm,
                                             void* stream) {
    int rc = camera_grid_check(n_alpha, n_beta, mu0, d_alpha, d_beta, d_l, d_q2, d_su, d_sm);
    if (rc != NP_OK) return rc;
    const long long n = (long long)n_alpha * n_beta;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 4096);
    camera_grid_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(a, mu0, n_alpha, n_beta, a1, a2, b1, b2, input_limit,
                                                                  d_alpha, d_beta, d_l, d_q2, d_su, d_sm);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return gk_fail(NP_ERR_KERNEL, "camera grid: %s", cudaGetErrorString(e));
    return NP_OK;
}

extern "C" int np_geokerr_camera_grid_host(double a, double mu0, int n_alpha, int n_beta, double a1, double a2,
                                           double b1, double b2, double input_limit, double* alpha, double* beta,
                                           double* l, double* q2, double* su, double* sm) {
    int rc = camera_grid_check(n_alpha, n_beta, mu0, alpha, beta, l, q2, su, sm);
    if (rc != NP_OK) return rc;
    const long long n = (long long)n_alpha * n_beta;
    for (long long k = 0; k < n; ++k)
        camera_grid_one(a, mu0, n_alpha, n_beta, a1, a2, b1, b2, input_limit, k, alpha[k], beta[k], l[k], q2[k], su[k],
                        sm[k]);
    return NP_OK;
}

// ---------------------------------------------------------------------------
// Equatorial crossings by Jacobi amplitude (equator_cf.cuh), one ray per
// thread on the device and the same function on the host.
namespace {
constexpr int kDiskXMax = 16;

__host__ __device__ inline void disk_crossings_one(int i, double a, const double* u0, const double* mu0,
                                                   const double* l, const double* q2, const double* su,
                                                   const double* sm, double u_far, double u_lo, double u_hi, int K,
                                                   double* xu, double* xphi, int32_t* nx, int32_t* status) {
    double u[kDiskXMax];
    int32_t br[kDiskXMax];
    const np::gkcf::EqX o = np::gkcf::equator_crossings(a, l[i], q2[i], u0[i], mu0[i], su[i], sm[i], u_far, u_lo,
                                                         u_hi, K, u, nullptr, br);
    for (int k = 0; k < K; ++k) xu[(long long)i * K + k] = k < o.n ? u[k] : 0.0;
    if (xphi) {
        double ph[kDiskXMax];
        if (o.n > 0) np::gkcf::crossing_phi(a, l[i], q2[i], u0[i], mu0[i], su[i], sm[i], u_far, o.n, u, br, ph);
        for (int k = 0; k < K; ++k) xphi[(long long)i * K + k] = k < o.n ? ph[k] : 0.0;
    }
    nx[i] = o.n;
    if (status) status[i] = o.status;
}

__global__ void disk_crossings_kernel(int n, double a, const double* u0, const double* mu0, const double* l,
                                      const double* q2, const double* su, const double* sm, double u_far, double u_lo,
                                      double u_hi, int K, double* xu, double* xphi, int32_t* nx, int32_t* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) disk_crossings_one(i, a, u0, mu0, l, q2, su, sm, u_far, u_lo, u_hi, K, xu, xphi, nx, status);
}

int disk_crossings_check(int n, double a, double u_far, double u_lo, double u_hi, int K, const void* p0,
                         const void* p1, const void* p2, const void* p3, const void* p4, const void* p5,
                         const void* p6, const void* p7) {
    if (n < 0 || K <= 0 || K > kDiskXMax) return gk_fail(NP_ERR_INVALID, "disk crossings: bad sizes (1 <= K <= 16)");
    if (!(fabs(a) < 1.0)) return gk_fail(NP_ERR_INVALID, "spin must satisfy |a| < 1");
    if (!(u_far >= 0.0) || !(u_lo <= u_hi)) return gk_fail(NP_ERR_INVALID, "disk crossings: bad u window");
    if (n > 0 && (!p0 || !p1 || !p2 || !p3 || !p4 || !p5 || !p6 || !p7))
        return gk_fail(NP_ERR_INVALID, "NULL argument");
    return NP_OK;
}
}  // namespace

extern "C" int np_geokerr_disk_crossings_device(int n, double a, const double* d_u0, const double* d_mu0,
                                                const double* d_l, const double* d_q2, const double* d_su,
                                                const double* d_sm, double u_far, double u_lo, double u_hi, int K,
                                                double* d_xu, double* d_xphi, int32_t* d_nx, int32_t* d_status,
                                                void* stream) {
    int rc = disk_crossings_check(n, a, u_far, u_lo, u_hi, K, d_u0, d_mu0, d_l, d_q2, d_su, d_sm, d_xu, d_nx);
    if (rc != NP_OK || n == 0) return rc;
    disk_crossings_kernel<<<(n + 63) / 64, 64, 0, (cudaStream_t)stream>>>(n, a, d_u0, d_mu0, d_l, d_q2, d_su, d_sm,
                                                                          u_far, u_lo, u_hi, K, d_xu, d_xphi, d_nx,
                                                                          d_status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return gk_fail(NP_ERR_KERNEL, "disk crossings: %s", cudaGetErrorString(e));
    return NP_OK;
}

extern "C" int np_geokerr_disk_crossings_host(int n, double a, const double* u0, const double* mu0, const double* l,
                                              const double* q2, const double* su, const double* sm, double u_far,
                                              double u_lo, double u_hi, int K, double* xu, double* xphi, int32_t* nx,
                                              int32_t* status) {
    int rc = disk_crossings_check(n, a, u_far, u_lo, u_hi, K, u0, mu0, l, q2, su, sm, xu, nx);
    if (rc != NP_OK) return rc;
    for (int i = 0; i < n; ++i) disk_crossings_one(i, a, u0, mu0, l, q2, su, sm, u_far, u_lo, u_hi, K, xu, xphi, nx, status);
    return NP_OK;
}
