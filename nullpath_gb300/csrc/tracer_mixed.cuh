// tracer_mixed.cuh -- mixed-precision Kerr ray tracer (FP32 bulk, FP64 islands).
//
// The same Hamiltonian H = 1/2 g^{mu nu} p_mu p_nu and the same RK4 step law
// as the FP64 path (render.cu:185,207), written in Carter's separated form
//
//   2 Sigma H = Delta p_r^2 + p_theta^2 - P(r)^2 / Delta + L^2 / sin^2(theta)
//               - 2 a E L + a^2 E^2 sin^2(theta),      P(r) = (r^2 + a^2) E - a L,
//
// whose analytic r- and theta-derivatives need three reciprocals and one
// sincos per evaluation instead of the fifteen divisions of the contravariant
// block form (bh_kerr.h:600-727).  p_t = -E and p_phi = L are conserved, so
// only (r, theta, p_r, p_theta) are integrated (plus phi when requested).
//
// Precision: right-hand sides in FP32; the state is kept as an unevaluated
// (hi, lo) FP32 pair and every RK4 increment is added with an error-free
// two-sum, so rounding does not accumulate over thousands of steps.  Steps
// within 0.1 M of the outer horizon and steps across a radial or polar
// turning point are taken in FP64; rays whose impact parameter lies within
// 1e-3 M of the critical curve are handed to the FP64 tracer whole.
#pragma once

#include "np_common.cuh"
#include "tracer_fp64.cuh"

namespace np {

struct RayConst {
    float E, L, a, a2, aL, a2E2, L2, twoaEL, M, rp, rm;
};

struct F5 { float r, th, pr, pth, ph; };

// Carter-form Hamilton equations in FP32.
template <bool PHI>
__device__ __forceinline__ F5 rhs_carter_f(float r, float th, float pr, float pth, const RayConst& c) {
    float sn, cs;
    sincosf(th, &sn, &cs);
    float s2 = fmaxf(sn * sn, 1e-30f);
    float is2 = __frcp_rn(s2);
    float r2 = r * r;
    float Sig = fmaf(c.a2, cs * cs, r2);
    float iS = __frcp_rn(Sig);
    float Del = (r - c.rp) * (r - c.rm);
    float iD = __frcp_rn(Del);
    float P = fmaf(r2 + c.a2, c.E, -c.aL);
    float PiD = P * iD;
    float W = fmaf(c.L2, is2, fmaf(c.a2E2, s2, -c.twoaEL));
    float F = fmaf(Del * pr, pr, fmaf(pth, pth, fmaf(-P, PiD, W)));
    float Del_r = 2.0f * (r - c.M);
    float F_r = fmaf(Del_r, fmaf(pr, pr, PiD * PiD), -4.0f * r * c.E * PiD);
    float sc2 = 2.0f * sn * cs;
    float F_t = sc2 * fmaf(-c.L2 * is2, is2, c.a2E2);
    F5 d;
    d.r = Del * pr * iS;
    d.th = pth * iS;
    d.pr = -0.5f * iS * fmaf(-2.0f * r * iS, F, F_r);
    d.pth = -0.5f * iS * fmaf(c.a2 * sc2 * iS, F, F_t);
    d.ph = PHI ? iS * fmaf(c.a, PiD, fmaf(c.L, is2, -c.a * c.E)) : 0.0f;
    return d;
}

struct D5 { double r, th, pr, pth, ph; };

// The same equations in FP64 (island steps); zero inside r_+ + 1e-12 as the
// reference does (bh_kerr.h:684-690).
__device__ __forceinline__ D5 rhs_carter_d(const D5& y, double E, double L, double a, double M,
                                           double rp, double rm) {
    D5 d{0, 0, 0, 0, 0};
    if (y.r <= rp + 1e-12) return d;
    double sn, cs;
    sincos(y.th, &sn, &cs);
    double s2 = fmax(sn * sn, 1e-30), is2 = 1.0 / s2;
    double r = y.r, r2 = r * r, a2 = a * a;
    double Sig = r2 + a2 * cs * cs, iS = 1.0 / Sig;
    double Del = (r - rp) * (r - rm), iD = 1.0 / Del;
    double P = (r2 + a2) * E - a * L, PiD = P * iD;
    double W = L * L * is2 + a2 * E * E * s2 - 2.0 * a * E * L;
    double F = Del * y.pr * y.pr + y.pth * y.pth - P * PiD + W;
    double Del_r = 2.0 * (r - M);
    double F_r = Del_r * (y.pr * y.pr + PiD * PiD) - 4.0 * r * E * PiD;
    double sc2 = 2.0 * sn * cs;
    double F_t = sc2 * (a2 * E * E - L * L * is2 * is2);
    d.r = Del * y.pr * iS;
    d.th = y.pth * iS;
    d.pr = -0.5 * iS * (F_r - 2.0 * r * iS * F);
    d.pth = -0.5 * iS * (F_t + a2 * sc2 * iS * F);
    d.ph = iS * (a * PiD + L * is2 - a * E);
    return d;
}

__device__ __forceinline__ D5 add5(const D5& y, double h, const D5& k) {
    return D5{y.r + h * k.r, y.th + h * k.th, y.pr + h * k.pr, y.pth + h * k.pth, y.ph + h * k.ph};
}

// Error-free transformation a + b = s + e (Knuth two-sum).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

struct HiLo { float hi, lo; };
__device__ __forceinline__ double hl_d(const HiLo& v) { return (double)v.hi + (double)v.lo; }
__device__ __forceinline__ HiLo d_hl(double x) { float h = (float)x; return HiLo{h, (float)(x - (double)h)}; }
__device__ __forceinline__ void hl_add(HiLo& v, float d) {
    float s, e;
    two_sum(v.hi, d, s, e);
    e = __fadd_rn(e, v.lo);
    v.hi = __fadd_rn(s, e);                  // renormalise (fast two-sum)
    v.lo = __fsub_rn(e, __fsub_rn(v.hi, s));
}

// theta - pi/2 of a (hi, lo) angle, exact for |theta - pi/2| < pi/2.
__device__ __forceinline__ float dtheta_eq(const HiLo& th) {
    const float PI2_HI = 1.57079637050628662109375f;          // (float)(pi/2)
    const float PI2_LO = -4.37113900018624283e-8f;             // pi/2 - PI2_HI
    return __fadd_rn(__fsub_rn(th.hi, PI2_HI), __fsub_rn(th.lo, PI2_LO));
}

// Closeness of a ray to the critical curve: R(r) = P(r)^2 - Delta K has a
// double root at the spherical photon orbit r_c exactly for critical rays.
// r_c solves R'(r) = 0, i.e. the depressed cubic
//   4 E^2 r^3 + (4 a^2 E^2 - 4 a E L - 2 K) r + 2 M K = 0,
// and near the critical curve R(r_c)/(E^2 r_c^4) ~ -(dR/db) db / r_c^4.  The
// scale 0.385/M is that derivative for the Schwarzschild photon sphere, so
// the test reads |b - b_crit| < db_thr.  Returns true when the ray is closer
// than db_thr (in M).
__device__ __forceinline__ bool near_critical(double E, double L, double Q, double a, double M,
                                              double rp, double db_thr) {
    double K = Q + (L - a * E) * (L - a * E);
    double c3 = 4.0 * E * E;
    double c1 = 4.0 * a * a * E * E - 4.0 * a * E * L - 2.0 * K;
    double c0 = 2.0 * M * K;
    // largest real root of c3 r^3 + c1 r + c0 by Newton from above
    double r = fmax(3.0 * M, sqrt(fmax(0.0, -c1 / c3)) + 2.0 * M) + 4.0 * M;
    for (int it = 0; it < 40; ++it) {
        double f = (c3 * r * r + c1) * r + c0;
        double fp = 3.0 * c3 * r * r + c1;
        if (fp <= 0.0) break;
        double dr = f / fp;
        r -= dr;
        if (fabs(dr) < 1e-13 * r) break;
    }
    if (!(r > rp)) return false;
    double r2 = r * r, a2 = a * a;
    double P = (r2 + a2) * E - a * L;
    double Del = r2 - 2.0 * M * r + a2;
    double R = P * P - Del * K;
    double eps = fabs(R) / (E * E * r2 * r2);
    return eps < 0.385 * db_thr / M;
}

// Per-lane ray of the mixed tracer.  PHI integrates phi and records the
// first four equatorial crossings for the per-ray report.
template <bool PHI>
struct RayMixed {
    HiLo r, th, pr, pth, ph;
    float k[5];                  // f(y) at the current state (first stage of the next step)
    RayConst c;
    double E, L;                 // conserved momenta in FP64
    double min_r, first_r;
    double xr[PHI ? 4 : 1], xphi[PHI ? 4 : 1];
    float disk[3];
    int step, orders, crossings, status;
    unsigned fp64_steps;
};

template <bool PHI>
__device__ __forceinline__ void mixed_set_k(RayMixed<PHI>& R) {
    F5 f = rhs_carter_f<PHI>(R.r.hi, R.th.hi, R.pr.hi, R.pth.hi, R.c);
    R.k[0] = f.r; R.k[1] = f.th; R.k[2] = f.pr; R.k[3] = f.pth; R.k[4] = f.ph;
}

template <bool PHI>
__device__ __forceinline__ void mixed_init(const SceneDev& s, const Momentum& m, RayMixed<PHI>& R) {
    R.E = -m.pt; R.L = m.pph;
    R.c.E = (float)R.E; R.c.L = (float)R.L; R.c.a = (float)s.a; R.c.a2 = (float)(s.a * s.a);
    R.c.aL = (float)(s.a * R.L); R.c.a2E2 = (float)(s.a * s.a * R.E * R.E);
    R.c.L2 = (float)(R.L * R.L); R.c.twoaEL = (float)(2.0 * s.a * R.E * R.L);
    R.c.M = (float)s.M; R.c.rp = (float)s.r_plus; R.c.rm = (float)s.r_minus;
    R.r = d_hl(s.r_cam); R.th = d_hl(s.th_cam); R.pr = d_hl(m.pr); R.pth = d_hl(m.pth); R.ph = d_hl(s.ph_cam);
    R.min_r = s.r_cam; R.first_r = 0.0;
    R.disk[0] = R.disk[1] = R.disk[2] = 0.0f;
    R.step = 0; R.orders = 0; R.crossings = 0; R.status = 2; R.fp64_steps = 0;
    if (PHI) for (int k = 0; k < 4; ++k) { R.xr[k] = 0.0; R.xphi[k] = 0.0; }
    mixed_set_k(R);
}

// One FP64 RK4 step from (hi, lo) state; returns false when the ray fell
// through the horizon or reached a pole (bh_kerr.h:770-773).
template <bool PHI>
__device__ __forceinline__ bool mixed_step_fp64(const SceneDev& s, RayMixed<PHI>& R, double h) {
    D5 y{hl_d(R.r), hl_d(R.th), hl_d(R.pr), hl_d(R.pth), PHI ? hl_d(R.ph) : 0.0};
    const double E = R.E, L = R.L, a = s.a, M = s.M, rp = s.r_plus, rm = s.r_minus;
    D5 k1 = rhs_carter_d(y, E, L, a, M, rp, rm);
    D5 k2 = rhs_carter_d(add5(y, 0.5 * h, k1), E, L, a, M, rp, rm);
    D5 k3 = rhs_carter_d(add5(y, 0.5 * h, k2), E, L, a, M, rp, rm);
    D5 k4 = rhs_carter_d(add5(y, h, k3), E, L, a, M, rp, rm);
    double h6 = h / 6.0;
    y.r += h6 * (k1.r + 2.0 * k2.r + 2.0 * k3.r + k4.r);
    y.th += h6 * (k1.th + 2.0 * k2.th + 2.0 * k3.th + k4.th);
    y.pr += h6 * (k1.pr + 2.0 * k2.pr + 2.0 * k3.pr + k4.pr);
    y.pth += h6 * (k1.pth + 2.0 * k2.pth + 2.0 * k3.pth + k4.pth);
    if (PHI) y.ph += h6 * (k1.ph + 2.0 * k2.ph + 2.0 * k3.ph + k4.ph);
    R.r = d_hl(y.r); R.th = d_hl(y.th); R.pr = d_hl(y.pr); R.pth = d_hl(y.pth);
    if (PHI) R.ph = d_hl(y.ph);
    R.fp64_steps++;
    return y.r > rp + 1e-9 && y.th > 1e-9 && y.th < kPi - 1e-9;
}

// Advances one step; returns true when the ray terminated.
template <bool PHI>
__device__ __forceinline__ bool mixed_advance(const SceneDev& s, RayMixed<PHI>& R, unsigned long long& evals) {
    if (R.step >= s.max_steps) { R.status = 2; return true; }
    const float rf = R.r.hi;
    const double h = s.h_unit * fmin(fmax(1.0, (double)rf / s.M), 100.0);
    // start of step (for crossings and island redo)
    const HiLo r0 = R.r, th0 = R.th, pr0 = R.pr, pth0 = R.pth, ph0 = R.ph;
    const float k0r = R.k[0], k0t = R.k[1], k0p = R.k[4];
    bool ok;
    if ((s.islands & kIslandHorizon) && (double)rf < s.r_plus + kHorizonBand) {
        ok = mixed_step_fp64(s, R, h);
        evals += 4;
    } else {
        const float hf = (float)h, hh = 0.5f * hf;
        F5 k2 = rhs_carter_f<PHI>(R.r.hi + fmaf(hh, R.k[0], R.r.lo), R.th.hi + fmaf(hh, R.k[1], R.th.lo),
                                  R.pr.hi + fmaf(hh, R.k[2], R.pr.lo), R.pth.hi + fmaf(hh, R.k[3], R.pth.lo), R.c);
        F5 k3 = rhs_carter_f<PHI>(R.r.hi + fmaf(hh, k2.r, R.r.lo), R.th.hi + fmaf(hh, k2.th, R.th.lo),
                                  R.pr.hi + fmaf(hh, k2.pr, R.pr.lo), R.pth.hi + fmaf(hh, k2.pth, R.pth.lo), R.c);
        F5 k4 = rhs_carter_f<PHI>(R.r.hi + fmaf(hf, k3.r, R.r.lo), R.th.hi + fmaf(hf, k3.th, R.th.lo),
                                  R.pr.hi + fmaf(hf, k3.pr, R.pr.lo), R.pth.hi + fmaf(hf, k3.pth, R.pth.lo), R.c);
        const float h6 = (float)(h / 6.0);
        hl_add(R.r, h6 * (R.k[0] + 2.0f * (k2.r + k3.r) + k4.r));
        hl_add(R.th, h6 * (R.k[1] + 2.0f * (k2.th + k3.th) + k4.th));
        hl_add(R.pr, h6 * (R.k[2] + 2.0f * (k2.pr + k3.pr) + k4.pr));
        hl_add(R.pth, h6 * (R.k[3] + 2.0f * (k2.pth + k3.pth) + k4.pth));
        if (PHI) hl_add(R.ph, h6 * (R.k[4] + 2.0f * (k2.ph + k3.ph) + k4.ph));
        evals += 3;
        bool turn = ((pr0.hi > 0.0f) != (R.pr.hi > 0.0f)) || ((pth0.hi > 0.0f) != (R.pth.hi > 0.0f));
        if ((s.islands & kIslandTurning) && turn) {
            R.r = r0; R.th = th0; R.pr = pr0; R.pth = pth0; R.ph = ph0;
            ok = mixed_step_fp64(s, R, h);
            evals += 4;
        } else {
            ok = (double)R.r.hi > s.r_plus + 1e-9 && R.th.hi > 1e-9f && (double)R.th.hi < kPi - 1e-9;
        }
    }
    R.step++;
    if (!ok) { R.status = 1; return true; }
    mixed_set_k(R);
    evals += 1;
    double rn = hl_d(R.r);
    R.min_r = fmin(R.min_r, rn);
    float dp = dtheta_eq(th0), dc = dtheta_eq(R.th);
    bool sc = (dp > 0.0f && dc < 0.0f) || (dp < 0.0f && dc > 0.0f);
    bool nz = (fabsf(dp) < 1e-8f && fabsf(dc) >= 1e-8f) || (fabsf(dc) < 1e-8f && fabsf(dp) >= 1e-8f);
    if (sc || nz) {
        double d0 = dp, d1 = dc;
        double alpha = fabs(d0) / (fabs(d0) + fabs(d1) + 1e-30);
        double r_0 = hl_d(r0);
        double rc, phc = 0.0;
        if (s.crossing == NP_CROSS_HERMITE && sc) {
            double u = hermite_root(d0, d1, h * (double)k0t, h * (double)R.k[1], alpha);
            rc = hermite_eval(r_0, rn, h * (double)k0r, h * (double)R.k[0], u);
            if (PHI) phc = hermite_eval(hl_d(ph0), hl_d(R.ph), h * (double)k0p, h * (double)R.k[4], u);
        } else {
            rc = r_0 + alpha * (rn - r_0);
            if (PHI) phc = hl_d(ph0) + alpha * (hl_d(R.ph) - hl_d(ph0));
        }
        if (PHI) {
            if (R.crossings < 4) { R.xr[R.crossings] = rc; R.xphi[R.crossings] = phc; }
        }
        R.crossings++;
        if (R.orders < s.max_orders && rc >= s.rin && rc <= s.rout) {
            float g = (float)doppler_g(rc, -R.E, R.L, s.M, s.a);
            shade_disk((float)rc, g, s.qf, s.gain, R.disk);
            if (R.orders == 0) R.first_r = rc;
            R.orders++;
        }
    }
    if (rn > s.r_far && R.step > 11) { R.status = 0; return true; }
    return false;
}

// |H| at the current state, for the invariant report (E and L are exact).
template <bool PHI>
__device__ __forceinline__ void mixed_invariants(const SceneDev& s, const RayMixed<PHI>& R, double r, double th, float* inv3) {
    double sn, cs;
    sincos(th, &sn, &cs);
    double s2 = fmax(sn * sn, 1e-30), a = s.a, a2 = a * a, E = R.E, L = R.L;
    double Sig = r * r + a2 * cs * cs;
    double Del = (r - s.r_plus) * (r - s.r_minus);
    double P = (r * r + a2) * E - a * L;
    double pr = hl_d(R.pr), pth = hl_d(R.pth);
    double F = Del * pr * pr + pth * pth - P * P / Del + L * L / s2 - 2.0 * a * E * L + a2 * E * E * s2;
    atomic_max_nonneg(&inv3[0], (float)fabs(0.5 * F / Sig));
    atomic_max_nonneg(&inv3[1], 0.0f);
    atomic_max_nonneg(&inv3[2], 0.0f);
}

}  // namespace np
