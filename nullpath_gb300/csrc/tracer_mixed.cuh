// tracer_mixed.cuh -- mixed-precision Kerr ray tracer (FP32 bulk, FP64 islands).
//
// The same Hamiltonian H = 1/2 g^{mu nu} p_mu p_nu and the same RK4 step law
// as the FP64 path (render.cu:185,207), written in Carter's separated form
//
//   2 Sigma H = Delta p_r^2 + p_theta^2 - P(r)^2 / Delta + L^2 / sin^2(theta)
//               - 2 a E L + a^2 E^2 sin^2(theta),      P(r) = (r^2 + a^2) E - a L,
//
// whose analytic r- and theta-derivatives need three reciprocals and one
// sincos per evaluation instead of the divisions of the contravariant block
// form (bh_kerr.h:600-727).  p_t = -E and p_phi = L are conserved, so only
// (r, theta, p_r, p_theta) are integrated (plus phi for the per-ray report).
//
// Precision.  Right-hand sides are FP32; the state is an unevaluated
// (hi, lo) FP32 pair and every RK4 increment is added with an error-free
// two-sum, so rounding does not accumulate over thousands of steps.  FP64 is
// used only where the scene's island mask asks for it:
//   horizon   steps that start within 0.1 M of r_+;
//   turning   steps across a sign change of p_r or p_theta (redone in FP64);
//   critical  rays with |b - b_crit| < 1e-3 M (traced whole in FP64 by
//             dedicated warps).
// GB300 issues FP64 at 1/64 of the FP32 rate and a warp pays for an FP64
// instruction whatever its active-lane count, so the per-step path holds no
// FP64 instruction at all and island steps of different lanes are batched:
// a lane that needs one parks until enough lanes of its warp are parked (or
// none is left stepping) and the warp then takes all their FP64 steps at once.
#pragma once

#include "np_common.cuh"

namespace np {

__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

struct HiLo { float hi, lo; };
__host__ __device__ __forceinline__ double hl_d(const HiLo& v) { return (double)v.hi + (double)v.lo; }
__host__ __device__ __forceinline__ HiLo d_hl(double x) { float h = (float)x; return HiLo{h, (float)(x - (double)h)}; }

// Error-free a + b = s + e (Knuth two-sum), then renormalised into v.
__device__ __forceinline__ void hl_add(HiLo& v, float d) {
    float s = __fadd_rn(v.hi, d);
    float bb = __fsub_rn(s, v.hi);
    float e = __fadd_rn(__fsub_rn(v.hi, __fsub_rn(s, bb)), __fsub_rn(d, bb));
    e = __fadd_rn(e, v.lo);
    v.hi = __fadd_rn(s, e);
    v.lo = __fsub_rn(e, __fsub_rn(v.hi, s));
}

// Packed FP32 pairs: the f32x2 arithmetic of sm_100-class GPUs does two
// IEEE round-to-nearest operations in one instruction.  The FP32 step is
// issue-bound, and its (r, theta) and (p_r, p_theta) updates pair up
// exactly; on the 1280x720x4 frame this took the kernel from 85.1 to 81.4 ms.
struct P2 { unsigned long long v; };
__device__ __forceinline__ P2 p2(float a, float b) {
    P2 r; asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b)); return r;
}
__device__ __forceinline__ void p2_get(P2 x, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(x.v));
}
__device__ __forceinline__ P2 add2(P2 a, P2 b) { P2 r; asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v)); return r; }
__device__ __forceinline__ P2 sub2(P2 a, P2 b) { P2 r; asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v)); return r; }
__device__ __forceinline__ P2 mul2(P2 a, P2 b) { P2 r; asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v)); return r; }
__device__ __forceinline__ P2 fma2(P2 a, P2 b, P2 c) {
    P2 r; asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v)); return r;
}
// hl_add on two (hi, lo) pairs at once.
__device__ __forceinline__ void hl_add2(P2& hi, P2& lo, P2 d) {
    P2 s = add2(hi, d);
    P2 bb = sub2(s, hi);
    P2 e = add2(sub2(hi, sub2(s, bb)), sub2(d, bb));
    e = add2(e, lo);
    hi = add2(s, e);
    lo = sub2(e, sub2(hi, s));
}

// theta - pi/2 of a (hi, lo) angle, exact while |theta - pi/2| < pi/2.
__device__ __forceinline__ float dtheta_eq(const HiLo& th) {
    const float PI2_HI = 1.57079637050628662109375f;   // fl(pi/2)
    const float PI2_LO = -4.37113900018624283e-8f;      // pi/2 - fl(pi/2)
    return __fadd_rn(__fsub_rn(th.hi, PI2_HI), __fsub_rn(th.lo, PI2_LO));
}

// Constants of one ray (FP32) and of the spacetime.
struct RayK {
    float E, L, aL, a2E2, L2, twoaEL;
};
struct SpaceK {
    float a, a2, M, rp, rm;
};

struct F5 { float r, th, pr, pth, ph; };

// sin and cos of theta on [0, pi] (and a little beyond) in FP32 without
// general range reduction.  theta is folded to |z| <= pi/4 with two-part
// constants, z = theta, theta - pi/2 or pi - theta (exact differences where
// they matter), so both results keep full relative accuracy near the poles
// and near the equator; then the Taylor series of sin through z^11 and of
// cos through z^10 (truncation below 2e-10 for |z| <= pi/4), in Horner form.
// Host builds (the accuracy probe) compile this with FP contraction off, so
// the plain operators round like the device intrinsics.
__host__ __device__ __forceinline__ float add_rn(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
__host__ __device__ __forceinline__ float sub_rn(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}

__host__ __device__ __forceinline__ void sincos_polar(float th, float& sn, float& cs) {
    const float PI_HI = 3.14159274101257324f, PI_LO = -8.74227766e-8f;       // fl(pi), pi - fl(pi)
    const float PI2_HI = 1.57079637050628662f, PI2_LO = -4.37113883e-8f;    // fl(pi/2), pi/2 - fl(pi/2)
    const bool mid = th >= 0.785398163f, top = th > 2.35619449f;
    float z = top ? add_rn(sub_rn(PI_HI, th), PI_LO) : (mid ? sub_rn(sub_rn(th, PI2_HI), PI2_LO) : th);
    float z2 = z * z;
    float ps = fmaf(z2, -1.0f / 39916800.0f, 1.0f / 362880.0f);
    ps = fmaf(z2, ps, -1.0f / 5040.0f);
    ps = fmaf(z2, ps, 1.0f / 120.0f);
    ps = fmaf(z2, ps, -1.0f / 6.0f);
    ps = z * fmaf(z2, ps, 1.0f);
    float pc = fmaf(z2, -1.0f / 3628800.0f, 1.0f / 40320.0f);
    pc = fmaf(z2, pc, -1.0f / 720.0f);
    pc = fmaf(z2, pc, 1.0f / 24.0f);
    pc = fmaf(z2, pc, -0.5f);
    pc = fmaf(z2, pc, 1.0f);
    // [0, pi/4): (sin z, cos z); [pi/4, 3pi/4]: (cos z, -sin z); (3pi/4, ...]: (sin z, -cos z)
    const bool mid_only = mid && !top;
    sn = mid_only ? pc : ps;
    cs = mid_only ? -ps : (top ? -pc : pc);
}

// Carter-form Hamilton equations in FP32.
template <bool PHI>
__device__ __forceinline__ F5 rhs_f(float r, float th, float pr, float pth, const RayK& c, const SpaceK& k) {
    float sn, cs;
    sincos_polar(th, sn, cs);
    float s2 = fmaxf(sn * sn, 1e-30f);
    float is2 = rcp_approx(s2);
    float r2 = r * r;
    float Sig = fmaf(k.a2, cs * cs, r2);
    float iS = rcp_approx(Sig);
    float Del = (r - k.rp) * (r - k.rm);
    float iD = rcp_approx(Del);
    float P = fmaf(r2 + k.a2, c.E, -c.aL);
    float PiD = P * iD;
    float W = fmaf(c.L2, is2, fmaf(c.a2E2, s2, -c.twoaEL));
    float F = fmaf(Del * pr, pr, fmaf(pth, pth, fmaf(-P, PiD, W)));
    float Del_r = 2.0f * (r - k.M);
    float F_r = fmaf(Del_r, fmaf(pr, pr, PiD * PiD), -4.0f * r * c.E * PiD);
    float sc2 = 2.0f * sn * cs;
    float F_t = sc2 * fmaf(-c.L2 * is2, is2, c.a2E2);
    F5 d;
    d.r = Del * pr * iS;
    d.th = pth * iS;
    d.pr = -0.5f * iS * fmaf(-2.0f * r * iS, F, F_r);
    d.pth = -0.5f * iS * fmaf(k.a2 * sc2 * iS, F, F_t);
    d.ph = PHI ? iS * fmaf(k.a, PiD, fmaf(c.L, is2, -k.a * c.E)) : 0.0f;
    return d;
}

struct D5 { double r, th, pr, pth, ph; };

// The same equations in FP64 (island steps and near-critical rays), given
// sin and cos of theta; zero inside r_+ + 1e-12 as the reference does
// (bh_kerr.h:684-690).  GB300 issues FP64 at 1/64 of the FP32 rate, so the
// three reciprocals share one division.
__device__ __forceinline__ D5 rhs_dsc(const D5& y, double sn, double cs, double E, double L, double a, double M,
                                      double rp, double rm) {
    D5 d{0, 0, 0, 0, 0};
    if (y.r <= rp + 1e-12) return d;
    double s2 = fmax(sn * sn, 1e-30);
    double r = y.r, r2 = r * r, a2 = a * a;
    double Sig = r2 + a2 * cs * cs;
    double Del = (r - rp) * (r - rm);
    double SD = Sig * Del, inv = 1.0 / (s2 * SD);
    double is2 = SD * inv, iS = s2 * Del * inv, iD = s2 * Sig * inv;
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

__device__ __forceinline__ D5 rhs_d(const D5& y, double E, double L, double a, double M, double rp, double rm) {
    double sn, cs;
    sincos(y.th, &sn, &cs);
    return rhs_dsc(y, sn, cs, E, L, a, M, rp, rm);
}

// sin and cos of theta0 + d from those of theta0.  An RK4 stage moves theta
// by a small angle d; sin d and cos d come from their Taylor series through
// d^13 and d^12 (truncation below 1e-18 for |d| <= 1/4) and the angle-
// addition formulas, about half the FP64 instructions of sincos.  Larger d
// falls back to sincos.
__device__ __forceinline__ void stage_sincos_d(double th0, double sn0, double cs0, double d, double& sn, double& cs) {
    if (fabs(d) <= 0.25) {
        const double z = d * d;
        const double sd = d * (1.0 + z * (-1.0 / 6.0 + z * (1.0 / 120.0 + z * (-1.0 / 5040.0 + z * (1.0 / 362880.0 +
                              z * (-1.0 / 39916800.0 + z * (1.0 / 6227020800.0)))))));
        const double cd = 1.0 + z * (-0.5 + z * (1.0 / 24.0 + z * (-1.0 / 720.0 + z * (1.0 / 40320.0 +
                              z * (-1.0 / 3628800.0 + z * (1.0 / 479001600.0))))));
        sn = sn0 * cd + cs0 * sd;
        cs = cs0 * cd - sn0 * sd;
    } else {
        sincos(th0 + d, &sn, &cs);
    }
}

__device__ __forceinline__ D5 add5(const D5& y, double h, const D5& k) {
    return D5{y.r + h * k.r, y.th + h * k.th, y.pr + h * k.pr, y.pth + h * k.pth, y.ph + h * k.ph};
}

// One FP64 RK4 step of the Carter system whose first stage k1 = f(y) is
// known, with sin/cos of y.th.
__device__ __forceinline__ D5 rk4_d_k1(const D5& y, double sn0, double cs0, const D5& k1, double h, double E,
                                       double L, double a, double M, double rp, double rm, bool phi) {
    double sn, cs;
    const double hh = 0.5 * h;
    stage_sincos_d(y.th, sn0, cs0, hh * k1.th, sn, cs);
    D5 k2 = rhs_dsc(add5(y, hh, k1), sn, cs, E, L, a, M, rp, rm);
    stage_sincos_d(y.th, sn0, cs0, hh * k2.th, sn, cs);
    D5 k3 = rhs_dsc(add5(y, hh, k2), sn, cs, E, L, a, M, rp, rm);
    stage_sincos_d(y.th, sn0, cs0, h * k3.th, sn, cs);
    D5 k4 = rhs_dsc(add5(y, h, k3), sn, cs, E, L, a, M, rp, rm);
    double h6 = h * (1.0 / 6.0);
    D5 o;
    o.r = y.r + h6 * (k1.r + 2.0 * (k2.r + k3.r) + k4.r);
    o.th = y.th + h6 * (k1.th + 2.0 * (k2.th + k3.th) + k4.th);
    o.pr = y.pr + h6 * (k1.pr + 2.0 * (k2.pr + k3.pr) + k4.pr);
    o.pth = y.pth + h6 * (k1.pth + 2.0 * (k2.pth + k3.pth) + k4.pth);
    o.ph = phi ? y.ph + h6 * (k1.ph + 2.0 * (k2.ph + k3.ph) + k4.ph) : y.ph;
    return o;
}

__device__ __forceinline__ D5 rk4_d(const D5& y, double h, double E, double L, double a, double M,
                                    double rp, double rm, bool phi) {
    double sn, cs;
    sincos(y.th, &sn, &cs);
    return rk4_d_k1(y, sn, cs, rhs_dsc(y, sn, cs, E, L, a, M, rp, rm), h, E, L, a, M, rp, rm, phi);
}

// Redshift g = E / (u^t (E - Omega L)) of a prograde Keplerian emitter on
// the equator (the physics of bh_kerr.h:833-862, with k.u expanded), FP32.
__device__ __forceinline__ float doppler_g_f(float r, float E, float L, float M, float a) {
    float Ms = fmaxf(1e-12f, M);
    float x = fmaxf(1.0f, r / Ms);
    float Om = 1.0f / ((a / Ms + x * sqrtf(x)) * Ms);
    float ir = 1.0f / r;
    float gtt = -(1.0f - 2.0f * M * ir);
    float gtp = -2.0f * M * a * ir;
    float gpp = r * r + a * a + 2.0f * M * a * a * ir;
    float den = -(gtt + Om * (2.0f * gtp + gpp * Om));
    float ut = rsqrtf(fmaxf(den, 1e-24f));
    float ku = ut * (E - Om * L);
    float g = E / fmaxf(ku, 1e-18f);
    return fmaxf(g, 0.0f);
}

// Root in [0, 1] of the cubic Hermite interpolant of d = theta - pi/2 over
// one step (d0, d1 of opposite sign; slopes m0, m1 = h dtheta/dlambda),
// safeguarded Newton from the linear estimate.
__device__ __forceinline__ float hermite_root_f(float d0, float d1, float m0, float m1, float s_lin) {
    float s = s_lin, lo = 0.0f, hi = 1.0f;
#pragma unroll 1
    for (int it = 0; it < 6; ++it) {
        float s2 = s * s, s3 = s2 * s;
        float h00 = 2.0f * s3 - 3.0f * s2 + 1.0f, h10 = s3 - 2.0f * s2 + s;
        float h01 = 1.0f - h00, h11 = s3 - s2;
        float p = h00 * d0 + h10 * m0 + h01 * d1 + h11 * m1;
        float dh00 = 6.0f * (s2 - s);
        float dp = dh00 * (d0 - d1) + (3.0f * s2 - 4.0f * s + 1.0f) * m0 + (3.0f * s2 - 2.0f * s) * m1;
        if ((p > 0.0f) == (d0 > 0.0f)) lo = s; else hi = s;
        float sn = (dp != 0.0f) ? s - p / dp : 0.5f * (lo + hi);
        if (!(sn > lo && sn < hi)) sn = 0.5f * (lo + hi);
        bool done = fabsf(sn - s) < 1e-7f;
        s = sn;
        if (done) break;
    }
    return s;
}

// Per-lane ray of the mixed tracer.
template <bool PHI>
struct MRay {
    HiLo r, th, pr, pth, ph;
    float k[5];                  // f(y) at the current state (first stage of the next step)
    HiLo E, L;                   // conserved momenta (p_t = -E, p_phi = L)
    RayK c;
    float min_r, first_r, h_pend, h_adapt;
    float disk[3];
    int step, orders, crossings, status;
    bool pending;                // parked for an FP64 island step of size h_pend
    bool pend_halves;            // the island step is two half steps (adaptive mode)
    unsigned fp64_steps;
    float xr[PHI ? 4 : 1], xphi[PHI ? 4 : 1];
    double xr_d[PHI ? 4 : 1];
};

template <bool PHI>
__device__ __forceinline__ void mray_consts(MRay<PHI>& R, float a) {
    const float E = R.E.hi, L = R.L.hi;
    R.c.E = E; R.c.L = L;
    R.c.aL = a * L;
    float aE = a * E;
    R.c.a2E2 = aE * aE;
    R.c.L2 = L * L;
    R.c.twoaEL = 2.0f * aE * L;
}

template <bool PHI>
__device__ __forceinline__ void mray_set_k(MRay<PHI>& R, const SpaceK& k) {
    F5 f = rhs_f<PHI>(R.r.hi, R.th.hi, R.pr.hi, R.pth.hi, R.c, k);
    R.k[0] = f.r; R.k[1] = f.th; R.k[2] = f.pr; R.k[3] = f.pth; R.k[4] = f.ph;
}

template <bool PHI>
__device__ __forceinline__ void mray_start(MRay<PHI>& R, const SceneDev& s, const SpaceK& k) {
    R.r = HiLo{s.r_cam_hi, s.r_cam_lo};
    R.th = HiLo{s.th_cam_hi, s.th_cam_lo};
    R.ph = HiLo{s.ph_cam_hi, s.ph_cam_lo};
    R.min_r = s.r_cam_hi; R.first_r = 0.0f; R.h_pend = 0.0f; R.h_adapt = 0.0f; R.pend_halves = false;
    R.disk[0] = R.disk[1] = R.disk[2] = 0.0f;
    R.step = 0; R.orders = 0; R.crossings = 0; R.status = 2;
    R.pending = false; R.fp64_steps = 0;
    if (PHI) for (int i = 0; i < 4; ++i) { R.xr[i] = 0.0f; R.xphi[i] = 0.0f; R.xr_d[i] = 0.0; }
    mray_consts(R, k.a);
    mray_set_k(R, k);
}

// Common tail of a step (FP32 or island): termination, next k1, crossing,
// escape.  (r0, th0, k0r, k0t, ph0, k0p) describe the start of the step.
template <bool PHI>
__device__ __forceinline__ bool mray_finish_step(MRay<PHI>& R, const SceneDev& s, const SpaceK& k, float h,
                                                 const HiLo& r0, const HiLo& th0, float k0r, float k0t,
                                                 const HiLo& ph0, float k0p) {
    R.step++;
    bool ok = R.r.hi > s.r_plus_f + 1e-6f * s.r_plus_f && R.th.hi > 1e-7f && R.th.hi < s.pi_lim_f;
    if (!ok) { R.status = 1; return true; }
    mray_set_k(R, k);
    R.min_r = fminf(R.min_r, R.r.hi);
    float dp = dtheta_eq(th0), dc = dtheta_eq(R.th);
    bool sc = (dp > 0.0f && dc < 0.0f) || (dp < 0.0f && dc > 0.0f);
    bool nz = (fabsf(dp) < 1e-8f && fabsf(dc) >= 1e-8f) || (fabsf(dc) < 1e-8f && fabsf(dp) >= 1e-8f);
    if (sc || nz) {
        float alpha = fabsf(dp) / (fabsf(dp) + fabsf(dc) + 1e-30f);
        float u = alpha;
        if (s.crossing == NP_CROSS_HERMITE && sc) u = hermite_root_f(dp, dc, h * k0t, h * R.k[1], alpha);
        // r(u) = r0 + h01 (r1 - r0) + h10 m0 + h11 m1, with r1 - r0 formed from the pairs
        float dr = (R.r.hi - r0.hi) + (R.r.lo - r0.lo);
        float corr;
        if (s.crossing == NP_CROSS_HERMITE && sc) {
            float u2 = u * u, u3 = u2 * u;
            corr = (3.0f * u2 - 2.0f * u3) * dr + (u3 - 2.0f * u2 + u) * (h * k0r) + (u3 - u2) * (h * R.k[0]);
        } else {
            corr = u * dr;
        }
        float rc_lo = r0.lo + corr;
        float rc = r0.hi + rc_lo;
        if (PHI && R.crossings < 4) {
            float dph = (R.ph.hi - ph0.hi) + (R.ph.lo - ph0.lo);
            float cph;
            if (s.crossing == NP_CROSS_HERMITE && sc) {
                float u2 = u * u, u3 = u2 * u;
                cph = (3.0f * u2 - 2.0f * u3) * dph + (u3 - 2.0f * u2 + u) * (h * k0p) + (u3 - u2) * (h * R.k[4]);
            } else {
                cph = u * dph;
            }
            R.xr[R.crossings] = rc;
            R.xr_d[R.crossings] = (double)r0.hi + (double)rc_lo;
            R.xphi[R.crossings] = (float)((double)ph0.hi + (double)(ph0.lo + cph));
        }
        R.crossings++;
        if (R.orders < s.max_orders && rc >= s.rin_f && rc <= s.rout_f) {
            float g = doppler_g_f(rc, R.E.hi, R.L.hi, k.M, k.a);
            shade_disk(rc, g, s.qf, s.gain, R.disk);
            if (R.orders == 0) R.first_r = rc;
            R.orders++;
        }
    }
    if (R.r.hi > s.r_far_f && R.step > 11) { R.status = 0; return true; }
    return false;
}

// Step size of render.cu:185,207 for the current radius (FP32).
__device__ __forceinline__ float mray_h(const SceneDev& s, float r) {
    return s.h_unit_f * fminf(fmaxf(1.0f, r * s.inv_M_f), 100.0f);
}
// Largest adaptive step: BH_RK_HMAX (bh_common.h:253) for reference scenes,
// 10 x the fixed step law for scenes in units of M.
__device__ __forceinline__ float mray_hmax(const SceneDev& s, float r) {
    return s.ref_units ? s.hmax_f : s.hmax_f * fminf(fmaxf(1.0f, r * s.inv_M_f), 100.0f);
}

// Result of an FP32 attempt.
enum { STEP_CONT = 0, STEP_DONE = 1, STEP_PARK = 2 };

// One FP32 step, or parks the lane for an FP64 island step.
template <bool PHI>
__device__ __forceinline__ int mray_step32(MRay<PHI>& R, const SceneDev& s, const SpaceK& k) {
    if (R.step >= s.max_steps) { R.status = 2; return STEP_DONE; }
    const float h = mray_h(s, R.r.hi);
    if ((s.islands & kIslandHorizon) && R.r.hi < s.r_band_f) {
        R.pending = true; R.h_pend = h;
        return STEP_PARK;
    }
    const HiLo r0 = R.r, th0 = R.th, pr0 = R.pr, pth0 = R.pth, ph0 = R.ph;
    const float k0r = R.k[0], k0t = R.k[1], k0p = R.k[4];
    const float hh = 0.5f * h;
    // (r, theta) and (p_r, p_theta) as packed pairs
    const P2 hiA = p2(R.r.hi, R.th.hi), loA = p2(R.r.lo, R.th.lo);
    const P2 hiB = p2(R.pr.hi, R.pth.hi), loB = p2(R.pr.lo, R.pth.lo);
    const P2 hh2 = p2(hh, hh), h2 = p2(h, h);
    float a0, a1, b0, b1;
    const P2 k1A = p2(R.k[0], R.k[1]), k1B = p2(R.k[2], R.k[3]);
    p2_get(add2(hiA, fma2(hh2, k1A, loA)), a0, a1);
    p2_get(add2(hiB, fma2(hh2, k1B, loB)), b0, b1);
    F5 k2 = rhs_f<PHI>(a0, a1, b0, b1, R.c, k);
    const P2 k2A = p2(k2.r, k2.th), k2B = p2(k2.pr, k2.pth);
    p2_get(add2(hiA, fma2(hh2, k2A, loA)), a0, a1);
    p2_get(add2(hiB, fma2(hh2, k2B, loB)), b0, b1);
    F5 k3 = rhs_f<PHI>(a0, a1, b0, b1, R.c, k);
    const P2 k3A = p2(k3.r, k3.th), k3B = p2(k3.pr, k3.pth);
    p2_get(add2(hiA, fma2(h2, k3A, loA)), a0, a1);
    p2_get(add2(hiB, fma2(h2, k3B, loB)), b0, b1);
    F5 k4 = rhs_f<PHI>(a0, a1, b0, b1, R.c, k);
    const float h6 = h * (1.0f / 6.0f);
    const P2 h62 = p2(h6, h6), two = p2(2.0f, 2.0f);
    P2 dA = mul2(h62, add2(fma2(two, add2(k2A, k3A), k1A), p2(k4.r, k4.th)));
    P2 dB = mul2(h62, add2(fma2(two, add2(k2B, k3B), k1B), p2(k4.pr, k4.pth)));
    P2 nhA = hiA, nlA = loA, nhB = hiB, nlB = loB;
    hl_add2(nhA, nlA, dA);
    hl_add2(nhB, nlB, dB);
    p2_get(nhA, R.r.hi, R.th.hi); p2_get(nlA, R.r.lo, R.th.lo);
    p2_get(nhB, R.pr.hi, R.pth.hi); p2_get(nlB, R.pr.lo, R.pth.lo);
    if (PHI) hl_add(R.ph, h6 * (R.k[4] + 2.0f * (k2.ph + k3.ph) + k4.ph));
    if (s.islands & kIslandTurning) {
        bool turn = ((pr0.hi > 0.0f) != (R.pr.hi > 0.0f)) || ((pth0.hi > 0.0f) != (R.pth.hi > 0.0f));
        if (turn) {
            R.r = r0; R.th = th0; R.pr = pr0; R.pth = pth0; R.ph = ph0;
            R.pending = true; R.h_pend = h;
            return STEP_PARK;
        }
    }
    return mray_finish_step(R, s, k, h, r0, th0, k0r, k0t, ph0, k0p) ? STEP_DONE : STEP_CONT;
}

// The parked FP64 step of size h_pend.
template <bool PHI>
__device__ __forceinline__ bool mray_island(MRay<PHI>& R, const SceneDev& s, const SpaceK& k) {
    const HiLo r0 = R.r, th0 = R.th, ph0 = R.ph;
    const float k0r = R.k[0], k0t = R.k[1], k0p = R.k[4];
    const float h = R.h_pend;
    D5 y{hl_d(R.r), hl_d(R.th), hl_d(R.pr), hl_d(R.pth), PHI ? hl_d(R.ph) : 0.0};
    const double E = hl_d(R.E), L = hl_d(R.L);
    D5 o;
    if (R.pend_halves) {
        o = rk4_d(y, 0.5 * (double)h, E, L, s.a, s.M, s.r_plus, s.r_minus, PHI);
        o = rk4_d(o, 0.5 * (double)h, E, L, s.a, s.M, s.r_plus, s.r_minus, PHI);
    } else {
        o = rk4_d(y, (double)h, E, L, s.a, s.M, s.r_plus, s.r_minus, PHI);
    }
    R.r = d_hl(o.r); R.th = d_hl(o.th); R.pr = d_hl(o.pr); R.pth = d_hl(o.pth);
    if (PHI) R.ph = d_hl(o.ph);
    R.pending = false;
    R.fp64_steps++;
    return mray_finish_step(R, s, k, h, r0, th0, k0r, k0t, ph0, k0p);
}

// Signed closeness of a ray to the critical curve.  R(r) = P(r)^2 - Delta K
// (K = Q + (L - aE)^2) has a double root at the spherical photon orbit r_c
// exactly for critical rays; r_c solves R'(r) = 0, the depressed cubic
//   4 E^2 r^3 + (4 a^2 E^2 - 4 a E L - 2 K) r + 2 M K = 0.
// Returns R(r_c) / (E^2 r_c^4): positive for rays that fall in (no radial
// turning point outside the horizon), negative for rays that turn, and a
// huge positive value when R has no minimum outside r_+ (captured).  Near the
// curve |R(r_c)| / (E^2 r_c^4) ~ |dR/db| |b - b_crit| / r_c^4.
__host__ __device__ __forceinline__ double critical_gap(double E, double L, double Q, double a, double M, double rp) {
    double K = Q + (L - a * E) * (L - a * E);
    double c3 = 4.0 * E * E;
    double c1 = 4.0 * a * a * E * E - 4.0 * a * E * L - 2.0 * K;
    double c0 = 2.0 * M * K;
    // largest real root by Newton from above (the cubic is convex there)
    double r = sqrt(fmax(0.0, -c1 / c3)) + 4.0 * M;
#pragma unroll 1
    for (int it = 0; it < 30; ++it) {
        double f = (c3 * r * r + c1) * r + c0;
        double fp = 3.0 * c3 * r * r + c1;
        if (fp <= 0.0) break;
        double dr = f / fp;
        r -= dr;
        if (fabs(dr) < 1e-12 * r) break;
    }
    if (!(r > rp)) return 1e300;
    double r2 = r * r, a2 = a * a;
    double P = (r2 + a2) * E - a * L;
    double Del = r2 - 2.0 * M * r + a2;
    return (P * P - Del * K) / (E * E * r2 * r2);
}

// |b - b_crit| < db_thr (in M): the scale 0.385/M is |dR/db| / r_c^4 of the
// Schwarzschild photon sphere.
__host__ __device__ __forceinline__ bool near_critical(double E, double L, double Q, double a, double M,
                                                       double rp, double db_thr) {
    double g = critical_gap(E, L, Q, a, M, rp);
    return g < 1e299 && fabs(g) < 0.385 * db_thr / M;
}

// near_critical with an FP32 screen: the FP32 gap (Newton on the same
// cubic to 1e-6 relative, then the same ratio) is within about 1e-6 of the
// FP64 one, so a ray whose FP32 gap is beyond 4x the threshold, or whose
// photon-orbit radius lies clearly inside the horizon, is not near-critical;
// every other ray takes the FP64 test.  The decisions equal near_critical's;
// most rays skip its FP64 Newton iterations (GB300 runs FP64 at 1/64 rate).
__device__ __forceinline__ bool near_critical_screened(double E, double L, double Q, double a, double M, double rp,
                                                       double db_thr) {
    const float Ef = (float)E, Lf = (float)L, Qf = (float)Q, af = (float)a, Mf = (float)M, rpf = (float)rp;
    const float K = Qf + (Lf - af * Ef) * (Lf - af * Ef);
    const float c3 = 4.0f * Ef * Ef;
    const float c1 = 4.0f * af * af * Ef * Ef - 4.0f * af * Ef * Lf - 2.0f * K;
    const float c0 = 2.0f * Mf * K;
    float r = sqrtf(fmaxf(0.0f, -c1 / c3)) + 4.0f * Mf;
    bool conv = false;
#pragma unroll 1
    for (int it = 0; it < 30; ++it) {
        const float f = (c3 * r * r + c1) * r + c0;
        const float fp = 3.0f * c3 * r * r + c1;
        if (fp <= 0.0f) break;
        const float dr = f / fp;
        r -= dr;
        if (fabsf(dr) < 1e-6f * r) { conv = true; break; }
    }
    if (conv && isfinite(r)) {
        if (r < rpf * (1.0f - 1e-4f)) return false;
        if (r > rpf * (1.0f + 1e-4f)) {
            const float r2 = r * r;
            const float P = (r2 + af * af) * Ef - af * Lf;
            const float Del = r2 - 2.0f * Mf * r + af * af;
            const float g = (P * P - Del * K) / (Ef * Ef * r2 * r2);
            if (isfinite(g) && fabsf(g) > 4.0f * 0.385f * (float)(db_thr / M)) return false;
        }
    }
    return near_critical(E, L, Q, a, M, rp, db_thr);
}

// RK4 increments d = h/6 (k1 + 2 k2 + 2 k3 + k4) of (r, theta, p_r, p_theta[, phi])
// from a (hi, lo) state whose first stage k1 is known.
template <bool PHI>
__device__ __forceinline__ void rk4_incr(const HiLo& r, const HiLo& th, const HiLo& pr, const HiLo& pth,
                                         const float k1[5], float h, const RayK& c, const SpaceK& k, float d[5]) {
    const float hh = 0.5f * h;
    F5 k2 = rhs_f<PHI>(r.hi + fmaf(hh, k1[0], r.lo), th.hi + fmaf(hh, k1[1], th.lo),
                       pr.hi + fmaf(hh, k1[2], pr.lo), pth.hi + fmaf(hh, k1[3], pth.lo), c, k);
    F5 k3 = rhs_f<PHI>(r.hi + fmaf(hh, k2.r, r.lo), th.hi + fmaf(hh, k2.th, th.lo),
                       pr.hi + fmaf(hh, k2.pr, pr.lo), pth.hi + fmaf(hh, k2.pth, pth.lo), c, k);
    F5 k4 = rhs_f<PHI>(r.hi + fmaf(h, k3.r, r.lo), th.hi + fmaf(h, k3.th, th.lo),
                       pr.hi + fmaf(h, k3.pr, pr.lo), pth.hi + fmaf(h, k3.pth, pth.lo), c, k);
    const float h6 = h * (1.0f / 6.0f);
    d[0] = h6 * (k1[0] + 2.0f * (k2.r + k3.r) + k4.r);
    d[1] = h6 * (k1[1] + 2.0f * (k2.th + k3.th) + k4.th);
    d[2] = h6 * (k1[2] + 2.0f * (k2.pr + k3.pr) + k4.pr);
    d[3] = h6 * (k1[3] + 2.0f * (k2.pth + k3.pth) + k4.pth);
    d[4] = PHI ? h6 * (k1[4] + 2.0f * (k2.ph + k3.ph) + k4.ph) : 0.0f;
}

__device__ __forceinline__ bool mray_alive(const SceneDev& s, float r, float th) {
    return r > s.r_plus_f + 1e-6f * s.r_plus_f && th > 1e-7f && th < s.pi_lim_f;
}

// One accepted adaptive step (step doubling with the error norm and step
// factors of bh_kerr.h:1058-1105 and the retry loop of render.cu:187-205),
// or a park for an FP64 island.  The error is measured on the compensated
// increments, |d_full - (d_half1 + d_half2)| / (atol + rtol max|y|) over
// r, theta, p_r, p_theta, so FP32 rounding of the state does not enter it.
template <bool PHI>
__device__ __forceinline__ int mray_step32_adaptive(MRay<PHI>& R, const SceneDev& s, const SpaceK& k) {
    if (R.step >= s.max_steps) { R.status = 2; return STEP_DONE; }
    const float hb = fminf(fmaxf(mray_h(s, R.r.hi), s.hmin_f), mray_hmax(s, R.r.hi));
    if ((s.islands & kIslandHorizon) && R.r.hi < s.r_band_f) {
        R.pending = true; R.pend_halves = false; R.h_pend = hb;
        return STEP_PARK;
    }
    float h = (R.h_adapt > 0.0f) ? R.h_adapt : hb;
    h = fminf(fmaxf(h, s.hmin_f), mray_hmax(s, R.r.hi));
    const HiLo r0 = R.r, th0 = R.th, pr0 = R.pr, pth0 = R.pth, ph0 = R.ph;
    const float k0r = R.k[0], k0t = R.k[1], k0p = R.k[4];
    const float rtol = s.rtol_f, atol = s.atol_f;
#pragma unroll 1
    for (int att = 0; att < 8; ++att) {
        float dF[5], dA[5], dB[5];
        rk4_incr<PHI>(r0, th0, pr0, pth0, R.k, h, R.c, k, dF);
        rk4_incr<PHI>(r0, th0, pr0, pth0, R.k, 0.5f * h, R.c, k, dA);
        HiLo r1 = r0, t1 = th0, p1 = pr0, q1 = pth0;
        hl_add(r1, dA[0]); hl_add(t1, dA[1]); hl_add(p1, dA[2]); hl_add(q1, dA[3]);
        F5 f1 = rhs_f<PHI>(r1.hi, t1.hi, p1.hi, q1.hi, R.c, k);
        float k1b[5] = {f1.r, f1.th, f1.pr, f1.pth, f1.ph};
        rk4_incr<PHI>(r1, t1, p1, q1, k1b, 0.5f * h, R.c, k, dB);
        const float rF = r0.hi + dF[0], tF = th0.hi + dF[1];
        const float r2 = r1.hi + dB[0], t2 = t1.hi + dB[1];
        bool alive = mray_alive(s, rF, tF) && mray_alive(s, r1.hi, t1.hi) && mray_alive(s, r2, t2);
        if (!alive) {
            h *= 0.5f;
        } else {
            float e = 0.0f;
            const float y0v[4] = {r0.hi, th0.hi, pr0.hi, pth0.hi};
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                float full = dF[i], half = dA[i] + dB[i];
                float sc = atol + rtol * fmaxf(fabsf(y0v[i] + full), fabsf(y0v[i] + half));
                // never ask for less than the FP32 rounding of the increments
                // themselves (~8 ulp), or a tight rtol rejects every step
                sc = fmaxf(sc, 5e-7f * (fabsf(full) + fabsf(dA[i]) + fabsf(dB[i])));
                e = fmaxf(e, fabsf(full - half) / fmaxf(sc, 1e-30f));
            }
            if (e <= 1.0f) {
                // accept the two half steps
                R.r = r1; R.th = t1; R.pr = p1; R.pth = q1;
                hl_add(R.r, dB[0]); hl_add(R.th, dB[1]); hl_add(R.pr, dB[2]); hl_add(R.pth, dB[3]);
                if (PHI) { hl_add(R.ph, dA[4]); hl_add(R.ph, dB[4]); }
                float fac = fminf(2.0f, 0.9f * __powf(fmaxf(1e-12f, e), -0.2f));
                R.h_adapt = fminf(fmaxf(h * fac, s.hmin_f), mray_hmax(s, R.r.hi));
                if (s.islands & kIslandTurning) {
                    bool turn = ((pr0.hi > 0.0f) != (R.pr.hi > 0.0f)) || ((pth0.hi > 0.0f) != (R.pth.hi > 0.0f));
                    if (turn) {
                        R.r = r0; R.th = th0; R.pr = pr0; R.pth = pth0; R.ph = ph0;
                        R.pending = true; R.pend_halves = true; R.h_pend = h;
                        return STEP_PARK;
                    }
                }
                return mray_finish_step(R, s, k, h, r0, th0, k0r, k0t, ph0, k0p) ? STEP_DONE : STEP_CONT;
            }
            h *= fmaxf(0.1f, 0.9f * __powf(fmaxf(1e-12f, e), -0.25f));
        }
        h = fmaxf(h, s.hmin_f);
        if (h <= s.hmin_f * 1.01f) break;
    }
    R.step++;
    R.status = 1;                 // no acceptable step: the reference counts the ray as captured
    return STEP_DONE;
}

// ---------------------------------------------------------------------------
// FP64 Carter-form ray for near-critical rays (traced whole in FP64).  With
// REC phi is integrated and the first four crossings are recorded.
template <bool REC>
struct DRay {
    D5 y, f;                     // state and f(state), the first stage of the next step
    double sn, cs;               // sin and cos of y.th
    double E, L;
    double min_r, first_r;
    float disk[3];
    int step, orders, crossings, status;
    double xr[REC ? 4 : 1], xphi[REC ? 4 : 1];
};

template <bool REC>
__device__ __forceinline__ void dray_start(DRay<REC>& R, const SceneDev& s, double E, double L, double pr, double pth) {
    R.y = D5{s.r_cam, s.th_cam, pr, pth, s.ph_cam};
    R.E = E; R.L = L;
    sincos(R.y.th, &R.sn, &R.cs);
    R.f = rhs_dsc(R.y, R.sn, R.cs, E, L, s.a, s.M, s.r_plus, s.r_minus);
    R.min_r = s.r_cam; R.first_r = 0.0;
    R.disk[0] = R.disk[1] = R.disk[2] = 0.0f;
    R.step = 0; R.orders = 0; R.crossings = 0; R.status = 2;
    if (REC) for (int i = 0; i < 4; ++i) { R.xr[i] = 0.0; R.xphi[i] = 0.0; }
}

// One FP64 step with the same step law, crossing rule and shading.
template <bool REC>
__device__ __forceinline__ bool dray_step(DRay<REC>& R, const SceneDev& s) {
    if (R.step >= s.max_steps) { R.status = 2; return true; }
    const double h = s.h_unit * fmin(fmax(1.0, R.y.r / s.M), 100.0);
    const D5 y0 = R.y, f0 = R.f;
    R.y = rk4_d_k1(y0, R.sn, R.cs, f0, h, R.E, R.L, s.a, s.M, s.r_plus, s.r_minus, REC);
    R.step++;
    bool ok = R.y.r > s.r_plus + 1e-9 && R.y.th > 1e-9 && R.y.th < kPi - 1e-9;
    if (!ok) { R.status = 1; return true; }
    sincos(R.y.th, &R.sn, &R.cs);
    R.f = rhs_dsc(R.y, R.sn, R.cs, R.E, R.L, s.a, s.M, s.r_plus, s.r_minus);
    const D5& f1 = R.f;
    R.min_r = fmin(R.min_r, R.y.r);
    double dp = y0.th - kPi * 0.5, dc = R.y.th - kPi * 0.5;
    bool sc = (dp > 0 && dc < 0) || (dp < 0 && dc > 0);
    bool nz = (fabs(dp) < 1e-8 && fabs(dc) >= 1e-8) || (fabs(dc) < 1e-8 && fabs(dp) >= 1e-8);
    if (sc || nz) {
        double alpha = fabs(dp) / (fabs(dp) + fabs(dc) + 1e-30);
        double rc, phc;
        if (s.crossing == NP_CROSS_HERMITE && sc) {
            double u = hermite_root(dp, dc, h * f0.th, h * f1.th, alpha);
            rc = hermite_eval(y0.r, R.y.r, h * f0.r, h * f1.r, u);
            phc = hermite_eval(y0.ph, R.y.ph, h * f0.ph, h * f1.ph, u);
        } else {
            rc = y0.r + alpha * (R.y.r - y0.r);
            phc = y0.ph + alpha * (R.y.ph - y0.ph);
        }
        if (REC && R.crossings < 4) { R.xr[R.crossings] = rc; R.xphi[R.crossings] = phc; }
        R.crossings++;
        if (R.orders < s.max_orders && rc >= s.rin && rc <= s.rout) {
            float g = (float)doppler_g(rc, -R.E, R.L, s.M, s.a);
            shade_disk((float)rc, g, s.qf, s.gain, R.disk);
            if (R.orders == 0) R.first_r = rc;
            R.orders++;
        }
    }
    if (R.y.r > s.r_far && R.step > 11) { R.status = 0; return true; }
    return false;
}

// ===========================================================================
// Embedded 7(8) integration in compensated FP32 (the mixed path's
// NP_INTEG_RKF78), with crossings landed on the equator by Henon's method.
//
// Fehlberg's 7(8) pair (E. Fehlberg, NASA TR R-287, 1968): 13 stages, the
// 8th-order solution propagated, local error estimate h 41/840 (k1 + k11 -
// k12 - k13).  Error control (one attempt per call): the weighted max norm of
// that estimate over r, theta, p_r, p_theta with the scene's rtol / atol,
// never below the FP32 rounding of the step's own increment; the step factor
// 0.9 e^(-1/8), clamped to [0.2, 5] after an accepted step and to [0.1, 0.9]
// after a rejected one.  The state stays an unevaluated (hi, lo) pair per
// component, and theta reaches sin/cos as (hi, lo) too: near the equator
// cos(theta) = -sin(theta - pi/2) is then exact to the pair's precision
// instead of to the FP32 ulp of theta (6e-8 rad), which is what the disk
// crossing radius is most sensitive to.
//
// Henon's method (M. Henon, Physica D 5, 1982): when an accepted step crosses
// theta = pi/2, one more 7(8) step is taken from the step's start with theta
// as the independent variable, dy/dtheta = f(y) / f_theta(y), of size
// pi/2 - theta_0.  It lands on the equator exactly, so the crossing radius
// carries the integrator's own error and no interpolant error.

// sin and cos of the angle hi + lo (|lo| well below ulp(hi)), folded as
// sincos_polar does but with the low part kept in the folded argument.
__host__ __device__ __forceinline__ void sincos_polar_hl(float th, float lo, float& sn, float& cs) {
    const float PI_HI = 3.14159274101257324f, PI_LO = -8.74227766e-8f;
    const float PI2_HI = 1.57079637050628662f, PI2_LO = -4.37113883e-8f;
    const bool mid = th >= 0.785398163f, top = th > 2.35619449f;
    float z = top ? add_rn(sub_rn(PI_HI, th), sub_rn(PI_LO, lo))
                  : (mid ? add_rn(sub_rn(th, PI2_HI), sub_rn(lo, PI2_LO)) : add_rn(th, lo));
    float z2 = z * z;
    float ps = fmaf(z2, -1.0f / 39916800.0f, 1.0f / 362880.0f);
    ps = fmaf(z2, ps, -1.0f / 5040.0f);
    ps = fmaf(z2, ps, 1.0f / 120.0f);
    ps = fmaf(z2, ps, -1.0f / 6.0f);
    ps = z * fmaf(z2, ps, 1.0f);
    float pc = fmaf(z2, -1.0f / 3628800.0f, 1.0f / 40320.0f);
    pc = fmaf(z2, pc, -1.0f / 720.0f);
    pc = fmaf(z2, pc, 1.0f / 24.0f);
    pc = fmaf(z2, pc, -0.5f);
    pc = fmaf(z2, pc, 1.0f);
    const bool mid_only = mid && !top;
    sn = mid_only ? pc : ps;
    cs = mid_only ? -ps : (top ? -pc : pc);
}

// rhs_f with theta given as (hi, lo).
template <bool PHI>
__device__ __forceinline__ F5 rhs_fhl(float r, float th, float tlo, float pr, float pth, const RayK& c,
                                      const SpaceK& k) {
    float sn, cs;
    sincos_polar_hl(th, tlo, sn, cs);
    float s2 = fmaxf(sn * sn, 1e-30f);
    float is2 = rcp_approx(s2);
    float r2 = r * r;
    float Sig = fmaf(k.a2, cs * cs, r2);
    float iS = rcp_approx(Sig);
    float Del = (r - k.rp) * (r - k.rm);
    float iD = rcp_approx(Del);
    float P = fmaf(r2 + k.a2, c.E, -c.aL);
    float PiD = P * iD;
    float W = fmaf(c.L2, is2, fmaf(c.a2E2, s2, -c.twoaEL));
    float F = fmaf(Del * pr, pr, fmaf(pth, pth, fmaf(-P, PiD, W)));
    float Del_r = 2.0f * (r - k.M);
    float F_r = fmaf(Del_r, fmaf(pr, pr, PiD * PiD), -4.0f * r * c.E * PiD);
    float sc2 = 2.0f * sn * cs;
    float F_t = sc2 * fmaf(-c.L2 * is2, is2, c.a2E2);
    F5 d;
    d.r = Del * pr * iS;
    d.th = pth * iS;
    d.pr = -0.5f * iS * fmaf(-2.0f * r * iS, F, F_r);
    d.pth = -0.5f * iS * fmaf(k.a2 * sc2 * iS, F, F_t);
    d.ph = PHI ? iS * fmaf(k.a, PiD, fmaf(c.L, is2, -k.a * c.E)) : 0.0f;
    return d;
}

template <typename T> struct V5 { T r, th, pr, pth, ph; };
template <typename T> struct V4 { T r, th, pr, pth; };

template <typename T>
__device__ __forceinline__ V4<T> v4(const V5<T>& k) { return V4<T>{k.r, k.th, k.pr, k.pth}; }

// One Fehlberg 7(8) combination.  ev(S) returns f at the stage input y0 +
// h S (the caller forms it from its own state representation); k1 = f(y0)
// is given.  Outputs the increments d = h sum b_i k_i and the error estimate
// err = h 41/840 (k1 + k11 - k12 - k13) of (r, theta, p_r, p_theta).
template <typename T, bool PHI, class Ev>
__device__ __forceinline__ void f78_combine(const V5<T>& K1, T h, Ev ev, V5<T>& d, V4<T>& err) {
    const V4<T> k1 = v4(K1);
#define NP78_S(expr) V4<T>{expr(r), expr(th), expr(pr), expr(pth)}
#define NP78_E2(c) (T(2.0 / 27) * k1.c)
    V5<T> f = ev(NP78_S(NP78_E2));
    const V4<T> k2 = v4(f);
#define NP78_E3(c) (T(1.0 / 36) * k1.c + T(1.0 / 12) * k2.c)
    f = ev(NP78_S(NP78_E3));
    const V4<T> k3 = v4(f);
#define NP78_E4(c) (T(1.0 / 24) * k1.c + T(1.0 / 8) * k3.c)
    f = ev(NP78_S(NP78_E4));
    const V4<T> k4 = v4(f);
#define NP78_E5(c) (T(5.0 / 12) * k1.c + T(-25.0 / 16) * k3.c + T(25.0 / 16) * k4.c)
    f = ev(NP78_S(NP78_E5));
    const V4<T> k5 = v4(f);
#define NP78_E6(c) (T(1.0 / 20) * k1.c + T(1.0 / 4) * k4.c + T(1.0 / 5) * k5.c)
    f = ev(NP78_S(NP78_E6));
    const V4<T> k6 = v4(f);
    V5<T> sb{T(34.0 / 105) * f.r, T(34.0 / 105) * f.th, T(34.0 / 105) * f.pr, T(34.0 / 105) * f.pth,
             PHI ? T(34.0 / 105) * f.ph : T(0)};
#define NP78_ACC(w)                                                                                      \
    sb.r += T(w) * f.r; sb.th += T(w) * f.th; sb.pr += T(w) * f.pr; sb.pth += T(w) * f.pth;              \
    if (PHI) sb.ph += T(w) * f.ph;
#define NP78_E7(c) (T(-25.0 / 108) * k1.c + T(125.0 / 108) * k4.c + T(-65.0 / 27) * k5.c + T(125.0 / 54) * k6.c)
    f = ev(NP78_S(NP78_E7));
    const V4<T> k7 = v4(f);
    NP78_ACC(9.0 / 35)
#define NP78_E8(c) (T(31.0 / 300) * k1.c + T(61.0 / 225) * k5.c + T(-2.0 / 9) * k6.c + T(13.0 / 900) * k7.c)
    f = ev(NP78_S(NP78_E8));
    const V4<T> k8 = v4(f);
    NP78_ACC(9.0 / 35)
#define NP78_E9(c) (T(2.0) * k1.c + T(-53.0 / 6) * k4.c + T(704.0 / 45) * k5.c + T(-107.0 / 9) * k6.c + \
                    T(67.0 / 90) * k7.c + T(3.0) * k8.c)
    f = ev(NP78_S(NP78_E9));
    const V4<T> k9 = v4(f);
    NP78_ACC(9.0 / 280)
#define NP78_E10(c) (T(-91.0 / 108) * k1.c + T(23.0 / 108) * k4.c + T(-976.0 / 135) * k5.c + T(311.0 / 54) * k6.c + \
                     T(-19.0 / 60) * k7.c + T(17.0 / 6) * k8.c + T(-1.0 / 12) * k9.c)
    f = ev(NP78_S(NP78_E10));
    const V4<T> k10 = v4(f);
    NP78_ACC(9.0 / 280)
#define NP78_E11(c) (T(2383.0 / 4100) * k1.c + T(-341.0 / 164) * k4.c + T(4496.0 / 1025) * k5.c +                \
                     T(-301.0 / 82) * k6.c + T(2133.0 / 4100) * k7.c + T(45.0 / 82) * k8.c + T(45.0 / 164) * k9.c + \
                     T(18.0 / 41) * k10.c)
    f = ev(NP78_S(NP78_E11));
    const V4<T> k11 = v4(f);
#define NP78_E12(c) (T(3.0 / 205) * k1.c + T(-6.0 / 41) * k6.c + T(-3.0 / 205) * k7.c + T(-3.0 / 41) * k8.c + \
                     T(3.0 / 41) * k9.c + T(6.0 / 41) * k10.c)
    f = ev(NP78_S(NP78_E12));
    const V4<T> k12 = v4(f);
    NP78_ACC(41.0 / 840)
#define NP78_E13(c) (T(-1777.0 / 4100) * k1.c + T(-341.0 / 164) * k4.c + T(4496.0 / 1025) * k5.c +                \
                     T(-289.0 / 82) * k6.c + T(2193.0 / 4100) * k7.c + T(51.0 / 82) * k8.c + T(33.0 / 164) * k9.c + \
                     T(12.0 / 41) * k10.c + k12.c)
    f = ev(NP78_S(NP78_E13));
    NP78_ACC(41.0 / 840)
    d = V5<T>{h * sb.r, h * sb.th, h * sb.pr, h * sb.pth, PHI ? h * sb.ph : T(0)};
    const T e1 = T(41.0 / 840) * h;
    err = V4<T>{e1 * ((k1.r + k11.r) - (k12.r + f.r)), e1 * ((k1.th + k11.th) - (k12.th + f.th)),
                e1 * ((k1.pr + k11.pr) - (k12.pr + f.pr)), e1 * ((k1.pth + k11.pth) - (k12.pth + f.pth))};
#undef NP78_S
#undef NP78_ACC
#undef NP78_E2
#undef NP78_E3
#undef NP78_E4
#undef NP78_E5
#undef NP78_E6
#undef NP78_E7
#undef NP78_E8
#undef NP78_E9
#undef NP78_E10
#undef NP78_E11
#undef NP78_E12
#undef NP78_E13
}

// Weighted max norm of a 7(8) error estimate: scale atol + rtol max(|y0|,
// |y0 + d|) per component, never below `floor_rel` |d| (the rounding of the
// increment itself in the arithmetic at hand).  A non-finite increment or
// estimate (a stage that left the domain, e.g. inside the horizon) gives an
// infinite norm: fmax alone would drop a NaN and accept the step.
template <typename T>
__device__ __forceinline__ T f78_norm(const V4<T>& y0, const V5<T>& d, const V4<T>& err, T rtol, T atol, T floor_rel) {
    T e = T(0);
    const T y[4] = {y0.r, y0.th, y0.pr, y0.pth};
    const T dd[4] = {d.r, d.th, d.pr, d.pth};
    const T ee[4] = {err.r, err.th, err.pr, err.pth};
    bool finite = true;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        T sc = atol + rtol * fmax(fabs(y[i]), fabs(y[i] + dd[i]));
        sc = fmax(sc, floor_rel * fabs(dd[i]));
        e = fmax(e, fabs(ee[i]) / fmax(sc, T(1e-30)));
        finite = finite && isfinite(dd[i]) && isfinite(ee[i]);
    }
    return finite ? e : T(1e30);
}

// Step-size factor after an attempt with error norm e.
__device__ __forceinline__ float f78_factor(float e, bool accepted) {
    const float f = 0.9f * __powf(fmaxf(e, 1e-12f), -0.125f);
    return accepted ? fminf(5.0f, fmaxf(0.2f, f)) : fminf(0.9f, fmaxf(0.1f, f));
}

// An ingoing ray (p_r < 0) at radius r is certainly captured when the radial
// potential R(r') = P(r')^2 - Delta(r') K, P = (r'^2 + a^2) E - a L,
// K = Q + (L - a E)^2, stays positive on [r_+, r]: it has no turning point
// left.  P increases with r' (E > 0) and Delta increases on [r_+, r], so
// min P^2 > Delta(r) K over the interval is sufficient.  FP64, a few
// operations; used once per ray entering the horizon band.
__device__ __forceinline__ bool capture_certified(double r, double th, double pr, double pth, double E, double L,
                                                  double a, double M, double rp, double rm) {
    if (!(pr < 0.0) || !(E > 0.0)) return false;
    double sn, cs;
    sincos(th, &sn, &cs);
    const double Q = pth * pth + cs * cs * (L * L / fmax(sn * sn, 1e-300) - a * a * E * E);
    const double K = Q + (L - a * E) * (L - a * E);
    const double Pp = (rp * rp + a * a) * E - a * L, Pr = (r * r + a * a) * E - a * L;
    const double minP = Pp > 0.0 ? Pp : (Pr < 0.0 ? -Pr : 0.0);
    const double Del = (r - rp) * (r - rm);
    return K >= 0.0 && minP * minP > Del * K * (1.0 + 1e-9) + 1e-300;
}

// A step whose theta starts moving towards the equator and ends moving
// away from it on the same side has crossed the equator twice (the polar
// motion of a ray with Q > 0 oscillates symmetrically about it): such a
// step is rejected, so that no crossing pair is missed.
__host__ __device__ __forceinline__ bool double_crossing(float dth0, float pth0, float dth1, float pth1) {
    const bool same = (dth0 > 0.0f) == (dth1 > 0.0f);
    const bool toward = (pth0 > 0.0f) == (dth0 < 0.0f);
    const bool away = (pth1 > 0.0f) == (dth1 > 0.0f);
    return same && toward && away;
}

// FP32 evaluation at the stage y0 + h S of a (hi, lo) state.
template <bool PHI>
struct Ev78f {
    const HiLo &r, &th, &pr, &pth;
    float h;
    const RayK& c;
    const SpaceK& k;
    __device__ __forceinline__ V5<float> operator()(const V4<float>& S) const {
        F5 f = rhs_fhl<PHI>(r.hi + fmaf(h, S.r, r.lo), th.hi, fmaf(h, S.th, th.lo), pr.hi + fmaf(h, S.pr, pr.lo),
                            pth.hi + fmaf(h, S.pth, pth.lo), c, k);
        return V5<float>{f.r, f.th, f.pr, f.pth, f.ph};
    }
};

// The same with theta as the independent variable (Henon): returns
// (dr, 1, dp_r, dp_theta, dphi) / dtheta at the stage theta0 + dth S.
template <bool PHI>
struct Ev78fHenon {
    const HiLo &r, &th, &pr, &pth;
    float dth;
    const RayK& c;
    const SpaceK& k;
    __device__ __forceinline__ V5<float> operator()(const V4<float>& S) const {
        F5 f = rhs_fhl<PHI>(r.hi + fmaf(dth, S.r, r.lo), th.hi, fmaf(dth, S.th, th.lo), pr.hi + fmaf(dth, S.pr, pr.lo),
                            pth.hi + fmaf(dth, S.pth, pth.lo), c, k);
        const float it = 1.0f / f.th;
        return V5<float>{f.r * it, 1.0f, f.pr * it, f.pth * it, PHI ? f.ph * it : 0.0f};
    }
};

// Crossing of theta = pi/2 inside an accepted FP32 step from (r0, th0, pr0,
// pth0, ph0) with f(y0) = k0: Henon step of size -dtheta_eq(th0).  Returns
// the crossing radius (hi, lo) and azimuth; false when the step is
// ill-conditioned (f_theta ~ 0 somewhere: a grazing ray), in which case the
// caller falls back to the Hermite interpolant.
template <bool PHI>
__device__ __forceinline__ bool henon78_f(const HiLo& r0, const HiLo& th0, const HiLo& pr0, const HiLo& pth0,
                                          const HiLo& ph0, const float k0[5], const RayK& c, const SpaceK& k,
                                          HiLo& rc, float& phc) {
    const float dth = -dtheta_eq(th0);
    const float it = 1.0f / k0[1];
    const V5<float> g1{k0[0] * it, 1.0f, k0[2] * it, k0[3] * it, PHI ? k0[4] * it : 0.0f};
    V5<float> d;
    V4<float> err;
    f78_combine<float, PHI>(g1, dth, Ev78fHenon<PHI>{r0, th0, pr0, pth0, dth, c, k}, d, err);
    if (!isfinite(d.r) || !(fabsf(d.r) < 1e4f)) return false;
    rc = r0;
    hl_add(rc, d.r);
    if (PHI) phc = (float)((double)ph0.hi + (double)(ph0.lo + d.ph));
    return true;
}

// FP64 stage evaluation of the Carter system (islands and near-critical
// rays): sin/cos of the stage angle by angle addition from those of theta0.
struct Ev78d {
    const D5& y;
    double sn0, cs0, h, E, L, a, M, rp, rm;
    __device__ __forceinline__ V5<double> operator()(const V4<double>& S) const {
        double sn, cs;
        stage_sincos_d(y.th, sn0, cs0, h * S.th, sn, cs);
        D5 z{y.r + h * S.r, y.th + h * S.th, y.pr + h * S.pr, y.pth + h * S.pth, 0.0};
        D5 f = rhs_dsc(z, sn, cs, E, L, a, M, rp, rm);
        return V5<double>{f.r, f.th, f.pr, f.pth, f.ph};
    }
};

struct Ev78dHenon {
    const D5& y;
    double sn0, cs0, dth, E, L, a, M, rp, rm;
    __device__ __forceinline__ V5<double> operator()(const V4<double>& S) const {
        double sn, cs;
        stage_sincos_d(y.th, sn0, cs0, dth * S.th, sn, cs);
        D5 z{y.r + dth * S.r, y.th + dth * S.th, y.pr + dth * S.pr, y.pth + dth * S.pth, 0.0};
        D5 f = rhs_dsc(z, sn, cs, E, L, a, M, rp, rm);
        const double it = 1.0 / f.th;
        return V5<double>{f.r * it, 1.0, f.pr * it, f.pth * it, f.ph * it};
    }
};

// FP64 Henon crossing from y0 (sin/cos sn0, cs0, f(y0) = f0); false when
// ill-conditioned.
__device__ __forceinline__ bool henon78_d(const D5& y0, double sn0, double cs0, const D5& f0, double E, double L,
                                          double a, double M, double rp, double rm, double& rc, double& phc) {
    const double dth = kPi * 0.5 - y0.th;
    const double it = 1.0 / f0.th;
    const V5<double> g1{f0.r * it, 1.0, f0.pr * it, f0.pth * it, f0.ph * it};
    V5<double> d;
    V4<double> err;
    f78_combine<double, true>(g1, dth, Ev78dHenon{y0, sn0, cs0, dth, E, L, a, M, rp, rm}, d, err);
    if (!isfinite(d.r) || !(fabs(d.r) < 1e4)) return false;
    rc = y0.r + d.r;
    phc = y0.ph + d.ph;
    return true;
}

// Records one equatorial crossing at radius rc (FP32 ray): per-ray report and
// disk shading.
template <bool PHI>
__device__ __forceinline__ void mray_record_crossing(MRay<PHI>& R, const SceneDev& s, const SpaceK& k, float rc,
                                                     double rc_d, float phc) {
    if (PHI && R.crossings < 4) {
        R.xr[R.crossings] = rc;
        R.xr_d[R.crossings] = rc_d;
        R.xphi[R.crossings] = phc;
    }
    R.crossings++;
    if (R.orders < s.max_orders && rc >= s.rin_f && rc <= s.rout_f) {
        float g = doppler_g_f(rc, R.E.hi, R.L.hi, k.M, k.a);
        shade_disk(rc, g, s.qf, s.gain, R.disk);
        if (R.orders == 0) R.first_r = rc;
        R.orders++;
    }
}

// f(y) of the current state with theta as (hi, lo) (first stage of the next 7(8) step).
template <bool PHI>
__device__ __forceinline__ void mray_set_k78(MRay<PHI>& R, const SpaceK& k) {
    F5 f = rhs_fhl<PHI>(R.r.hi, R.th.hi, R.th.lo, R.pr.hi, R.pth.hi, R.c, k);
    R.k[0] = f.r; R.k[1] = f.th; R.k[2] = f.pr; R.k[3] = f.pth; R.k[4] = f.ph;
}

// Tail of an accepted 7(8) step (FP32 or island): termination, next k1,
// crossing (Henon, Hermite fallback), escape.  y0 / k0 describe the start
// of the step; h is the step taken.
template <bool PHI>
__device__ __forceinline__ bool mray_finish78(MRay<PHI>& R, const SceneDev& s, const SpaceK& k, float h,
                                              const HiLo& r0, const HiLo& th0, const HiLo& pr0, const HiLo& pth0,
                                              const HiLo& ph0, const float k0[5]) {
    R.step++;
    bool ok = R.r.hi > s.r_plus_f + 1e-6f * s.r_plus_f && R.th.hi > 1e-7f && R.th.hi < s.pi_lim_f;
    if (!ok) { R.status = 1; return true; }
    mray_set_k78(R, k);
    R.min_r = fminf(R.min_r, R.r.hi);
    const float dp = dtheta_eq(th0), dc = dtheta_eq(R.th);
    if ((dp > 0.0f && dc < 0.0f) || (dp < 0.0f && dc > 0.0f)) {
        HiLo rc;
        float phc = 0.0f;
        if (!(s.crossing == NP_CROSS_ROOT && henon78_f<PHI>(r0, th0, pr0, pth0, ph0, k0, R.c, k, rc, phc))) {
            // cubic Hermite in lambda over the step (also the fallback of a
            // grazing crossing), or linear in theta
            const float lin = fabsf(dp) / (fabsf(dp) + fabsf(dc));
            float u = s.crossing == NP_CROSS_LINEAR ? lin : hermite_root_f(dp, dc, h * k0[1], h * R.k[1], lin);
            float dr = (R.r.hi - r0.hi) + (R.r.lo - r0.lo);
            float u2 = u * u, u3 = u2 * u;
            const bool lin_only = s.crossing == NP_CROSS_LINEAR;
            rc = r0;
            hl_add(rc, lin_only ? u * dr
                                : (3.0f * u2 - 2.0f * u3) * dr + (u3 - 2.0f * u2 + u) * (h * k0[0]) + (u3 - u2) * (h * R.k[0]));
            if (PHI) {
                float dph = (R.ph.hi - ph0.hi) + (R.ph.lo - ph0.lo);
                float cph = lin_only ? u * dph
                                     : (3.0f * u2 - 2.0f * u3) * dph + (u3 - 2.0f * u2 + u) * (h * k0[4]) + (u3 - u2) * (h * R.k[4]);
                phc = (float)((double)ph0.hi + (double)(ph0.lo + cph));
            }
        }
        mray_record_crossing(R, s, k, rc.hi + rc.lo, hl_d(rc), phc);
    }
    if (R.r.hi > s.r_far_f && R.step > 11) { R.status = 0; return true; }
    return false;
}

// One FP32 7(8) attempt.  Accepted: the state advances (STEP_CONT or
// STEP_DONE).  Rejected: h shrinks and the lane returns STEP_CONT without a
// step, so one lane's retries never stall its warp.  Island steps park the
// lane with h_pend (horizon band; turning points when the mask asks).
template <bool PHI>
__device__ __forceinline__ int mray_step78(MRay<PHI>& R, const SceneDev& s, const SpaceK& k, bool& accepted) {
    accepted = false;
    if (R.step >= s.max_steps) { R.status = 2; return STEP_DONE; }
    // a step moves r by about h (|dr/dlambda| ~ E): at most half the radius
    float h = fminf(R.h_adapt > 0.0f ? R.h_adapt : mray_h(s, R.r.hi), 0.5f * R.r.hi);
    if ((s.islands & kIslandHorizon) && R.r.hi < s.r_band_f) {
        // inside the band: a ray that provably falls in ends here (it reaches
        // r_+ without another crossing of the disk, which lies outside the
        // band); any other takes FP64 island steps
        if (s.cert_capture &&
            capture_certified(hl_d(R.r), hl_d(R.th), hl_d(R.pr), hl_d(R.pth), hl_d(R.E), hl_d(R.L), s.a, s.M,
                              s.r_plus, s.r_minus)) {
            R.step++; R.status = 1; R.min_r = s.r_plus_f;
            return STEP_DONE;
        }
        // or the whole ray is handed to the FP64 closed form (status 3)
        if (s.band_cf) { R.status = 3; return STEP_DONE; }
        R.pending = true; R.h_pend = h;
        return STEP_PARK;
    }
    const V5<float> k1{R.k[0], R.k[1], R.k[2], R.k[3], R.k[4]};
    V5<float> d;
    V4<float> err;
    f78_combine<float, PHI>(k1, h, Ev78f<PHI>{R.r, R.th, R.pr, R.pth, h, R.c, k}, d, err);
    float e = f78_norm<float>(V4<float>{R.r.hi, R.th.hi, R.pr.hi, R.pth.hi}, d, err, s.rtol_f, s.atol78_f, 0.0f);
    {
        const float dth0 = dtheta_eq(R.th);
        if (double_crossing(dth0, R.pth.hi, dth0 + d.th, R.pth.hi + d.pth)) e = fmaxf(e, 2.0f);
    }
    if (!(e <= 1.0f)) {
        h *= isfinite(e) ? f78_factor(e, false) : 0.1f;
        R.h_adapt = h;
        if (h < s.hmin_f) { R.step++; R.status = 1; return STEP_DONE; }
        return STEP_CONT;
    }
    accepted = true;
    const HiLo r0 = R.r, th0 = R.th, pr0 = R.pr, pth0 = R.pth, ph0 = R.ph;
    const float k0[5] = {R.k[0], R.k[1], R.k[2], R.k[3], R.k[4]};
    hl_add(R.r, d.r); hl_add(R.th, d.th); hl_add(R.pr, d.pr); hl_add(R.pth, d.pth);
    if (PHI) hl_add(R.ph, d.ph);
    R.h_adapt = h * f78_factor(e, true);
    if (s.islands & kIslandTurning) {
        bool turn = ((pr0.hi > 0.0f) != (R.pr.hi > 0.0f)) || ((pth0.hi > 0.0f) != (R.pth.hi > 0.0f));
        if (turn) {
            R.r = r0; R.th = th0; R.pr = pr0; R.pth = pth0; R.ph = ph0;
            R.pending = true; R.h_pend = h;
            accepted = false;
            return STEP_PARK;
        }
    }
    return mray_finish78(R, s, k, h, r0, th0, pr0, pth0, ph0, k0) ? STEP_DONE : STEP_CONT;
}

// The parked FP64 7(8) step: a by-value core and the FP32-side
// bookkeeping.  The core is inlined: a call would make the FP32 loop save
// its live registers around it, which cost more than the FP64 stage storage
// (islands are rare, and the FP32 stage vectors are dead while one runs).
struct Isl78In { double r, th, pr, pth, ph, E, L, h, a, M, rp, rm, rtol, atol, hmin; int root; };
struct Isl78Out { double r, th, pr, pth, ph, h_taken, h_next, rc, phc; int ok, crossed, attempts; };

// Attempts from h until one is accepted (at most 24, h shrinking); an
// accepted step that crosses the equator is landed on it by an FP64 Henon
// step when `root` is set.
__device__ __forceinline__ Isl78Out island78_core(const Isl78In in) {
    Isl78Out o{};
    const D5 y{in.r, in.th, in.pr, in.pth, in.ph};
    double sn0, cs0;
    sincos(y.th, &sn0, &cs0);
    const D5 f0 = rhs_dsc(y, sn0, cs0, in.E, in.L, in.a, in.M, in.rp, in.rm);
    const V5<double> k1{f0.r, f0.th, f0.pr, f0.pth, f0.ph};
    double h = in.h, e = 0.0;
    V5<double> d{};
    int att = 0;
    bool acc = false;
#pragma unroll 1
    for (; att < 24; ++att) {
        V4<double> err;
        f78_combine<double, true>(k1, h, Ev78d{y, sn0, cs0, h, in.E, in.L, in.a, in.M, in.rp, in.rm}, d, err);
        e = f78_norm<double>(V4<double>{y.r, y.th, y.pr, y.pth}, d, err, in.rtol, in.atol, 1e-15);
        if (double_crossing((float)(y.th - kPi * 0.5), (float)y.pth, (float)(y.th + d.th - kPi * 0.5),
                            (float)(y.pth + d.pth)))
            e = fmax(e, 2.0);
        if (e <= 1.0) { acc = true; break; }
        h *= isfinite(e) ? (double)f78_factor((float)e, false) : 0.1;
        if (h < in.hmin) break;
    }
    o.attempts = att + 1;
    if (!acc) return o;
    o.ok = 1;
    o.r = y.r + d.r; o.th = y.th + d.th; o.pr = y.pr + d.pr; o.pth = y.pth + d.pth; o.ph = y.ph + d.ph;
    o.h_taken = h;
    o.h_next = h * (double)f78_factor((float)e, true);
    const double dp = y.th - kPi * 0.5, dc = o.th - kPi * 0.5;
    if (in.root && ((dp > 0.0 && dc < 0.0) || (dp < 0.0 && dc > 0.0)))
        o.crossed = henon78_d(y, sn0, cs0, f0, in.E, in.L, in.a, in.M, in.rp, in.rm, o.rc, o.phc) ? 1 : 0;
    return o;
}

// The parked FP64 island step of an FP32 ray (h_pend): FP64 attempts at the
// scene's FP64 tolerance, then the common tail.  `attempts` returns the
// attempts taken.
template <bool PHI>
__device__ __forceinline__ bool mray_island78(MRay<PHI>& R, const SceneDev& s, const SpaceK& k, int& attempts) {
    const HiLo r0 = R.r, th0 = R.th, pr0 = R.pr, pth0 = R.pth, ph0 = R.ph;
    const float k0[5] = {R.k[0], R.k[1], R.k[2], R.k[3], R.k[4]};
    Isl78In in;
    in.r = hl_d(R.r); in.th = hl_d(R.th); in.pr = hl_d(R.pr); in.pth = hl_d(R.pth); in.ph = PHI ? hl_d(R.ph) : 0.0;
    in.E = hl_d(R.E); in.L = hl_d(R.L); in.h = (double)R.h_pend;
    in.a = s.a; in.M = s.M; in.rp = s.r_plus; in.rm = s.r_minus;
    // the FP32 step's own tolerance: the island changes the arithmetic of
    // the step, not its accuracy target (near-critical rays use rtol_fp64)
    in.rtol = s.rtol; in.atol = (double)s.atol78_f; in.hmin = s.hmin; in.root = s.crossing == NP_CROSS_ROOT;
    const Isl78Out o = island78_core(in);
    attempts = o.attempts;
    R.pending = false;
    R.fp64_steps++;
    if (!o.ok) { R.step++; R.status = 1; return true; }
    R.r = d_hl(o.r); R.th = d_hl(o.th); R.pr = d_hl(o.pr); R.pth = d_hl(o.pth);
    if (PHI) R.ph = d_hl(o.ph);
    R.h_adapt = (float)o.h_next;
    if (o.crossed) {
        // landed on the equator in FP64: record here; the common tail below
        // is not used, so it cannot count the crossing twice
        R.step++;
        bool ok = R.r.hi > s.r_plus_f + 1e-6f * s.r_plus_f && R.th.hi > 1e-7f && R.th.hi < s.pi_lim_f;
        if (!ok) { R.status = 1; return true; }
        mray_set_k78(R, k);
        R.min_r = fminf(R.min_r, R.r.hi);
        mray_record_crossing(R, s, k, (float)o.rc, o.rc, (float)o.phc);
        if (R.r.hi > s.r_far_f && R.step > 11) { R.status = 0; return true; }
        return false;
    }
    return mray_finish78(R, s, k, (float)o.h_taken, r0, th0, pr0, pth0, ph0, k0);
}

// ---------------------------------------------------------------------------
// Near-critical rays traced whole in FP64 with the 7(8) pair at the
// scene's FP64 tolerance and Henon crossings.
template <bool REC>
struct DRay78 {
    D5 y, f;
    double sn, cs, E, L, h;
    double min_r, first_r;
    float disk[3];
    int step, orders, crossings, status;
    double xr[REC ? 4 : 1], xphi[REC ? 4 : 1];
};

template <bool REC>
__device__ __forceinline__ void dray78_start(DRay78<REC>& R, const SceneDev& s, double E, double L, double pr,
                                             double pth) {
    R.y = D5{s.r_cam, s.th_cam, pr, pth, s.ph_cam};
    R.E = E; R.L = L;
    sincos(R.y.th, &R.sn, &R.cs);
    R.f = rhs_dsc(R.y, R.sn, R.cs, E, L, s.a, s.M, s.r_plus, s.r_minus);
    R.h = s.h_unit * fmin(fmax(1.0, R.y.r / s.M), 100.0);
    R.min_r = s.r_cam; R.first_r = 0.0;
    R.disk[0] = R.disk[1] = R.disk[2] = 0.0f;
    R.step = 0; R.orders = 0; R.crossings = 0; R.status = 2;
    if (REC) for (int i = 0; i < 4; ++i) { R.xr[i] = 0.0; R.xphi[i] = 0.0; }
}

// One attempt; returns true when the ray is done.  `accepted` tells whether
// a step was taken.
template <bool REC>
__device__ __forceinline__ bool dray78_step(DRay78<REC>& R, const SceneDev& s, bool& accepted) {
    accepted = false;
    if (R.step >= s.max_steps) { R.status = 2; return true; }
    if (s.cert_capture && R.y.r < (double)s.r_band_f &&
        capture_certified(R.y.r, R.y.th, R.y.pr, R.y.pth, R.E, R.L, s.a, s.M, s.r_plus, s.r_minus)) {
        R.step++; R.status = 1; R.min_r = s.r_plus;
        return true;
    }
    const V5<double> k1{R.f.r, R.f.th, R.f.pr, R.f.pth, R.f.ph};
    V5<double> d;
    V4<double> err;
    f78_combine<double, true>(k1, R.h, Ev78d{R.y, R.sn, R.cs, R.h, R.E, R.L, s.a, s.M, s.r_plus, s.r_minus}, d, err);
    double e = f78_norm<double>(V4<double>{R.y.r, R.y.th, R.y.pr, R.y.pth}, d, err, s.rtol64, s.atol, 1e-15);
    if (double_crossing((float)(R.y.th - kPi * 0.5), (float)R.y.pth, (float)(R.y.th + d.th - kPi * 0.5),
                        (float)(R.y.pth + d.pth)))
        e = fmax(e, 2.0);
    if (!(e <= 1.0)) {
        R.h *= isfinite(e) ? (double)f78_factor((float)e, false) : 0.1;
        if (R.h < s.hmin) { R.step++; R.status = 1; return true; }
        return false;
    }
    accepted = true;
    const D5 y0 = R.y, f0 = R.f;
    const double sn0 = R.sn, cs0 = R.cs;
    const double h_taken = R.h;
    R.y = D5{y0.r + d.r, y0.th + d.th, y0.pr + d.pr, y0.pth + d.pth, y0.ph + d.ph};
    R.h *= (double)f78_factor((float)e, true);
    R.step++;
    bool ok = R.y.r > s.r_plus + 1e-9 && R.y.th > 1e-9 && R.y.th < kPi - 1e-9;
    if (!ok) { R.status = 1; return true; }
    sincos(R.y.th, &R.sn, &R.cs);
    R.f = rhs_dsc(R.y, R.sn, R.cs, R.E, R.L, s.a, s.M, s.r_plus, s.r_minus);
    R.min_r = fmin(R.min_r, R.y.r);
    const double dp = y0.th - kPi * 0.5, dc = R.y.th - kPi * 0.5;
    if ((dp > 0 && dc < 0) || (dp < 0 && dc > 0)) {
        double rc, phc;
        if (!(s.crossing == NP_CROSS_ROOT &&
              henon78_d(y0, sn0, cs0, f0, R.E, R.L, s.a, s.M, s.r_plus, s.r_minus, rc, phc))) {
            // cubic Hermite in lambda over the step (also the fallback of a
            // grazing crossing), or linear in theta
            const double lin = fabs(dp) / (fabs(dp) + fabs(dc));
            if (s.crossing == NP_CROSS_LINEAR) {
                rc = y0.r + lin * (R.y.r - y0.r);
                phc = y0.ph + lin * (R.y.ph - y0.ph);
            } else {
                const double hs = h_taken;
                const double u = hermite_root(dp, dc, hs * f0.th, hs * R.f.th, lin);
                rc = hermite_eval(y0.r, R.y.r, hs * f0.r, hs * R.f.r, u);
                phc = hermite_eval(y0.ph, R.y.ph, hs * f0.ph, hs * R.f.ph, u);
            }
        }
        if (REC && R.crossings < 4) { R.xr[R.crossings] = rc; R.xphi[R.crossings] = phc; }
        R.crossings++;
        if (R.orders < s.max_orders && rc >= s.rin && rc <= s.rout) {
            float g = (float)doppler_g(rc, -R.E, R.L, s.M, s.a);
            shade_disk((float)rc, g, s.qf, s.gain, R.disk);
            if (R.orders == 0) R.first_r = rc;
            R.orders++;
        }
    }
    if (R.y.r > s.r_far && R.step > 11) { R.status = 0; return true; }
    return false;
}

}  // namespace np
