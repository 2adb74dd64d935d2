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

}  // namespace np
