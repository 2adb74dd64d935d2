// tracer_df.cuh -- the FP64-class steps of the mixed 7(8) path in
// double-float arithmetic (dfloat.cuh) on the FP32 pipes.
//
// The island steps (turning points, the horizon band) and the near-critical
// rays of the mixed path need far more than FP32's 24 bits, and GB300 issues
// FP64 at 1/64 of the FP32 rate.  Here they run the same Fehlberg 7(8) pair,
// Carter-form right-hand side and Henon crossing as the native FP64 versions
// in tracer_mixed.cuh, on double-float numbers (48-bit significands; an
// addition is 20 FP32 operations, a multiplication 8).  The lane's (hi, lo)
// FP32 state is already a double-float, so nothing converts through FP64.
#pragma once

#include "dfloat.cuh"
#include "tracer_mixed.cuh"

namespace np {

// Spacetime constants as double-floats (from the scene's FP64 values, split
// on the host).
struct DfK {
    DF a, a2, M, rp, rm;
};
__device__ __forceinline__ DfK dfk_of(const SceneDev& s) {
    DfK k;
    k.a = DF(s.a_hl[0], s.a_hl[1]);
    k.a2 = k.a * k.a;
    k.M = DF(s.M_hl[0], s.M_hl[1]);
    k.rp = DF(s.rp_hl[0], s.rp_hl[1]);
    k.rm = DF(s.rm_hl[0], s.rm_hl[1]);
    return k;
}
__device__ __forceinline__ DF df_of(const HiLo& v) { return DF(v.hi, v.lo); }
__device__ __forceinline__ HiLo hl_of(const DF& v) { return HiLo{v.hi, v.lo}; }

// Carter-form Hamilton equations (as rhs_dsc) on double-floats, given sin
// and cos of theta; zero inside r_+ (plus a relative 1e-12).
__device__ __forceinline__ V5<DF> rhs_carter_df(const V4<DF>& y, DF sn, DF cs, DF E, DF L, const DfK& k) {
    const DF zero(0.0f, 0.0f);
    if (!(y.r > k.rp * DF(1.0 + 1e-12))) return V5<DF>{zero, zero, zero, zero, zero};
    DF s2 = sn * sn;
    if (!(s2.hi > 1e-30f)) s2 = DF(1e-30f, 0.0f);
    const DF r2 = y.r * y.r;
    const DF Sig = r2 + k.a2 * (cs * cs);
    const DF Del = (y.r - k.rp) * (y.r - k.rm);
    const DF SD = Sig * Del;
    const DF inv = DF(1.0f, 0.0f) / (s2 * SD);
    const DF is2 = SD * inv, iS = (s2 * Del) * inv, iD = (s2 * Sig) * inv;
    const DF P = (r2 + k.a2) * E - k.a * L, PiD = P * iD;
    const DF aE = k.a * E;
    const DF W = (L * L) * is2 + (aE * aE) * s2 - (aE * L) * 2.0f;
    const DF F = (Del * y.pr) * y.pr + y.pth * y.pth - P * PiD + W;
    const DF Del_r = (y.r - k.M) * 2.0f;
    const DF F_r = Del_r * (y.pr * y.pr + PiD * PiD) - (y.r * E) * PiD * 4.0f;
    const DF sc2 = (sn * cs) * 2.0f;
    const DF F_t = sc2 * (aE * aE - (L * L) * is2 * is2);
    V5<DF> d;
    d.r = (Del * y.pr) * iS;
    d.th = y.pth * iS;
    d.pr = iS * (F_r - (y.r * iS) * F * 2.0f) * -0.5f;
    d.pth = iS * (F_t + (k.a2 * sc2) * iS * F) * -0.5f;
    d.ph = iS * (k.a * PiD + L * is2 - aE);
    return d;
}

// sin and cos of theta0 + d from those of theta0: the Taylor series of sin d
// through d^11 and cos d through d^12 (truncation < 2e-22 for |d| <= 1/8)
// and the angle-addition formulas; larger d evaluates df_sincos.
__device__ __forceinline__ void df_stage_sincos(DF th0, DF sn0, DF cs0, DF d, DF& sn, DF& cs) {
    if (fabsf(d.hi) <= 0.125f) {
        const DF z = d * d;
        DF ps = DF(-1.0 / 39916800.0);
        ps = ps * z + DF(1.0 / 362880.0);
        ps = ps * z + DF(-1.0 / 5040.0);
        ps = ps * z + DF(1.0 / 120.0);
        ps = ps * z + DF(-1.0 / 6.0);
        ps = ps * z + DF(1.0f, 0.0f);
        const DF sd = ps * d;
        DF pc = DF(1.0 / 479001600.0);
        pc = pc * z + DF(-1.0 / 3628800.0);
        pc = pc * z + DF(1.0 / 40320.0);
        pc = pc * z + DF(-1.0 / 720.0);
        pc = pc * z + DF(1.0 / 24.0);
        pc = pc * z + DF(-0.5);
        pc = pc * z + DF(1.0f, 0.0f);
        sn = sn0 * pc + cs0 * sd;
        cs = cs0 * pc - sn0 * sd;
    } else {
        df_sincos(th0 + d, sn, cs);
    }
}

struct Ev78df {
    const V4<DF>& y;
    DF sn0, cs0, h, E, L;
    const DfK& k;
    __device__ __forceinline__ V5<DF> operator()(const V4<DF>& S) const {
        DF sn, cs;
        df_stage_sincos(y.th, sn0, cs0, h * S.th, sn, cs);
        const V4<DF> z{y.r + h * S.r, y.th + h * S.th, y.pr + h * S.pr, y.pth + h * S.pth};
        return rhs_carter_df(z, sn, cs, E, L, k);
    }
};

struct Ev78dfHenon {
    const V4<DF>& y;
    DF sn0, cs0, dth, E, L;
    const DfK& k;
    __device__ __forceinline__ V5<DF> operator()(const V4<DF>& S) const {
        DF sn, cs;
        df_stage_sincos(y.th, sn0, cs0, dth * S.th, sn, cs);
        const V4<DF> z{y.r + dth * S.r, y.th + dth * S.th, y.pr + dth * S.pr, y.pth + dth * S.pth};
        const V5<DF> f = rhs_carter_df(z, sn, cs, E, L, k);
        const DF it = DF(1.0f, 0.0f) / f.th;
        return V5<DF>{f.r * it, DF(1.0f, 0.0f), f.pr * it, f.pth * it, f.ph * it};
    }
};

// pi/2 as a double-float.
__device__ __forceinline__ DF df_half_pi() { return DF(1.57079637050628662109375f, -4.37113882867379e-08f); }

// Henon crossing from y0 (sin/cos sn0, cs0, f(y0) = f0) in double-floats;
// false when ill-conditioned.
__device__ __forceinline__ bool henon78_df(const V4<DF>& y0, DF ph0, DF sn0, DF cs0, const V5<DF>& f0, DF E, DF L,
                                           const DfK& k, DF& rc, DF& phc) {
    const DF dth = df_half_pi() - y0.th;
    const DF it = DF(1.0f, 0.0f) / f0.th;
    const V5<DF> g1{f0.r * it, DF(1.0f, 0.0f), f0.pr * it, f0.pth * it, f0.ph * it};
    V5<DF> d;
    V4<DF> err;
    f78_combine<DF, true>(g1, dth, Ev78dfHenon{y0, sn0, cs0, dth, E, L, k}, d, err);
    if (!isfinite(d.r) || !(fabsf(d.r.hi) < 1e4f)) return false;
    rc = y0.r + d.r;
    phc = ph0 + d.ph;
    return true;
}

// ---------------------------------------------------------------------------
// One double-float 7(8) step, by value and not inlined: the island steps of
// FP32 rays and the steps of near-critical rays share this one instance (its
// code is long, and inlining it at every call site multiplies compile time).
// Attempts from h until one is accepted (at most max_att, h shrinking by the
// controller); an accepted step that crosses the equator is landed on it by
// a double-float Henon step when `root` is set.
struct DfIn {
    DF r, th, pr, pth, ph, E, L;
    float h, rtol, atol, hmin;
    int root, max_att;
};
struct DfOut {
    DF r, th, pr, pth, ph, rc, phc;
    float h_taken, h_next, e;
    int ok, crossed, attempts;
};

__device__ __noinline__ DfOut step78_df(const DfIn in, const DfK K) {
    DfOut o;
    const V4<DF> y{in.r, in.th, in.pr, in.pth};
    DF sn0, cs0;
    df_sincos(y.th, sn0, cs0);
    const V5<DF> f0 = rhs_carter_df(y, sn0, cs0, in.E, in.L, K);
    float hf = in.h;
    V5<DF> d;
    float e = 0.0f;
    bool acc = false;
    int att = 0;
#pragma unroll 1
    while (att < in.max_att) {
        ++att;
        const DF h(hf, 0.0f);
        V4<DF> err;
        f78_combine<DF, true>(f0, h, Ev78df{y, sn0, cs0, h, in.E, in.L, K}, d, err);
        e = df_to_float(f78_norm<DF>(y, d, err, DF(in.rtol, 0.0f), DF(in.atol, 0.0f), DF(1e-13f, 0.0f)));
        const float dth0 = df_to_float(y.th - df_half_pi());
        if (double_crossing(dth0, y.pth.hi, dth0 + df_to_float(d.th), df_to_float(y.pth + d.pth))) e = fmaxf(e, 2.0f);
        if (e <= 1.0f) { acc = true; break; }
        hf *= isfinite(e) ? f78_factor(e, false) : 0.1f;
        if (hf < in.hmin) break;
    }
    o.attempts = att;
    o.e = e;
    o.ok = acc ? 1 : 0;
    o.crossed = 0;
    o.h_taken = hf;
    o.h_next = acc ? hf * f78_factor(e, true) : hf;
    if (!acc) return o;
    o.r = y.r + d.r; o.th = y.th + d.th; o.pr = y.pr + d.pr; o.pth = y.pth + d.pth; o.ph = in.ph + d.ph;
    const float dp = df_to_float(y.th - df_half_pi()), dc = df_to_float(o.th - df_half_pi());
    if (in.root && ((dp > 0.0f && dc < 0.0f) || (dp < 0.0f && dc > 0.0f)))
        o.crossed = henon78_df(y, in.ph, sn0, cs0, f0, in.E, in.L, K, o.rc, o.phc) ? 1 : 0;
    return o;
}

// Island step of an FP32 ray in double-floats at the scene's rtol, then the
// common tail.  `attempts` returns the attempts taken.
template <bool PHI>
__device__ __forceinline__ bool mray_island78_df(MRay<PHI>& R, const SceneDev& s, const SpaceK& k, int& attempts) {
    const HiLo r0 = R.r, th0 = R.th, pr0 = R.pr, pth0 = R.pth, ph0 = R.ph;
    const float k0[5] = {R.k[0], R.k[1], R.k[2], R.k[3], R.k[4]};
    DfIn in;
    in.r = df_of(R.r); in.th = df_of(R.th); in.pr = df_of(R.pr); in.pth = df_of(R.pth); in.ph = df_of(R.ph);
    in.E = df_of(R.E); in.L = df_of(R.L);
    in.h = R.h_pend; in.rtol = s.rtol_f; in.atol = s.atol78_f; in.hmin = s.hmin_f;
    in.root = s.crossing == NP_CROSS_ROOT; in.max_att = 24;
    const DfOut o = step78_df(in, dfk_of(s));
    attempts = o.attempts;
    R.pending = false;
    R.fp64_steps++;
    if (!o.ok) { R.step++; R.status = 1; return true; }
    R.r = hl_of(o.r); R.th = hl_of(o.th); R.pr = hl_of(o.pr); R.pth = hl_of(o.pth);
    if (PHI) R.ph = hl_of(o.ph);
    R.h_adapt = o.h_next;
    if (o.crossed) {
        // landed on the equator in double-float: record here; the common tail
        // is not used, so it cannot count the crossing twice
        R.step++;
        bool ok = R.r.hi > s.r_plus_f + 1e-6f * s.r_plus_f && R.th.hi > 1e-7f && R.th.hi < s.pi_lim_f;
        if (!ok) { R.status = 1; return true; }
        mray_set_k78(R, k);
        R.min_r = fminf(R.min_r, R.r.hi);
        mray_record_crossing(R, s, k, df_to_float(o.rc), df_to_double(o.rc), df_to_float(o.phc));
        if (R.r.hi > s.r_far_f && R.step > 11) { R.status = 0; return true; }
        return false;
    }
    return mray_finish78(R, s, k, o.h_taken, r0, th0, pr0, pth0, ph0, k0);
}

// ---------------------------------------------------------------------------
// Near-critical rays traced whole in double-floats with the 7(8) pair at
// rtol_fp64 and double-float Henon crossings (one attempt per call).
template <bool REC>
struct DRay78df {
    DF r, th, pr, pth, ph, E, L;
    float h;
    float min_r, first_r;
    float disk[3];
    int step, orders, crossings, status;
    double xr[REC ? 4 : 1], xphi[REC ? 4 : 1];
};

template <bool REC>
__device__ __forceinline__ void dray78df_start(DRay78df<REC>& R, const SceneDev& s, const HiLo& E, const HiLo& L,
                                               const HiLo& pr, const HiLo& pth) {
    R.r = DF(s.r_cam_hi, s.r_cam_lo); R.th = DF(s.th_cam_hi, s.th_cam_lo);
    R.pr = df_of(pr); R.pth = df_of(pth); R.ph = DF(s.ph_cam_hi, s.ph_cam_lo);
    R.E = df_of(E); R.L = df_of(L);
    R.h = mray_h(s, s.r_cam_hi);
    R.min_r = s.r_cam_hi; R.first_r = 0.0f;
    R.disk[0] = R.disk[1] = R.disk[2] = 0.0f;
    R.step = 0; R.orders = 0; R.crossings = 0; R.status = 2;
    if (REC) for (int i = 0; i < 4; ++i) { R.xr[i] = 0.0; R.xphi[i] = 0.0; }
}

// One attempt; returns true when the ray is done; `accepted` tells whether a
// step was taken.
template <bool REC>
__device__ __forceinline__ bool dray78df_step(DRay78df<REC>& R, const SceneDev& s, bool& accepted) {
    accepted = false;
    if (R.step >= s.max_steps) { R.status = 2; return true; }
    if (s.cert_capture && R.r.hi < s.r_band_f &&
        capture_certified(df_to_double(R.r), df_to_double(R.th), df_to_double(R.pr), df_to_double(R.pth),
                          df_to_double(R.E), df_to_double(R.L), s.a, s.M, s.r_plus, s.r_minus)) {
        R.step++; R.status = 1; R.min_r = s.r_plus_f;
        return true;
    }
    DfIn in;
    in.r = R.r; in.th = R.th; in.pr = R.pr; in.pth = R.pth; in.ph = R.ph; in.E = R.E; in.L = R.L;
    in.h = fminf(R.h, 0.5f * R.r.hi); in.rtol = s.rtol64_f; in.atol = s.atol64_f; in.hmin = s.hmin_f;
    in.root = s.crossing == NP_CROSS_ROOT; in.max_att = 1;
    const DfOut o = step78_df(in, dfk_of(s));
    if (!o.ok) {
        R.h = o.h_taken * (isfinite(o.e) ? f78_factor(o.e, false) : 0.1f);
        if (R.h < s.hmin_f) { R.step++; R.status = 1; return true; }
        return false;
    }
    accepted = true;
    const DF r0 = R.r, th0 = R.th, ph0 = R.ph;
    R.r = o.r; R.th = o.th; R.pr = o.pr; R.pth = o.pth; R.ph = o.ph;
    R.h = o.h_next;
    R.step++;
    bool ok = R.r.hi > s.r_plus_f + 1e-6f * s.r_plus_f && R.th.hi > 1e-7f && R.th.hi < s.pi_lim_f;
    if (!ok) { R.status = 1; return true; }
    R.min_r = fminf(R.min_r, R.r.hi);
    const float dp = df_to_float(th0 - df_half_pi()), dc = df_to_float(R.th - df_half_pi());
    if ((dp > 0.0f && dc < 0.0f) || (dp < 0.0f && dc > 0.0f)) {
        DF rc = o.rc, phc = o.phc;
        if (!o.crossed) {
            // linear in theta over the step (grazing crossings, or another crossing mode)
            const float u = fabsf(dp) / (fabsf(dp) + fabsf(dc));
            rc = r0 + (R.r - r0) * u;
            phc = ph0 + (R.ph - ph0) * u;
        }
        if (REC && R.crossings < 4) { R.xr[R.crossings] = df_to_double(rc); R.xphi[R.crossings] = df_to_double(phc); }
        R.crossings++;
        const float rcf = df_to_float(rc);
        if (R.orders < s.max_orders && rcf >= s.rin_f && rcf <= s.rout_f) {
            const float g = doppler_g_f(rcf, R.E.hi, R.L.hi, (float)s.M, (float)s.a);
            shade_disk(rcf, g, s.qf, s.gain, R.disk);
            if (R.orders == 0) R.first_r = rcf;
            R.orders++;
        }
    }
    if (R.r.hi > s.r_far_f && R.step > 11) { R.status = 0; return true; }
    return false;
}

}  // namespace np
