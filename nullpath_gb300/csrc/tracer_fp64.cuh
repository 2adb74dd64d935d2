// tracer_fp64.cuh -- the reference renderer's FP64 Hamiltonian integrator
// (render.cu:161-251) as a per-lane state machine for the persistent kernel.
//
// Formulation, floors and termination rules follow include/bh_kerr.h
// (600-774 fixed RK4, 987-1105 adaptive step doubling); all eight phase-space
// components are integrated and the stage combination uses the compensated
// sum of bh_common.h:485-493.  This is the FP64 baseline form.
#pragma once

#include "np_common.cuh"

namespace np {

struct St8 { double t, r, th, ph, pt, pr, pth, pph; };

__device__ __forceinline__ St8 axpy8(const St8& y, double h, const St8& k) {
    return St8{y.t + h * k.t, y.r + h * k.r, y.th + h * k.th, y.ph + h * k.ph,
               y.pt + h * k.pt, y.pr + h * k.pr, y.pth + h * k.pth, y.pph + h * k.pph};
}

__device__ __forceinline__ double r_plus_of(double M, double a) {
    double d = M * M - a * a;
    if (d < 0.0) d = 0.0;
    return M + sqrt(d);
}

// Hamilton's equations with the analytic inverse-metric derivatives
// (bh_kerr.h:600-727), fused into one routine that shares sin/cos.
__device__ __forceinline__ void rhs_ref(const St8& y, double M, double a, double rp, St8& f) {
    if (y.r <= rp + 1e-12 || y.r <= 1e-12) { f = St8{0, 0, 0, 0, 0, 0, 0, 0}; return; }
    double s, c;
    sincos(y.th, &s, &c);
    const double r = y.r, r2 = r * r, a2 = a * a;
    // inverse metric with floors (bh_kerr.h:600-617)
    double s2f = fmax(kEps, s * s);
    double Sgf = fmax(kEps, r2 + a2 * c * c);
    double Del = r2 - 2.0 * M * r + a2;
    double Af = (r2 + a2) * (r2 + a2) - a2 * Del * s2f;
    double g_rr = fmax(kEps, Del) / Sgf;
    double g_hh = 1.0 / Sgf;
    double g_tt = -Af / fmax(kEps, Sgf * Del);
    double g_tp = -2.0 * M * a * r / fmax(kEps, Sgf * Del);
    double g_pp = (Del - a2 * s2f) / fmax(kEps, Sgf * Del * s2f);
    // derivatives (bh_kerr.h:624-672)
    double s2 = (s * s > 1e-30) ? s * s : 1e-30;
    double B = r2 + a2;
    double Sig = r2 + a2 * c * c;
    double A = B * B - a2 * Del * s2;
    double D = Sig * Del;
    double D2 = D * D + 1e-48;
    double ds2 = 2.0 * s * c;
    double Sig_r = 2.0 * r, Sig_t = -2.0 * a2 * s * c;
    double Del_r = 2.0 * (r - M);
    double A_r = 4.0 * r * B - a2 * Del_r * s2;
    double A_t = -a2 * Del * ds2;
    double D_r = Sig_r * Del + Sig * Del_r;
    double D_t = Sig_t * Del;
    double inv_D2 = 1.0 / D2;
    double tt_r = -(A_r * D - A * D_r) * inv_D2;
    double tt_t = -(A_t * D - A * D_t) * inv_D2;
    double Nn = 2.0 * M * a * r, Nn_r = 2.0 * M * a;
    double tp_r = -(Nn_r * D - Nn * D_r) * inv_D2;
    double tp_t = (Nn * D_t) * inv_D2;
    double inv_S2 = 1.0 / (Sig * Sig);
    double rr_r = (Del_r * Sig - Del * Sig_r) * inv_S2;
    double rr_t = -(Del * Sig_t) * inv_S2;
    double hh_r = -Sig_r * inv_S2;
    double hh_t = -Sig_t * inv_S2;
    double P = Del - a2 * s2, P_t = -a2 * ds2;
    double Q = Del * Sig * s2 + 1e-48;
    double Q_r = Del_r * Sig * s2 + Del * Sig_r * s2;
    double Q_t = Del * Sig_t * s2 + Del * Sig * ds2;
    double inv_Q2 = 1.0 / (Q * Q + 1e-48);
    double pp_r = (Del_r * Q - P * Q_r) * inv_Q2;
    double pp_t = (P_t * Q - P * Q_t) * inv_Q2;

    f.t = g_tt * y.pt + g_tp * y.pph;
    f.r = g_rr * y.pr;
    f.th = g_hh * y.pth;
    f.ph = g_tp * y.pt + g_pp * y.pph;
    f.pt = 0.0;
    f.pph = 0.0;
    Klein<double> sr, st;
    sr.add(tt_r * y.pt * y.pt); sr.add(2.0 * tp_r * y.pt * y.pph); sr.add(pp_r * y.pph * y.pph);
    sr.add(rr_r * y.pr * y.pr); sr.add(hh_r * y.pth * y.pth);
    st.add(tt_t * y.pt * y.pt); st.add(2.0 * tp_t * y.pt * y.pph); st.add(pp_t * y.pph * y.pph);
    st.add(rr_t * y.pr * y.pr); st.add(hh_t * y.pth * y.pth);
    f.pr = -0.5 * sr.value();
    f.pth = -0.5 * st.value();
}

__device__ __forceinline__ double combine4(double k1, double k2, double k3, double k4) {
    Klein<double> k; k.add(k1); k.add(2.0 * k2); k.add(2.0 * k3); k.add(k4);
    return k.value();
}

// One RK4 step; k1 (= f(y)) is returned for the crossing interpolant.
__device__ __forceinline__ void rk4_ref(const St8& y, double M, double a, double rp, double h, St8& out, St8& k1) {
    St8 k2, k3, k4;
    rhs_ref(y, M, a, rp, k1);
    rhs_ref(axpy8(y, 0.5 * h, k1), M, a, rp, k2);
    rhs_ref(axpy8(y, 0.5 * h, k2), M, a, rp, k3);
    rhs_ref(axpy8(y, h, k3), M, a, rp, k4);
    double h6 = h / 6.0;
    out.t = y.t + h6 * combine4(k1.t, k2.t, k3.t, k4.t);
    out.r = y.r + h6 * combine4(k1.r, k2.r, k3.r, k4.r);
    out.th = y.th + h6 * combine4(k1.th, k2.th, k3.th, k4.th);
    out.ph = y.ph + h6 * combine4(k1.ph, k2.ph, k3.ph, k4.ph);
    out.pt = y.pt + h6 * combine4(k1.pt, k2.pt, k3.pt, k4.pt);
    out.pr = y.pr + h6 * combine4(k1.pr, k2.pr, k3.pr, k4.pr);
    out.pth = y.pth + h6 * combine4(k1.pth, k2.pth, k3.pth, k4.pth);
    out.pph = y.pph + h6 * combine4(k1.pph, k2.pph, k3.pph, k4.pph);
}

// Step doubling (bh_kerr.h:1058-1105); returns the growth factor on
// acceptance (y advanced), 0 on rejection (h shrunk).
__device__ __forceinline__ double adaptive_ref(St8& y, double M, double a, double rp, double& h,
                                               double rtol, double atol, St8& k1) {
    St8 full, half1, half2, kd;
    rk4_ref(y, M, a, rp, h, full, k1);
    double h2 = 0.5 * h;
    rk4_ref(y, M, a, rp, h2, half1, kd);
    rk4_ref(half1, M, a, rp, h2, half2, kd);
    auto alive = [&](const St8& z) { return z.r > rp + 1e-12 && z.th > 1e-9 && z.th < kPi - 1e-9; };
    if (!(alive(full) && alive(half1) && alive(half2))) { h *= 0.5; return 0.0; }
    auto nerr = [&](double u, double v) {
        double sc = atol + rtol * fmax(fabs(u), fabs(v));
        return fabs(u - v) / fmax(sc, 1e-30);
    };
    double e = fmax(fmax(nerr(full.r, half2.r), nerr(full.th, half2.th)),
                    fmax(fmax(nerr(full.ph, half2.ph), nerr(full.pr, half2.pr)),
                         fmax(nerr(full.pth, half2.pth), nerr(full.pph, half2.pph))));
    if (e <= 1.0) {
        y = half2;
        return fmin(2.0, kSafety * pow(fmax(1e-12, e), -0.2));
    }
    h *= fmax(0.1, kSafety * pow(fmax(1e-12, e), -0.25));
    return 0.0;
}

// Fehlberg's embedded 7(8) pair (E. Fehlberg, NASA TR R-287, 1968): 13
// stages, the 8th-order solution propagated, the local error estimate
// h 41/840 (k1 + k11 - k12 - k13).  The metric depends on (r, theta) only
// and p_t, p_phi are constants, so a stage input needs the (r, theta, p_r,
// p_theta) parts of earlier stages; t and phi are accumulated into the
// solution as each stage is evaluated.  Returns the weighted error norm
// over (r, theta, phi, p_r, p_theta, p_phi) (p_phi's error is zero).
struct K4 { double r, th, pr, pth; };

__device__ __forceinline__ K4 k4_of(const St8& f) { return K4{f.r, f.th, f.pr, f.pth}; }

__device__ __forceinline__ double rkf78_ref(const St8& y, double M, double a, double rp, double h, double rtol,
                                            double atol, St8& out, St8& k1full) {
    St8 z = y, f;
    double st = 0.0, sph = 0.0, eph = 0.0;   // h-free sums of b_i k_i.t, b_i k_i.ph, e_i k_i.ph
    auto eval = [&](double b, double e) {
        rhs_ref(z, M, a, rp, f);
        st += b * f.t; sph += b * f.ph; eph += e * f.ph;
        return k4_of(f);
    };
    auto set = [&](double dr, double dth, double dpr, double dpth) {
        z.r = y.r + h * dr; z.th = y.th + h * dth; z.pr = y.pr + h * dpr; z.pth = y.pth + h * dpth;
    };
    const double e1 = 41.0 / 840.0;
    K4 k1 = eval(0.0, e1);
    k1full = f;
    set(2.0 / 27 * k1.r, 2.0 / 27 * k1.th, 2.0 / 27 * k1.pr, 2.0 / 27 * k1.pth);
    K4 k2 = eval(0.0, 0.0);
#define NP_S3(c) (1.0 / 36 * k1.c + 1.0 / 12 * k2.c)
    set(NP_S3(r), NP_S3(th), NP_S3(pr), NP_S3(pth));
    K4 k3 = eval(0.0, 0.0);
#define NP_S4(c) (1.0 / 24 * k1.c + 1.0 / 8 * k3.c)
    set(NP_S4(r), NP_S4(th), NP_S4(pr), NP_S4(pth));
    K4 k4 = eval(0.0, 0.0);
#define NP_S5(c) (5.0 / 12 * k1.c - 25.0 / 16 * k3.c + 25.0 / 16 * k4.c)
    set(NP_S5(r), NP_S5(th), NP_S5(pr), NP_S5(pth));
    K4 k5 = eval(0.0, 0.0);
#define NP_S6(c) (1.0 / 20 * k1.c + 1.0 / 4 * k4.c + 1.0 / 5 * k5.c)
    set(NP_S6(r), NP_S6(th), NP_S6(pr), NP_S6(pth));
    K4 k6 = eval(34.0 / 105, 0.0);
#define NP_S7(c) (-25.0 / 108 * k1.c + 125.0 / 108 * k4.c - 65.0 / 27 * k5.c + 125.0 / 54 * k6.c)
    set(NP_S7(r), NP_S7(th), NP_S7(pr), NP_S7(pth));
    K4 k7 = eval(9.0 / 35, 0.0);
#define NP_S8(c) (31.0 / 300 * k1.c + 61.0 / 225 * k5.c - 2.0 / 9 * k6.c + 13.0 / 900 * k7.c)
    set(NP_S8(r), NP_S8(th), NP_S8(pr), NP_S8(pth));
    K4 k8 = eval(9.0 / 35, 0.0);
#define NP_S9(c) (2.0 * k1.c - 53.0 / 6 * k4.c + 704.0 / 45 * k5.c - 107.0 / 9 * k6.c + 67.0 / 90 * k7.c + 3.0 * k8.c)
    set(NP_S9(r), NP_S9(th), NP_S9(pr), NP_S9(pth));
    K4 k9 = eval(9.0 / 280, 0.0);
#define NP_S10(c) (-91.0 / 108 * k1.c + 23.0 / 108 * k4.c - 976.0 / 135 * k5.c + 311.0 / 54 * k6.c \
                   - 19.0 / 60 * k7.c + 17.0 / 6 * k8.c - 1.0 / 12 * k9.c)
    set(NP_S10(r), NP_S10(th), NP_S10(pr), NP_S10(pth));
    K4 k10 = eval(9.0 / 280, 0.0);
#define NP_S11(c) (2383.0 / 4100 * k1.c - 341.0 / 164 * k4.c + 4496.0 / 1025 * k5.c - 301.0 / 82 * k6.c \
                   + 2133.0 / 4100 * k7.c + 45.0 / 82 * k8.c + 45.0 / 164 * k9.c + 18.0 / 41 * k10.c)
    set(NP_S11(r), NP_S11(th), NP_S11(pr), NP_S11(pth));
    K4 k11 = eval(0.0, e1);
#define NP_S12(c) (3.0 / 205 * k1.c - 6.0 / 41 * k6.c - 3.0 / 205 * k7.c - 3.0 / 41 * k8.c + 3.0 / 41 * k9.c \
                   + 6.0 / 41 * k10.c)
    set(NP_S12(r), NP_S12(th), NP_S12(pr), NP_S12(pth));
    K4 k12 = eval(41.0 / 840, -e1);
#define NP_S13(c) (-1777.0 / 4100 * k1.c - 341.0 / 164 * k4.c + 4496.0 / 1025 * k5.c - 289.0 / 82 * k6.c \
                   + 2193.0 / 4100 * k7.c + 51.0 / 82 * k8.c + 33.0 / 164 * k9.c + 12.0 / 41 * k10.c + k12.c)
    set(NP_S13(r), NP_S13(th), NP_S13(pr), NP_S13(pth));
    K4 k13 = eval(41.0 / 840, -e1);
#define NP_B8(c) (34.0 / 105 * k6.c + 9.0 / 35 * k7.c + 9.0 / 35 * k8.c + 9.0 / 280 * k9.c + 9.0 / 280 * k10.c \
                  + 41.0 / 840 * k12.c + 41.0 / 840 * k13.c)
#define NP_E(c) (e1 * (k1.c + k11.c - k12.c - k13.c))
    out = y;
    out.t = y.t + h * st;
    out.ph = y.ph + h * sph;
    out.r = y.r + h * NP_B8(r);
    out.th = y.th + h * NP_B8(th);
    out.pr = y.pr + h * NP_B8(pr);
    out.pth = y.pth + h * NP_B8(pth);
    auto w = [&](double err, double u, double v) {
        double sc = atol + rtol * fmax(fabs(u), fabs(v));
        return fabs(h * err) / fmax(sc, 1e-30);
    };
    double e = fmax(fmax(w(NP_E(r), y.r, out.r), w(NP_E(th), y.th, out.th)),
                    fmax(fmax(w(eph, y.ph, out.ph), w(NP_E(pr), y.pr, out.pr)), w(NP_E(pth), y.pth, out.pth)));
#undef NP_S3
#undef NP_S4
#undef NP_S5
#undef NP_S6
#undef NP_S7
#undef NP_S8
#undef NP_S9
#undef NP_S10
#undef NP_S11
#undef NP_S12
#undef NP_S13
#undef NP_B8
#undef NP_E
    return e;
}

// Hamiltonian H = g^{mu nu} p_mu p_nu / 2, its scale Hs = the same sum of
// absolute terms (so |H| / Hs is the relative cancellation error, which
// stays meaningful near the horizon where the terms grow like 1/Delta),
// and Carter's constant Q = p_theta^2 + cos^2 theta (L^2 / sin^2 theta -
// a^2 E^2) of a state.
__device__ __forceinline__ void h_and_q(const St8& y, double M, double a, double& H, double& Hs, double& Q) {
    double sn, c;
    sincos(y.th, &sn, &c);
    double r2 = y.r * y.r, a2 = a * a;
    double s2 = fmax(kEps, sn * sn);
    double Sig = fmax(kEps, r2 + a2 * c * c);
    double Del = r2 - 2.0 * M * y.r + a2;
    double A = (r2 + a2) * (r2 + a2) - a2 * Del * s2;
    double grr = fmax(kEps, Del) / Sig, ghh = 1.0 / Sig;
    double gtt = -A / fmax(kEps, Sig * Del), gtp = -2.0 * M * a * y.r / fmax(kEps, Sig * Del);
    double gpp = (Del - a2 * s2) / fmax(kEps, Sig * Del * s2);
    double t0 = gtt * y.pt * y.pt, t1 = 2.0 * gtp * y.pt * y.pph, t2 = gpp * y.pph * y.pph;
    double t3 = grr * y.pr * y.pr, t4 = ghh * y.pth * y.pth;
    H = 0.5 * (t0 + t1 + t2 + t3 + t4);
    Hs = 0.5 * (fabs(t0) + fabs(t1) + fabs(t2) + fabs(t3) + fabs(t4));
    Q = y.pth * y.pth + c * c * (y.pph * y.pph / s2 - a2 * y.pt * y.pt);
}

__device__ __forceinline__ void invariants_ref(const SceneDev& s, const St8& y, double pt0, double pph0, float* inv3) {
    double sn, c;
    sincos(y.th, &sn, &c);
    double r2 = y.r * y.r, a2 = s.a * s.a;
    double s2 = fmax(kEps, sn * sn);
    double Sig = fmax(kEps, r2 + a2 * c * c);
    double Del = r2 - 2.0 * s.M * y.r + a2;
    double A = (r2 + a2) * (r2 + a2) - a2 * Del * s2;
    double grr = fmax(kEps, Del) / Sig, ghh = 1.0 / Sig;
    double gtt = -A / fmax(kEps, Sig * Del), gtp = -2.0 * s.M * s.a * y.r / fmax(kEps, Sig * Del);
    double gpp = (Del - a2 * s2) / fmax(kEps, Sig * Del * s2);
    double H = 0.5 * (gtt * y.pt * y.pt + 2.0 * gtp * y.pt * y.pph + gpp * y.pph * y.pph
                      + grr * y.pr * y.pr + ghh * y.pth * y.pth);
    atomic_max_nonneg(&inv3[0], (float)fabs(H));
    atomic_max_nonneg(&inv3[1], (float)(fabs(y.pt - pt0) / fmax(1e-12, fabs(pt0))));
    atomic_max_nonneg(&inv3[2], (float)(fabs(y.pph - pph0) / fmax(1e-12, fabs(pph0))));
}

// Per-lane ray of the FP64 tracer.  With REC the first four equatorial
// crossings (any radius) are recorded for the per-ray report.  q0 and qs
// are Carter's constant at the camera and its drift scale max(|Q0|,
// (E M)^2); dH and dQ the largest |H| / Hs and |Q - Q0| / qs seen (drift
// tracking only).
template <bool REC>
struct RayFP64 {
    St8 y, prev;
    double min_r, h_adapt, first_r, pt0, pph0;
    double q0, qs, dH, dQ;
    double cur_H, cur_Q;                   // H and Q at the current state (the invariant gate's reference)
    double x_h, x_dp, x_alpha;             // pending root-found crossing: step size, start offset, linear guess
    double xr[REC ? 4 : 1], xphi[REC ? 4 : 1];
    float disk[3];
    int step, orders, crossings, status;   // status: 0 escaped, 1 captured, 2 step cap
    int att;                               // rejected 7(8) attempts of the current step
    bool xpend;                            // the last step crossed the equator; its root is not yet found
};

template <bool REC>
__device__ __forceinline__ void fp64_init(const SceneDev& s, const Momentum& m, RayFP64<REC>& R) {
    R.y = St8{0.0, s.r_cam, s.th_cam, s.ph_cam, m.pt, m.pr, m.pth, m.pph};
    R.prev = R.y;
    R.min_r = s.r_cam;
    R.h_adapt = 0.0;
    R.first_r = 0.0;
    R.pt0 = m.pt; R.pph0 = m.pph;
    double H0, Hs0, Q0;
    h_and_q(R.y, s.M, s.a, H0, Hs0, Q0);
    R.q0 = Q0;
    R.cur_H = H0; R.cur_Q = Q0;
    R.att = 0;
    R.qs = fmax(fabs(Q0), m.pt * m.pt * s.M * s.M);
    R.dH = fabs(H0) / fmax(Hs0, 1e-300);
    R.dQ = 0.0;
    R.disk[0] = R.disk[1] = R.disk[2] = 0.0f;
    R.step = 0; R.orders = 0; R.crossings = 0; R.status = 2;
    R.xpend = false; R.x_h = R.x_dp = R.x_alpha = 0.0;
    if (REC) for (int k = 0; k < 4; ++k) { R.xr[k] = 0.0; R.xphi[k] = 0.0; }
}

// Integrator families of fp64_advance: RK4 and step doubling (chosen by
// the scene at run time), or the embedded 7(8) pair.
constexpr int kFp64Rk4 = 0;
constexpr int kFp64Rkf78 = 1;

// One step of size h from y with the family's single-step map (the
// crossing root finder re-integrates the crossing step with it).
template <int MODE>
__device__ __forceinline__ void fp64_single_step(const SceneDev& s, const St8& y, double h, St8& out,
                                                 unsigned long long& evals) {
    St8 k1;
    if (MODE == kFp64Rkf78) {
        rkf78_ref(y, s.M, s.a, s.r_plus, h, s.rtol, s.atol, out, k1);
        evals += 13;
    } else {
        rk4_ref(y, s.M, s.a, s.r_plus, h, out, k1);
        evals += 4;
    }
}

// Crossing of theta = pi/2 inside the step prev -> (prev advanced by h):
// Newton iteration on the fraction u of the step, each iterate a fresh
// single step of u h from prev, safeguarded by the sign bracket [0, 1].
// Returns the state at the crossing.
template <int MODE>
__device__ __forceinline__ St8 fp64_root_crossing(const SceneDev& s, const St8& prev, double h, double dp, double u0,
                                                  unsigned long long& evals) {
    const double hp = kPi * 0.5;
    double lo = 0.0, hi = 1.0, u = u0;
    St8 z = prev, f;
    for (int it = 0; it < 10; ++it) {
        fp64_single_step<MODE>(s, prev, u * h, z, evals);
        double g = z.th - hp;
        if (g == 0.0) break;
        if ((g > 0.0) == (dp > 0.0)) lo = u; else hi = u;
        rhs_ref(z, s.M, s.a, s.r_plus, f);
        evals += 1;
        double dg = h * f.th;
        double un = (dg != 0.0) ? u - g / dg : 0.5 * (lo + hi);
        if (!(un > lo && un < hi)) un = 0.5 * (lo + hi);
        bool done = fabs(un - u) < 1e-15;
        u = un;
        if (done) break;
    }
    return z;
}

// Book-keeping of one equatorial crossing at radius rc, azimuth phc (alpha
// the linear fraction of the step, for the conserved momenta there).
template <bool REC>
__device__ __forceinline__ void fp64_record_crossing(const SceneDev& s, RayFP64<REC>& R, double rc, double phc,
                                                     double alpha, float* inv3) {
    if (REC) {
        if (R.crossings < 4) { R.xr[R.crossings] = rc; R.xphi[R.crossings] = phc; }
    }
    R.crossings++;
    if (R.orders < s.max_orders && rc >= s.rin && rc <= s.rout) {
        double pt = R.prev.pt + alpha * (R.y.pt - R.prev.pt);
        double pph = R.prev.pph + alpha * (R.y.pph - R.prev.pph);
        float g = (float)doppler_g(rc, pt, pph, s.M, s.a);
        shade_disk((float)rc, g, s.qf, s.gain, R.disk);
        if (R.orders == 0) R.first_r = rc;
        R.orders++;
        if (s.check_inv && inv3) {
            St8 cr = R.y; cr.r = rc; cr.th = kPi * 0.5; cr.pt = pt; cr.pph = pph;
            invariants_ref(s, cr, R.pt0, R.pph0, inv3);
        }
    }
}

// End of an accepted step: the next step starts here; escape test.
template <bool REC>
__device__ __forceinline__ bool fp64_step_tail(const SceneDev& s, RayFP64<REC>& R) {
    R.prev = R.y;
    if (R.y.r > s.r_far && R.step > 11) { R.status = 0; return true; }
    return false;
}

// Advances the ray by one accepted step; returns true when it terminated.
// `evals` counts right-hand-side evaluations; with TRK the drift of H and
// Q is tracked over the accepted steps.  With DEFER a root-found crossing
// is left pending (R.xpend) for fp64_resolve, which a warp runs for all its
// pending lanes at once: a lone lane's root search would otherwise hold the
// other 31 lanes of its warp for about four single steps.
template <int MODE, bool TRK, bool DEFER = false, bool REC>
__device__ __forceinline__ bool fp64_advance(const SceneDev& s, RayFP64<REC>& R, float* inv3, unsigned long long& evals) {
    if (R.step >= s.max_steps) { R.status = 2; return true; }
    const double M = s.M, a = s.a, rp = s.r_plus;
    double scale = fmin(fmax(1.0, R.y.r / (0.5 * s.Rs)), 100.0);
    bool ok = false;
    double h_used = 0.0;
    St8 k1;
    if (MODE == kFp64Rkf78) {
        // One attempt per call: a rejected attempt shrinks h and returns, so
        // a lane that needs many attempts (near the horizon) takes them over
        // several passes of the warp's loop while the other lanes step.
        // Same step bounds as step doubling; controller 0.9 e^(-1/8) within
        // [0.2, 4] on acceptance, [0.1, 0.9] on rejection, halving on a
        // horizon or gate rejection; at most 24 attempts per step, and a
        // step that fails at the smallest h ends the ray as captured (the
        // limits of step doubling).  The gate bounds this step's change of
        // H and Q (not their drift since the camera, which no step size could
        // undo) and is not applied at the smallest step.
        const double hmin = s.hmin, hmax = s.ref_units ? s.hmax : s.hmax * scale;
        double h = (R.h_adapt > 0.0) ? R.h_adapt : s.h_unit * scale;
        h = fmin(fmax(h, hmin), hmax);
        St8 out;
        double e = rkf78_ref(R.y, M, a, rp, h, s.rtol, s.atol, out, k1);
        evals += 13;
        bool alive = out.r > rp + 1e-12 && out.th > 1e-9 && out.th < kPi - 1e-9 && e == e;
        bool acc = alive && e <= 1.0;
        bool gated = false;
        double H = 0.0, Hs = 0.0, Q = 0.0;
        if (acc && s.inv_gate > 0.0) {
            h_and_q(out, M, a, H, Hs, Q);
            if (h > hmin * 1.01) {
                gated = fabs(H - R.cur_H) > s.inv_gate * Hs || fabs(Q - R.cur_Q) > s.inv_gate * R.qs;
                acc = !gated;
            }
        }
        if (!acc) {
            R.att++;
            if (h <= hmin * 1.01 || R.att >= 24) { R.step++; R.status = 1; return true; }
            double fac = (!alive || gated) ? 0.5 : fmin(0.9, fmax(0.1, kSafety * pow(e, -0.125)));
            R.h_adapt = fmax(h * fac, hmin);
            return false;
        }
        R.att = 0;
        ok = true; h_used = h;
        R.y = out;
        if (s.inv_gate > 0.0) { R.cur_H = H; R.cur_Q = Q; }
        double sc2 = fmin(fmax(1.0, out.r / (0.5 * s.Rs)), 100.0);
        double grow = fmin(4.0, fmax(0.2, kSafety * pow(fmax(e, 1e-16), -0.125)));
        R.h_adapt = fmin(fmax(h * grow, hmin), s.ref_units ? s.hmax : s.hmax * sc2);
    } else if (s.integrator == NP_INTEG_ADAPTIVE) {
        // bounds: BH_RK_HMIN/HMAX (bh_common.h:245,253) for reference scenes;
        // hmax scaled like the fixed step law for scenes in units of M
        const double hmin = s.hmin, hmax = s.ref_units ? s.hmax : s.hmax * scale;
        double hb = fmin(fmax(s.h_unit * scale, hmin), hmax);
        double h = (R.h_adapt > 0.0) ? R.h_adapt : hb;
        h = fmin(fmax(h, hmin), hmax);
        for (int att = 0; att < 8; ++att) {
            double ht = h;
            double fac = adaptive_ref(R.y, M, a, rp, ht, s.rtol, s.atol, k1);
            evals += 12;
            if (fac > 0.0) {
                ok = true; h_used = ht;
                double sc2 = fmin(fmax(1.0, R.y.r / (0.5 * s.Rs)), 100.0);
                R.h_adapt = fmin(fmax(ht * fac, hmin), s.ref_units ? s.hmax : s.hmax * sc2);
                break;
            }
            h = fmax(ht, hmin);
            if (h <= hmin * 1.01) break;
        }
    } else {
        h_used = s.h_unit * scale;
        St8 out;
        rk4_ref(R.y, M, a, rp, h_used, out, k1);
        evals += 4;
        R.y = out;
        ok = R.y.r > rp + 1e-9 && R.y.th > 1e-9 && R.y.th < kPi - 1e-9;
    }
    R.step++;
    if (!ok) { R.status = 1; return true; }
    if (TRK) {
        double H, Hs, Q;
        h_and_q(R.y, M, a, H, Hs, Q);
        R.dH = fmax(R.dH, fabs(H) / fmax(Hs, 1e-300));
        R.dQ = fmax(R.dQ, fabs(Q - R.q0) / R.qs);
    }
    R.min_r = fmin(R.min_r, R.y.r);
    const double hp = kPi * 0.5;
    double dp = R.prev.th - hp, dc = R.y.th - hp;
    bool sc = (dp > 0 && dc < 0) || (dp < 0 && dc > 0);
    bool nz = (fabs(dp) < 1e-8 && fabs(dc) >= 1e-8) || (fabs(dc) < 1e-8 && fabs(dp) >= 1e-8);
    if (sc || nz) {
        double alpha = fabs(dp) / (fabs(dp) + fabs(dc) + 1e-30);
        double rc, phc;
        if (s.crossing == NP_CROSS_ROOT && sc) {
            if (DEFER) {
                // the root is found later, together with other lanes' (fp64_resolve)
                R.xpend = true; R.x_h = h_used; R.x_dp = dp; R.x_alpha = alpha;
                return false;
            }
            St8 z = fp64_root_crossing<MODE>(s, R.prev, h_used, dp, alpha, evals);
            rc = z.r;
            phc = z.ph;
        } else if (s.crossing == NP_CROSS_HERMITE && sc) {
            St8 f1;
            rhs_ref(R.y, M, a, rp, f1);
            evals += 1;
            double u = hermite_root(dp, dc, h_used * k1.th, h_used * f1.th, alpha);
            rc = hermite_eval(R.prev.r, R.y.r, h_used * k1.r, h_used * f1.r, u);
            phc = hermite_eval(R.prev.ph, R.y.ph, h_used * k1.ph, h_used * f1.ph, u);
        } else {
            rc = R.prev.r + alpha * (R.y.r - R.prev.r);
            phc = R.prev.ph + alpha * (R.y.ph - R.prev.ph);
        }
        fp64_record_crossing(s, R, rc, phc, alpha, inv3);
    }
    return fp64_step_tail(s, R);
}

// Root of a crossing deferred by fp64_advance<MODE, TRK, true>, then the
// rest of that step; returns true when the ray terminated.
template <int MODE, bool REC>
__device__ __forceinline__ bool fp64_resolve(const SceneDev& s, RayFP64<REC>& R, float* inv3,
                                             unsigned long long& evals) {
    St8 z = fp64_root_crossing<MODE>(s, R.prev, R.x_h, R.x_dp, R.x_alpha, evals);
    R.xpend = false;
    fp64_record_crossing(s, R, z.r, z.ph, R.x_alpha, inv3);
    return fp64_step_tail(s, R);
}

}  // namespace np
