/*
 * np_oracle.cpp -- CPU FP64 oracle of the Kerr render path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA kernels
 * in nullpath_gb300/csrc: only tests/, __graft_entry__.smoke() and the CPU
 * baseline legs of bench.py load it.  The product never links or calls it.
 *
 * It restates, in plain double-precision C++, the per-pixel body of the
 * reference renderer:
 *   camera ray + jitter ........ render.cu:137-159, 88-99
 *   camera tetrads ............. include/bh_kerr.h:781-826 (static), 910-967 (ZAMO), 880-884
 *   inverse metric + derivs .... include/bh_kerr.h:600-617, 624-672
 *   Hamilton's equations ....... include/bh_kerr.h:679-727
 *   fixed RK4 .................. include/bh_kerr.h:734-774
 *   adaptive step doubling ..... include/bh_kerr.h:987-1105, render.cu:187-205
 *   compensated sums ........... include/bh_common.h:451-493
 *   disk crossings + shading ... render.cu:210-251, 65-86
 *   colour selection ........... render.cu:312-363
 *   Doppler factor ............. include/bh_kerr.h:833-862
 * plus the benchmark-scene extensions (lengths in M, stratified seeded
 * jitter, r^-q emissivity, configurable disk edges / escape radius / step
 * cap, cubic-Hermite crossing location) that the CUDA path also implements,
 * and the research mode of the reference's accuracy plan (docs/PLAN.md:
 * 35-66): Fehlberg's embedded 7(8) pair (NASA TR R-287, 1968) as a plain
 * tableau loop, the invariant gate on each step's change of H and Carter's
 * Q, root-found crossings and the per-ray drift report.
 *
 * Compile with -ffp-contract=off so that no fused multiply-add changes the
 * rounding between x86 and Arm hosts.
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <algorithm>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/np_render.h"

namespace npo {

static const double kPi = 3.141592653589793238462643383279502884;
static const float kPiF = 3.14159265358979323846f;
static const double kEps = 1e-12;       // BH_EPS_D, bh_common.h:77
static const double kEpsSin = 1e-12;    // BH_EPS_SIN_D, bh_common.h:93
static const double kHMin = 1e-6;       // BH_RK_HMIN, bh_common.h:245
static const double kHMax = 0.2;        // BH_RK_HMAX, bh_common.h:253
static const double kSafety = 0.9;      // BH_RK_SAFETY, bh_common.h:236

struct State { double t, r, th, ph, pt, pr, pth, pph; };

// Second-order compensated (Kahan-Babuska / Klein 2006) accumulator, the
// summation the reference applies to the Hamiltonian terms
// (bh_common.h:451-483).
struct Klein {
    double s = 0.0, c1 = 0.0, c2 = 0.0;
    void add(double x) {
        double t = s + x;
        double e = (std::fabs(s) >= std::fabs(x)) ? (s - t) + x : (x - t) + s;
        s = t;
        double u = c1 + e;
        double ee = (std::fabs(c1) >= std::fabs(e)) ? (c1 - u) + e : (e - u) + c1;
        c1 = u;
        c2 += ee;
    }
    double value() const { return s + c1 + c2; }
};

// k1 + 2 k2 + 2 k3 + k4 through the compensated accumulator (bh_common.h:485-493).
static inline double rk4_combine(double k1, double k2, double k3, double k4) {
    Klein k; k.add(k1); k.add(2.0 * k2); k.add(2.0 * k3); k.add(k4);
    return k.value();
}

// Covariant Boyer-Lindquist blocks (bh_kerr.h:575-592).
static void metric_cov(double M, double a, double r, double th,
                       double& gtt, double& gtp, double& gpp, double& grr, double& ghh) {
    double c = std::cos(th), s = std::sin(th), s2 = s * s;
    double r2 = r * r, a2 = a * a;
    double Sig = r2 + a2 * c * c;
    double Del = r2 - 2.0 * M * r + a2;
    double A = (r2 + a2) * (r2 + a2) - a2 * Del * s2;
    gtt = -(1.0 - 2.0 * M * r / std::fmax(kEps, Sig));
    gtp = -2.0 * M * a * r * s2 / std::fmax(kEps, Sig);
    gpp = A * s2 / std::fmax(kEps, Sig);
    grr = Sig / std::fmax(kEps, Del);
    ghh = Sig;
}

// Contravariant blocks with the reference's floors (bh_kerr.h:600-617).
static void metric_inv(double M, double a, double r, double th, double g[5]) {
    double c = std::cos(th), s = std::sin(th);
    double s2 = std::fmax(kEpsSin, s * s);
    double r2 = r * r, a2 = a * a;
    double Sig = std::fmax(kEps, r2 + a2 * c * c);
    double Del = r2 - 2.0 * M * r + a2;
    double A = (r2 + a2) * (r2 + a2) - a2 * Del * s2;
    g[3] = std::fmax(kEps, Del) / Sig;                       // g^rr
    g[4] = 1.0 / Sig;                                          // g^thth
    g[0] = -A / std::fmax(kEps, Sig * Del);                    // g^tt
    g[1] = -2.0 * M * a * r / std::fmax(kEps, Sig * Del);      // g^tphi
    g[2] = (Del - a2 * s2) / std::fmax(kEps, Sig * Del * s2);  // g^phiphi
}

// Analytic d/dr and d/dtheta of the contravariant blocks (bh_kerr.h:624-672).
// dr[k], dth[k] follow the order tt, tphi, phiphi, rr, thth.
static void metric_inv_derivs(double M, double a, double r, double th, double dr[5], double dth[5]) {
    double s = std::sin(th), c = std::cos(th);
    double s2 = (s * s > 1e-30) ? s * s : 1e-30;
    double r2 = r * r, a2 = a * a;
    double B = r2 + a2;
    double Sig = r2 + a2 * c * c;
    double Del = r2 - 2.0 * M * r + a2;
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
    dr[0] = -(A_r * D - A * D_r) / D2;
    dth[0] = -(A_t * D - A * D_t) / D2;
    double N = 2.0 * M * a * r, N_r = 2.0 * M * a;
    dr[1] = -(N_r * D - N * D_r) / D2;
    dth[1] = -(0.0 * D - N * D_t) / D2;
    dr[3] = (Del_r * Sig - Del * Sig_r) / (Sig * Sig);
    dth[3] = -(Del * Sig_t) / (Sig * Sig);
    dr[4] = -Sig_r / (Sig * Sig);
    dth[4] = -Sig_t / (Sig * Sig);
    double P = Del - a2 * s2, P_r = Del_r, P_t = -a2 * ds2;
    double Q = Del * Sig * s2 + 1e-48;
    double Q_r = Del_r * Sig * s2 + Del * Sig_r * s2;
    double Q_t = Del * Sig_t * s2 + Del * Sig * ds2;
    double Q2 = Q * Q + 1e-48;
    dr[2] = (P_r * Q - P * Q_r) / Q2;
    dth[2] = (P_t * Q - P * Q_t) / Q2;
}

static inline double r_plus(double M, double a) {
    double d = M * M - a * a;
    if (d < 0.0) d = 0.0;
    return M + std::sqrt(d);
}

// Hamilton's equations x' = g^{mu nu} p_nu, p' = -1/2 dg p p (bh_kerr.h:679-727).
static void rhs(const State& y, double M, double a, State& f) {
    if (y.r <= r_plus(M, a) + 1e-12 || y.r <= 1e-12) { f = State{}; return; }
    double g[5], gr[5], gt[5];
    metric_inv(M, a, y.r, y.th, g);
    metric_inv_derivs(M, a, y.r, y.th, gr, gt);
    f.t = g[0] * y.pt + g[1] * y.pph;
    f.r = g[3] * y.pr;
    f.th = g[4] * y.pth;
    f.ph = g[1] * y.pt + g[2] * y.pph;
    f.pt = 0.0;
    f.pph = 0.0;
    Klein sr, st;
    sr.add(gr[0] * y.pt * y.pt); sr.add(2.0 * gr[1] * y.pt * y.pph); sr.add(gr[2] * y.pph * y.pph);
    sr.add(gr[3] * y.pr * y.pr); sr.add(gr[4] * y.pth * y.pth);
    st.add(gt[0] * y.pt * y.pt); st.add(2.0 * gt[1] * y.pt * y.pph); st.add(gt[2] * y.pph * y.pph);
    st.add(gt[3] * y.pr * y.pr); st.add(gt[4] * y.pth * y.pth);
    f.pr = -0.5 * sr.value();
    f.pth = -0.5 * st.value();
}

static inline State axpy(const State& y, double h, const State& k) {
    return State{y.t + h * k.t, y.r + h * k.r, y.th + h * k.th, y.ph + h * k.ph,
                 y.pt + h * k.pt, y.pr + h * k.pr, y.pth + h * k.pth, y.pph + h * k.pph};
}

// One classical RK4 step with the compensated stage combination
// (bh_kerr.h:734-774 and 987-1032); k1 is returned for the crossing
// interpolant.
static void rk4(const State& y, double M, double a, double h, State& out, State* k1_out) {
    State k1, k2, k3, k4;
    rhs(y, M, a, k1);
    rhs(axpy(y, 0.5 * h, k1), M, a, k2);
    rhs(axpy(y, 0.5 * h, k2), M, a, k3);
    rhs(axpy(y, h, k3), M, a, k4);
    double h6 = h / 6.0;
    out = y;
    out.t += h6 * rk4_combine(k1.t, k2.t, k3.t, k4.t);
    out.r += h6 * rk4_combine(k1.r, k2.r, k3.r, k4.r);
    out.th += h6 * rk4_combine(k1.th, k2.th, k3.th, k4.th);
    out.ph += h6 * rk4_combine(k1.ph, k2.ph, k3.ph, k4.ph);
    out.pt += h6 * rk4_combine(k1.pt, k2.pt, k3.pt, k4.pt);
    out.pr += h6 * rk4_combine(k1.pr, k2.pr, k3.pr, k4.pr);
    out.pth += h6 * rk4_combine(k1.pth, k2.pth, k3.pth, k4.pth);
    out.pph += h6 * rk4_combine(k1.pph, k2.pph, k3.pph, k4.pph);
    if (k1_out) *k1_out = k1;
}

// Continue-flag of the fixed-step integrator (bh_kerr.h:770-773).
static inline bool alive_fixed(const State& y, double M, double a) {
    return y.r > r_plus(M, a) + 1e-9 && y.th > 1e-9 && y.th < kPi - 1e-9;
}
// Continue-flag of the adaptive sub-steps (bh_kerr.h:1028-1031).
static inline bool alive_adaptive(const State& y, double M, double a) {
    return y.r > r_plus(M, a) + 1e-12 && y.th > 1e-9 && y.th < kPi - 1e-9;
}

// Step doubling with the reference's error norm and step factors
// (bh_kerr.h:1058-1105).  Returns the growth factor (> 0) on acceptance.
static double adaptive_step(State& y, double M, double a, double& h, double rtol, double atol,
                            State* k1_out) {
    State full, half1, half2, k1;
    rk4(y, M, a, h, full, &k1);
    double h2 = 0.5 * h;
    rk4(y, M, a, h2, half1, nullptr);
    rk4(half1, M, a, h2, half2, nullptr);
    bool ok = alive_adaptive(full, M, a) && alive_adaptive(half1, M, a) && alive_adaptive(half2, M, a);
    if (!ok) { h *= 0.5; return 0.0; }
    auto nerr = [&](double u, double v) {
        double sc = atol + rtol * std::fmax(std::fabs(u), std::fabs(v));
        return std::fabs(u - v) / std::fmax(sc, 1e-30);
    };
    double e = std::fmax(std::fmax(nerr(full.r, half2.r), nerr(full.th, half2.th)),
                         std::fmax(std::fmax(nerr(full.ph, half2.ph), nerr(full.pr, half2.pr)),
                                   std::fmax(nerr(full.pth, half2.pth), nerr(full.pph, half2.pph))));
    if (e <= 1.0) {
        y = half2;
        if (k1_out) *k1_out = k1;
        return std::fmin(2.0, kSafety * std::pow(std::fmax(1e-12, e), -0.2));
    }
    h *= std::fmax(0.1, kSafety * std::pow(std::fmax(1e-12, e), -0.25));
    return 0.0;
}

// Fehlberg 7(8) tableau (E. Fehlberg, NASA TR R-287, 1968, table X):
// 13 stages, rows of the coupling matrix, 8th-order weights, and the
// error weights (7th minus 8th order: 41/840 on k1, k11 and -41/840 on k12, k13).
static const double kF78A[13][12] = {
    {},
    {2.0 / 27},
    {1.0 / 36, 1.0 / 12},
    {1.0 / 24, 0, 1.0 / 8},
    {5.0 / 12, 0, -25.0 / 16, 25.0 / 16},
    {1.0 / 20, 0, 0, 1.0 / 4, 1.0 / 5},
    {-25.0 / 108, 0, 0, 125.0 / 108, -65.0 / 27, 125.0 / 54},
    {31.0 / 300, 0, 0, 0, 61.0 / 225, -2.0 / 9, 13.0 / 900},
    {2.0, 0, 0, -53.0 / 6, 704.0 / 45, -107.0 / 9, 67.0 / 90, 3.0},
    {-91.0 / 108, 0, 0, 23.0 / 108, -976.0 / 135, 311.0 / 54, -19.0 / 60, 17.0 / 6, -1.0 / 12},
    {2383.0 / 4100, 0, 0, -341.0 / 164, 4496.0 / 1025, -301.0 / 82, 2133.0 / 4100, 45.0 / 82, 45.0 / 164, 18.0 / 41},
    {3.0 / 205, 0, 0, 0, 0, -6.0 / 41, -3.0 / 205, -3.0 / 41, 3.0 / 41, 6.0 / 41, 0},
    {-1777.0 / 4100, 0, 0, -341.0 / 164, 4496.0 / 1025, -289.0 / 82, 2193.0 / 4100, 51.0 / 82, 33.0 / 164,
     12.0 / 41, 0, 1.0},
};
static const double kF78B[13] = {0, 0, 0, 0, 0, 34.0 / 105, 9.0 / 35, 9.0 / 35, 9.0 / 280, 9.0 / 280, 0,
                                 41.0 / 840, 41.0 / 840};
static const double kF78E[13] = {41.0 / 840, 0, 0, 0, 0, 0, 0, 0, 0, 0, 41.0 / 840, -41.0 / 840, -41.0 / 840};

static inline double& comp(State& y, int i) {
    double* p[8] = {&y.t, &y.r, &y.th, &y.ph, &y.pt, &y.pr, &y.pth, &y.pph};
    return *p[i];
}
static inline double compc(const State& y, int i) {
    const double p[8] = {y.t, y.r, y.th, y.ph, y.pt, y.pr, y.pth, y.pph};
    return p[i];
}

// One 7(8) step: out = 8th-order solution; returns the error norm over
// (r, theta, phi, p_r, p_theta, p_phi) with the step-doubling weights.
static double rkf78(const State& y, double M, double a, double h, double rtol, double atol, State& out) {
    State k[13];
    for (int j = 0; j < 13; ++j) {
        State z = y;
        for (int c = 0; c < 8; ++c) {
            double acc = 0.0;
            for (int i = 0; i < j; ++i) acc += kF78A[j][i] * compc(k[i], c);
            comp(z, c) = comp(z, c) + h * acc;
        }
        rhs(z, M, a, k[j]);
    }
    out = y;
    double e = 0.0;
    for (int c = 0; c < 8; ++c) {
        double acc = 0.0, err = 0.0;
        for (int i = 0; i < 13; ++i) { acc += kF78B[i] * compc(k[i], c); err += kF78E[i] * compc(k[i], c); }
        comp(out, c) = compc(y, c) + h * acc;
        if (c == 1 || c == 2 || c == 3 || c == 5 || c == 6 || c == 7) {
            double sc = atol + rtol * std::fmax(std::fabs(compc(y, c)), std::fabs(compc(out, c)));
            e = std::fmax(e, std::fabs(h * err) / std::fmax(sc, 1e-30));
        }
    }
    return e;
}

// Hamiltonian, the sum of its absolute terms, and Carter's constant of a state.
static void h_and_q(const State& y, double M, double a, double& H, double& Hs, double& Q) {
    double g[5];
    metric_inv(M, a, y.r, y.th, g);
    const double t[5] = {g[0] * y.pt * y.pt, 2.0 * g[1] * y.pt * y.pph, g[2] * y.pph * y.pph, g[3] * y.pr * y.pr,
                         g[4] * y.pth * y.pth};
    H = 0.5 * (t[0] + t[1] + t[2] + t[3] + t[4]);
    Hs = 0.5 * (std::fabs(t[0]) + std::fabs(t[1]) + std::fabs(t[2]) + std::fabs(t[3]) + std::fabs(t[4]));
    double c = std::cos(y.th), sn = std::sin(y.th);
    double s2 = std::fmax(kEps, sn * sn);
    Q = y.pth * y.pth + c * c * (y.pph * y.pph / s2 - a * a * y.pt * y.pt);
}

// Static-observer tetrad -> covariant momentum (bh_kerr.h:781-826).
static State camera_static(double M, double a, double r, double th, double ph,
                           double nr, double nth, double nph) {
    State s{}; s.r = r; s.th = th; s.ph = ph;
    double gtt, gtp, gpp, grr, ghh;
    metric_cov(M, a, r, th, gtt, gtp, gpp, grr, ghh);
    double ut = 1.0 / std::sqrt(std::fmax(kEps, -gtt));
    double er = 1.0 / std::sqrt(std::fmax(kEps, grr));
    double eh = 1.0 / std::sqrt(std::fmax(kEps, ghh));
    double ept, epp;
    if (std::fabs(gtp) > kEps) {
        double beta = -gtt / gtp;
        Klein n2; n2.add(gtt); n2.add(2.0 * gtp * beta); n2.add(gpp * beta * beta);
        double inv = 1.0 / std::sqrt(std::fmax(kEps, std::fabs(n2.value())));
        ept = inv; epp = beta * inv;
    } else {
        ept = 0.0; epp = 1.0 / std::sqrt(std::fmax(kEps, gpp));
    }
    double Pt = ut + nph * ept, Pr = nr * er, Ph = nth * eh, Pp = nph * epp;
    s.pt = gtt * Pt + gtp * Pp;
    s.pr = grr * Pr;
    s.pth = ghh * Ph;
    s.pph = gtp * Pt + gpp * Pp;
    return s;
}

// ZAMO tetrad -> covariant momentum (bh_kerr.h:910-967).
static State camera_zamo(double M, double a, double r, double th, double ph,
                         double nr, double nth, double nph) {
    State s{}; s.r = r; s.th = th; s.ph = ph;
    double c = std::cos(th), sn = std::sin(th);
    double r2 = r * r, a2 = a * a;
    double Sig = std::fmax(kEps, r2 + a2 * c * c);
    double Del = r2 - 2.0 * M * r + a2;
    double A = std::fmax(kEps, (r2 + a2) * (r2 + a2) - a2 * Del * sn * sn);
    double alpha = std::sqrt(std::fmax(kEps, Del * Sig / A));
    double omega = 2.0 * M * a * r / A;
    double et_t = 1.0 / std::fmax(kEps, alpha);
    double et_p = omega / std::fmax(kEps, alpha);
    double er_r = std::sqrt(std::fmax(kEps, Del / Sig));
    double eh_h = 1.0 / std::sqrt(Sig);
    double ep_p = std::sqrt(std::fmax(kEps, Sig / A)) / std::fmax(kEps, std::fabs(sn));
    double Pt = et_t, Pr = nr * er_r, Ph = nth * eh_h, Pp = et_p + nph * ep_p;
    double gtt, gtp, gpp, grr, ghh;
    metric_cov(M, a, r, th, gtt, gtp, gpp, grr, ghh);
    s.pt = gtt * Pt + gtp * Pp;
    s.pr = grr * Pr;
    s.pth = ghh * Ph;
    s.pph = gtp * Pt + gpp * Pp;
    return s;
}

static inline bool static_timelike(double M, double a, double r, double th) {
    double gtt, gtp, gpp, grr, ghh;
    metric_cov(M, a, r, th, gtt, gtp, gpp, grr, ghh);
    return gtt < 0.0;
}

// Redshift of a prograde Keplerian emitter at the crossing (bh_kerr.h:833-862).
static double doppler_g(double r, double pt, double pph, double M, double a) {
    double gtt, gtp, gpp, grr, ghh;
    metric_cov(M, a, r, kPi * 0.5, gtt, gtp, gpp, grr, ghh);
    double Ms = std::fmax(kEps, M);
    double Om = 1.0 / (a / Ms + std::pow(std::fmax(1.0, r / Ms), 1.5)) / Ms;
    Klein d; d.add(gtt); d.add(2.0 * gtp * Om); d.add(gpp * Om * Om);
    double den = -d.value();
    double ut = 1.0 / std::sqrt(den > 1e-24 ? den : 1e-24);
    double up = Om * ut;
    Klein k; k.add(pt * ut); k.add(pph * up);
    double ku = -k.value();
    double g = -pt / (ku > 1e-18 ? ku : 1e-18);
    return g > 0.0 ? g : 0.0;
}

// Integer hash of render.cu:88-99 (reference jitter).
static inline uint32_t wang_hash(uint32_t v) {
    v = (v ^ 61u) ^ (v >> 16);
    v *= 9u;
    v = v ^ (v >> 4);
    v *= 0x27d4eb2du;
    v = v ^ (v >> 15);
    return v;
}
static inline float wang_unit(uint32_t v) { return (float)(wang_hash(v) & 0x00ffffffu) * (1.0f / 16777216.0f); }

// 32-bit finaliser "lowbias32" (C. Wellons, public domain hash prospector);
// the stratified sampler's counter-based generator.
static inline uint32_t mix32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du;
    x ^= x >> 15; x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
static inline double strat_unit(uint32_t seed, uint32_t pix, uint32_t sample, uint32_t dim) {
    uint32_t h = mix32(mix32(mix32(seed + 0x9e3779b9u * (dim + 1u)) ^ pix) ^ (sample * 0x85ebca6bu));
    return (double)(h >> 8) * (1.0 / 16777216.0);
}

// Scene quantities shared by all pixels.
struct Frame {
    bool ref_units;               // lengths in Rs, float-rounded camera (render.cu)
    double M, a, Rs, r_cam, th_cam, ph_cam;
    float Mf, Rsf;
    float aspect_f, tan_half_f;   // reference camera in float (render.cu:137-139)
    double aspect, tan_half;
    double rin, rout, r_far, q;
    float gain;
    double h_unit;                // step = h_unit * clamp(r/M, 1, 100)
    bool zamo;
    int max_steps, max_orders, integrator, crossing, bg_mode, disk_on, jitter, strata;
    float bg_sigma_rad, bg_peak;
    uint32_t seed;
    double rtol, atol, inv_gate;
    float crit_rho[256];          // NP_JITTER_CRITICAL: critical-curve radius per position angle
    double crit_band;
};

// R(r_c) / (E^2 r_c^4) at the largest root r_c of R'(r) = 0 for
// R(r) = P^2 - Delta K: > 0 for rays without a radial turning point outside
// the horizon (captured), < 0 for turning rays; 1e300 when R has no minimum
// outside r_+ (captured).
static double critical_gap(double E, double L, double Q, double a, double M, double rp) {
    double K = Q + (L - a * E) * (L - a * E);
    double c3 = 4.0 * E * E;
    double c1 = 4.0 * a * a * E * E - 4.0 * a * E * L - 2.0 * K;
    double c0 = 2.0 * M * K;
    double r = std::sqrt(std::fmax(0.0, -c1 / c3)) + 4.0 * M;
    for (int it = 0; it < 30; ++it) {
        double fv = (c3 * r * r + c1) * r + c0;
        double fp = 3.0 * c3 * r * r + c1;
        if (fp <= 0.0) break;
        double dr = fv / fp;
        r -= dr;
        if (std::fabs(dr) < 1e-12 * r) break;
    }
    if (!(r > rp)) return 1e300;
    double r2 = r * r, a2 = a * a;
    double P = (r2 + a2) * E - a * L;
    double Del = r2 - 2.0 * M * r + a2;
    return (P * P - Del * K) / (E * E * r2 * r2);
}

static Frame make_frame(const np_scene_t& s) {
    Frame f{};
    f.ref_units = (s.units == NP_UNITS_RS);
    if (f.ref_units) {
        float Mf = (float)s.mass;
        float Rsf = 2.0f * Mf;
        float af = (float)s.spin * Mf;
        float rcf = (float)s.r_cam * Rsf;
        float thf = (float)s.theta_deg * kPiF / 180.0f;
        float phf = (float)s.phi_deg * kPiF / 180.0f;
        f.Mf = Mf; f.Rsf = Rsf;
        f.M = Mf; f.a = af; f.Rs = Rsf; f.r_cam = rcf; f.th_cam = thf; f.ph_cam = phf;
        f.aspect_f = (float)s.width / (float)s.height;
        float fov = (float)s.fov_y_deg * kPiF / 180.0f;
        f.tan_half_f = std::tan(0.5f * fov);
        f.h_unit = (double)(float)s.step_scale;   // INTEGRATION_STEP_SIZE is a float (bh_common.h:213)
    } else {
        f.M = s.mass; f.a = s.spin * s.mass; f.Rs = 2.0 * s.mass;
        f.Mf = (float)f.M; f.Rsf = (float)f.Rs;
        f.r_cam = s.r_cam * s.mass;
        f.th_cam = s.theta_deg * kPi / 180.0;
        f.ph_cam = s.phi_deg * kPi / 180.0;
        f.aspect = (double)s.width / (double)s.height;
        f.tan_half = std::tan(0.5 * s.fov_y_deg * kPi / 180.0);
        f.h_unit = s.step_scale;
    }
    f.rin = s.disk_rin > 0.0 ? s.disk_rin : 3.0 * f.Rs;
    f.rout = s.disk_rout > 0.0 ? s.disk_rout : 20.0 * f.Rs;
    f.r_far = s.escape_r > 0.0 ? s.escape_r : f.r_cam + 10.0 * f.Rs;
    f.q = s.emissivity_q;
    f.gain = (float)s.disk_gain;
    f.zamo = (s.camera == NP_CAMERA_ZAMO) || !static_timelike(f.M, f.a, f.r_cam, f.th_cam);
    f.max_steps = s.max_steps;
    f.max_orders = std::max(1, s.disk_max_orders);
    f.integrator = s.integrator;
    f.inv_gate = s.inv_gate > 0.0 ? s.inv_gate : 0.0;
    f.crossing = s.crossing;
    f.bg_mode = s.background;
    f.disk_on = s.disk_on;
    f.jitter = s.jitter;
    f.seed = s.seed;
    int m = (int)std::floor(std::sqrt((double)std::max(1, s.spp)));
    f.strata = std::max(1, m);
    f.bg_sigma_rad = (float)s.bg_sigma_deg * kPiF / 180.0f;
    f.bg_peak = (float)s.bg_brightness;
    f.rtol = s.rtol; f.atol = s.atol;
    f.crit_band = 0.02;
    if (s.jitter == NP_JITTER_CRITICAL) {
        // bisection on the tangent-plane radius along each position angle
        const double rho_max = f.ref_units ? (double)f.tan_half_f * std::sqrt((double)f.aspect_f * f.aspect_f + 1.0)
                                           : f.tan_half * std::sqrt(f.aspect * f.aspect + 1.0);
        const double rp = f.M + std::sqrt(std::fmax(0.0, f.M * f.M - f.a * f.a));
        const double c = std::cos(f.th_cam), sn = std::sin(f.th_cam);
        auto captured = [&](double rho, double psi) {
            double cx = rho * std::cos(psi), cy = rho * std::sin(psi), cz = -1.0;
            double nrm = 1.0 / std::sqrt(cx * cx + cy * cy + cz * cz);
            State y = f.zamo ? camera_zamo(f.M, f.a, f.r_cam, f.th_cam, f.ph_cam, cz * nrm, cy * nrm, cx * nrm)
                             : camera_static(f.M, f.a, f.r_cam, f.th_cam, f.ph_cam, cz * nrm, cy * nrm, cx * nrm);
            double E = -y.pt, L = y.pph;
            double Q = y.pth * y.pth + c * c * (L * L / (sn * sn) - f.a * f.a * E * E);
            return critical_gap(E, L, Q, f.a, f.M, rp) > 0.0;
        };
        for (int i = 0; i < 256; ++i) {
            double psi = -kPi + 2.0 * kPi * (double)i / 256.0;
            double lo = 0.0, hi = rho_max, out;
            if (!captured(lo, psi)) out = 0.0;
            else if (captured(hi, psi)) out = rho_max;
            else {
                for (int it = 0; it < 60; ++it) {
                    double mid = 0.5 * (lo + hi);
                    if (captured(mid, psi)) lo = mid; else hi = mid;
                }
                out = 0.5 * (lo + hi);
            }
            f.crit_rho[i] = (float)out;
        }
    }
    return f;
}

// Odd samples of NP_JITTER_CRITICAL move along their position angle to
// rho_c(psi) (1 + band (2u - 1)) in the tangent plane.
static void critical_remap(const Frame& f, uint32_t pix, uint32_t sample, double& cx, double& cy) {
    double psi = std::atan2(cy, cx);
    double t = (psi + kPi) * (256.0 / (2.0 * kPi));
    int i0 = (int)std::floor(t);
    double fr = t - (double)i0;
    i0 = ((i0 % 256) + 256) % 256;
    int i1 = (i0 + 1) % 256;
    double rc = (1.0 - fr) * (double)f.crit_rho[i0] + fr * (double)f.crit_rho[i1];
    double u = strat_unit(f.seed, pix, sample, 2);
    double rho = rc * (1.0 + f.crit_band * (2.0 * u - 1.0));
    cx = rho * std::cos(psi);
    cy = rho * std::sin(psi);
}

// Camera direction for sample `sample` of pixel (x, y) (render.cu:143-159),
// or of the continuous image position (fx, fy) when `explicit_pos`.
struct Dir { double nr, nth, nph; float cam_x, cam_y; };

static Dir camera_dir(const Frame& f, const np_scene_t& s, int x, int y, uint32_t sample,
                      bool explicit_pos, double fx, double fy) {
    Dir d{};
    if (f.ref_units) {
        float px, py;
        if (explicit_pos) { px = (float)fx; py = (float)fy; }
        else if (f.jitter == NP_JITTER_WANGHASH) {
            float jx = wang_unit((uint32_t)(x * 73856093u ^ y * 19349663u ^ sample * 83492791u)) - 0.5f;
            float jy = wang_unit((uint32_t)(x * 83492791u ^ y * 2654435761u ^ sample * 19349663u)) - 0.5f;
            px = x + 0.5f + jx; py = y + 0.5f + jy;
        } else {
            uint32_t pix = (uint32_t)(y * s.width + x);
            int m = f.strata;
            uint32_t c = sample % (uint32_t)(m * m);
            px = (float)(x + ((double)(c % m) + strat_unit(f.seed, pix, sample, 0)) / m);
            py = (float)(y + ((double)(c / m) + strat_unit(f.seed, pix, sample, 1)) / m);
        }
        float ndc_x = (px / (float)s.width) * 2.0f - 1.0f;
        float ndc_y = (py / (float)s.height) * 2.0f - 1.0f;
        float cx = ndc_x * f.aspect_f * f.tan_half_f;
        float cy = -ndc_y * f.tan_half_f;
        if (!explicit_pos && f.jitter == NP_JITTER_CRITICAL && (sample & 1u)) {
            double dx = cx, dy = cy;
            critical_remap(f, (uint32_t)(y * s.width + x), sample, dx, dy);
            cx = (float)dx; cy = (float)dy;
        }
        float cz = -1.0f;
        float nrm = 1.0f / std::sqrt(cx * cx + cy * cy + cz * cz);
        cx *= nrm; cy *= nrm; cz *= nrm;
        d.nr = cz; d.nth = cy; d.nph = cx; d.cam_x = cx; d.cam_y = cy;
    } else {
        double px, py;
        if (explicit_pos) { px = fx; py = fy; }
        else if (f.jitter == NP_JITTER_WANGHASH) {
            float jx = wang_unit((uint32_t)(x * 73856093u ^ y * 19349663u ^ sample * 83492791u)) - 0.5f;
            float jy = wang_unit((uint32_t)(x * 83492791u ^ y * 2654435761u ^ sample * 19349663u)) - 0.5f;
            px = x + 0.5 + jx; py = y + 0.5 + jy;
        } else {
            uint32_t pix = (uint32_t)(y * s.width + x);
            int m = f.strata;
            uint32_t c = sample % (uint32_t)(m * m);
            px = x + ((double)(c % m) + strat_unit(f.seed, pix, sample, 0)) / m;
            py = y + ((double)(c / m) + strat_unit(f.seed, pix, sample, 1)) / m;
        }
        double ndc_x = (px / s.width) * 2.0 - 1.0;
        double ndc_y = (py / s.height) * 2.0 - 1.0;
        double cx = ndc_x * f.aspect * f.tan_half;
        double cy = -ndc_y * f.tan_half;
        if (!explicit_pos && f.jitter == NP_JITTER_CRITICAL && (sample & 1u))
            critical_remap(f, (uint32_t)(y * s.width + x), sample, cx, cy);
        double cz = -1.0;
        double nrm = 1.0 / std::sqrt(cx * cx + cy * cy + cz * cz);
        cx *= nrm; cy *= nrm; cz *= nrm;
        d.nr = cz; d.nth = cy; d.nph = cx; d.cam_x = (float)cx; d.cam_y = (float)cy;
    }
    return d;
}

// Disk emission I = j(r) g^3 (1, .75, .45) (render.cu:65-72, j = r^-q).
static inline void shade_disk(float r, float g, float q, float out[3]) {
    float j = std::pow(std::fmax(r, 1.0f), -q);
    float I = j * g * g * g;
    out[0] = 1.0f * I; out[1] = 0.75f * I; out[2] = 0.45f * I;
}

static inline float clamp01(float v) { return std::fmin(std::fmax(v, 0.0f), 1.0f); }

// Sky gradient with a bright band (render.cu:74-86).
static inline void shade_sky(float u, float v, float out[3]) {
    (void)u;
    float t = clamp01(v);
    float c0 = 0.02f * (1 - t) + 0.08f * t;
    float c1 = 0.03f * (1 - t) + 0.09f * t;
    float c2 = 0.05f * (1 - t) + 0.12f * t;
    float band = std::exp(-50.0f * (v - 0.5f) * (v - 0.5f));
    c0 += 0.4f * band; c1 += 0.35f * band; c2 += 0.3f * band;
    out[0] = clamp01(c0); out[1] = clamp01(c1); out[2] = clamp01(c2);
}

struct RayOut {
    bool captured = false;
    int status = 0;               // 0 escaped, 1 captured, 2 step cap
    int orders = 0;               // disk hits
    int crossings = 0;            // equatorial crossings (any radius)
    float disk[3] = {0, 0, 0};
    double min_r = 0.0;
    double xr[4] = {0, 0, 0, 0}, xphi[4] = {0, 0, 0, 0};
    double first_hit_r = 0.0;
    long steps = 0;
    State last{};
    double pt0 = 0.0, pph0 = 0.0;
    double dH = 0.0, dQ = 0.0;    // max |H| / Hs, max |Q - Q0| / max(|Q0|, (E M)^2)
    float inv[3] = {0, 0, 0};
};

static inline void inv_update(float inv[3], float H, float E, float L) {
    inv[0] = std::fmax(inv[0], H); inv[1] = std::fmax(inv[1], E); inv[2] = std::fmax(inv[2], L);
}

static void invariants_at(const Frame& f, const State& y, double pt0, double pph0, float inv[3]) {
    double g[5];
    metric_inv(f.M, f.a, y.r, y.th, g);
    double H = 0.5 * (g[0] * y.pt * y.pt + 2.0 * g[1] * y.pt * y.pph + g[2] * y.pph * y.pph
                      + g[3] * y.pr * y.pr + g[4] * y.pth * y.pth);
    inv_update(inv, (float)std::fabs(H),
               (float)(std::fabs(y.pt - pt0) / std::fmax(1e-12, std::fabs(pt0))),
               (float)(std::fabs(y.pph - pph0) / std::fmax(1e-12, std::fabs(pph0))));
}

// Solves theta(s) = pi/2 on the cubic Hermite interpolant of one step
// (values y0, y1 and slopes h*f0, h*f1) by safeguarded Newton iteration.
static double hermite_root(double d0, double d1, double m0, double m1, double s_lin) {
    // p(s) = h00(s) d0 + h10(s) m0 + h01(s) d1 + h11(s) m1, d = theta - pi/2;
    // d0 and d1 have opposite signs, so [0, 1] brackets a root.
    double s = s_lin, lo = 0.0, hi = 1.0;
    for (int it = 0; it < 8; ++it) {
        double s2 = s * s, s3 = s2 * s;
        double p = (2 * s3 - 3 * s2 + 1) * d0 + (s3 - 2 * s2 + s) * m0 + (-2 * s3 + 3 * s2) * d1 + (s3 - s2) * m1;
        double dp = (6 * s2 - 6 * s) * d0 + (3 * s2 - 4 * s + 1) * m0 + (-6 * s2 + 6 * s) * d1 + (3 * s2 - 2 * s) * m1;
        if ((p > 0) == (d0 > 0)) lo = s; else hi = s;
        double sn = (dp != 0.0) ? s - p / dp : 0.5 * (lo + hi);
        if (!(sn > lo && sn < hi)) sn = 0.5 * (lo + hi);
        bool done = std::fabs(sn - s) < 1e-15;
        s = sn;
        if (done) break;
    }
    return s;
}
static inline double hermite_eval(double y0, double y1, double m0, double m1, double s) {
    double s2 = s * s, s3 = s2 * s;
    return (2 * s3 - 3 * s2 + 1) * y0 + (s3 - 2 * s2 + s) * m0 + (-2 * s3 + 3 * s2) * y1 + (s3 - s2) * m1;
}

// Single step of the integrator family (RK4 for RK4 and step doubling).
static void single_step(const Frame& f, const State& y, double h, State& out) {
    if (f.integrator == NP_INTEG_RKF78) rkf78(y, f.M, f.a, h, f.rtol, f.atol, out);
    else rk4(y, f.M, f.a, h, out, nullptr);
}

// theta = pi/2 inside the step prev -> prev + h: Newton on the step
// fraction u with fresh single steps of u h from prev, kept inside the sign
// bracket [0, 1] (bisection when Newton leaves it).
static State root_crossing(const Frame& f, const State& prev, double h, double dp, double u0) {
    const double hp = kPi * 0.5;
    double lo = 0.0, hi = 1.0, u = u0;
    State z = prev, fz;
    for (int it = 0; it < 10; ++it) {
        single_step(f, prev, u * h, z);
        double g = z.th - hp;
        if (g == 0.0) break;
        if ((g > 0.0) == (dp > 0.0)) lo = u; else hi = u;
        rhs(z, f.M, f.a, fz);
        double dg = h * fz.th;
        double un = (dg != 0.0) ? u - g / dg : 0.5 * (lo + hi);
        if (!(un > lo && un < hi)) un = 0.5 * (lo + hi);
        bool done = std::fabs(un - u) < 1e-15;
        u = un;
        if (done) break;
    }
    return z;
}

// Traces one ray in FP64 following render.cu:161-251.
static void trace(const Frame& f, const Dir& d, bool track_inv, RayOut& o, bool track_drift = false) {
    State y = f.zamo ? camera_zamo(f.M, f.a, f.r_cam, f.th_cam, f.ph_cam, d.nr, d.nth, d.nph)
                     : camera_static(f.M, f.a, f.r_cam, f.th_cam, f.ph_cam, d.nr, d.nth, d.nph);
    o.pt0 = y.pt; o.pph0 = y.pph;
    double H0, Hs0, Q0;
    h_and_q(y, f.M, f.a, H0, Hs0, Q0);
    const double E2 = y.pt * y.pt, qs = std::fmax(std::fabs(Q0), E2 * f.M * f.M);
    double cur_H = H0, cur_Q = Q0;   // the invariant gate's reference: H and Q at the current state
    o.dH = std::fabs(H0) / std::fmax(Hs0, 1e-300);
    o.min_r = y.r;
    State prev = y;
    double h_adapt = 0.0;
    const double half_pi = kPi * 0.5;
    int step = 0;
    o.status = 2;
    for (step = 0; step < f.max_steps; ++step) {
        double scale = std::fmin(std::fmax(1.0, y.r / (0.5 * f.Rs)), 100.0);
        bool ok = false;
        double h_used = 0.0;
        State k1{};
        if (f.integrator == NP_INTEG_RKF78) {
            // step bounds of step doubling; factors 0.9 e^(-1/8) in [0.2, 4]
            // on acceptance, [0.1, 0.9] on rejection, halving on a gate or
            // horizon rejection; the gate bounds the step's change of H and
            // Q and is not applied at the smallest step
            const double hmin = f.ref_units ? kHMin : kHMin * f.M;
            const double hmax = f.ref_units ? kHMax : 10.0 * f.h_unit * scale;
            double h = (h_adapt > 0.0) ? h_adapt : f.h_unit * scale;
            h = std::fmin(std::fmax(h, hmin), hmax);
            for (int att = 0; att < 24; ++att) {
                State out;
                double e = rkf78(y, f.M, f.a, h, f.rtol, f.atol, out);
                bool alive = alive_adaptive(out, f.M, f.a) && e == e;
                bool acc = alive && e <= 1.0, gated = false;
                double H = 0.0, Hs = 0.0, Q = 0.0;
                if (acc && f.inv_gate > 0.0) {
                    h_and_q(out, f.M, f.a, H, Hs, Q);
                    if (h > hmin * 1.01) {
                        gated = std::fabs(H - cur_H) > f.inv_gate * Hs || std::fabs(Q - cur_Q) > f.inv_gate * qs;
                        acc = !gated;
                    }
                }
                if (acc) {
                    ok = true; h_used = h;
                    rhs(y, f.M, f.a, k1);
                    y = out;
                    if (f.inv_gate > 0.0) { cur_H = H; cur_Q = Q; }
                    double sc2 = std::fmin(std::fmax(1.0, y.r / (0.5 * f.Rs)), 100.0);
                    double grow = std::fmin(4.0, std::fmax(0.2, kSafety * std::pow(std::fmax(e, 1e-16), -0.125)));
                    h_adapt = std::fmin(std::fmax(h * grow, hmin), f.ref_units ? kHMax : 10.0 * f.h_unit * sc2);
                    break;
                }
                if (h <= hmin * 1.01) break;
                double fac = (!alive || gated) ? 0.5 : std::fmin(0.9, std::fmax(0.1, kSafety * std::pow(e, -0.125)));
                h = std::fmax(h * fac, hmin);
            }
        } else if (f.integrator == NP_INTEG_ADAPTIVE) {
            // BH_RK_HMIN/HMAX for reference scenes; in units of M the largest
            // step is 10 x the fixed step law at the current radius
            const double hmin = f.ref_units ? kHMin : kHMin * f.M;
            const double hmax = f.ref_units ? kHMax : 10.0 * f.h_unit * scale;
            double hb = std::fmin(std::fmax(f.h_unit * scale, hmin), hmax);
            double h = (h_adapt > 0.0) ? h_adapt : hb;
            h = std::fmin(std::fmax(h, hmin), hmax);
            for (int att = 0; att < 8; ++att) {
                double ht = h;
                double fac = adaptive_step(y, f.M, f.a, ht, f.rtol, f.atol, &k1);
                if (fac > 0.0) {
                    ok = true; h_used = ht;
                    double sc2 = std::fmin(std::fmax(1.0, y.r / (0.5 * f.Rs)), 100.0);
                    h_adapt = std::fmin(std::fmax(ht * fac, hmin), f.ref_units ? kHMax : 10.0 * f.h_unit * sc2);
                    break;
                }
                h = std::fmax(ht, hmin);
                if (h <= hmin * 1.01) break;
            }
        } else {
            h_used = f.h_unit * scale;
            State out;
            rk4(y, f.M, f.a, h_used, out, &k1);
            y = out;
            ok = alive_fixed(y, f.M, f.a);
        }
        o.steps++;
        if (!ok) { o.captured = true; o.status = 1; break; }
        if (track_drift) {
            double H, Hs, Q;
            h_and_q(y, f.M, f.a, H, Hs, Q);
            o.dH = std::fmax(o.dH, std::fabs(H) / std::fmax(Hs, 1e-300));
            o.dQ = std::fmax(o.dQ, std::fabs(Q - Q0) / qs);
        }
        o.min_r = std::fmin(o.min_r, y.r);
        double dp = prev.th - half_pi, dc = y.th - half_pi;
        const double eps = 1e-8;
        bool sign_change = (dp > 0 && dc < 0) || (dp < 0 && dc > 0);
        bool near_zero = (std::fabs(dp) < eps && std::fabs(dc) >= eps) || (std::fabs(dc) < eps && std::fabs(dp) >= eps);
        if (sign_change || near_zero) {
            double alpha = std::fabs(dp) / (std::fabs(dp) + std::fabs(dc) + 1e-30);
            double rc, phc;
            if (f.crossing == NP_CROSS_ROOT && sign_change) {
                State z = root_crossing(f, prev, h_used, dp, alpha);
                rc = z.r;
                phc = z.ph;
            } else if (f.crossing == NP_CROSS_HERMITE && sign_change) {
                State f1;
                rhs(y, f.M, f.a, f1);
                double s = hermite_root(dp, dc, h_used * k1.th, h_used * f1.th, alpha);
                rc = hermite_eval(prev.r, y.r, h_used * k1.r, h_used * f1.r, s);
                phc = hermite_eval(prev.ph, y.ph, h_used * k1.ph, h_used * f1.ph, s);
            } else {
                rc = prev.r + alpha * (y.r - prev.r);
                phc = prev.ph + alpha * (y.ph - prev.ph);
            }
            if (o.crossings < 4) { o.xr[o.crossings] = rc; o.xphi[o.crossings] = phc; }
            o.crossings++;
            if (o.orders < f.max_orders && rc >= f.rin && rc <= f.rout) {
                double pt = prev.pt + alpha * (y.pt - prev.pt);
                double pph = prev.pph + alpha * (y.pph - prev.pph);
                float g = (float)doppler_g(rc, pt, pph, f.M, f.a);
                float c[3];
                shade_disk((float)rc, g, (float)f.q, c);
                o.disk[0] += c[0] * f.gain; o.disk[1] += c[1] * f.gain; o.disk[2] += c[2] * f.gain;
                if (o.orders == 0) o.first_hit_r = rc;
                o.orders++;
                if (track_inv) {
                    State cr = y; cr.r = rc; cr.th = half_pi; cr.pt = pt; cr.pph = pph;
                    invariants_at(f, cr, o.pt0, o.pph0, o.inv);
                }
            }
        }
        prev = y;
        if (y.r > f.r_far && step > 10) { o.status = 0; break; }
    }
    o.last = y;
}

// Colour of one traced sample (render.cu:312-359).
static void sample_colour(const Frame& f, const Dir& d, RayOut& o, bool track_inv, float col[3]) {
    if (o.captured) {
        if (f.bg_mode == NP_BG_POINT) {
            float rph = 1.5f * f.Rsf;
            float w = std::fmax(0.02f * f.Rsf, 0.005f * f.Rsf + 0.02f * f.bg_sigma_rad * f.Rsf);
            float dr = (float)o.min_r - rph;
            float I = f.bg_peak * std::exp(-0.5f * (dr / w) * (dr / w)) + 0.0f;
            col[0] = col[1] = col[2] = I;
        } else {
            col[0] = col[1] = col[2] = 0.0f;
        }
    } else if (o.orders > 0 && f.disk_on) {
        col[0] = o.disk[0]; col[1] = o.disk[1]; col[2] = o.disk[2];
    } else {
        if (track_inv) invariants_at(f, o.last, o.pt0, o.pph0, o.inv);
        if (f.bg_mode == NP_BG_POINT) {
            float rph = 1.5f * f.Rsf;
            float w = std::fmax(0.02f * f.Rsf, 0.005f * f.Rsf + 0.02f * f.bg_sigma_rad * f.Rsf);
            float dr = (float)o.min_r - rph;
            float I = f.bg_peak * std::exp(-0.5f * (dr / w) * (dr / w)) + 0.02f;
            col[0] = col[1] = col[2] = I;
        } else {
            shade_sky(d.cam_x * 0.5f + 0.5f, d.cam_y * 0.5f + 0.5f, col);
        }
    }
}

}  // namespace npo

using namespace npo;

extern "C" {

// Renders rows [y_begin, y_end) of the scene into full-frame planar buffers
// (rgb float[3][H][W], rcross float[H][W]); inv3 may be NULL.
int npo_render(const np_scene_t* sc, int y_begin, int y_end, float* rgb, float* rcross,
               float* inv3, int nthreads) {
    if (!sc || !rgb || sc->width <= 0 || sc->height <= 0 || sc->spp <= 0) return NP_ERR_INVALID;
    const np_scene_t s = *sc;
    Frame f = make_frame(s);
    const int W = s.width, H = s.height;
    y_begin = std::max(0, y_begin); y_end = std::min(H, y_end);
    const long npx = (long)W * (y_end - y_begin);
    const size_t plane = (size_t)W * H;
    const bool inv = s.check_invariants && inv3;
    float inv_all[3] = {0, 0, 0};
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel
    {
        float inv_loc[3] = {0, 0, 0};
#pragma omp for schedule(dynamic, 16)
        for (long i = 0; i < npx; ++i) {
            int x = (int)(i % W);
            int y = y_begin + (int)(i / W);
            float acc[3] = {0, 0, 0};
            float rc0 = 0.0f;
            for (int sm = 0; sm < s.spp; ++sm) {
                uint32_t sid = (uint32_t)(s.sample_offset + sm);
                Dir d = camera_dir(f, s, x, y, sid, false, 0, 0);
                RayOut o;
                trace(f, d, inv, o);
                float col[3];
                sample_colour(f, d, o, inv, col);
                acc[0] += col[0]; acc[1] += col[1]; acc[2] += col[2];
                if (sm == 0) rc0 = (float)o.first_hit_r;
                if (inv) { inv_loc[0] = std::fmax(inv_loc[0], o.inv[0]);
                           inv_loc[1] = std::fmax(inv_loc[1], o.inv[1]);
                           inv_loc[2] = std::fmax(inv_loc[2], o.inv[2]); }
            }
            size_t p = (size_t)y * W + x;
            rgb[p] = acc[0]; rgb[plane + p] = acc[1]; rgb[2 * plane + p] = acc[2];
            if (rcross) rcross[p] = rc0;
        }
        if (inv) {
#pragma omp critical
            { inv_update(inv_all, inv_loc[0], inv_loc[1], inv_loc[2]); }
        }
    }
    if (inv) { inv3[0] = std::fmax(inv3[0], inv_all[0]); inv3[1] = std::fmax(inv3[1], inv_all[1]);
               inv3[2] = std::fmax(inv3[2], inv_all[2]); }
    return NP_OK;
}

// Traces explicit image positions; layout as np_trace_rays_device.
// steps (may be NULL) receives the number of integration steps per ray.
int npo_trace_rays(const np_scene_t* sc, int n, const double* px, const double* py,
                   double* consts, double* cross, int32_t* status, int32_t* steps, int nthreads) {
    if (!sc || n < 0 || !px || !py) return NP_ERR_INVALID;
    const np_scene_t s = *sc;
    Frame f = make_frame(s);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = 0; i < n; ++i) {
        Dir d = camera_dir(f, s, 0, 0, 0, true, px[i], py[i]);
        RayOut o;
        trace(f, d, false, o);
        if (consts) {
            double c = std::cos(f.th_cam), sn = std::sin(f.th_cam);
            State y0 = f.zamo ? camera_zamo(f.M, f.a, f.r_cam, f.th_cam, f.ph_cam, d.nr, d.nth, d.nph)
                              : camera_static(f.M, f.a, f.r_cam, f.th_cam, f.ph_cam, d.nr, d.nth, d.nph);
            double E = -y0.pt, L = y0.pph;
            double Q = y0.pth * y0.pth + c * c * (L * L / (sn * sn) - f.a * f.a * E * E);
            (void)Q;
            consts[4 * i + 0] = y0.pt;
            consts[4 * i + 1] = y0.pph;
            consts[4 * i + 2] = y0.pr;
            consts[4 * i + 3] = y0.pth;
        }
        if (cross) for (int k = 0; k < 4; ++k) { cross[8 * i + 2 * k] = o.xr[k]; cross[8 * i + 2 * k + 1] = o.xphi[k]; }
        if (status) status[i] = o.status + 16 * std::min(o.crossings, 15);
        if (steps) steps[i] = (int32_t)o.steps;
    }
    return NP_OK;
}

// Conserved-quantity drift of explicit rays; layout as np_trace_invariants_device.
// Camera momenta (p_t, p_phi, p_r, p_theta) of the rays of sample
// `sample_offset` (the sample whose first crossing np_render_device reports
// in rcross) of every pixel of rows [y_begin, y_end): consts[4 * ((y -
// y_begin) * width + x) + 0..3].  The camera restatement of render.cu:137-170
// as npo_render uses it.
int npo_frame_rays(const np_scene_t* sc, int y_begin, int y_end, double* consts) {
    if (!sc || !consts || y_begin < 0 || y_end > sc->height || y_begin > y_end) return NP_ERR_INVALID;
    const np_scene_t s = *sc;
    Frame f = make_frame(s);
    for (int y = y_begin; y < y_end; ++y)
        for (int x = 0; x < s.width; ++x) {
            Dir d = camera_dir(f, s, x, y, (uint32_t)s.sample_offset, false, 0.0, 0.0);
            State y0 = f.zamo ? camera_zamo(f.M, f.a, f.r_cam, f.th_cam, f.ph_cam, d.nr, d.nth, d.nph)
                              : camera_static(f.M, f.a, f.r_cam, f.th_cam, f.ph_cam, d.nr, d.nth, d.nph);
            double* c = consts + 4 * ((size_t)(y - y_begin) * s.width + x);
            c[0] = y0.pt; c[1] = y0.pph; c[2] = y0.pr; c[3] = y0.pth;
        }
    return NP_OK;
}

int npo_trace_invariants(const np_scene_t* sc, int n, const double* px, const double* py, double* drift,
                         int32_t* steps, int nthreads) {
    if (!sc || n < 0 || !px || !py || !drift) return NP_ERR_INVALID;
    const np_scene_t s = *sc;
    Frame f = make_frame(s);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = 0; i < n; ++i) {
        Dir d = camera_dir(f, s, 0, 0, 0, true, px[i], py[i]);
        RayOut o;
        trace(f, d, false, o, true);
        drift[2 * i] = o.dH;
        drift[2 * i + 1] = o.dQ;
        if (steps) steps[i] = (int32_t)o.steps;
    }
    return NP_OK;
}

// The 7(8) tableau (rows of A, weights b8, error weights) for order checks.
void npo_rkf78_tableau(double* A, double* b, double* e) {
    for (int j = 0; j < 13; ++j) {
        for (int i = 0; i < 13; ++i) A[13 * j + i] = i < 12 ? kF78A[j][i] : 0.0;
        b[j] = kF78B[j];
        e[j] = kF78E[j];
    }
}

int npo_abi_version(void) { return NP_ABI_VERSION; }

int npo_critical_curve(const np_scene_t* sc, float* rho) {
    if (!sc || !rho) return -1;
    np_scene_t s = *sc;
    s.jitter = NP_JITTER_CRITICAL;
    Frame f = make_frame(s);
    for (int i = 0; i < 256; ++i) rho[i] = f.crit_rho[i];
    return 0;
}

// Raw metric blocks (order tt, tphi, phiphi, rr, thth) for unit checks.
void npo_metric_inv(double M, double a, double r, double th, double* g5) { metric_inv(M, a, r, th, g5); }
void npo_metric_inv_derivs(double M, double a, double r, double th, double* dr5, double* dth5) {
    metric_inv_derivs(M, a, r, th, dr5, dth5);
}

}  // extern "C"
