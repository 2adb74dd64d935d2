// adjoint.cu -- differentiable Kerr render: forward pass with checkpoints and a
// hand-written reverse (adjoint) sweep through the RK4 steps, on sm_103a.
//
// Image model (per sample): colour = gain * (w . base) * sum_k r_k^-q g_k^3 over
// the disk crossings of the ray (render.cu:65-72, 229-231 with emissivity
// index q), the sky or black otherwise; the image is the mean over samples.
// Parameters differentiated: spin a, camera inclination theta_cam, disk gain,
// emissivity index q.  The forward integrator is the Carter-form Hamiltonian
// RK4 of the mixed path with the reference step law h = h0 clamp(r/M, 1, 100)
// (render.cu:185,207), shortened near the polar axis by the factor
// sin(theta) / (sin(theta) + 0.05), and cubic-Hermite crossing location, in
// FP32 or FP64.  The axis factor keeps the discrete map smooth for rays that
// pass close to a pole (L ~ 0): there the theta equation's L^2/sin^3(theta)
// term turns the ray within a few times theta_min, which the plain step law
// steps over, so that the map's derivative is not that of its secant.
//
// Backward: the forward stores the state every K steps (checkpoints); the
// reverse sweep walks the checkpoint segments from last to first, recomputes
// the K states of a segment into a per-ray buffer, and back-propagates the
// adjoint state through each RK4 step (stages re-evaluated from the stored
// state) with the vector-Jacobian product of the right-hand side, adding the
// gradient of every disk crossing (implicit root of the Hermite interpolant)
// on the way.  Classification changes (disk edge, capture, escape) are not
// differentiated: the gradient is that of the image with every ray's event
// structure held fixed.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <algorithm>

#include <cuda_runtime.h>

#include "np_render.h"
#include "np_common.cuh"

using namespace np;

namespace {

thread_local std::string g_adj_error;
int adj_fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_adj_error = buf;
    np_record_error(buf);
    return code;
}

// Scene constants of the differentiable path (host-prepared, double).
struct AdjScene {
    int W, H, spp, sample_offset, strata, jitter, max_orders, disk_on, K, max_seg;
    unsigned seed;
    long long npix, total;
    double M, a, r_cam, th_cam, ph_cam, tan_half, aspect, h_unit, rin, rout, r_far, gain, q, r_plus, r_minus;
    int max_steps;
};

// Width of the step law's polar-axis factor sin(theta) / (sin(theta) + sigma).
constexpr double kPoleSigma = 0.05;

// ---------------------------------------------------------------------------
// Forward-mode numbers with two tangents (d/da, d/dtheta_cam) for ray set-up.
struct Dual2 {
    double v, a, t;
};
__device__ __forceinline__ Dual2 dc(double x) { return Dual2{x, 0.0, 0.0}; }
__device__ __forceinline__ Dual2 operator+(Dual2 x, Dual2 y) { return Dual2{x.v + y.v, x.a + y.a, x.t + y.t}; }
__device__ __forceinline__ Dual2 operator-(Dual2 x, Dual2 y) { return Dual2{x.v - y.v, x.a - y.a, x.t - y.t}; }
__device__ __forceinline__ Dual2 operator-(Dual2 x) { return Dual2{-x.v, -x.a, -x.t}; }
__device__ __forceinline__ Dual2 operator*(Dual2 x, Dual2 y) {
    return Dual2{x.v * y.v, x.a * y.v + x.v * y.a, x.t * y.v + x.v * y.t};
}
__device__ __forceinline__ Dual2 operator/(Dual2 x, Dual2 y) {
    double iv = 1.0 / y.v, q = x.v * iv;
    return Dual2{q, (x.a - q * y.a) * iv, (x.t - q * y.t) * iv};
}
__device__ __forceinline__ Dual2 dsqrt(Dual2 x) {
    double s = sqrt(x.v), h = 0.5 / s;
    return Dual2{s, x.a * h, x.t * h};
}

// Static-observer / ZAMO camera momentum with tangents (bh_kerr.h:781-826,
// 910-967), as functions of a and theta_cam.
struct DMom { Dual2 pt, pr, pth, pph; };
__device__ DMom camera_dual(const AdjScene& s, double nr, double nth, double nph, bool zamo) {
    const Dual2 a{s.a, 1.0, 0.0};
    const Dual2 th{s.th_cam, 0.0, 1.0};
    const Dual2 sn{sin(s.th_cam), 0.0, cos(s.th_cam)};
    const Dual2 cs{cos(s.th_cam), 0.0, -sin(s.th_cam)};
    (void)th;
    const Dual2 M = dc(s.M), r = dc(s.r_cam);
    Dual2 s2 = sn * sn, r2 = r * r, a2 = a * a;
    Dual2 Sig = r2 + a2 * cs * cs;
    Dual2 Del = r2 - dc(2.0) * M * r + a2;
    Dual2 A = (r2 + a2) * (r2 + a2) - a2 * Del * s2;
    Dual2 gtt = -(dc(1.0) - dc(2.0) * M * r / Sig);
    Dual2 gtp = -(dc(2.0) * M * a * r * s2 / Sig);
    Dual2 gpp = A * s2 / Sig;
    Dual2 grr = Sig / Del;
    Dual2 ghh = Sig;
    Dual2 Pt, Pp, Pr, Ph;
    if (!zamo) {
        Dual2 ut = dc(1.0) / dsqrt(-gtt);
        Dual2 er = dc(1.0) / dsqrt(grr);
        Dual2 eh = dc(1.0) / dsqrt(ghh);
        Dual2 ept, epp;
        if (fabs(gtp.v) > kEps) {
            Dual2 beta = -gtt / gtp;
            Dual2 n2 = gtt + dc(2.0) * gtp * beta + gpp * beta * beta;
            Dual2 inv = dc(1.0) / dsqrt(n2.v < 0.0 ? -n2 : n2);
            ept = inv; epp = beta * inv;
        } else {
            ept = dc(0.0); epp = dc(1.0) / dsqrt(gpp);
        }
        Pt = ut + dc(nph) * ept; Pr = dc(nr) * er; Ph = dc(nth) * eh; Pp = dc(nph) * epp;
    } else {
        Dual2 alpha = dsqrt(Del * Sig / A);
        Dual2 omega = dc(2.0) * M * a * r / A;
        Pt = dc(1.0) / alpha;
        Pp = omega / alpha + dc(nph) * dsqrt(Sig / A) / (sn.v < 0.0 ? -sn : sn);
        Pr = dc(nr) * dsqrt(Del / Sig);
        Ph = dc(nth) / dsqrt(Sig);
    }
    DMom m;
    m.pt = gtt * Pt + gtp * Pp;
    m.pr = grr * Pr;
    m.pth = ghh * Ph;
    m.pph = gtp * Pt + gpp * Pp;
    return m;
}

// Camera direction of a sample (lengths in M, stratified or wanghash jitter;
// same arithmetic as camera_dir of the render path in units of M).
__device__ void adj_dir(const AdjScene& s, long long item, double& nr, double& nth, double& nph, float& cam_y,
                        long long& p, int& sl) {
    p = item % s.npix;
    sl = (int)(item / s.npix);
    int x = (int)(p % s.W), y = (int)(p / s.W);
    uint32_t sample = (uint32_t)(s.sample_offset + sl);
    double px, py;
    if (s.jitter == NP_JITTER_WANGHASH) {
        float jx = wang_unit((uint32_t)(x * 73856093u ^ y * 19349663u ^ sample * 83492791u)) - 0.5f;
        float jy = wang_unit((uint32_t)(x * 83492791u ^ y * 2654435761u ^ sample * 19349663u)) - 0.5f;
        px = x + 0.5 + jx; py = y + 0.5 + jy;
    } else {
        uint32_t pix = (uint32_t)(y * s.W + x);
        int m = s.strata;
        uint32_t c = sample % (uint32_t)(m * m);
        px = __dadd_rn((double)x, __ddiv_rn(__dadd_rn((double)(c % m), strat_unit(s.seed, pix, sample, 0)), (double)m));
        py = __dadd_rn((double)y, __ddiv_rn(__dadd_rn((double)(c / m), strat_unit(s.seed, pix, sample, 1)), (double)m));
    }
    double ndc_x = __dsub_rn(__dmul_rn(__ddiv_rn(px, (double)s.W), 2.0), 1.0);
    double ndc_y = __dsub_rn(__dmul_rn(__ddiv_rn(py, (double)s.H), 2.0), 1.0);
    double cx = __dmul_rn(__dmul_rn(ndc_x, s.aspect), s.tan_half);
    double cy = __dmul_rn(-ndc_y, s.tan_half);
    double cz = -1.0;
    double n2 = __dadd_rn(__dadd_rn(__dmul_rn(cx, cx), __dmul_rn(cy, cy)), __dmul_rn(cz, cz));
    double nrm = __ddiv_rn(1.0, __dsqrt_rn(n2));
    nr = __dmul_rn(cz, nrm); nth = __dmul_rn(cy, nrm); nph = __dmul_rn(cx, nrm);
    cam_y = (float)nth;
}

// ---------------------------------------------------------------------------
// Carter-form right-hand side and its vector-Jacobian product.
template <typename R>
struct V4 { R r, th, pr, pth; };

template <typename R>
struct Par { R E, L, a, M; };

template <typename R>
__device__ __forceinline__ V4<R> rhs(const V4<R>& y, const Par<R>& p) {
    R sn = sin(y.th), cs = cos(y.th);
    R s2 = sn * sn, is2 = R(1) / s2;
    R A = p.a * p.a;
    R Sig = y.r * y.r + A * cs * cs, iS = R(1) / Sig;
    R Del = y.r * y.r - R(2) * p.M * y.r + A, iD = R(1) / Del;
    R P = (y.r * y.r + A) * p.E - p.a * p.L, PiD = P * iD;
    R W = p.L * p.L * is2 + A * p.E * p.E * s2 - R(2) * p.a * p.E * p.L;
    R F = Del * y.pr * y.pr + y.pth * y.pth - P * PiD + W;
    R Fr = R(2) * (y.r - p.M) * (y.pr * y.pr + PiD * PiD) - R(4) * y.r * p.E * PiD;
    R sc2 = R(2) * sn * cs;
    R Ft = sc2 * (A * p.E * p.E - p.L * p.L * is2 * is2);
    V4<R> d;
    d.r = Del * y.pr * iS;
    d.th = y.pth * iS;
    d.pr = R(-0.5) * iS * (Fr - R(2) * y.r * iS * F);
    d.pth = R(-0.5) * iS * (Ft + A * sc2 * iS * F);
    return d;
}

// gy += g^T df/dy, gp += g^T df/d(E, L, a) for output adjoint g.
template <typename R>
__device__ __forceinline__ void rhs_vjp(const V4<R>& y, const Par<R>& p, const V4<R>& g, V4<R>& gy, R& gE, R& gL,
                                        R& ga) {
    const R r = y.r, pr = y.pr, pth = y.pth, E = p.E, L = p.L, a = p.a, M = p.M;
    // forward values
    R sn = sin(y.th), cs = cos(y.th);
    R s2 = sn * sn, is2 = R(1) / s2;
    R A = a * a, AE2 = A * E * E, L2 = L * L;
    R Sig = r * r + A * cs * cs, iS = R(1) / Sig;
    R Del = r * r - R(2) * M * r + A, iD = R(1) / Del;
    R P = (r * r + A) * E - a * L, PiD = P * iD;
    R W = L2 * is2 + AE2 * s2 - R(2) * a * E * L;
    R F = Del * pr * pr + pth * pth - P * PiD + W;
    R Delr = R(2) * (r - M);
    R Fr = Delr * (pr * pr + PiD * PiD) - R(4) * r * E * PiD;
    R sc2 = R(2) * sn * cs;
    R Ft = sc2 * (AE2 - L2 * is2 * is2);
    R X = Fr - R(2) * r * iS * F;
    R Yv = Ft + A * sc2 * iS * F;
    // reverse
    R g_iS = R(0), g_F = R(0), g_Fr = R(0), g_Ft = R(0), g_A = R(0), g_sc2 = R(0), g_Del = R(0);
    R g_r = R(0), g_pr = R(0), g_pth = R(0), g_E = R(0), g_L = R(0), g_a = R(0);
    R g_X = R(-0.5) * iS * g.pr;
    g_iS += R(-0.5) * X * g.pr;
    R g_Y = R(-0.5) * iS * g.pth;
    g_iS += R(-0.5) * Yv * g.pth;
    g_Fr += g_X;
    g_r += g_X * (R(-2) * iS * F);
    g_iS += g_X * (R(-2) * r * F);
    g_F += g_X * (R(-2) * r * iS);
    g_Ft += g_Y;
    g_A += g_Y * sc2 * iS * F;
    g_sc2 += g_Y * A * iS * F;
    g_iS += g_Y * A * sc2 * F;
    g_F += g_Y * A * sc2 * iS;
    g_pth += g.th * iS;
    g_iS += g.th * pth;
    g_Del += g.r * pr * iS;
    g_pr += g.r * Del * iS;
    g_iS += g.r * Del * pr;
    // Ft = sc2 (AE2 - L2 is2^2)
    R g_AE2 = g_Ft * sc2;
    R g_L2 = g_Ft * (-sc2 * is2 * is2);
    R g_is2 = g_Ft * (R(-2) * sc2 * L2 * is2);
    g_sc2 += g_Ft * (AE2 - L2 * is2 * is2);
    // Fr = Delr (pr^2 + PiD^2) - 4 r E PiD
    R g_Delr = g_Fr * (pr * pr + PiD * PiD);
    g_pr += g_Fr * Delr * R(2) * pr;
    R g_PiD = g_Fr * (Delr * R(2) * PiD - R(4) * r * E);
    g_r += g_Fr * (R(-4) * E * PiD);
    g_E += g_Fr * (R(-4) * r * PiD);
    g_r += R(2) * g_Delr;
    // F = Del pr^2 + pth^2 - P PiD + W
    g_Del += g_F * pr * pr;
    g_pr += g_F * R(2) * Del * pr;
    g_pth += g_F * R(2) * pth;
    R g_P = g_F * (-PiD);
    g_PiD += g_F * (-P);
    R g_W = g_F;
    // W = L2 is2 + AE2 s2 - 2 a E L
    g_L2 += g_W * is2;
    g_is2 += g_W * L2;
    g_AE2 += g_W * s2;
    R g_s2 = g_W * AE2;
    g_a += g_W * (R(-2) * E * L);
    g_E += g_W * (R(-2) * a * L);
    g_L += g_W * (R(-2) * a * E);
    // PiD = P iD
    g_P += g_PiD * iD;
    R g_iD = g_PiD * P;
    // P = (r^2 + A) E - a L
    g_r += g_P * R(2) * r * E;
    g_A += g_P * E;
    g_E += g_P * (r * r + A);
    g_a += g_P * (-L);
    g_L += g_P * (-a);
    // iD = 1/Del, Del = r^2 - 2 M r + A
    g_Del += g_iD * (-iD * iD);
    g_r += g_Del * (R(2) * r - R(2) * M);
    g_A += g_Del;
    // iS = 1/Sig, Sig = r^2 + A c^2
    R g_Sig = g_iS * (-iS * iS);
    g_r += g_Sig * R(2) * r;
    g_A += g_Sig * cs * cs;
    R g_cs = g_Sig * R(2) * A * cs;
    // is2 = 1/s2, s2 = s^2, sc2 = 2 s c
    g_s2 += g_is2 * (-is2 * is2);
    R g_sn = g_s2 * R(2) * sn;
    g_sn += g_sc2 * R(2) * cs;
    g_cs += g_sc2 * R(2) * sn;
    // AE2 = A E^2, L2 = L^2, A = a^2
    g_A += g_AE2 * E * E;
    g_E += g_AE2 * R(2) * A * E;
    g_L += g_L2 * R(2) * L;
    g_a += g_A * R(2) * a;
    gy.r += g_r;
    gy.th += g_sn * cs - g_cs * sn;
    gy.pr += g_pr;
    gy.pth += g_pth;
    gE += g_E;
    gL += g_L;
    ga += g_a;
}

template <typename R>
__device__ __forceinline__ V4<R> axpy4(const V4<R>& y, R h, const V4<R>& k) {
    return V4<R>{y.r + h * k.r, y.th + h * k.th, y.pr + h * k.pr, y.pth + h * k.pth};
}

// Step size h = h0 clamp(r/M, 1, 100) sin(theta) / (sin(theta) + sigma) and
// its partial derivatives dh/dr, dh/dtheta.
template <typename R>
__device__ __forceinline__ R step_h(const AdjScene& s, R r, R th, R& dhdr, R& dhdth) {
    R x = r / R(s.M);
    R hr, dhr;
    if (x <= R(1)) { hr = R(s.h_unit); dhr = R(0); }
    else if (x >= R(100)) { hr = R(s.h_unit * 100.0); dhr = R(0); }
    else { hr = R(s.h_unit) * x; dhr = R(s.h_unit / s.M); }
    const R sn = sin(th), cs = cos(th);
    const R den = sn + R(kPoleSigma);
    const R f = sn / den;
    dhdr = dhr * f;
    dhdth = hr * R(kPoleSigma) * cs / (den * den);
    return hr * f;
}

template <typename R>
__device__ __forceinline__ V4<R> rk4_step(const V4<R>& y, const Par<R>& p, R h, V4<R>& k1) {
    k1 = rhs(y, p);
    V4<R> k2 = rhs(axpy4(y, R(0.5) * h, k1), p);
    V4<R> k3 = rhs(axpy4(y, R(0.5) * h, k2), p);
    V4<R> k4 = rhs(axpy4(y, h, k3), p);
    R h6 = h / R(6);
    return V4<R>{y.r + h6 * (k1.r + R(2) * (k2.r + k3.r) + k4.r), y.th + h6 * (k1.th + R(2) * (k2.th + k3.th) + k4.th),
                 y.pr + h6 * (k1.pr + R(2) * (k2.pr + k3.pr) + k4.pr),
                 y.pth + h6 * (k1.pth + R(2) * (k2.pth + k3.pth) + k4.pth)};
}

// Reverse of one RK4 step: given gy1 = dJ/dy_{n+1}, adds the contributions to
// gy0 (= dJ/dy_n), to the constants' adjoints and returns dJ/dh.
template <typename R>
__device__ __forceinline__ R rk4_step_vjp(const V4<R>& y, const Par<R>& p, R h, const V4<R>& gy1, V4<R>& gy0, R& gE,
                                          R& gL, R& ga) {
    V4<R> k1 = rhs(y, p);
    V4<R> y2 = axpy4(y, R(0.5) * h, k1);
    V4<R> k2 = rhs(y2, p);
    V4<R> y3 = axpy4(y, R(0.5) * h, k2);
    V4<R> k3 = rhs(y3, p);
    V4<R> y4 = axpy4(y, h, k3);
    V4<R> k4 = rhs(y4, p);
    R h6 = h / R(6), h3 = h / R(3);
    R gh = (gy1.r * (k1.r + R(2) * (k2.r + k3.r) + k4.r) + gy1.th * (k1.th + R(2) * (k2.th + k3.th) + k4.th) +
            gy1.pr * (k1.pr + R(2) * (k2.pr + k3.pr) + k4.pr) + gy1.pth * (k1.pth + R(2) * (k2.pth + k3.pth) + k4.pth)) /
           R(6);
    V4<R> gk1{gy1.r * h6, gy1.th * h6, gy1.pr * h6, gy1.pth * h6};
    V4<R> gk2{gy1.r * h3, gy1.th * h3, gy1.pr * h3, gy1.pth * h3};
    V4<R> gk3 = gk2;
    V4<R> gk4 = gk1;
    gy0.r += gy1.r; gy0.th += gy1.th; gy0.pr += gy1.pr; gy0.pth += gy1.pth;
    // k4 = f(y4), y4 = y + h k3
    V4<R> g4{R(0), R(0), R(0), R(0)};
    rhs_vjp(y4, p, gk4, g4, gE, gL, ga);
    gy0.r += g4.r; gy0.th += g4.th; gy0.pr += g4.pr; gy0.pth += g4.pth;
    gk3.r += h * g4.r; gk3.th += h * g4.th; gk3.pr += h * g4.pr; gk3.pth += h * g4.pth;
    gh += g4.r * k3.r + g4.th * k3.th + g4.pr * k3.pr + g4.pth * k3.pth;
    // k3 = f(y3), y3 = y + h/2 k2
    V4<R> g3{R(0), R(0), R(0), R(0)};
    rhs_vjp(y3, p, gk3, g3, gE, gL, ga);
    gy0.r += g3.r; gy0.th += g3.th; gy0.pr += g3.pr; gy0.pth += g3.pth;
    R hh = R(0.5) * h;
    gk2.r += hh * g3.r; gk2.th += hh * g3.th; gk2.pr += hh * g3.pr; gk2.pth += hh * g3.pth;
    gh += R(0.5) * (g3.r * k2.r + g3.th * k2.th + g3.pr * k2.pr + g3.pth * k2.pth);
    // k2 = f(y2), y2 = y + h/2 k1
    V4<R> g2{R(0), R(0), R(0), R(0)};
    rhs_vjp(y2, p, gk2, g2, gE, gL, ga);
    gy0.r += g2.r; gy0.th += g2.th; gy0.pr += g2.pr; gy0.pth += g2.pth;
    gk1.r += hh * g2.r; gk1.th += hh * g2.th; gk1.pr += hh * g2.pr; gk1.pth += hh * g2.pth;
    gh += R(0.5) * (g2.r * k1.r + g2.th * k1.th + g2.pr * k1.pr + g2.pth * k1.pth);
    // k1 = f(y)
    rhs_vjp(y, p, gk1, gy0, gE, gL, ga);
    return gh;
}

// Redshift factor (bh_kerr.h:833-862 with k.u expanded) and its partial
// derivatives with respect to r, E, L, a (forward mode, closed form).
template <typename R>
__device__ __forceinline__ R doppler_d(R r, R E, R L, R a, R M, R& dr, R& dE, R& dL, R& da) {
    // Omega = 1 / (a/M + (r/M)^(3/2)) / M  (r >= M on the disk)
    R x = r / M, sx = sqrt(x);
    R D = a / M + x * sx;
    R Om = R(1) / (D * M);
    R dOm_dr = -Om / D * (R(1.5) * sx / M);
    R dOm_da = -Om / D * (R(1) / M);
    R ir = R(1) / r;
    R gtt = -(R(1) - R(2) * M * ir), gtp = -R(2) * M * a * ir, gpp = r * r + a * a + R(2) * M * a * a * ir;
    R dgtt_dr = -R(2) * M * ir * ir, dgtp_dr = R(2) * M * a * ir * ir, dgpp_dr = R(2) * r - R(2) * M * a * a * ir * ir;
    R dgtp_da = -R(2) * M * ir, dgpp_da = R(2) * a + R(4) * M * a * ir;
    R den = -(gtt + R(2) * gtp * Om + gpp * Om * Om);
    R dden_dOm = -(R(2) * gtp + R(2) * gpp * Om);
    R dden_dr = -(dgtt_dr + R(2) * dgtp_dr * Om + dgpp_dr * Om * Om) + dden_dOm * dOm_dr;
    R dden_da = -(R(2) * dgtp_da * Om + dgpp_da * Om * Om) + dden_dOm * dOm_da;
    R sd = sqrt(den);
    R B = E - Om * L;
    R g = E * sd / B;                           // = E / (u^t (E - Omega L)), u^t = 1/sqrt(den)
    R dg_dsd = E / B, dg_dB = -g / B;
    R dsd_dden = R(0.5) / sd;
    dr = dg_dsd * dsd_dden * dden_dr + dg_dB * (-L * dOm_dr);
    da = dg_dsd * dsd_dden * dden_da + dg_dB * (-L * dOm_da);
    dE = sd / B + dg_dB;
    dL = dg_dB * (-Om);
    return g;
}

// Hermite crossing: root u of p(u) = h00 d0 + h10 m0 + h01 d1 + h11 m1 and
// r_c = h00 r0 + h10 hr0 + h01 r1 + h11 hr1 (hr = h dr/dlambda).
template <typename R>
__device__ __forceinline__ R herm_root(R d0, R d1, R m0, R m1) {
    R s = fabs(d0) / (fabs(d0) + fabs(d1) + R(1e-30)), lo = R(0), hi = R(1);
#pragma unroll 1
    for (int it = 0; it < 30; ++it) {
        R s2 = s * s, s3 = s2 * s;
        R p = (R(2) * s3 - R(3) * s2 + R(1)) * d0 + (s3 - R(2) * s2 + s) * m0 + (R(3) * s2 - R(2) * s3) * d1 + (s3 - s2) * m1;
        R dp = (R(6) * s2 - R(6) * s) * (d0 - d1) + (R(3) * s2 - R(4) * s + R(1)) * m0 + (R(3) * s2 - R(2) * s) * m1;
        if ((p > R(0)) == (d0 > R(0))) lo = s; else hi = s;
        R sn = (dp != R(0)) ? s - p / dp : R(0.5) * (lo + hi);
        if (!(sn > lo && sn < hi)) sn = R(0.5) * (lo + hi);
        bool done = fabs(sn - s) < R(sizeof(R) == 4 ? 1e-7 : 1e-15);
        s = sn;
        if (done) break;
    }
    return s;
}

// Per-ray forward record.
struct RayRec {
    int steps, status, orders;
};

// Forward integration of one ray.  With `ck` non-null the state (and the disk
// hits so far) is stored every K steps: ck[j] = state after j K steps.
template <typename R>
__device__ void trace_fwd(const AdjScene& s, const V4<R>& y0, const Par<R>& p, V4<R>* ck, int* ck_orders, RayRec& rec,
                          R& disk_sum, R* xr = nullptr) {
    V4<R> y = y0;
    V4<R> f0 = rhs(y, p);
    const R hp = R(1.5707963267948966);
    const R rp = R(s.r_plus);
    rec.steps = 0; rec.status = 2; rec.orders = 0;
    disk_sum = R(0);
    for (int n = 0; n < s.max_steps; ++n) {
        if (ck && n % s.K == 0) { ck[n / s.K] = y; ck_orders[n / s.K] = rec.orders; }
        R dhdr, dhdth;
        R h = step_h<R>(s, y.r, y.th, dhdr, dhdth);
        V4<R> k1;
        V4<R> y1 = rk4_step(y, p, h, k1);
        rec.steps = n + 1;
        bool ok = y1.r > rp * R(1.000001) && y1.th > R(1e-7) && y1.th < R(3.1415925);
        if (!ok) { rec.status = 1; return; }
        V4<R> f1 = rhs(y1, p);
        R d0 = y.th - hp, d1 = y1.th - hp;
        if ((d0 > R(0) && d1 < R(0)) || (d0 < R(0) && d1 > R(0))) {
            R u = herm_root(d0, d1, h * f0.th, h * f1.th);
            R u2 = u * u, u3 = u2 * u;
            R rc = (R(2) * u3 - R(3) * u2 + R(1)) * y.r + (u3 - R(2) * u2 + u) * h * f0.r + (R(3) * u2 - R(2) * u3) * y1.r +
                   (u3 - u2) * h * f1.r;
            if (rec.orders < s.max_orders && rc >= R(s.rin) && rc <= R(s.rout)) {
                R dr, dE, dL, da;
                R g = doppler_d(rc, p.E, p.L, p.a, p.M, dr, dE, dL, da);
                disk_sum += pow(rc, -R(s.q)) * g * g * g;
                if (xr && rec.orders < 4) xr[rec.orders] = rc;
                rec.orders++;
            }
        }
        y = y1;
        f0 = f1;
        if (y.r > R(s.r_far) && n + 1 > 11) { rec.status = 0; return; }
    }
}

// Colour of a sample from the forward record (render.cu:312-359 rules).
__device__ __forceinline__ void adj_colour(const AdjScene& s, const RayRec& rec, double disk_sum, float cam_y, float col[3]) {
    if (rec.status == 1 || !(rec.orders > 0 && s.disk_on)) {
        if (rec.status == 1) { col[0] = col[1] = col[2] = 0.0f; }
        else shade_sky(cam_y * 0.5f + 0.5f, col);
    } else {
        float I = (float)(s.gain * disk_sum);
        col[0] = 1.0f * I; col[1] = 0.75f * I; col[2] = 0.45f * I;
    }
}

struct AdjBuffers {
    float* srgb;            // [spp][3][npix] per-sample colours
    int32_t* sig;           // [spp][npix] event signature: status + 4 * orders
    unsigned char* ck;      // per-ray checkpoint slots
    unsigned char* seg;     // per-thread segment buffers of the reverse sweep
    double* grad;           // [total][4] per-sample gradients (a, theta, gain, q)
    unsigned long long* work;   // next ray of the reverse sweep (zeroed before each sweep)
    size_t ck_stride, seg_stride;   // bytes per ray
};

template <typename R>
__device__ __forceinline__ void ray_setup(const AdjScene& s, long long item, V4<R>& y0, Par<R>& p, DMom& dm,
                                          float& cam_y, long long& pix, int& sl, bool zamo) {
    double nr, nth, nph;
    adj_dir(s, item, nr, nth, nph, cam_y, pix, sl);
    dm = camera_dual(s, nr, nth, nph, zamo);
    y0 = V4<R>{R(s.r_cam), R(s.th_cam), R(dm.pr.v), R(dm.pth.v)};
    p = Par<R>{R(-dm.pt.v), R(dm.pph.v), R(s.a), R(s.M)};
}

template <typename R>
__global__ void adj_forward_kernel(const AdjScene s, AdjBuffers b, int zamo, int store) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < s.total;
         i += (long long)gridDim.x * blockDim.x) {
        V4<R> y0; Par<R> p; DMom dm; float cam_y; long long pix; int sl;
        ray_setup<R>(s, i, y0, p, dm, cam_y, pix, sl, zamo != 0);
        V4<R>* ck = store ? (V4<R>*)(b.ck + (size_t)i * b.ck_stride) : nullptr;
        int* cko = store ? (int*)(b.ck + (size_t)i * b.ck_stride + (size_t)s.max_seg * sizeof(V4<R>)) : nullptr;
        RayRec rec;
        R disk;
        trace_fwd<R>(s, y0, p, ck, cko, rec, disk);
        if (store) {
            int* recp = cko + s.max_seg;
            recp[0] = rec.steps; recp[1] = rec.status; recp[2] = rec.orders;
        }
        float col[3];
        adj_colour(s, rec, (double)disk, cam_y, col);
        float* base = b.srgb + (size_t)sl * 3 * s.npix;
        base[pix] = col[0]; base[s.npix + pix] = col[1]; base[2 * s.npix + pix] = col[2];
        b.sig[(size_t)sl * s.npix + pix] = rec.status + 4 * rec.orders;
    }
}

// Mean over samples.
__global__ void adj_resolve_kernel(const float* srgb, float* img, long long npix, int spp) {
    long long n = 3 * npix;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float acc = 0.0f;
        for (int s = 0; s < spp; ++s) acc += srgb[(size_t)s * n + i];
        img[i] = acc / (float)spp;
    }
}

// Reverse sweep.  gimg = dLoss/dimage [3][npix]; writes per-sample gradients
// (d/da, d/dtheta_cam, d/dgain, d/dq) to b.grad.
// A resident grid whose threads take rays one at a time from a global
// counter (rays differ in length by orders of magnitude, so a static
// assignment leaves a long tail); the segment buffer belongs to the thread,
// so its memory scales with the grid, not with the rays.
template <typename R>
__global__ void adj_backward_kernel(const AdjScene s, AdjBuffers b, const float* __restrict__ gimg, int zamo) {
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    V4<R>* seg = (V4<R>*)(b.seg + (size_t)tid * b.seg_stride);
    for (long long i = (long long)atomicAdd(b.work, 1ull); i < s.total; i = (long long)atomicAdd(b.work, 1ull)) {
        double* out = b.grad + (size_t)i * 4;
        out[0] = out[1] = out[2] = out[3] = 0.0;
        V4<R>* ck = (V4<R>*)(b.ck + (size_t)i * b.ck_stride);
        int* cko = (int*)(b.ck + (size_t)i * b.ck_stride + (size_t)s.max_seg * sizeof(V4<R>));
        const int* recp = cko + s.max_seg;
        const int N = recp[0], status = recp[1], orders = recp[2];
        if (status == 1 || orders == 0 || !s.disk_on) continue;     // colour does not depend on the parameters
        V4<R> y0; Par<R> p; DMom dm; float cam_y; long long pix; int sl;
        ray_setup<R>(s, i, y0, p, dm, cam_y, pix, sl, zamo != 0);
        // dL/dcolour of this sample = gimg / spp; colour = gain * (w . base) * sum_k f_k
        const double inv = 1.0 / s.spp;
        const double B = (1.0 * gimg[pix] + 0.75 * gimg[s.npix + pix] + 0.45 * gimg[2 * s.npix + pix]) * inv;
        if (B == 0.0) continue;
        const R cf = R(s.gain * B);     // dJ/d(sum_k f_k)
        V4<R> gy{R(0), R(0), R(0), R(0)};
        R gE = R(0), gL = R(0), ga = R(0);
        double g_gain = 0.0, g_q = 0.0;
        const R hp = R(1.5707963267948966);
        const int nseg = (N + s.K - 1) / s.K;
        for (int j = nseg - 1; j >= 0; --j) {
            const int n0 = j * s.K, n1 = min(N, n0 + s.K);
            // recompute the segment's states y_{n0} .. y_{n1}
            seg[0] = ck[j];
            int hits_before = cko[j];
            for (int n = n0; n < n1; ++n) {
                R dhdr, dhdth;
                R h = step_h<R>(s, seg[n - n0].r, seg[n - n0].th, dhdr, dhdth);
                V4<R> k1;
                seg[n - n0 + 1] = rk4_step(seg[n - n0], p, h, k1);
            }
            // disk hits in this segment, in order (the order index decides whether a hit counts)
            int hit_index[64];
            int nh = 0;
            {
                int hits = hits_before;
                for (int n = n0; n < n1 && nh < 64; ++n) {
                    const V4<R>& ya = seg[n - n0];
                    const V4<R>& yb = seg[n - n0 + 1];
                    if (n == N - 1 && status == 1) break;
                    R d0 = ya.th - hp, d1 = yb.th - hp;
                    if (!((d0 > R(0) && d1 < R(0)) || (d0 < R(0) && d1 > R(0)))) continue;
                    R dhdr, dhdth;
                    R h = step_h<R>(s, ya.r, ya.th, dhdr, dhdth);
                    V4<R> fa = rhs(ya, p), fb = rhs(yb, p);
                    R u = herm_root(d0, d1, h * fa.th, h * fb.th);
                    R u2 = u * u, u3 = u2 * u;
                    R rc = (R(2) * u3 - R(3) * u2 + R(1)) * ya.r + (u3 - R(2) * u2 + u) * h * fa.r +
                           (R(3) * u2 - R(2) * u3) * yb.r + (u3 - u2) * h * fb.r;
                    if (hits < s.max_orders && rc >= R(s.rin) && rc <= R(s.rout)) { hit_index[nh++] = n; hits++; }
                }
            }
            // reverse through the segment
            int hcur = nh - 1;
            for (int n = n1 - 1; n >= n0; --n) {
                const V4<R> ya = seg[n - n0];
                const V4<R> yb = seg[n - n0 + 1];
                R dhdr, dhdth;
                R h = step_h<R>(s, ya.r, ya.th, dhdr, dhdth);
                R gh = R(0);
                V4<R> gya{R(0), R(0), R(0), R(0)};
                if (hcur >= 0 && hit_index[hcur] == n) {
                    --hcur;
                    // crossing gradient: J_k = cf * rc^-q g^3
                    V4<R> fa = rhs(ya, p), fb = rhs(yb, p);
                    R d0 = ya.th - hp, d1 = yb.th - hp, m0 = h * fa.th, m1 = h * fb.th;
                    R u = herm_root(d0, d1, m0, m1);
                    R u2 = u * u, u3 = u2 * u;
                    R h00 = R(2) * u3 - R(3) * u2 + R(1), h10 = u3 - R(2) * u2 + u, h01 = R(3) * u2 - R(2) * u3, h11 = u3 - u2;
                    R e00 = R(6) * u2 - R(6) * u, e10 = R(3) * u2 - R(4) * u + R(1), e01 = -e00, e11 = R(3) * u2 - R(2) * u;
                    R rc = h00 * ya.r + h10 * h * fa.r + h01 * yb.r + h11 * h * fb.r;
                    R drg, dEg, dLg, dag;
                    R g = doppler_d(rc, p.E, p.L, p.a, p.M, drg, dEg, dLg, dag);
                    R rq = pow(rc, -R(s.q));
                    R fk = rq * g * g * g;
                    g_gain += (double)(B * (double)fk);
                    g_q += (double)(-(double)cf * log((double)rc) * (double)fk);
                    R gJ_rc = cf * (-R(s.q) * fk / rc + rq * R(3) * g * g * drg);
                    gE += cf * rq * R(3) * g * g * dEg;
                    gL += cf * rq * R(3) * g * g * dLg;
                    ga += cf * rq * R(3) * g * g * dag;
                    // r_c through the implicit root u and directly
                    R drc_du = e00 * ya.r + e10 * h * fa.r + e01 * yb.r + e11 * h * fb.r;
                    R dp_du = e00 * d0 + e10 * m0 + e01 * d1 + e11 * m1;
                    R kappa = -gJ_rc * drc_du / dp_du;
                    R g_d0 = kappa * h00, g_m0 = kappa * h10, g_d1 = kappa * h01, g_m1 = kappa * h11;
                    gya.r += gJ_rc * h00;
                    gy.r += gJ_rc * h01;                    // y_{n+1} adjoint lives in gy
                    V4<R> gfa{gJ_rc * h10 * h, g_m0 * h, R(0), R(0)};
                    V4<R> gfb{gJ_rc * h11 * h, g_m1 * h, R(0), R(0)};
                    gh += gJ_rc * (h10 * fa.r + h11 * fb.r) + g_m0 * fa.th + g_m1 * fb.th;
                    gya.th += g_d0;
                    gy.th += g_d1;
                    rhs_vjp(ya, p, gfa, gya, gE, gL, ga);
                    rhs_vjp(yb, p, gfb, gy, gE, gL, ga);
                }
                // through the step y_{n+1} = Phi(y_n, h(r_n))
                gh += rk4_step_vjp(ya, p, h, gy, gya, gE, gL, ga);
                gya.r += gh * dhdr;
                gya.th += gh * dhdth;
                gy = gya;
            }
        }
        // camera set-up: y0 = (r_cam, theta_cam, p_r, p_theta), E = -p_t, L = p_phi
        double da = (double)ga + (double)gy.pr * dm.pr.a + (double)gy.pth * dm.pth.a - (double)gE * dm.pt.a +
                    (double)gL * dm.pph.a;
        double dth = (double)gy.th + (double)gy.pr * dm.pr.t + (double)gy.pth * dm.pth.t - (double)gE * dm.pt.t +
                     (double)gL * dm.pph.t;
        out[0] = da * s.M;         // d/d(spin), a = spin M
        out[1] = dth;              // d/d(theta_cam) in radians
        out[2] = g_gain;
        out[3] = g_q;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI (include/np_render.h).

struct np_adjoint {
    int device = -1;
    int precision = NP_PREC_MIXED;
    AdjScene s{};
    int zamo = 0;
    AdjBuffers b{};
    int bwd_blocks = 1;      // grid of the reverse sweep (its threads own the segment buffers)
    size_t bytes = 0;
    void* base = nullptr;
    bool have_forward = false;
};

namespace {

int prepare_adj(const np_scene_t& sc, int K, AdjScene& s, int& zamo) {
    if (sc.units != NP_UNITS_M) return adj_fail(NP_ERR_INVALID, "the differentiable render needs lengths in M");
    if (sc.integrator != NP_INTEG_RK4) return adj_fail(NP_ERR_INVALID, "the differentiable render uses fixed-step RK4");
    if (sc.crossing != NP_CROSS_HERMITE) return adj_fail(NP_ERR_INVALID, "the differentiable render uses Hermite crossings");
    if (sc.background != NP_BG_GRADIENT) return adj_fail(NP_ERR_INVALID, "the differentiable render uses the gradient sky");
    if (K < 1 || K > 4096) return adj_fail(NP_ERR_INVALID, "checkpoint interval K must be in [1, 4096]");
    int v = np_scene_validate(&sc);
    if (v != NP_OK) return v;
    memset(&s, 0, sizeof(s));
    s.W = sc.width; s.H = sc.height; s.spp = sc.spp; s.sample_offset = sc.sample_offset;
    s.strata = std::max(1, (int)std::floor(std::sqrt((double)std::max(1, sc.spp))));
    s.jitter = sc.jitter; s.seed = sc.seed;
    s.max_orders = std::max(1, sc.disk_max_orders); s.disk_on = sc.disk_on; s.K = K;
    s.max_steps = sc.max_steps;
    s.max_seg = (sc.max_steps + K - 1) / K + 1;
    s.npix = (long long)sc.width * sc.height; s.total = s.npix * sc.spp;
    s.M = sc.mass; s.a = sc.spin * sc.mass; s.r_cam = sc.r_cam * sc.mass;
    s.th_cam = sc.theta_deg * kPi / 180.0; s.ph_cam = sc.phi_deg * kPi / 180.0;
    s.aspect = (double)sc.width / sc.height; s.tan_half = std::tan(0.5 * sc.fov_y_deg * kPi / 180.0);
    s.h_unit = sc.step_scale;
    s.rin = sc.disk_rin > 0 ? sc.disk_rin : 6.0 * sc.mass;
    s.rout = sc.disk_rout > 0 ? sc.disk_rout : 40.0 * sc.mass;
    s.r_far = sc.escape_r > 0 ? sc.escape_r : s.r_cam + 20.0 * sc.mass;
    s.gain = sc.disk_gain; s.q = sc.emissivity_q;
    double disc = std::max(0.0, s.M * s.M - s.a * s.a);
    s.r_plus = s.M + std::sqrt(disc); s.r_minus = s.M - std::sqrt(disc);
    double r = s.r_cam, th = s.th_cam, a = s.a, M = s.M;
    double gtt = -(1.0 - 2.0 * M * r / (r * r + a * a * std::cos(th) * std::cos(th)));
    zamo = (sc.camera == NP_CAMERA_ZAMO) || !(gtt < 0.0);
    return NP_OK;
}

}  // namespace

extern "C" {

np_adjoint_t* np_adjoint_create(void) { return new np_adjoint(); }

void np_adjoint_destroy(np_adjoint_t* h) {
    if (!h) return;
    if (h->base) cudaFree(h->base);
    delete h;
}


int np_adjoint_forward(np_adjoint_t* h, const np_scene_t* scene, int precision, int K, float* d_img,
                       float* d_sample_rgb, int32_t* d_sample_sig, void* stream_v, np_adjoint_stats_t* stats) {
    if (!h || !scene || !d_img) return adj_fail(NP_ERR_INVALID, "NULL argument");
    if (precision != NP_PREC_FP64 && precision != NP_PREC_MIXED) return adj_fail(NP_ERR_INVALID, "Invalid precision.");
    AdjScene s;
    int zamo = 0;
    int rc = prepare_adj(*scene, K, s, zamo);
    if (rc != NP_OK) return rc;
    const size_t rsz = precision == NP_PREC_FP64 ? sizeof(V4<double>) : sizeof(V4<float>);
    const size_t ck_stride = ((size_t)s.max_seg * (rsz + sizeof(int)) + 3 * sizeof(int) + 15) & ~(size_t)15;
    const size_t seg_stride = ((size_t)(K + 1) * rsz + 15) & ~(size_t)15;
    const size_t n = (size_t)s.total;
    // reverse-sweep grid: the resident blocks of 64 threads, at most as many
    // as the rays need, and few enough that the segment buffers stay within
    // 256 MiB (at least one block per SM)
    int dev = 0, sms = 1, occ = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (precision == NP_PREC_FP64)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, adj_backward_kernel<double>, 64, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, adj_backward_kernel<float>, 64, 0);
    long long bwd = std::min<long long>((s.total + 63) / 64, (long long)sms * std::max(1, occ));
    bwd = std::min<long long>(bwd, std::max<long long>(sms, (256ll << 20) / (long long)(seg_stride * 64)));
    bwd = std::max<long long>(1, bwd);
    const size_t nthreads = (size_t)bwd * 64;
    const size_t need = n * 3 * sizeof(float) + n * sizeof(int32_t) + n * ck_stride + nthreads * seg_stride +
                        n * 4 * sizeof(double) + 1024 + 256;
    cudaStream_t st = (cudaStream_t)stream_v;
    if (h->bytes < need) {
        if (h->base) { cudaStreamSynchronize(st); cudaFree(h->base); h->base = nullptr; h->bytes = 0; }
        if (cudaMalloc(&h->base, need) != cudaSuccess)
            return adj_fail(NP_ERR_ALLOC, "cudaMalloc of %zu bytes for the adjoint workspace failed", need);
        h->bytes = need;
    }
    char* p = (char*)h->base;
    AdjBuffers b;
    b.srgb = d_sample_rgb ? d_sample_rgb : (float*)p; p += n * 3 * sizeof(float);
    b.sig = d_sample_sig ? d_sample_sig : (int32_t*)p; p += n * sizeof(int32_t);
    p = (char*)(((uintptr_t)p + 255) & ~(uintptr_t)255);
    b.ck = (unsigned char*)p; p += n * ck_stride;
    b.seg = (unsigned char*)p; p += nthreads * seg_stride;
    p = (char*)(((uintptr_t)p + 255) & ~(uintptr_t)255);
    b.grad = (double*)p; p += n * 4 * sizeof(double);
    p = (char*)(((uintptr_t)p + 255) & ~(uintptr_t)255);
    b.work = (unsigned long long*)p;
    b.ck_stride = ck_stride; b.seg_stride = seg_stride;
    const int threads = 128;
    const int blocks = (int)std::min<long long>((s.total + threads - 1) / threads, (long long)sms * 64);
    cudaEvent_t e0, e1;
    if (stats) { cudaEventCreate(&e0); cudaEventCreate(&e1); cudaEventRecord(e0, st); }
    if (precision == NP_PREC_FP64) adj_forward_kernel<double><<<blocks, threads, 0, st>>>(s, b, zamo, 1);
    else adj_forward_kernel<float><<<blocks, threads, 0, st>>>(s, b, zamo, 1);
    adj_resolve_kernel<<<(int)std::min<long long>((3 * s.npix + 255) / 256, (long long)sms * 16), 256, 0, st>>>(
        b.srgb, d_img, s.npix, s.spp);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return adj_fail(NP_ERR_KERNEL, "%s", cudaGetErrorString(e));
    if (stats) {
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0; cudaEventElapsedTime(&ms, e0, e1);
        stats->forward_ms = ms;
        stats->workspace_bytes = need;
        stats->checkpoint_bytes_per_ray = ck_stride;
        cudaEventDestroy(e0); cudaEventDestroy(e1);
    }
    h->s = s; h->zamo = zamo; h->b = b; h->precision = precision; h->have_forward = true;
    h->bwd_blocks = (int)bwd;
    return NP_OK;
}

int np_adjoint_backward(np_adjoint_t* h, const float* d_grad_img, double* h_grad4, double* d_sample_grad,
                        void* stream_v, np_adjoint_stats_t* stats) {
    if (!h || !d_grad_img || !h_grad4) return adj_fail(NP_ERR_INVALID, "NULL argument");
    if (!h->have_forward) return adj_fail(NP_ERR_INVALID, "np_adjoint_forward must run first");
    cudaStream_t st = (cudaStream_t)stream_v;
    const AdjScene& s = h->s;
    const int threads = 64;
    const int blocks = h->bwd_blocks;   // the grid the forward sized the segment buffers for
    cudaEvent_t e0, e1;
    if (stats) { cudaEventCreate(&e0); cudaEventCreate(&e1); cudaEventRecord(e0, st); }
    if (cudaMemsetAsync(h->b.work, 0, sizeof(unsigned long long), st) != cudaSuccess)
        return adj_fail(NP_ERR_KERNEL, "cudaMemsetAsync of the reverse-sweep counter failed");
    if (h->precision == NP_PREC_FP64) adj_backward_kernel<double><<<blocks, threads, 0, st>>>(s, h->b, d_grad_img, h->zamo);
    else adj_backward_kernel<float><<<blocks, threads, 0, st>>>(s, h->b, d_grad_img, h->zamo);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return adj_fail(NP_ERR_KERNEL, "%s", cudaGetErrorString(e));
    if (stats) cudaEventRecord(e1, st);
    // deterministic reduction on the host (per-sample gradients in sample order)
    const size_t n = (size_t)s.total;
    double* hg = (double*)malloc(n * 4 * sizeof(double));
    if (!hg) return adj_fail(NP_ERR_ALLOC, "host allocation failed");
    if (d_sample_grad) {
        e = cudaMemcpyAsync(d_sample_grad, h->b.grad, n * 4 * sizeof(double), cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) { free(hg); return adj_fail(NP_ERR_KERNEL, "%s", cudaGetErrorString(e)); }
    }
    e = cudaMemcpyAsync(hg, h->b.grad, n * 4 * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { free(hg); return adj_fail(NP_ERR_KERNEL, "%s", cudaGetErrorString(e)); }
    double acc[4] = {0, 0, 0, 0};
    for (size_t i = 0; i < n; ++i)
        for (int k = 0; k < 4; ++k) acc[k] += hg[4 * i + k];
    free(hg);
    for (int k = 0; k < 4; ++k) h_grad4[k] = acc[k];
    if (stats) {
        float ms = 0; cudaEventElapsedTime(&ms, e0, e1);
        stats->backward_ms = ms;
        cudaEventDestroy(e0); cudaEventDestroy(e1);
    }
    return NP_OK;
}

}  // extern "C"
