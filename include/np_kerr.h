/*
 * np_kerr.h -- the reference's physics-header API (bh_common.h, bh_types.h,
 * bh_kerr.h, bh_schwarzschild.h of NullPath) for host C++ and CUDA device
 * code, implemented anew.
 *
 * Code written against those headers compiles against this one unchanged:
 * same type names and members (GeodesicState, GeodesicStateD, RayStatus,
 * SchwarzschildMetric, BhKleinSum), same function names, argument order,
 * return conventions and numerical floors.  Every function is
 * __host__ __device__ under nvcc (the reference marks some device-only) and
 * plain inline under a host compiler.
 *
 *   constants, helpers, compensated sum ... bh_common.h:50-253, 371-493
 *   RayStatus ............................. bh_common.h:295-331
 *   SchwarzschildMetric, GeodesicState .... bh_types.h:52-150, 163-251
 *   Kerr metric blocks (FP32 / FP64) ...... bh_kerr.h:81-250 / 575-672
 *   Hamiltonian, Hamilton's equations ..... bh_kerr.h:252-345 / 679-727
 *   fixed RK4 ............................. bh_kerr.h:358-398 / 734-774
 *   camera tetrads ........................ bh_kerr.h:431-479 / 781-826, 880-967
 *   Doppler factor of the disk ............ bh_kerr.h:506-535 / 833-862
 *   RK4 step and step doubling (FP64) ..... bh_kerr.h:987-1105
 *   Schwarzschild equations and RK4 ....... bh_schwarzschild.h:68-295
 *
 * Units: G = c = 1; M the mass, a = J/M (|a| < M), Boyer-Lindquist
 * (t, r, theta, phi) with covariant momenta (p_t, p_r, p_theta, p_phi).
 * The hot paths of the renderer (nullpath_gb300/csrc) use their own
 * Carter-form kernels; this header is the per-ray building-block API.
 */
#ifndef NP_KERR_H
#define NP_KERR_H

#include <cmath>

#if defined(__CUDACC__)
#define NP_HD __host__ __device__
#else
#define NP_HD
#endif

/* ---- constants (bh_common.h:50-253) ----------------------------------- */
constexpr float BH_PI = 3.14159265358979323846f;
constexpr double BH_PI_D = 3.141592653589793238462643383279502884;
constexpr float BH_EPS = 1e-6f;
constexpr double BH_EPS_D = 1e-12;
constexpr float BH_EPS_SIN = 1e-6f;
constexpr double BH_EPS_SIN_D = 1e-12;
constexpr float BH_SCHWARZSCHILD_MULTIPLIER = 2.0f;
constexpr float BH_PHOTON_SPHERE_MULTIPLIER = 1.5f;
constexpr int BH_MAX_INTEGRATION_STEPS_DEFAULT = 10000;
constexpr float BH_INTEGRATION_STEP_DEFAULT = 0.01f;
constexpr double BH_RK_REL_TOL = 1e-10;
constexpr double BH_RK_ABS_TOL = 1e-12;
constexpr double BH_RK_SAFETY = 0.9;
constexpr double BH_RK_HMIN = 1e-6;
constexpr double BH_RK_HMAX = 0.2;

/* Outcome of a traced ray (bh_common.h:295-331). */
enum class RayStatus : int { Escaped = 0, Captured = 1, PhotonSphere = 2, Inconclusive = 3 };

namespace np_kerr_detail {
NP_HD inline float sqrt_(float x) { return sqrtf(x); }
NP_HD inline double sqrt_(double x) { return sqrt(x); }
NP_HD inline float rsqrt_(float x) {
#if defined(__CUDA_ARCH__)
    return rsqrtf(x);
#else
    return 1.0f / sqrtf(x);
#endif
}
NP_HD inline double rsqrt_(double x) {
#if defined(__CUDA_ARCH__)
    return rsqrt(x);
#else
    return 1.0 / sqrt(x);
#endif
}
NP_HD inline float sin_(float x) { return sinf(x); }
NP_HD inline double sin_(double x) { return sin(x); }
NP_HD inline float cos_(float x) { return cosf(x); }
NP_HD inline double cos_(double x) { return cos(x); }
NP_HD inline float max_(float x, float y) { return fmaxf(x, y); }
NP_HD inline double max_(double x, double y) { return fmax(x, y); }
NP_HD inline float abs_(float x) { return fabsf(x); }
NP_HD inline double abs_(double x) { return fabs(x); }
}  // namespace np_kerr_detail

/* ---- small helpers (bh_common.h:127-190, 371-445) ---------------------- */
NP_HD inline float bh_r_s(float M) { return BH_SCHWARZSCHILD_MULTIPLIER * M; }
NP_HD inline float bh_r_ph(float Rs) { return BH_PHOTON_SPHERE_MULTIPLIER * Rs; }
/* b_crit = 3 sqrt(3) M = (3 sqrt(3) / 2) Rs for Schwarzschild. */
NP_HD inline float bh_bcrit_from_M(float M) { return 3.0f * sqrtf(3.0f) * M; }
NP_HD inline float bh_bcrit_from_Rs(float Rs) { return 0.5f * 3.0f * sqrtf(3.0f) * Rs; }
NP_HD inline float bh_to_M_units(float x, float M) { return x / fmaxf(M, BH_EPS); }
NP_HD inline float bh_to_Rs_units(float x, float Rs) { return x / fmaxf(Rs, BH_EPS); }
NP_HD inline float bh_abs(float x) { return fabsf(x); }
NP_HD inline double bh_abs(double x) { return fabs(x); }
NP_HD inline float bh_clamp(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
NP_HD inline float bh_clamp01(float x) { return bh_clamp(x, 0.0f, 1.0f); }
NP_HD inline float bh_safe_sin2(float theta) {
    float s = sinf(theta);
    return fmaxf(BH_EPS_SIN, s * s);
}
NP_HD inline float bh_safe_div(float num, float den, float eps = BH_EPS) {
    float d = fabsf(den) < eps ? copysignf(eps, den) : den;
    return num / d;
}

/* Second-order compensated (Kahan-Babuska-Klein) summation: the running sum,
 * its first-order error and the error of that error are carried separately
 * (A. Klein, "A generalized Kahan-Babuska-summation-algorithm", Computing 76,
 * 2006), bh_common.h:451-484. */
template <typename Real>
struct BhKleinSum {
    Real sum, cs, ccs;
    NP_HD BhKleinSum() : sum(Real(0)), cs(Real(0)), ccs(Real(0)) {}
    NP_HD void add(Real x) {
        using np_kerr_detail::abs_;
        Real t = sum + x;
        Real lost = abs_(sum) >= abs_(x) ? (sum - t) + x : (x - t) + sum;
        sum = t;
        Real t2 = cs + lost;
        Real lost2 = abs_(cs) >= abs_(lost) ? (cs - t2) + lost : (lost - t2) + cs;
        cs = t2;
        ccs = ccs + lost2;
    }
    NP_HD Real result() const { return sum + cs + ccs; }
};

/* k1 + 2 k2 + 2 k3 + k4 with the compensated sum (bh_common.h:485-493). */
template <typename Real>
NP_HD inline Real bh_rk4_sum(Real k1, Real k2, Real k3, Real k4) {
    BhKleinSum<Real> s;
    s.add(k1);
    s.add(Real(2) * k2);
    s.add(Real(2) * k3);
    s.add(k4);
    return s.result();
}

/* ---- states (bh_types.h:163-251, bh_kerr.h:553-556) -------------------- */
struct GeodesicState {
    float t, r, theta, phi;          /* Boyer-Lindquist position */
    float pt, pr, ptheta, pphi;      /* covariant momentum */
    NP_HD GeodesicState() : t(0), r(0), theta(0), phi(0), pt(0), pr(0), ptheta(0), pphi(0) {}
};

struct GeodesicStateD {
    double t, r, theta, phi;
    double pt, pr, ptheta, pphi;
};

/* Schwarzschild metric of mass m (bh_types.h:52-150). */
struct SchwarzschildMetric {
    float mass;
    float Rs;
    NP_HD explicit SchwarzschildMetric(float m) : mass(m), Rs(BH_SCHWARZSCHILD_MULTIPLIER * m) {}
    NP_HD float g_tt(float r) const { return -(1.0f - Rs / r); }
    NP_HD float g_rr(float r) const { return 1.0f / fmaxf(BH_EPS, 1.0f - Rs / r); }
    NP_HD float g_theta_theta(float r) const { return r * r; }
    NP_HD float g_phi_phi(float r, float theta) const {
        float s = sinf(theta);
        return r * r * s * s;
    }
};

namespace np_kerr_detail {

/* Sigma, Delta, A and the trigonometry of one point. */
template <typename R>
struct KerrPoint {
    R s, c, r2, a2, Sig, Del, B;
    NP_HD KerrPoint(R M, R a, R r, R th) {
        s = sin_(th);
        c = cos_(th);
        r2 = r * r;
        a2 = a * a;
        Sig = r2 + a2 * c * c;
        Del = r2 - R(2) * M * r + a2;
        B = r2 + a2;
    }
};

template <typename R>
NP_HD inline void cov_blocks(R M, R a, R r, R th, R eps, bool floor_sigma, R& g_tt, R& g_tphi, R& g_phiphi,
                             R& g_rr, R& g_thth) {
    KerrPoint<R> p(M, a, r, th);
    const R s2 = p.s * p.s;
    const R A = p.B * p.B - p.a2 * p.Del * s2;
    const R Sd = floor_sigma ? max_(eps, p.Sig) : p.Sig;
    g_tt = -(R(1) - R(2) * M * r / Sd);
    g_tphi = -R(2) * M * a * r * s2 / Sd;
    g_phiphi = A * s2 / Sd;
    g_rr = p.Sig / max_(eps, p.Del);
    g_thth = p.Sig;
}

/* Analytic r- and theta-derivatives of the five inverse-metric blocks,
 * written as quotients N/D with D = Sigma Delta (g^tt, g^tphi),
 * D = Sigma (g^rr, g^thth) and D = Delta Sigma sin^2 (g^phiphi). */
template <typename R>
NP_HD inline void contra_derivs(R M, R a, R r, R th, R s2, bool add_floor, R* d_r, R* d_th) {
    KerrPoint<R> p(M, a, r, th);
    const R A = p.B * p.B - p.a2 * p.Del * s2;
    const R ds2 = R(2) * p.s * p.c;
    const R Sig_r = R(2) * r, Sig_t = -R(2) * p.a2 * p.s * p.c;
    const R Del_r = R(2) * (r - M);
    const R A_r = R(4) * r * p.B - p.a2 * Del_r * s2;
    const R A_t = -p.a2 * p.Del * ds2;
    const R D = p.Sig * p.Del;
    const R D_r = Sig_r * p.Del + p.Sig * Del_r;
    const R D_t = Sig_t * p.Del;
    // denominators squared with the floors of the FP64 (additive) and FP32
    // (clamped) forms
    const R D2 = add_floor ? D * D + R(1e-48) : max_(R(1e-24), D * D);
    const R Nt = R(2) * M * a * r, Nt_r = R(2) * M * a;
    const R S2 = p.Sig * p.Sig;
    const R N = p.Del - p.a2 * s2;
    const R N_t = -p.a2 * ds2;
    const R Q = add_floor ? p.Del * p.Sig * s2 + R(1e-48) : p.Del * p.Sig * s2;
    const R Q_r = Del_r * p.Sig * s2 + p.Del * Sig_r * s2;
    const R Q_t = p.Del * Sig_t * s2 + p.Del * p.Sig * ds2;
    const R Q2 = add_floor ? Q * Q + R(1e-48) : max_(R(1e-24), Q * Q);
    d_r[0] = -(A_r * D - A * D_r) / D2;
    d_th[0] = -(A_t * D - A * D_t) / D2;
    d_r[1] = -(Nt_r * D - Nt * D_r) / D2;
    d_th[1] = Nt * D_t / D2;
    d_r[2] = (Del_r * Q - N * Q_r) / Q2;
    d_th[2] = (N_t * Q - N * Q_t) / Q2;
    d_r[3] = (Del_r * p.Sig - p.Del * Sig_r) / S2;
    d_th[3] = -(p.Del * Sig_t) / S2;
    d_r[4] = -Sig_r / S2;
    d_th[4] = -Sig_t / S2;
}

/* Hamilton's equations x' = g^{mu nu} p_nu, p' = -1/2 d g^{ab} p_a p_b,
 * the two force sums compensated. */
template <typename R, typename S>
NP_HD inline void hamilton(const S& st, const R g[5], const R d_r[5], const R d_th[5], S& d) {
    d.t = g[0] * st.pt + g[1] * st.pphi;
    d.r = g[3] * st.pr;
    d.theta = g[4] * st.ptheta;
    d.phi = g[1] * st.pt + g[2] * st.pphi;
    d.pt = R(0);
    d.pphi = R(0);
    BhKleinSum<R> fr, ft;
    fr.add(d_r[0] * st.pt * st.pt);
    fr.add(R(2) * d_r[1] * st.pt * st.pphi);
    fr.add(d_r[2] * st.pphi * st.pphi);
    fr.add(d_r[3] * st.pr * st.pr);
    fr.add(d_r[4] * st.ptheta * st.ptheta);
    ft.add(d_th[0] * st.pt * st.pt);
    ft.add(R(2) * d_th[1] * st.pt * st.pphi);
    ft.add(d_th[2] * st.pphi * st.pphi);
    ft.add(d_th[3] * st.pr * st.pr);
    ft.add(d_th[4] * st.ptheta * st.ptheta);
    d.pr = R(-0.5) * fr.result();
    d.ptheta = R(-0.5) * ft.result();
}

template <typename S, typename R>
NP_HD inline S stage(const S& y, R h, const S& k) {
    S o = y;
    o.t = y.t + h * k.t; o.r = y.r + h * k.r; o.theta = y.theta + h * k.theta; o.phi = y.phi + h * k.phi;
    o.pt = y.pt + h * k.pt; o.pr = y.pr + h * k.pr; o.ptheta = y.ptheta + h * k.ptheta; o.pphi = y.pphi + h * k.pphi;
    return o;
}

template <typename S, typename R>
NP_HD inline void rk4_combine(S& y, R h, const S& k1, const S& k2, const S& k3, const S& k4) {
    const R h6 = h / R(6);
    y.t += h6 * bh_rk4_sum(k1.t, k2.t, k3.t, k4.t);
    y.r += h6 * bh_rk4_sum(k1.r, k2.r, k3.r, k4.r);
    y.theta += h6 * bh_rk4_sum(k1.theta, k2.theta, k3.theta, k4.theta);
    y.phi += h6 * bh_rk4_sum(k1.phi, k2.phi, k3.phi, k4.phi);
    y.pt += h6 * bh_rk4_sum(k1.pt, k2.pt, k3.pt, k4.pt);
    y.pr += h6 * bh_rk4_sum(k1.pr, k2.pr, k3.pr, k4.pr);
    y.ptheta += h6 * bh_rk4_sum(k1.ptheta, k2.ptheta, k3.ptheta, k4.ptheta);
    y.pphi += h6 * bh_rk4_sum(k1.pphi, k2.pphi, k3.pphi, k4.pphi);
}

template <typename R>
NP_HD inline R horizon(R M, R a) {
    R d = M * M - a * a;
    if (d < R(0)) d = R(0);
    return M + sqrt_(d);
}

/* Static-observer tetrad: e_t along the Killing time, e_r, e_theta unit,
 * e_phi the unit vector in the (t, phi) plane orthogonal to e_t; the photon
 * direction (n_r, n_theta, n_phi) has local energy 1. */
template <typename R, typename S>
NP_HD inline S static_camera(R M, R a, R r_cam, R th, R ph, R nr, R nth, R nph, R eps, R tphi_eps, bool norm_floor_add) {
    S s{};
    s.t = R(0); s.r = r_cam; s.theta = th; s.phi = ph;
    R g_tt, g_tphi, g_phiphi, g_rr, g_thth;
    cov_blocks<R>(M, a, r_cam, th, eps, sizeof(R) == 8, g_tt, g_tphi, g_phiphi, g_rr, g_thth);
    const R ut = rsqrt_(max_(eps, -g_tt));
    const R er = rsqrt_(max_(eps, g_rr));
    const R eh = rsqrt_(max_(eps, g_thth));
    R ept, epp;
    if (abs_(g_tphi) > tphi_eps) {
        const R beta = -g_tt / g_tphi;
        BhKleinSum<R> n2;
        n2.add(g_tt);
        n2.add(R(2) * g_tphi * beta);
        n2.add(g_phiphi * beta * beta);
        const R inv = norm_floor_add ? rsqrt_(abs_(n2.result()) + R(1e-12)) : rsqrt_(max_(eps, abs_(n2.result())));
        ept = inv;
        epp = beta * inv;
    } else {
        ept = R(0);
        epp = rsqrt_(max_(eps, g_phiphi));
    }
    const R Pt = ut + nph * ept, Pr = nr * er, Ph = nth * eh, Pp = nph * epp;
    s.pt = g_tt * Pt + g_tphi * Pp;
    s.pr = g_rr * Pr;
    s.ptheta = g_thth * Ph;
    s.pphi = g_tphi * Pt + g_phiphi * Pp;
    return s;
}

}  // namespace np_kerr_detail

/* ---- Kerr metric blocks ------------------------------------------------ */
/* Covariant g_tt, g_tphi, g_phiphi, g_rr, g_thth (bh_kerr.h:81-98). */
NP_HD inline void kerr_blocks_cov(float M, float a, float r, float th, float& g_tt, float& g_tphi,
                                  float& g_phiphi, float& g_rr, float& g_thth) {
    np_kerr_detail::cov_blocks<float>(M, a, r, th, BH_EPS, false, g_tt, g_tphi, g_phiphi, g_rr, g_thth);
}
/* FP64, Sigma floored at BH_EPS_D (bh_kerr.h:575-592). */
NP_HD inline void kerr_blocks_cov_d(double M, double a, double r, double th, double& g_tt, double& g_tphi,
                                    double& g_phiphi, double& g_rr, double& g_thth) {
    np_kerr_detail::cov_blocks<double>(M, a, r, th, BH_EPS_D, true, g_tt, g_tphi, g_phiphi, g_rr, g_thth);
}

/* Contravariant blocks with the horizon and pole floors (bh_kerr.h:125-142). */
NP_HD inline void kerr_blocks_contra(float M, float a, float r, float th, float& gtt, float& gtphi,
                                     float& gphiphi, float& grr, float& gthth) {
    np_kerr_detail::KerrPoint<float> p(M, a, r, th);
    const float s2 = p.s * p.s;
    const float A = p.B * p.B - p.a2 * p.Del * s2;
    const float Sf = fmaxf(BH_EPS, p.Sig);
    const float SD = fmaxf(BH_EPS, p.Sig * p.Del);
    grr = fmaxf(BH_EPS, p.Del) / Sf;
    gthth = 1.0f / Sf;
    gtt = -A / SD;
    gtphi = -2.0f * M * a * r / SD;
    gphiphi = (p.Del - p.a2 * s2) / fmaxf(BH_EPS, p.Sig * p.Del * s2 + BH_EPS);
}
/* FP64 (bh_kerr.h:600-617). */
NP_HD inline void kerr_blocks_contra_d(double M, double a, double r, double th, double& gtt, double& gtphi,
                                       double& gphiphi, double& grr, double& gthth) {
    np_kerr_detail::KerrPoint<double> p(M, a, r, th);
    const double s2 = fmax(BH_EPS_SIN_D, p.s * p.s);
    const double Sf = fmax(BH_EPS_D, p.Sig);
    const double A = p.B * p.B - p.a2 * p.Del * s2;
    grr = fmax(BH_EPS_D, p.Del) / Sf;
    gthth = 1.0 / Sf;
    gtt = -A / fmax(BH_EPS_D, Sf * p.Del);
    gtphi = -2.0 * M * a * r / fmax(BH_EPS_D, Sf * p.Del);
    gphiphi = (p.Del - p.a2 * s2) / fmax(BH_EPS_D, Sf * p.Del * s2);
}

/* d/dr and d/dtheta of the contravariant blocks (bh_kerr.h:176-230). */
NP_HD inline void kerr_blocks_contra_derivs(float M, float a, float r, float th, float& gtt_r, float& gtphi_r,
                                            float& gphiphi_r, float& grr_r, float& gthth_r, float& gtt_th,
                                            float& gtphi_th, float& gphiphi_th, float& grr_th, float& gthth_th) {
    float dr[5], dt[5];
    const float s = sinf(th);
    np_kerr_detail::contra_derivs<float>(M, a, r, th, fmaxf(BH_EPS_SIN, s * s), false, dr, dt);
    gtt_r = dr[0]; gtphi_r = dr[1]; gphiphi_r = dr[2]; grr_r = dr[3]; gthth_r = dr[4];
    gtt_th = dt[0]; gtphi_th = dt[1]; gphiphi_th = dt[2]; grr_th = dt[3]; gthth_th = dt[4];
}
/* FP64 (bh_kerr.h:624-672). */
NP_HD inline void kerr_blocks_contra_derivs_d(double M, double a, double r, double th, double& gtt_r,
                                              double& gtphi_r, double& gphiphi_r, double& grr_r, double& gthth_r,
                                              double& gtt_th, double& gtphi_th, double& gphiphi_th, double& grr_th,
                                              double& gthth_th) {
    double dr[5], dt[5];
    const double s = sin(th);
    np_kerr_detail::contra_derivs<double>(M, a, r, th, (s * s > 1e-30 ? s * s : 1e-30), true, dr, dt);
    gtt_r = dr[0]; gtphi_r = dr[1]; gphiphi_r = dr[2]; grr_r = dr[3]; gthth_r = dr[4];
    gtt_th = dt[0]; gtphi_th = dt[1]; gphiphi_th = dt[2]; grr_th = dt[3]; gthth_th = dt[4];
}

/* H = 1/2 g^{mu nu} p_mu p_nu, compensated (bh_kerr.h:252-264). */
NP_HD inline float hamiltonian_kerr(const GeodesicState& s, float M, float a) {
    float g[5];
    kerr_blocks_contra(M, a, s.r, s.theta, g[0], g[1], g[2], g[3], g[4]);
    BhKleinSum<float> h;
    h.add(g[0] * s.pt * s.pt);
    h.add(2.0f * g[1] * s.pt * s.pphi);
    h.add(g[2] * s.pphi * s.pphi);
    h.add(g[3] * s.pr * s.pr);
    h.add(g[4] * s.ptheta * s.ptheta);
    return 0.5f * h.result();
}

/* Hamilton's equations; zero inside r_+ + 1e-3 (bh_kerr.h:294-345). */
NP_HD inline void computeGeodesicDerivativesKerr(const GeodesicState& st, float M, float a, GeodesicState& d) {
    const float rp = M + sqrtf(fmaxf(0.0f, M * M - a * a));
    if (st.r <= rp + 1e-3f || st.r <= 1e-6f) { d = GeodesicState(); return; }
    float g[5], dr[5], dt[5];
    kerr_blocks_contra(M, a, st.r, st.theta, g[0], g[1], g[2], g[3], g[4]);
    kerr_blocks_contra_derivs(M, a, st.r, st.theta, dr[0], dr[1], dr[2], dr[3], dr[4], dt[0], dt[1], dt[2], dt[3],
                              dt[4]);
    np_kerr_detail::hamilton<float>(st, g, dr, dt, d);
}
/* FP64; zero inside r_+ + 1e-12 (bh_kerr.h:679-727). */
NP_HD inline void computeGeodesicDerivativesKerrD(const GeodesicStateD& st, double M, double a, GeodesicStateD& d) {
    const double rp = np_kerr_detail::horizon(M, a);
    if (st.r <= rp + 1e-12 || st.r <= 1e-12) { d = GeodesicStateD{}; return; }
    double g[5], dr[5], dt[5];
    kerr_blocks_contra_d(M, a, st.r, st.theta, g[0], g[1], g[2], g[3], g[4]);
    kerr_blocks_contra_derivs_d(M, a, st.r, st.theta, dr[0], dr[1], dr[2], dr[3], dr[4], dt[0], dt[1], dt[2], dt[3],
                                dt[4]);
    np_kerr_detail::hamilton<double>(st, g, dr, dt, d);
}

/* One RK4 step in place; true while outside r_+ + 1e-3 and off the poles by
 * 1e-3 (bh_kerr.h:358-398). */
NP_HD inline bool integrateGeodesicKerr(GeodesicState& st, float M, float a, float h) {
    using np_kerr_detail::stage;
    GeodesicState k1, k2, k3, k4;
    computeGeodesicDerivativesKerr(st, M, a, k1);
    computeGeodesicDerivativesKerr(stage(st, 0.5f * h, k1), M, a, k2);
    computeGeodesicDerivativesKerr(stage(st, 0.5f * h, k2), M, a, k3);
    computeGeodesicDerivativesKerr(stage(st, h, k3), M, a, k4);
    np_kerr_detail::rk4_combine(st, h, k1, k2, k3, k4);
    const float rp = M + sqrtf(fmaxf(0.0f, M * M - a * a));
    return st.r > rp + 1e-3f && st.theta > 1e-3f && st.theta < BH_PI - 1e-3f;
}
/* FP64 (bh_kerr.h:734-774): margins 1e-9. */
NP_HD inline bool integrateGeodesicKerrD(GeodesicStateD& st, double M, double a, double h) {
    using np_kerr_detail::stage;
    GeodesicStateD k1, k2, k3, k4;
    computeGeodesicDerivativesKerrD(st, M, a, k1);
    computeGeodesicDerivativesKerrD(stage(st, 0.5 * h, k1), M, a, k2);
    computeGeodesicDerivativesKerrD(stage(st, 0.5 * h, k2), M, a, k3);
    computeGeodesicDerivativesKerrD(stage(st, h, k3), M, a, k4);
    np_kerr_detail::rk4_combine(st, h, k1, k2, k3, k4);
    const double rp = np_kerr_detail::horizon(M, a);
    return st.r > rp + 1e-9 && st.theta > 1e-9 && st.theta < BH_PI_D - 1e-9;
}

/* Camera ray of a static observer at (r_cam, theta_cam, phi_cam) with local
 * direction (n_r, n_theta, n_phi) (bh_kerr.h:431-479, 781-826). */
NP_HD inline GeodesicState init_ray_from_camera_general(float M, float a, float r_cam, float theta_cam,
                                                        float phi_cam, float n_r, float n_theta, float n_phi) {
    return np_kerr_detail::static_camera<float, GeodesicState>(M, a, r_cam, theta_cam, phi_cam, n_r, n_theta, n_phi,
                                                               BH_EPS, 1e-12f, true);
}
NP_HD inline GeodesicStateD init_ray_from_camera_general_d(double M, double a, double r_cam, double theta_cam,
                                                           double phi_cam, double n_r, double n_theta, double n_phi) {
    return np_kerr_detail::static_camera<double, GeodesicStateD>(M, a, r_cam, theta_cam, phi_cam, n_r, n_theta, n_phi,
                                                                 BH_EPS_D, BH_EPS_D, false);
}

/* A static observer exists where g_tt < 0, outside the ergosphere
 * (bh_kerr.h:880-884). */
NP_HD inline bool kerr_static_timelike(double M, double a, double r, double th) {
    double g_tt, g_tphi, g_phiphi, g_rr, g_thth;
    kerr_blocks_cov_d(M, a, r, th, g_tt, g_tphi, g_phiphi, g_rr, g_thth);
    return g_tt < 0.0;
}

/* Camera ray of the zero-angular-momentum observer: lapse alpha and frame
 * rotation omega (bh_kerr.h:910-967). */
NP_HD inline GeodesicStateD init_ray_from_camera_zamo_d(double M, double a, double r_cam, double theta_cam,
                                                        double phi_cam, double n_r, double n_theta, double n_phi) {
    GeodesicStateD s{};
    s.t = 0.0; s.r = r_cam; s.theta = theta_cam; s.phi = phi_cam;
    const double c = cos(theta_cam), sn = sin(theta_cam);
    const double r2 = r_cam * r_cam, a2 = a * a;
    const double Sig = fmax(BH_EPS_D, r2 + a2 * c * c);
    const double Del = r2 - 2.0 * M * r_cam + a2;
    const double A = fmax(BH_EPS_D, (r2 + a2) * (r2 + a2) - a2 * Del * sn * sn);
    const double alpha = sqrt(fmax(BH_EPS_D, Del * Sig / A));
    const double omega = 2.0 * M * a * r_cam / A;
    const double Pt = 1.0 / fmax(BH_EPS_D, alpha);
    const double Pp = omega / fmax(BH_EPS_D, alpha) + n_phi * (sqrt(fmax(BH_EPS_D, Sig / A)) / fmax(BH_EPS_D, fabs(sn)));
    const double Pr = n_r * sqrt(fmax(BH_EPS_D, Del / Sig));
    const double Ph = n_theta * (1.0 / sqrt(Sig));
    double g_tt, g_tphi, g_phiphi, g_rr, g_thth;
    kerr_blocks_cov_d(M, a, r_cam, theta_cam, g_tt, g_tphi, g_phiphi, g_rr, g_thth);
    s.pt = g_tt * Pt + g_tphi * Pp;
    s.pr = g_rr * Pr;
    s.ptheta = g_thth * Ph;
    s.pphi = g_tphi * Pt + g_phiphi * Pp;
    return s;
}

/* Redshift g = E_inf / (-k.u) of a prograde Keplerian emitter
 * Omega = 1 / (a + r^{3/2}) on the equator (bh_kerr.h:506-535). */
NP_HD inline float doppler_g_general(const GeodesicState& st, float M, float a) {
    float g_tt, g_tphi, g_phiphi, g_rr, g_thth;
    kerr_blocks_cov(M, a, st.r, BH_PI * 0.5f, g_tt, g_tphi, g_phiphi, g_rr, g_thth);
    const float Ms = fmaxf(BH_EPS, M);
    const float Om = 1.0f / (a / Ms + powf(fmaxf(1.0f, st.r / Ms), 1.5f)) / Ms;
    BhKleinSum<float> den;
    den.add(g_tt);
    den.add(2.0f * g_tphi * Om);
    den.add(g_phiphi * Om * Om);
    const float ut = np_kerr_detail::rsqrt_(fmaxf(BH_EPS, -den.result()));
    BhKleinSum<float> ku;
    ku.add(st.pt * ut);
    ku.add(st.pphi * (Om * ut));
    const float g = -st.pt / fmaxf(1e-9f, -ku.result());
    return fmaxf(0.0f, g);
}
/* FP64 (bh_kerr.h:833-862). */
NP_HD inline double doppler_g_general_d(const GeodesicStateD& st, double M, double a) {
    double g_tt, g_tphi, g_phiphi, g_rr, g_thth;
    kerr_blocks_cov_d(M, a, st.r, BH_PI_D * 0.5, g_tt, g_tphi, g_phiphi, g_rr, g_thth);
    const double Ms = fmax(BH_EPS_D, M);
    const double Om = 1.0 / (a / Ms + pow(fmax(1.0, st.r / Ms), 1.5)) / Ms;
    BhKleinSum<double> den;
    den.add(g_tt);
    den.add(2.0 * g_tphi * Om);
    den.add(g_phiphi * Om * Om);
    const double dn = -den.result();
    const double ut = np_kerr_detail::rsqrt_(dn > 1e-24 ? dn : 1e-24);
    BhKleinSum<double> ku;
    ku.add(st.pt * ut);
    ku.add(st.pphi * (Om * ut));
    const double k = -ku.result();
    const double g = -st.pt / (k > 1e-18 ? k : 1e-18);
    return g > 0.0 ? g : 0.0;
}

/* One FP64 RK4 step s -> s_out; true while outside r_+ + 1e-12 and off the
 * poles by 1e-9 (bh_kerr.h:987-1032). */
NP_HD inline bool rk4_step_d(const GeodesicStateD& s, double M, double a, double h, GeodesicStateD& s_out) {
    using np_kerr_detail::stage;
    GeodesicStateD k1, k2, k3, k4;
    computeGeodesicDerivativesKerrD(s, M, a, k1);
    computeGeodesicDerivativesKerrD(stage(s, 0.5 * h, k1), M, a, k2);
    computeGeodesicDerivativesKerrD(stage(s, 0.5 * h, k2), M, a, k3);
    computeGeodesicDerivativesKerrD(stage(s, h, k3), M, a, k4);
    s_out = s;
    np_kerr_detail::rk4_combine(s_out, h, k1, k2, k3, k4);
    const double rp = np_kerr_detail::horizon(M, a);
    return s_out.r > rp + 1e-12 && s_out.theta > 1e-9 && s_out.theta < BH_PI_D - 1e-9;
}

/* Step doubling (bh_kerr.h:1058-1105): one step of h against two of h/2; the
 * error is the largest |full - half| / (abs_tol + rel_tol max(|full|, |half|))
 * over r, theta, phi, p_r, p_theta, p_phi.  On acceptance (error <= 1) s takes
 * the two half steps and the growth factor min(2, 0.9 e^-0.2) is returned;
 * otherwise s is unchanged, h shrinks by max(0.1, 0.9 e^-0.25) and 0 is
 * returned.  A step that leaves the domain halves h and returns 0. */
NP_HD inline double rk4_adaptive_step_d(GeodesicStateD& s, double M, double a, double& h,
                                        double rel_tol = BH_RK_REL_TOL, double abs_tol = BH_RK_ABS_TOL) {
    GeodesicStateD full, half1, half2;
    const bool ok = rk4_step_d(s, M, a, h, full) & rk4_step_d(s, M, a, 0.5 * h, half1);
    if (!(ok && rk4_step_d(half1, M, a, 0.5 * h, half2))) {
        h *= 0.5;
        return 0.0;
    }
    const double f[6] = {full.r, full.theta, full.phi, full.pr, full.ptheta, full.pphi};
    const double g[6] = {half2.r, half2.theta, half2.phi, half2.pr, half2.ptheta, half2.pphi};
    double e = 0.0;
    for (int i = 0; i < 6; ++i) {
        const double sc = abs_tol + rel_tol * fmax(fabs(f[i]), fabs(g[i]));
        e = fmax(e, fabs(f[i] - g[i]) / fmax(sc, 1e-30));
    }
    if (e <= 1.0) {
        s = half2;
        return fmin(2.0, BH_RK_SAFETY * pow(fmax(1e-12, e), -0.2));
    }
    h *= fmax(0.1, BH_RK_SAFETY * pow(fmax(1e-12, e), -0.25));
    return 0.0;
}

/* ---- Schwarzschild (bh_schwarzschild.h:68-295) ------------------------- */
/* H with g^tt = -1/A, g^rr = A, A = max(eps, 1 - Rs/r). */
NP_HD inline float hamiltonian_schwarzschild(const GeodesicState& s, float Rs) {
    const float A = fmaxf(BH_EPS, 1.0f - Rs / s.r);
    const float sn = sinf(s.theta);
    const float st2 = fmaxf(BH_EPS_SIN, sn * sn);
    const float r2 = s.r * s.r;
    return 0.5f * ((-1.0f / A) * s.pt * s.pt + A * s.pr * s.pr + (1.0f / r2) * s.ptheta * s.ptheta +
                   (1.0f / (r2 * st2)) * s.pphi * s.pphi);
}

/* Hamilton's equations of the Schwarzschild metric; zero inside Rs + 1e-3. */
NP_HD inline void computeGeodesicDerivatives(const GeodesicState& state, const SchwarzschildMetric& metric,
                                             GeodesicState& d) {
    const float r = state.r, Rs = metric.Rs;
    if (r <= Rs + 0.001f || r <= 0.001f) { d = GeodesicState(); return; }
    const float sn = sinf(state.theta), cs = cosf(state.theta);
    const float r2 = r * r, r3 = r2 * r;
    const float A = fmaxf(BH_EPS, 1.0f - Rs / r);
    const float s2 = fmaxf(BH_EPS_SIN, sn * sn);
    d.t = (-1.0f / A) * state.pt;
    d.r = A * state.pr;
    d.theta = state.ptheta / r2;
    d.phi = state.pphi / (r2 * s2);
    d.pt = 0.0f;
    d.pr = -0.5f * ((Rs / (r2 * A * A)) * state.pt * state.pt + (Rs / r2) * state.pr * state.pr +
                    (-2.0f / r3) * state.ptheta * state.ptheta + (-2.0f / (r3 * s2)) * state.pphi * state.pphi);
    const float sn_safe = fabsf(sn) < 1e-6f ? (sn >= 0.0f ? 1e-6f : -1e-6f) : sn;
    d.ptheta = (cs / (r2 * s2 * sn_safe)) * state.pphi * state.pphi;
    d.pphi = 0.0f;
}

/* One RK4 step (plain stage sum); true while outside Rs + 1e-3 and off the
 * poles by 1e-3. */
NP_HD inline bool integrateGeodesic(GeodesicState& state, const SchwarzschildMetric& metric, float h) {
    using np_kerr_detail::stage;
    GeodesicState k1, k2, k3, k4;
    computeGeodesicDerivatives(state, metric, k1);
    computeGeodesicDerivatives(stage(state, 0.5f * h, k1), metric, k2);
    computeGeodesicDerivatives(stage(state, 0.5f * h, k2), metric, k3);
    computeGeodesicDerivatives(stage(state, h, k3), metric, k4);
    const float h6 = h / 6.0f;
    state.t += h6 * (k1.t + 2.0f * k2.t + 2.0f * k3.t + k4.t);
    state.r += h6 * (k1.r + 2.0f * k2.r + 2.0f * k3.r + k4.r);
    state.theta += h6 * (k1.theta + 2.0f * k2.theta + 2.0f * k3.theta + k4.theta);
    state.phi += h6 * (k1.phi + 2.0f * k2.phi + 2.0f * k3.phi + k4.phi);
    state.pt += h6 * (k1.pt + 2.0f * k2.pt + 2.0f * k3.pt + k4.pt);
    state.pr += h6 * (k1.pr + 2.0f * k2.pr + 2.0f * k3.pr + k4.pr);
    state.ptheta += h6 * (k1.ptheta + 2.0f * k2.ptheta + 2.0f * k3.ptheta + k4.ptheta);
    state.pphi += h6 * (k1.pphi + 2.0f * k2.pphi + 2.0f * k3.pphi + k4.pphi);
    return state.r > metric.Rs + 0.001f && state.theta > 0.001f && state.theta < BH_PI - 0.001f;
}

/* Closest approach of an equatorial Schwarzschild photon with impact
 * parameter b (schwarzschild_blackhole.cu:24-37): the largest root of
 * r^3 - b^2 r + b^2 Rs = 0 in trigonometric form; false (no turning point
 * outside the horizon) for b <= b_crit = (3 sqrt(3)/2) Rs. */
NP_HD inline bool schwarzschild_rmin_analytic(float Rs, float b, float* rmin_out) {
    if (Rs <= 0.0f || b <= 0.0f || rmin_out == nullptr) return false;
    const double beta = (double)b / (double)Rs;
    const double beta_crit = 1.5 * sqrt(3.0);
    if (beta <= beta_crit) return false;
    double c = -beta_crit / beta;
    c = c < -1.0 ? -1.0 : (c > 1.0 ? 1.0 : c);
    const double x = (2.0 * beta / sqrt(3.0)) * cos(acos(c) / 3.0);
    *rmin_out = (float)(x * (double)Rs);
    const float rr = *rmin_out;
    return rr == rr && rr < 3.0e38f && rr > Rs;     // finite and outside the horizon
}

/* Deflection table of equatorial Schwarzschild photons (bh_types.h:281-300). */
struct GeodesicLookupTable {
    float* impact_parameters;
    float* deflection_angles;
    float* bending_angles;
    float* closest_approaches;
    int* ray_status;
    int num_entries;
    float mass;
};

#endif /* NP_KERR_H */
