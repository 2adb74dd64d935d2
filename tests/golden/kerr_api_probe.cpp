// Probe of the physics-header API: evaluates every function of the API on a
// fixed set of points, cameras and short integrations and prints one line per
// value ("name index value" with 17 significant digits).  Built two ways by
// the tests: against include/np_kerr.h (default), or with -DPROBE_REF against
// the reference's own headers, whose output is the committed golden file.
#include <cmath>
#include <cstdio>

#ifdef PROBE_REF
static inline double probe_rsqrt(double x) { return 1.0 / std::sqrt(x); }
static inline float probe_rsqrtf(float x) { return 1.0f / std::sqrt(x); }
#define rsqrt probe_rsqrt
#define rsqrtf probe_rsqrtf
#include "bh_common.h"
#include "bh_types.h"
#include "bh_kerr.h"
#include "bh_schwarzschild.h"
#else
#include "np_kerr.h"
#endif

static int g_idx = 0;
static void out(const char* name, double v) { std::printf("%s %d %.17g\n", name, g_idx, v); }
static void outs(const char* name, const GeodesicStateD& s) {
    out(name, s.t); out(name, s.r); out(name, s.theta); out(name, s.phi);
    out(name, s.pt); out(name, s.pr); out(name, s.ptheta); out(name, s.pphi);
}
static void outf(const char* name, const GeodesicState& s) {
    out(name, s.t); out(name, s.r); out(name, s.theta); out(name, s.phi);
    out(name, s.pt); out(name, s.pr); out(name, s.ptheta); out(name, s.pphi);
}

int main() {
    const double Ms[] = {1.0, 2.5};
    const double spins[] = {0.0, 0.5, 0.9, 0.998};
    const double rs[] = {3.0, 6.3, 20.0, 150.0};
    const double ths[] = {0.3, 1.2, 1.5707963267948966, 2.9};
    const double dirs[][3] = {{-0.95, 0.2, 0.24}, {-0.8, -0.45, 0.39}, {-0.99, 0.0, -0.14}, {0.3, 0.5, -0.81}};
    for (double M : Ms)
        for (double sp : spins)
            for (double rr : rs)
                for (double th : ths) {
                    ++g_idx;
                    const double a = sp * M, r = rr * M;
                    double v[10];
                    kerr_blocks_cov_d(M, a, r, th, v[0], v[1], v[2], v[3], v[4]);
                    for (int i = 0; i < 5; ++i) out("cov_d", v[i]);
                    kerr_blocks_contra_d(M, a, r, th, v[0], v[1], v[2], v[3], v[4]);
                    for (int i = 0; i < 5; ++i) out("contra_d", v[i]);
                    kerr_blocks_contra_derivs_d(M, a, r, th, v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8], v[9]);
                    for (int i = 0; i < 10; ++i) out("derivs_d", v[i]);
                    float f[10];
                    kerr_blocks_cov((float)M, (float)a, (float)r, (float)th, f[0], f[1], f[2], f[3], f[4]);
                    for (int i = 0; i < 5; ++i) out("cov_f", f[i]);
                    kerr_blocks_contra((float)M, (float)a, (float)r, (float)th, f[0], f[1], f[2], f[3], f[4]);
                    for (int i = 0; i < 5; ++i) out("contra_f", f[i]);
                    kerr_blocks_contra_derivs((float)M, (float)a, (float)r, (float)th, f[0], f[1], f[2], f[3], f[4],
                                              f[5], f[6], f[7], f[8], f[9]);
                    for (int i = 0; i < 10; ++i) out("derivs_f", f[i]);
                    out("static_timelike", kerr_static_timelike(M, a, r, th) ? 1.0 : 0.0);
                }
    // cameras, right-hand sides, integrations
    for (double sp : spins)
        for (const auto& d : dirs) {
            ++g_idx;
            const double M = 1.0, a = sp, r = 30.0, th = 1.3;
            const double n = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            const double nr = d[0] / n, nth = d[1] / n, nph = d[2] / n;
            GeodesicStateD s = init_ray_from_camera_general_d(M, a, r, th, 0.2, nr, nth, nph);
            outs("cam_d", s);
            outs("zamo_d", init_ray_from_camera_zamo_d(M, a, r, th, 0.2, nr, nth, nph));
            GeodesicState sf = init_ray_from_camera_general((float)M, (float)a, (float)r, (float)th, 0.2f,
                                                            (float)nr, (float)nth, (float)nph);
            outf("cam_f", sf);
            out("H_f", hamiltonian_kerr(sf, (float)M, (float)a));
            GeodesicStateD dd;
            computeGeodesicDerivativesKerrD(s, M, a, dd);
            outs("rhs_d", dd);
            GeodesicState df;
            computeGeodesicDerivativesKerr(sf, (float)M, (float)a, df);
            outf("rhs_f", df);
            GeodesicStateD y = s;
            bool ok = true;
            for (int k = 0; k < 60 && ok; ++k) ok = integrateGeodesicKerrD(y, M, a, 0.05 * y.r);
            outs("rk4_d", y);
            out("rk4_d_ok", ok ? 1.0 : 0.0);
            GeodesicState yf = sf;
            bool okf = true;
            for (int k = 0; k < 60 && okf; ++k) okf = integrateGeodesicKerr(yf, (float)M, (float)a, 0.05f * yf.r);
            outf("rk4_f", yf);
            GeodesicStateD z = s, zo;
            out("step_d_ok", rk4_step_d(z, M, a, 0.7, zo) ? 1.0 : 0.0);
            outs("step_d", zo);
            double h = 0.5;
            int acc = 0;
            for (int k = 0; k < 40; ++k) {
                double fac = rk4_adaptive_step_d(z, M, a, h, 1e-9, 1e-12);
                if (fac > 0.0) { ++acc; h *= fac; }
            }
            outs("adaptive_d", z);
            out("adaptive_h", h);
            out("adaptive_acc", acc);
            GeodesicStateD e = s;
            e.r = 7.5;
            out("doppler_d", doppler_g_general_d(e, M, a));
            GeodesicState ef = sf;
            ef.r = 7.5f;
            out("doppler_f", doppler_g_general(ef, (float)M, (float)a));
        }
    // Schwarzschild
    for (const auto& d : dirs) {
        ++g_idx;
        SchwarzschildMetric m(1.5f);
        GeodesicState s;
        s.r = 25.0f; s.theta = 1.1f; s.phi = 0.0f;
        s.pt = -1.0f; s.pr = (float)d[0]; s.ptheta = 25.0f * (float)d[1]; s.pphi = 25.0f * std::sin(1.1f) * (float)d[2];
        out("schw_H", hamiltonian_schwarzschild(s, m.Rs));
        GeodesicState ds;
        computeGeodesicDerivatives(s, m, ds);
        outf("schw_rhs", ds);
        bool ok = true;
        for (int k = 0; k < 80 && ok; ++k) ok = integrateGeodesic(s, m, 0.02f * s.r);
        outf("schw_rk4", s);
        out("schw_g", m.g_tt(9.0f) + m.g_rr(9.0f) + m.g_theta_theta(9.0f) + m.g_phi_phi(9.0f, 0.7f));
    }
    ++g_idx;
    out("bcrit", bh_bcrit_from_M(1.3f));
    out("bcrit_rs", bh_bcrit_from_Rs(2.6f));
    out("rph", bh_r_ph(bh_r_s(1.3f)));
    out("units", bh_to_M_units(7.0f, 0.0f) + bh_to_Rs_units(7.0f, 2.0f));
    out("safe_div", bh_safe_div(1.0f, -0.0f) + bh_safe_div(2.0f, 1e-9f) + bh_safe_div(3.0f, 4.0f));
    out("sin2", bh_safe_sin2(1e-5f));
    out("rk4sum", bh_rk4_sum(1e16, 1.0, -1e16, 3.0));
    out("status", (double)(int)RayStatus::Inconclusive);
    return 0;
}
