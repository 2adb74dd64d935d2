/*
 * ref_driver.cpp -- host driver around the REFERENCE's own physics headers.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file against the
 * unmodified reference headers where they lie (include/bh_common.h,
 * include/bh_types.h, include/bh_kerr.h of danielchristiancazares/NullPath)
 * into oracle/_ref/libnpref.so.  It exists to pin the oracle restatement in
 * np_oracle.cpp: the physics (metric blocks, analytic derivatives, RK4,
 * adaptive step doubling, camera tetrads, Doppler factor) comes from the
 * reference itself, and only the per-pixel loop of render.cu:141-363 is
 * restated here, because render.cu is a CUDA translation unit with a main().
 *
 * Reference semantics only: lengths in Rs, wanghash jitter, linear
 * crossing interpolation, fixed RK4 or the reference adaptive integrator.
 */
#include <cmath>
#include <cstdint>
#include <algorithm>

// Host stand-ins for the two device intrinsics the headers call.
static inline double np_host_rsqrt(double x) { return 1.0 / std::sqrt(x); }
static inline float np_host_rsqrtf(float x) { return 1.0f / std::sqrt(x); }
#define rsqrt np_host_rsqrt
#define rsqrtf np_host_rsqrtf

#include "bh_common.h"
#include "bh_types.h"
#include "bh_kerr.h"

#include "../include/np_render.h"

namespace {

inline unsigned wanghash_(unsigned a) {
    a = (a ^ 61u) ^ (a >> 16); a *= 9u; a = a ^ (a >> 4); a *= 0x27d4eb2d; a = a ^ (a >> 15);
    return a;
}
inline float rnd01_(unsigned s) { return (wanghash_(s) & 0x00ffffff) * (1.0f / 16777216.0f); }

struct Col { float x, y, z; };

inline Col shade_disk_(float r, float g, float q) {
    float j = powf(fmaxf(r, 1.0f), -q);
    float I = j * g * g * g;
    return Col{1.0f * I, 0.75f * I, 0.45f * I};
}
inline float c01(float v) { return fminf(fmaxf(v, 0.f), 1.f); }
inline Col shade_bg_(float u, float v) {
    (void)u;
    float t = c01(v);
    Col c{0.02f * (1 - t) + 0.08f * t, 0.03f * (1 - t) + 0.09f * t, 0.05f * (1 - t) + 0.12f * t};
    float band = expf(-50.0f * (v - 0.5f) * (v - 0.5f));
    c.x += 0.4f * band; c.y += 0.35f * band; c.z += 0.3f * band;
    return Col{c01(c.x), c01(c.y), c01(c.z)};
}

}  // namespace

extern "C" int npref_render(const np_scene_t* sc, int y_begin, int y_end, float* rgb, float* rcross) {
    if (!sc || !rgb || sc->units != NP_UNITS_RS) return -1;
    const int width = sc->width, height = sc->height;
    const float mass = (float)sc->mass, spin = (float)sc->spin, r_cam_Rs = (float)sc->r_cam;
    const float theta_cam = (float)sc->theta_deg * PI_F / 180.0f;
    const float phi_cam = (float)sc->phi_deg * PI_F / 180.0f;
    const float fov_y_deg = (float)sc->fov_y_deg;
    const int integrator_mode = sc->integrator, camera_mode = sc->camera;
    const int disk_on = sc->disk_on, disk_max_orders = std::max(1, sc->disk_max_orders);
    const float disk_gain = (float)sc->disk_gain, q = (float)sc->emissivity_q;
    const size_t plane = (size_t)width * height;
    y_begin = std::max(0, y_begin); y_end = std::min(height, y_end);
    long npx = (long)width * (y_end - y_begin);
#pragma omp parallel for schedule(dynamic, 16)
    for (long i = 0; i < npx; ++i) {
        int x = (int)(i % width), y = y_begin + (int)(i / width);
        SchwarzschildMetric metric(mass);
        float Rs = metric.Rs, M = mass, a = spin * M, r_cam = r_cam_Rs * Rs;
        float aspect = (float)width / (float)height;
        float fov_y = fov_y_deg * BH_PI / 180.0f;
        float tan_half = tanf(0.5f * fov_y);
        Col accum{0, 0, 0};
        float rc0 = 0.0f;
        for (int s = 0; s < sc->spp; ++s) {
            unsigned sample_id = (unsigned)(sc->sample_offset + s);
            float jx = rnd01_((unsigned)(x * 73856093u ^ y * 19349663u ^ sample_id * 83492791u)) - 0.5f;
            float jy = rnd01_((unsigned)(x * 83492791u ^ y * 2654435761u ^ sample_id * 19349663u)) - 0.5f;
            float ndc_x = ((x + 0.5f + jx) / (float)width) * 2.0f - 1.0f;
            float ndc_y = ((y + 0.5f + jy) / (float)height) * 2.0f - 1.0f;
            float cam_x = ndc_x * aspect * tan_half, cam_y = -ndc_y * tan_half, cam_z = -1.0f;
            float norm = rsqrtf(cam_x * cam_x + cam_y * cam_y + cam_z * cam_z);
            cam_x *= norm; cam_y *= norm; cam_z *= norm;
            float n_r = cam_z, n_theta = cam_y, n_phi = cam_x;
            GeodesicStateD state;
            bool static_ok = kerr_static_timelike((double)M, (double)a, (double)r_cam, (double)theta_cam);
            if (camera_mode == 1 || !static_ok)
                state = init_ray_from_camera_zamo_d(M, a, r_cam, theta_cam, phi_cam, n_r, n_theta, n_phi);
            else
                state = init_ray_from_camera_general_d(M, a, r_cam, theta_cam, phi_cam, n_r, n_theta, n_phi);
            double min_r = state.r;
            bool captured = false;
            int orders = 0;
            Col disk{0, 0, 0};
            GeodesicStateD prev = state;
            const double rin = sc->disk_rin > 0 ? sc->disk_rin : 3.0 * (double)Rs;
            const double rout = sc->disk_rout > 0 ? sc->disk_rout : 20.0 * (double)Rs;
            const double r_far = sc->escape_r > 0 ? sc->escape_r : (double)r_cam + 10.0 * (double)Rs;
            const double hstep = (double)(float)sc->step_scale;
            double h_adapt = 0.0;
            double first_r = 0.0;
            for (int step = 0; step < sc->max_steps; ++step) {
                double scale = fmin(fmax(1.0, state.r / (0.5 * (double)Rs)), 100.0);
                bool ok = false;
                if (integrator_mode == 1) {
                    double hb = fmin(fmax(hstep * scale, BH_RK_HMIN), BH_RK_HMAX);
                    double h = (h_adapt > 0.0) ? h_adapt : hb;
                    h = fmin(fmax(h, BH_RK_HMIN), BH_RK_HMAX);
                    for (int att = 0; att < 8; ++att) {
                        double ht = h;
                        double fac = rk4_adaptive_step_d(state, M, a, ht, sc->rtol, sc->atol);
                        if (fac > 0.0) { ok = true; h_adapt = fmin(fmax(ht * fac, BH_RK_HMIN), BH_RK_HMAX); break; }
                        h = fmax(ht, BH_RK_HMIN);
                        if (h <= BH_RK_HMIN * 1.01) break;
                    }
                } else {
                    ok = integrateGeodesicKerrD(state, M, a, hstep * scale);
                }
                if (!ok) { captured = true; break; }
                min_r = fmin(min_r, state.r);
                double dp = prev.theta - BH_PI_D * 0.5, dc = state.theta - BH_PI_D * 0.5;
                double eps = 1e-8;
                bool sc_ = (dp > 0 && dc < 0) || (dp < 0 && dc > 0);
                bool nz = (fabs(dp) < eps && fabs(dc) >= eps) || (fabs(dc) < eps && fabs(dp) >= eps);
                if ((sc_ || nz) && orders < disk_max_orders) {
                    double alpha = fabs(dp) / (fabs(dp) + fabs(dc) + 1e-30);
                    double r_cross = prev.r + alpha * (state.r - prev.r);
                    if (r_cross >= rin && r_cross <= rout) {
                        GeodesicStateD cross = state;
                        cross.r = r_cross; cross.theta = BH_PI_D * 0.5;
                        cross.pt = prev.pt + alpha * (state.pt - prev.pt);
                        cross.pphi = prev.pphi + alpha * (state.pphi - prev.pphi);
                        float g = (float)doppler_g_general_d(cross, M, a);
                        Col c = shade_disk_((float)r_cross, g, q);
                        disk.x += c.x * disk_gain; disk.y += c.y * disk_gain; disk.z += c.z * disk_gain;
                        if (orders == 0) first_r = r_cross;
                        orders++;
                    }
                }
                prev = state;
                if (state.r > r_far && step > 10) break;
            }
            Col color;
            const bool point = sc->background == NP_BG_POINT;
            const float bg_sigma_rad = (float)sc->bg_sigma_deg * PI_F / 180.0f;
            const float bg_peak = (float)sc->bg_brightness;
            if (captured) {
                if (point) {
                    float r_ph = 1.5f * Rs;
                    float w = fmaxf(0.02f * Rs, 0.005f * Rs + 0.02f * bg_sigma_rad * Rs);
                    float dr = ((float)min_r - r_ph);
                    float I = bg_peak * expf(-0.5f * (dr / w) * (dr / w)) + 0.0f;
                    color = Col{I, I, I};
                } else {
                    color = Col{0, 0, 0};
                }
            } else if (orders > 0 && disk_on) {
                color = disk;
            } else if (point) {
                float r_ph = 1.5f * Rs;
                float w = fmaxf(0.02f * Rs, 0.005f * Rs + 0.02f * bg_sigma_rad * Rs);
                float dr = ((float)min_r - r_ph);
                float I = bg_peak * expf(-0.5f * (dr / w) * (dr / w)) + 0.02f;
                color = Col{I, I, I};
            } else {
                color = shade_bg_(cam_x * 0.5f + 0.5f, cam_y * 0.5f + 0.5f);
            }
            accum.x += color.x; accum.y += color.y; accum.z += color.z;
            if (s == 0) rc0 = (float)first_r;
        }
        size_t p = (size_t)y * width + x;
        rgb[p] = accum.x; rgb[plane + p] = accum.y; rgb[2 * plane + p] = accum.z;
        if (rcross) rcross[p] = rc0;
    }
    return 0;
}

// Raw physics entry points of the reference headers, for unit checks.
extern "C" void npref_metric_inv(double M, double a, double r, double th, double* g5) {
    kerr_blocks_contra_d(M, a, r, th, g5[0], g5[1], g5[2], g5[3], g5[4]);
}
extern "C" void npref_metric_inv_derivs(double M, double a, double r, double th, double* dr5, double* dth5) {
    kerr_blocks_contra_derivs_d(M, a, r, th, dr5[0], dr5[1], dr5[2], dr5[3], dr5[4],
                                dth5[0], dth5[1], dth5[2], dth5[3], dth5[4]);
}
