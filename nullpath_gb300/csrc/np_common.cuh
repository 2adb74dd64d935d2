// np_common.cuh -- scene constants, sampling, shading and work distribution
// shared by the FP64 and mixed-precision Kerr tracers (sm_103a).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "np_render.h"

// Records the message np_last_error() returns (thread-local, np_render.cu).
void np_record_error(const char* msg);

// Streaming multiprocessors of the current device (1 if it cannot be read):
// grid-stride launches cap their grids at a multiple of it.
inline int np_device_sms() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        n <= 0)
        return 1;
    return n;
}

namespace np {

constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr float kPiF = 3.14159265358979323846f;
constexpr double kEps = 1e-12;     // floor of the FP64 metric blocks (bh_common.h:77)
constexpr double kHMin = 1e-6;     // bh_common.h:245
constexpr double kHMax = 0.2;      // bh_common.h:253
constexpr double kSafety = 0.9;    // bh_common.h:236

// Island selection of the mixed path (bit mask in SceneDev::islands).
constexpr int kIslandHorizon = 1;   // FP64 steps within kHorizonBand of r_+
constexpr int kIslandTurning = 2;   // FP64 redo of steps across a p_r / p_theta sign change
constexpr int kIslandCritical = 4;  // FP64 tracing of rays with |b - b_crit| < kCriticalDb
constexpr double kHorizonBand = 0.1;   // in M
constexpr double kCriticalDb = 1e-3;   // in M

// Per-scene constants, computed once on the host in double precision and
// passed by value (kernel parameters live in the constant bank, so every
// lane reads them as a broadcast).
constexpr int kCritN = 256;

struct SceneDev {
    int W, H, spp, sample_offset;
    long long npix, total;            // pixels, rays (= npix * spp)
    int ref_units, jitter, strata;
    unsigned seed;
    int integrator, max_steps, max_orders, crossing;
    int bg_mode, disk_on, check_inv, islands;
    double M, a, Rs, r_cam, th_cam, ph_cam, r_plus, r_minus;
    float aspect_f, tan_half_f;
    double aspect, tan_half;
    double rin, rout, r_far, q, h_unit, rtol, atol;
    float Rsf, gain, bg_sigma_rad, bg_peak, qf;
    // camera tetrad: p^t = T0 + n_phi T1, p^phi = P0 + n_phi P1,
    // p^r = n_r R1, p^theta = n_theta H1, then lowered with g_{mu nu}(camera)
    double T0, T1, P0, P1, R1, H1;
    double gtt, gtp, gpp, grr, ghh;
    double cos_cam, sin_cam;
    // FP32 copies for the mixed tracer's per-step path
    float r_cam_hi, r_cam_lo, th_cam_hi, th_cam_lo, ph_cam_hi, ph_cam_lo;
    float r_plus_f, r_band_f, pi_lim_f, rin_f, rout_f, r_far_f, h_unit_f, inv_M_f;
    float hmin_f, hmax_f, rtol_f, atol_f;
    double hmin, hmax;         // adaptive step bounds (hmax scales with r in units of M)
    double inv_gate;           // invariant gate of the embedded 7(8) integrator (0 = off)
    double rtol64;             // rtol of the FP64 7(8) islands and near-critical rays of the mixed path
    float atol78_f;            // atol of the FP32 7(8) steps: the scene's, at least 1e-9 M (FP32 resolution)
    int cert_capture;          // 7(8) path: rays certified to fall in end at the horizon band (disk outside it)
    int island_df;             // 7(8) path: FP64-class steps in double-float arithmetic
    int crit_cf;               // mixed path: near-critical rays in closed form (Mino-time solution)
    int band_cf;               // 7(8) mixed path: rays entering the horizon band (not certified to fall
                               // in) end there and are solved whole in closed form instead of FP64 steps
    float a_hl[2], M_hl[2], rp_hl[2], rm_hl[2];   // a, M, r_+, r_- as double-float pairs
    float rtol64_f, atol64_f;  // tolerances of the near-critical rays (double-float arithmetic)
    int island_batch;
    int cross_batch;           // pending root-found crossings that trigger a warp's search (FP64 tracer)
    // NP_JITTER_CRITICAL: tangent-plane radius of the critical curve at
    // kCritN equally spaced position angles from -pi, and the band half-width
    float crit_rho[kCritN];
    double crit_band;
};

// ---------------------------------------------------------------------------
// Jitter.  wang_hash is the integer hash of render.cu:88-99 (kept so that the
// reference sampling pattern is reproduced bit for bit); mix32 is the
// "lowbias32" finaliser (C. Wellons) used by the stratified sampler.
__host__ __device__ __forceinline__ uint32_t wang_hash(uint32_t v) {
    v = (v ^ 61u) ^ (v >> 16);
    v *= 9u;
    v = v ^ (v >> 4);
    v *= 0x27d4eb2du;
    v = v ^ (v >> 15);
    return v;
}
__host__ __device__ __forceinline__ float wang_unit(uint32_t v) {
    return (float)(wang_hash(v) & 0x00ffffffu) * (1.0f / 16777216.0f);
}
__host__ __device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du;
    x ^= x >> 15; x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
__host__ __device__ __forceinline__ double strat_unit(uint32_t seed, uint32_t pix, uint32_t sample, uint32_t dim) {
    uint32_t h = mix32(mix32(mix32(seed + 0x9e3779b9u * (dim + 1u)) ^ pix) ^ (sample * 0x85ebca6bu));
    return (double)(h >> 8) * (1.0 / 16777216.0);
}

// Critical-curve importance sampling (NP_JITTER_CRITICAL): odd samples move
// along their position angle psi in the camera's tangent plane to
// rho_c(psi) (1 + band (2u - 1)), u a seeded uniform, so that half the rays
// lie within +-band of the critical impact parameter (the tangent-plane
// radius is b / r_cam to first order).
__host__ __device__ __forceinline__ void critical_remap(const SceneDev& s, uint32_t pix, uint32_t sample, double& cx,
                                                        double& cy) {
    const double psi = atan2(cy, cx);
    const double t = (psi + kPi) * ((double)kCritN / (2.0 * kPi));
    int i0 = (int)floor(t);
    const double fr = t - (double)i0;
    i0 = ((i0 % kCritN) + kCritN) % kCritN;
    const int i1 = (i0 + 1) % kCritN;
    const double rc = (1.0 - fr) * (double)s.crit_rho[i0] + fr * (double)s.crit_rho[i1];
    const double u = strat_unit(s.seed, pix, sample, 2);
    const double rho = rc * (1.0 + s.crit_band * (2.0 * u - 1.0));
    cx = rho * cos(psi);
    cy = rho * sin(psi);
}

struct CamDir { double nr, nth, nph; float cam_x, cam_y; };

// Local direction of one sample.  The few float operations of the reference
// camera (render.cu:145-154) use round-to-nearest intrinsics so that no
// contraction changes their rounding.
__device__ __forceinline__ CamDir camera_dir(const SceneDev& s, int x, int y, uint32_t sample,
                                             bool explicit_pos, double fx, double fy) {
    CamDir d;
    if (s.ref_units) {
        float px, py;
        if (explicit_pos) { px = (float)fx; py = (float)fy; }
        else if (s.jitter == NP_JITTER_WANGHASH) {
            float jx = wang_unit((uint32_t)(x * 73856093u ^ y * 19349663u ^ sample * 83492791u)) - 0.5f;
            float jy = wang_unit((uint32_t)(x * 83492791u ^ y * 2654435761u ^ sample * 19349663u)) - 0.5f;
            px = __fadd_rn(__fadd_rn((float)x, 0.5f), jx);
            py = __fadd_rn(__fadd_rn((float)y, 0.5f), jy);
        } else {
            uint32_t pix = (uint32_t)(y * s.W + x);
            int m = s.strata;
            uint32_t c = sample % (uint32_t)(m * m);
            px = (float)(x + ((double)(c % m) + strat_unit(s.seed, pix, sample, 0)) / m);
            py = (float)(y + ((double)(c / m) + strat_unit(s.seed, pix, sample, 1)) / m);
        }
        float ndc_x = __fsub_rn(__fmul_rn(__fdiv_rn(px, (float)s.W), 2.0f), 1.0f);
        float ndc_y = __fsub_rn(__fmul_rn(__fdiv_rn(py, (float)s.H), 2.0f), 1.0f);
        float cx = __fmul_rn(__fmul_rn(ndc_x, s.aspect_f), s.tan_half_f);
        float cy = __fmul_rn(-ndc_y, s.tan_half_f);
        if (!explicit_pos && s.jitter == NP_JITTER_CRITICAL && (sample & 1u)) {
            double dx = cx, dy = cy;
            critical_remap(s, (uint32_t)(y * s.W + x), sample, dx, dy);
            cx = (float)dx; cy = (float)dy;
        }
        float cz = -1.0f;
        float n2 = __fadd_rn(__fadd_rn(__fmul_rn(cx, cx), __fmul_rn(cy, cy)), __fmul_rn(cz, cz));
        float nrm = __fdiv_rn(1.0f, __fsqrt_rn(n2));
        cx = __fmul_rn(cx, nrm); cy = __fmul_rn(cy, nrm); cz = __fmul_rn(cz, nrm);
        d.nr = cz; d.nth = cy; d.nph = cx; d.cam_x = cx; d.cam_y = cy;
    } else {
        double px, py;
        if (explicit_pos) { px = fx; py = fy; }
        else if (s.jitter == NP_JITTER_WANGHASH) {
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
        if (!explicit_pos && s.jitter == NP_JITTER_CRITICAL && (sample & 1u))
            critical_remap(s, (uint32_t)(y * s.W + x), sample, cx, cy);
        double cz = -1.0;
        double n2 = __dadd_rn(__dadd_rn(__dmul_rn(cx, cx), __dmul_rn(cy, cy)), __dmul_rn(cz, cz));
        double nrm = __ddiv_rn(1.0, __dsqrt_rn(n2));
        cx = __dmul_rn(cx, nrm); cy = __dmul_rn(cy, nrm); cz = __dmul_rn(cz, nrm);
        d.nr = cz; d.nth = cy; d.nph = cx; d.cam_x = (float)cx; d.cam_y = (float)cy;
    }
    return d;
}

// Covariant camera momentum from the precomputed tetrad (bh_kerr.h:815-823
// and 952-964 with the metric factored out), rounding as the CPU does.
struct Momentum { double pt, pr, pth, pph; };
__device__ __forceinline__ Momentum camera_momentum(const SceneDev& s, const CamDir& d) {
    double Pt = __dadd_rn(s.T0, __dmul_rn(d.nph, s.T1));
    double Pp = __dadd_rn(s.P0, __dmul_rn(d.nph, s.P1));
    double Pr = __dmul_rn(d.nr, s.R1);
    double Ph = __dmul_rn(d.nth, s.H1);
    Momentum m;
    m.pt = __dadd_rn(__dmul_rn(s.gtt, Pt), __dmul_rn(s.gtp, Pp));
    m.pr = __dmul_rn(s.grr, Pr);
    m.pth = __dmul_rn(s.ghh, Ph);
    m.pph = __dadd_rn(__dmul_rn(s.gtp, Pt), __dmul_rn(s.gpp, Pp));
    return m;
}

// Second-order compensated accumulator (Klein 2006), the summation of
// bh_common.h:451-483.
template <typename T>
struct Klein {
    T s, c1, c2;
    __device__ __forceinline__ Klein() : s(T(0)), c1(T(0)), c2(T(0)) {}
    __device__ __forceinline__ void add(T x) {
        T t = s + x;
        T e = (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
        s = t;
        T u = c1 + e;
        T ee = (fabs(c1) >= fabs(e)) ? (c1 - u) + e : (e - u) + c1;
        c1 = u;
        c2 += ee;
    }
    __device__ __forceinline__ T value() const { return s + c1 + c2; }
};

__device__ __forceinline__ void metric_cov_d(double M, double a, double r, double th,
                                             double& gtt, double& gtp, double& gpp, double& grr, double& ghh) {
    double sn, c;
    sincos(th, &sn, &c);
    double s2 = sn * sn, r2 = r * r, a2 = a * a;
    double Sig = r2 + a2 * c * c;
    double Del = r2 - 2.0 * M * r + a2;
    double A = (r2 + a2) * (r2 + a2) - a2 * Del * s2;
    gtt = -(1.0 - 2.0 * M * r / fmax(kEps, Sig));
    gtp = -2.0 * M * a * r * s2 / fmax(kEps, Sig);
    gpp = A * s2 / fmax(kEps, Sig);
    grr = Sig / fmax(kEps, Del);
    ghh = Sig;
}

// g = E_inf / E_emitter for a prograde Keplerian emitter at the equator
// (bh_kerr.h:833-862); only r and the conserved p_t, p_phi enter.
__device__ __forceinline__ double doppler_g(double r, double pt, double pph, double M, double a) {
    double gtt, gtp, gpp, grr, ghh;
    metric_cov_d(M, a, r, kPi * 0.5, gtt, gtp, gpp, grr, ghh);
    double Ms = fmax(kEps, M);
    double Om = 1.0 / (a / Ms + pow(fmax(1.0, r / Ms), 1.5)) / Ms;
    Klein<double> d; d.add(gtt); d.add(2.0 * gtp * Om); d.add(gpp * Om * Om);
    double den = -d.value();
    double ut = 1.0 / sqrt(den > 1e-24 ? den : 1e-24);
    double up = Om * ut;
    Klein<double> k; k.add(pt * ut); k.add(pph * up);
    double ku = -k.value();
    double g = -pt / (ku > 1e-18 ? ku : 1e-18);
    return g > 0.0 ? g : 0.0;
}

// I = r^-q g^3 (1, .75, .45) (render.cu:65-72 with the index q as a parameter).
__device__ __forceinline__ void shade_disk(float r, float g, float q, float gain, float acc[3]) {
    float j = powf(fmaxf(r, 1.0f), -q);
    float I = j * g * g * g;
    acc[0] += (1.0f * I) * gain;
    acc[1] += (0.75f * I) * gain;
    acc[2] += (0.45f * I) * gain;
}

__device__ __forceinline__ float clamp01f(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

// Sky gradient with a bright band (render.cu:74-86).
__device__ __forceinline__ void shade_sky(float v, float out[3]) {
    float t = clamp01f(v);
    float c0 = 0.02f * (1 - t) + 0.08f * t;
    float c1 = 0.03f * (1 - t) + 0.09f * t;
    float c2 = 0.05f * (1 - t) + 0.12f * t;
    float band = expf(-50.0f * (v - 0.5f) * (v - 0.5f));
    c0 += 0.4f * band; c1 += 0.35f * band; c2 += 0.3f * band;
    out[0] = clamp01f(c0); out[1] = clamp01f(c1); out[2] = clamp01f(c2);
}

// Final colour of one sample (render.cu:312-359); cam_y is the camera-frame
// direction's y component (sky gradient), min_r the closest approach.
__device__ __forceinline__ void sample_colour(const SceneDev& s, bool captured, int orders,
                                              const float disk[3], float min_r, float cam_y, float col[3]) {
    if (captured || !(orders > 0 && s.disk_on)) {
        if (s.bg_mode == NP_BG_POINT) {
            float rph = 1.5f * s.Rsf;
            float w = fmaxf(0.02f * s.Rsf, 0.005f * s.Rsf + 0.02f * s.bg_sigma_rad * s.Rsf);
            float dr = min_r - rph;
            float I = s.bg_peak * expf(-0.5f * (dr / w) * (dr / w)) + (captured ? 0.0f : 0.02f);
            col[0] = col[1] = col[2] = I;
        } else if (captured) {
            col[0] = col[1] = col[2] = 0.0f;
        } else {
            shade_sky(cam_y * 0.5f + 0.5f, col);
        }
    } else {
        col[0] = disk[0]; col[1] = disk[1]; col[2] = disk[2];
    }
}

// Non-negative float max through the ordered integer view (deterministic).
__device__ __forceinline__ void atomic_max_nonneg(float* addr, float v) {
    if (!(v >= 0.0f)) return;
    atomicMax(reinterpret_cast<int*>(addr), __float_as_int(v));
}

// Cubic Hermite helpers on one step (values y0, y1; slopes m0, m1 = h f).
__device__ __forceinline__ double hermite_eval(double y0, double y1, double m0, double m1, double s) {
    double s2 = s * s, s3 = s2 * s;
    return (2 * s3 - 3 * s2 + 1) * y0 + (s3 - 2 * s2 + s) * m0 + (-2 * s3 + 3 * s2) * y1 + (s3 - s2) * m1;
}
// Root of the Hermite interpolant of d = theta - pi/2 (d0, d1 of opposite
// sign), safeguarded Newton from the linear estimate.
__device__ __forceinline__ double hermite_root(double d0, double d1, double m0, double m1, double s_lin) {
    double s = s_lin, lo = 0.0, hi = 1.0;
    for (int it = 0; it < 8; ++it) {
        double s2 = s * s, s3 = s2 * s;
        double p = (2 * s3 - 3 * s2 + 1) * d0 + (s3 - 2 * s2 + s) * m0 + (-2 * s3 + 3 * s2) * d1 + (s3 - s2) * m1;
        double dp = (6 * s2 - 6 * s) * d0 + (3 * s2 - 4 * s + 1) * m0 + (-6 * s2 + 6 * s) * d1 + (3 * s2 - 2 * s) * m1;
        if ((p > 0) == (d0 > 0)) lo = s; else hi = s;
        double sn = (dp != 0.0) ? s - p / dp : 0.5 * (lo + hi);
        if (!(sn > lo && sn < hi)) sn = 0.5 * (lo + hi);
        bool done = fabs(sn - s) < 1e-15;
        s = sn;
        if (done) break;
    }
    return s;
}

// ---------------------------------------------------------------------------
// Work distribution.  Every warp owns a chunk of ray indices [base, end)
// taken from one global counter; lanes whose ray has finished take the next
// index of the chunk, so a warp keeps all 32 lanes busy while rays of very
// different lengths retire.  One atomic per chunk.
struct WarpQueue {
    long long base, end;
};

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Hands a fresh ray index to every lane in `need`; returns -1 for lanes that
// get none (queue drained).  Must be called by all 32 lanes.
__device__ __forceinline__ long long warp_take(WarpQueue& q, unsigned need, unsigned long long* counter,
                                               long long total, int chunk) {
    const int lane = threadIdx.x & 31;
    long long mine = -1;
    while (need) {
        long long avail = q.end - q.base;
        int n = __popc(need);
        if (avail <= 0) {
            long long nb = 0;
            if (lane == 0) nb = (long long)atomicAdd(counter, (unsigned long long)chunk);
            nb = __shfl_sync(0xffffffffu, nb, 0);
            if (nb >= total) { q.base = q.end = total; break; }
            q.base = nb;
            q.end = min(nb + (long long)chunk, total);
            avail = q.end - q.base;
        }
        int take = (int)min((long long)n, avail);
        // the first `take` lanes of `need` (in lane order) are served
        unsigned served = need;
        for (int k = n; k > take; --k) served &= ~(1u << (31 - __clz(served)));
        if ((served >> lane) & 1u) mine = q.base + __popc(served & lanemask_lt());
        q.base += take;
        need &= ~served;
    }
    return mine;
}

}  // namespace np
