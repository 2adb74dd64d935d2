// np_render.cu -- sm_103a Kerr renderer behind the C ABI of include/np_render.h.
//
// Kernels
//   render_fp64_kernel   FP64 reference-form integrator (render.cu:161-251),
//                        persistent, one ray per lane with per-lane refill.
//   render_mixed_kernel  FP32/compensated Carter-form integrator with FP64
//                        islands; near-critical rays are appended to a
//                        deferred list and solved by the first warps of the
//                        same launch, in FP64 closed form (equator_cf.cuh)
//                        or traced whole in FP64.
//   resolve_kernel       sums the per-sample colours of a pass in sample
//                        order into the planar image (progressive spp).
//   trace_rays_kernel    explicit rays, per-ray crossing report.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <cmath>
#include <algorithm>
#include <mutex>
#include <string>
#include <vector>
#include <type_traits>

#include "np_common.cuh"
#include "tracer_fp64.cuh"
#include "tracer_mixed.cuh"
#include "tracer_df.cuh"
#include "equator_cf.cuh"

using namespace np;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

}  // namespace

void np_record_error(const char* msg) { g_last_error = msg ? msg : ""; }

namespace {

#define NP_CU(expr, code)                                                          \
    do {                                                                           \
        cudaError_t e_ = (expr);                                                   \
        if (e_ != cudaSuccess)                                                     \
            return fail((code), "%s: %s", #expr, cudaGetErrorString(e_));          \
    } while (0)

constexpr int kBlock = 128;
constexpr int kChunk = 64;
constexpr int kStepsPerTurn = 4;   // FP32 steps per pass of the mixed tracer's scheduling loop

// Tunables (set through np_tune; the autotuner searches them).
struct Tuning {
    int island_batch = 8;   // parked lanes that trigger a batched FP64 island step
    // The same for the 7(8) path, whose island steps (FP64 7(8)) cost about
    // 80 FP32 steps: the warp waits until every lane with work is parked.
    // 1280x720x4 frame, every island: 8 / 16 / 32 lanes gave 206 / 152 / 117 ms.
    int island_batch78 = 32;
    // Lanes with a pending root-found crossing that trigger the warp's
    // search (FP64 tracer).  A search costs the warp about four single
    // steps; batching trades the stall of the other lanes against the wait
    // of the pending ones.  Research scene 1280x720x1 on GB300: 1 / 3 / 6 /
    // 12 lanes gave 329 / 367 / 393 / 402 k rays/s.
    int cross_batch = 12;
    int min_blocks = 4;     // register cap of the mixed tracer (blocks of 128 per SM)
    // The same for the mixed 7(8) tracer.  Its FP32 loop alone needs 103
    // registers; with the FP64 island step inlined, 168 fit without spills,
    // while the 128 of 4 blocks spill around the island step.  Measured on the
    // 1280x720x4 frame, 4 blocks are faster all the same: 17.5 vs 20.4 ms
    // without islands, 201 vs 206 ms with every island.
    int min_blocks78 = 4;
    int chunk = 64;         // ray indices a warp takes from the global counter at once
};
Tuning g_tune;

// Device-side counters of one call.
struct Counters {
    unsigned long long work;        // next ray index (main pass)
    unsigned long long work2;       // next deferred-list index
    unsigned long long deferred;    // deferred-list length
    unsigned long long rays, steps, fp64_steps, evals;
    unsigned long long closed_form;  // near-critical rays solved in closed form
    unsigned long long band;         // rays handed from the horizon band to the closed form
};

// ---------------------------------------------------------------------------
// Scene preparation (host, FP64).

void host_metric_cov(double M, double a, double r, double th,
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

// Radius of the critical curve in the camera's tangent plane at kCritN
// position angles psi_i = -pi + 2 pi i / kCritN: bisection on the radius for
// the sign change of critical_gap (captured inside, turning outside) of the
// camera ray through (rho cos psi, rho sin psi, -1), with the camera tetrad
// of the scene.  Clamped to [0, frame corner].
void build_critical_table(SceneDev& d) {
    const double rho_max = (d.ref_units ? (double)d.tan_half_f * std::sqrt((double)d.aspect_f * d.aspect_f + 1.0)
                                        : d.tan_half * std::sqrt(d.aspect * d.aspect + 1.0));
    const double c = d.cos_cam, sn = d.sin_cam;
    auto captured = [&](double rho, double psi) {
        const double cx = rho * std::cos(psi), cy = rho * std::sin(psi), cz = -1.0;
        const double nrm = 1.0 / std::sqrt(cx * cx + cy * cy + cz * cz);
        const double nr = cz * nrm, nth = cy * nrm, nph = cx * nrm;
        const double Pt = d.T0 + nph * d.T1, Pp = d.P0 + nph * d.P1, Pr = nr * d.R1, Ph = nth * d.H1;
        (void)Pr;
        const double pt = d.gtt * Pt + d.gtp * Pp, pth = d.ghh * Ph, pph = d.gtp * Pt + d.gpp * Pp;
        const double E = -pt, L = pph;
        const double Q = pth * pth + c * c * (L * L / (sn * sn) - d.a * d.a * E * E);
        return critical_gap(E, L, Q, d.a, d.M, d.r_plus) > 0.0;
    };
    for (int i = 0; i < kCritN; ++i) {
        const double psi = -kPi + 2.0 * kPi * (double)i / (double)kCritN;
        double lo = 0.0, hi = rho_max, out;
        if (!captured(lo, psi)) out = 0.0;
        else if (captured(hi, psi)) out = rho_max;
        else {
            for (int it = 0; it < 60; ++it) {
                const double mid = 0.5 * (lo + hi);
                if (captured(mid, psi)) lo = mid; else hi = mid;
            }
            out = 0.5 * (lo + hi);
        }
        d.crit_rho[i] = (float)out;
    }
}

// Builds the per-scene constants; camera tetrads follow bh_kerr.h:781-826
// (static observer) and 910-967 (ZAMO), the static observer falling back to
// the ZAMO inside the ergosphere (render.cu:163-170).
int prepare_scene(const np_scene_t& sc, SceneDev& d) {
    int v = np_scene_validate(&sc);
    if (v != NP_OK) return v;
    std::memset(&d, 0, sizeof(d));
    d.W = sc.width; d.H = sc.height; d.spp = sc.spp; d.sample_offset = sc.sample_offset;
    d.npix = (long long)sc.width * sc.height;
    d.total = d.npix * sc.spp;
    d.ref_units = sc.units == NP_UNITS_RS;
    d.jitter = sc.jitter; d.seed = sc.seed;
    d.strata = std::max(1, (int)std::floor(std::sqrt((double)std::max(1, sc.spp))));
    d.integrator = sc.integrator; d.max_steps = sc.max_steps;
    d.max_orders = std::max(1, sc.disk_max_orders);
    d.crossing = sc.crossing; d.bg_mode = sc.background; d.disk_on = sc.disk_on;
    d.check_inv = sc.check_invariants;
    d.islands = sc.islands;
    d.inv_gate = sc.inv_gate > 0.0 ? sc.inv_gate : 0.0;
    // Near-critical rays run whole in FP64 7(8) at the scene's rtol unless told
    // otherwise: at rtol 1e-8 their crossing radii stay within 1e-7 M (order 1)
    // and 2e-6 M (order 2) of the Mino-time solver, and a tighter tolerance
    // (formerly 1e-10) lengthened the frame's FP64 tail by 15 %.
    d.rtol64 = sc.rtol_fp64 > 0.0 ? sc.rtol_fp64 : sc.rtol;
    // Step doubling at a tight rtol works at the FP32 precision floor where p_r
    // or p_theta changes sign; its turning-point steps are always FP64.
    if (sc.integrator == NP_INTEG_ADAPTIVE) d.islands |= NP_ISLAND_TURNING;
    if (d.ref_units) {
        float Mf = (float)sc.mass, Rsf = 2.0f * Mf;
        float af = (float)sc.spin * Mf, rcf = (float)sc.r_cam * Rsf;
        d.M = Mf; d.a = af; d.Rs = Rsf; d.r_cam = rcf;
        d.th_cam = (float)sc.theta_deg * kPiF / 180.0f;
        d.ph_cam = (float)sc.phi_deg * kPiF / 180.0f;
        d.aspect_f = (float)sc.width / (float)sc.height;
        float fov = (float)sc.fov_y_deg * kPiF / 180.0f;
        d.tan_half_f = std::tan(0.5f * fov);
        d.h_unit = (double)(float)sc.step_scale;
        d.Rsf = Rsf;
    } else {
        d.M = sc.mass; d.a = sc.spin * sc.mass; d.Rs = 2.0 * sc.mass;
        d.r_cam = sc.r_cam * sc.mass;
        d.th_cam = sc.theta_deg * kPi / 180.0;
        d.ph_cam = sc.phi_deg * kPi / 180.0;
        d.aspect = (double)sc.width / (double)sc.height;
        d.tan_half = std::tan(0.5 * sc.fov_y_deg * kPi / 180.0);
        d.h_unit = sc.step_scale;
        d.Rsf = (float)d.Rs;
    }
    double disc = std::fmax(0.0, d.M * d.M - d.a * d.a);
    d.r_plus = d.M + std::sqrt(disc);
    d.r_minus = d.M - std::sqrt(disc);
    d.rin = sc.disk_rin > 0.0 ? sc.disk_rin : 3.0 * d.Rs;
    d.rout = sc.disk_rout > 0.0 ? sc.disk_rout : 20.0 * d.Rs;
    d.r_far = sc.escape_r > 0.0 ? sc.escape_r : d.r_cam + 10.0 * d.Rs;
    d.q = sc.emissivity_q; d.qf = (float)sc.emissivity_q;
    d.rtol = sc.rtol; d.atol = sc.atol;
    d.gain = (float)sc.disk_gain;
    d.bg_sigma_rad = (float)sc.bg_sigma_deg * kPiF / 180.0f;
    d.bg_peak = (float)sc.bg_brightness;

    {
        HiLo v = d_hl(d.r_cam); d.r_cam_hi = v.hi; d.r_cam_lo = v.lo;
        v = d_hl(d.th_cam); d.th_cam_hi = v.hi; d.th_cam_lo = v.lo;
        v = d_hl(d.ph_cam); d.ph_cam_hi = v.hi; d.ph_cam_lo = v.lo;
        d.r_plus_f = (float)d.r_plus;
        d.r_band_f = (float)(d.r_plus + kHorizonBand * d.M);
        d.pi_lim_f = 3.14159250f;              // largest float below pi - 1e-9
        d.rin_f = (float)d.rin; d.rout_f = (float)d.rout; d.r_far_f = (float)d.r_far;
        d.h_unit_f = (float)d.h_unit; d.inv_M_f = (float)(1.0 / d.M);
        if (d.ref_units) { d.hmin = kHMin; d.hmax = kHMax; }
        else { d.hmin = kHMin * d.M; d.hmax = 10.0 * d.h_unit; }
        d.hmin_f = (float)d.hmin; d.hmax_f = (float)d.hmax;
        d.rtol_f = (float)d.rtol; d.atol_f = (float)d.atol;
        d.atol78_f = (float)std::fmax(d.atol, 1e-9 * d.M);
        d.cert_capture = !d.disk_on || d.rin > d.r_plus + kHorizonBand * d.M;
        d.island_df = sc.island_arith == NP_ISLAND_ARITH_DF;
        d.crit_cf = sc.critical_solver == NP_CRITICAL_CLOSED_FORM;
        d.band_cf = d.crit_cf && (sc.islands & NP_ISLAND_HORIZON) && sc.integrator == NP_INTEG_RKF78 &&
                    d.a != 0.0 && d.cert_capture;
        auto split = [](double x, float* o) { o[0] = (float)x; o[1] = (float)(x - (double)o[0]); };
        split(d.a, d.a_hl); split(d.M, d.M_hl); split(d.r_plus, d.rp_hl); split(d.r_minus, d.rm_hl);
        d.rtol64_f = (float)d.rtol64; d.atol64_f = (float)std::fmax(d.atol, 1e-14 * d.M);
        d.island_batch = sc.integrator == NP_INTEG_RKF78 ? g_tune.island_batch78 : g_tune.island_batch;
        d.cross_batch = g_tune.cross_batch;
    }
    const double M = d.M, a = d.a, r = d.r_cam, th = d.th_cam;
    double gtt, gtp, gpp, grr, ghh;
    host_metric_cov(M, a, r, th, gtt, gtp, gpp, grr, ghh);
    d.gtt = gtt; d.gtp = gtp; d.gpp = gpp; d.grr = grr; d.ghh = ghh;
    d.cos_cam = std::cos(th); d.sin_cam = std::sin(th);
    bool zamo = (sc.camera == NP_CAMERA_ZAMO) || !(gtt < 0.0);
    if (!zamo) {
        double ut = 1.0 / std::sqrt(std::fmax(kEps, -gtt));
        double er = 1.0 / std::sqrt(std::fmax(kEps, grr));
        double eh = 1.0 / std::sqrt(std::fmax(kEps, ghh));
        double ept, epp;
        if (std::fabs(gtp) > kEps) {
            double beta = -gtt / gtp;
            // compensated |e_phi|^2 (bh_kerr.h:801-806)
            double s = 0.0, c1 = 0.0, c2 = 0.0;
            double terms[3] = {gtt, 2.0 * gtp * beta, gpp * beta * beta};
            for (double x : terms) {
                double t = s + x;
                double e = (std::fabs(s) >= std::fabs(x)) ? (s - t) + x : (x - t) + s;
                s = t;
                double u = c1 + e;
                double ee = (std::fabs(c1) >= std::fabs(e)) ? (c1 - u) + e : (e - u) + c1;
                c1 = u; c2 += ee;
            }
            double n2 = s + c1 + c2;
            double inv = 1.0 / std::sqrt(std::fmax(kEps, std::fabs(n2)));
            ept = inv; epp = beta * inv;
        } else {
            ept = 0.0; epp = 1.0 / std::sqrt(std::fmax(kEps, gpp));
        }
        d.T0 = ut; d.T1 = ept; d.P0 = 0.0; d.P1 = epp; d.R1 = er; d.H1 = eh;
    } else {
        double c = std::cos(th), sn = std::sin(th);
        double r2 = r * r, a2 = a * a;
        double Sig = std::fmax(kEps, r2 + a2 * c * c);
        double Del = r2 - 2.0 * M * r + a2;
        double A = std::fmax(kEps, (r2 + a2) * (r2 + a2) - a2 * Del * sn * sn);
        double alpha = std::sqrt(std::fmax(kEps, Del * Sig / A));
        double omega = 2.0 * M * a * r / A;
        d.T0 = 1.0 / std::fmax(kEps, alpha);
        d.T1 = 0.0;
        d.P0 = omega / std::fmax(kEps, alpha);
        d.P1 = std::sqrt(std::fmax(kEps, Sig / A)) / std::fmax(kEps, std::fabs(sn));
        d.R1 = std::sqrt(std::fmax(kEps, Del / Sig));
        d.H1 = 1.0 / std::sqrt(Sig);
    }
    d.crit_band = 0.02;
    if (sc.jitter == NP_JITTER_CRITICAL) build_critical_table(d);
    return NP_OK;
}

// ---------------------------------------------------------------------------
// Kernels.

__device__ __forceinline__ void ray_coords(const SceneDev& s, long long item, long long& p, int& sl,
                                           int& x, int& y, uint32_t& sid) {
    p = item % s.npix;
    sl = (int)(item / s.npix);
    x = (int)(p % s.W);
    y = (int)(p / s.W);
    sid = (uint32_t)(s.sample_offset + sl);
}

__device__ __forceinline__ void write_sample(const SceneDev& s, float* srgb, float* rcross,
                                             long long p, int sl, const float col[3], double first_r) {
    float* base = srgb + (size_t)sl * 3 * s.npix;
    base[p] = col[0];
    base[s.npix + p] = col[1];
    base[2 * s.npix + p] = col[2];
    if (sl == 0 && rcross) rcross[p] = (float)first_r;
}

__device__ __forceinline__ void flush_counters(Counters* ctr, unsigned long long rays, unsigned long long steps,
                                               unsigned long long f64, unsigned long long evals,
                                               unsigned long long cf = 0) {
    for (int o = 16; o > 0; o >>= 1) {
        rays += __shfl_down_sync(0xffffffffu, rays, o);
        steps += __shfl_down_sync(0xffffffffu, steps, o);
        f64 += __shfl_down_sync(0xffffffffu, f64, o);
        evals += __shfl_down_sync(0xffffffffu, evals, o);
        cf += __shfl_down_sync(0xffffffffu, cf, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&ctr->rays, rays);
        atomicAdd(&ctr->steps, steps);
        atomicAdd(&ctr->fp64_steps, f64);
        atomicAdd(&ctr->evals, evals);
        if (cf) atomicAdd(&ctr->closed_form, cf);
    }
}

// FP64 reference-form tracer over every ray index in [0, total).
template <int MODE>
__global__ void __launch_bounds__(kBlock)
render_fp64_kernel(const SceneDev s, float* __restrict__ srgb, float* __restrict__ rcross,
                   float* __restrict__ inv3, Counters* __restrict__ ctr) {
    const unsigned FULL = 0xffffffffu;
    unsigned long long* counter = &ctr->work;
    const long long total = s.total;
    WarpQueue q{0, 0};
    bool drained = false;
    RayFP64<false> R;
    CamDir dir;
    long long item = -1, p = 0;
    int sl = 0;
    bool have = false;
    unsigned long long n_rays = 0, n_steps = 0, n_evals = 0;
    while (true) {
        unsigned need = __ballot_sync(FULL, !have);
        if (need && !drained) {
            long long idx = warp_take(q, need, counter, total, kChunk);
            drained = q.base >= total;
            if (!have && idx >= 0) {
                item = idx;
                int x, y; uint32_t sid;
                ray_coords(s, item, p, sl, x, y, sid);
                dir = camera_dir(s, x, y, sid, false, 0.0, 0.0);
                fp64_init(s, camera_momentum(s, dir), R);
                have = true;
                n_rays++;
            }
        }
        if (!__any_sync(FULL, have)) break;
        // Root-found crossings wait until cross_batch lanes of the warp have
        // one (or no lane can step) and are then found together.
        unsigned pend = __ballot_sync(FULL, have && R.xpend);
        unsigned act = __ballot_sync(FULL, have && !R.xpend);
        bool done = false;
        if (pend && ((int)__popc(pend) >= s.cross_batch || !act)) {
            if (have && R.xpend) done = fp64_resolve<MODE>(s, R, inv3, n_evals);
        } else if (have && !R.xpend) {
            const int s0 = R.step;
            done = fp64_advance<MODE, false, true>(s, R, inv3, n_evals);
            n_steps += (unsigned long long)(R.step - s0);   // a rejected 7(8) attempt takes no step
        }
        if (done) {
            bool captured = R.status == 1;
            if (s.check_inv && inv3 && !captured && !(R.orders > 0 && s.disk_on))
                invariants_ref(s, R.y, R.pt0, R.pph0, inv3);
            float col[3];
            sample_colour(s, captured, R.orders, R.disk, (float)R.min_r, dir.cam_y, col);
            write_sample(s, srgb, rcross, p, sl, col, R.first_r);
            have = false;
        }
    }
    flush_counters(ctr, n_rays, n_steps, 0, n_evals);
}

// Per-ray initial data of the mixed path, structure of arrays:
//   a[i] = (p_r hi, p_r lo, p_theta hi, p_theta lo), b[i] = (E hi, E lo, L hi, L lo),
//   cy[i] = camera-frame y of the ray direction (sky colour), flag[i] = 1 for
//   near-critical rays (deferred to the FP64 warps, listed in `list`).
struct InitSoA {
    float4* a;
    float4* b;
    float* cy;
    unsigned char* flag;
    long long* list;
};

// Camera rays of one pass, fully parallel (one ray per thread).  All FP64
// work of ray generation happens here, with every lane of a warp active.
// Initial data of ray `li` of scene s, stored at index gi of the arrays;
// near-critical rays go to the deferred list (at most list_cap entries).
__device__ __forceinline__ void init_one(const SceneDev& s, long long li, long long gi, const InitSoA& soa,
                                         Counters* __restrict__ ctr, unsigned long long list_cap) {
    long long p; int sl, x, y; uint32_t sid;
    ray_coords(s, li, p, sl, x, y, sid);
    CamDir dir = camera_dir(s, x, y, sid, false, 0.0, 0.0);
    Momentum m = camera_momentum(s, dir);
    double E = -m.pt, L = m.pph;
    bool defer = false;
    if (s.islands & kIslandCritical) {
        double Q = m.pth * m.pth + s.cos_cam * s.cos_cam * (L * L / (s.sin_cam * s.sin_cam) - s.a * s.a * E * E);
        defer = near_critical_screened(E, L, Q, s.a, s.M, s.r_plus, kCriticalDb);
    }
    HiLo pr = d_hl(m.pr), pth = d_hl(m.pth), Eh = d_hl(E), Lh = d_hl(L);
    soa.a[gi] = make_float4(pr.hi, pr.lo, pth.hi, pth.lo);
    soa.b[gi] = make_float4(Eh.hi, Eh.lo, Lh.hi, Lh.lo);
    soa.cy[gi] = dir.cam_y;
    if (defer) {
        unsigned long long slot = atomicAdd(&ctr->deferred, 1ull);
        if (slot < list_cap) soa.list[slot] = gi;
        else defer = false;         // list full: the ray stays on the FP32 path
    }
    soa.flag[gi] = defer ? 1 : 0;
}

__global__ void __launch_bounds__(256)
ray_init_kernel(const SceneDev s, InitSoA soa, Counters* __restrict__ ctr) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < s.total;
         i += (long long)gridDim.x * blockDim.x)
        init_one(s, i, i, soa, ctr, (unsigned long long)s.total);
}

__device__ __forceinline__ void load_ray(const InitSoA& soa, long long i, MRay<false>& R, float& cam_y) {
    float4 a = soa.a[i], b = soa.b[i];
    R.pr = HiLo{a.x, a.y}; R.pth = HiLo{a.z, a.w};
    R.E = HiLo{b.x, b.y}; R.L = HiLo{b.z, b.w};
    cam_y = soa.cy[i];
}

// Mixed-precision tracer.  Warp 0 of the first `nd` blocks first traces the
// near-critical rays of `list` in FP64 (one block per SM, so their latency
// overlaps the FP32 work of the rest of the grid); every warp then traces
// FP32 rays from the shared counter, lanes refilling independently and
// parked island steps executed in batches.
// Integrator families of the mixed tracer (one kernel instantiation each, so
// the 7(8) stage storage does not raise the register count of the RK4 loop).
constexpr int kFamRk4 = 0;   // fixed RK4 and step doubling
constexpr int kFam78 = 1;    // embedded 7(8), FP64 islands and near-critical rays
constexpr int kFam78df = 2;  // embedded 7(8), the same in double-float arithmetic

template <int FAM> struct CritRay { using type = DRay<false>; };
template <> struct CritRay<kFam78> { using type = DRay78<false>; };
template <> struct CritRay<kFam78df> { using type = DRay78df<false>; };

// A near-critical ray in closed form (equator_cf.cuh): Carter's constants of
// the camera momentum in the units E = M = 1, the disk crossings of the
// Mino-time solution (radii in [rin, rout], at most max_orders), capture or
// escape, and the closest approach.  false when the ray is outside the
// closed forms (it is then integrated).
struct CritCF {
    int status, orders;
    float disk[3];
    double first_r, min_r;
};

__device__ __forceinline__ bool crit_constants(const SceneDev& s, const Momentum& m, double& l, double& q2,
                                               double& su, double& sm) {
    const double E = -m.pt, L = m.pph;
    const double Q = m.pth * m.pth + s.cos_cam * s.cos_cam * (L * L / (s.sin_cam * s.sin_cam) - s.a * s.a * E * E);
    l = L / (E * s.M);
    q2 = Q / (E * E * s.M * s.M);
    su = m.pr < 0.0 ? 1.0 : -1.0;
    sm = m.pth > 0.0 ? -1.0 : 1.0;
    return E > 0.0;
}

// Not inlined: the single-scene and batched kernels call the same function,
// so a ray gets the same bits from both, and the FP32 loops around the call
// sites keep their own register allocation.
__device__ __noinline__ bool crit_cf_solve(const SceneDev& s, const Momentum& m, CritCF& o) {
    double l, q2, su, sm;
    if (!crit_constants(s, m, l, q2, su, sm)) return false;
    double xu[8];
    const int kmax = s.disk_on ? min(s.max_orders, 8) : 0;
    const gkcf::EqX x = gkcf::equator_crossings(s.a / s.M, l, q2, s.M / s.r_cam, s.cos_cam, su, sm, s.M / s.r_far,
                                                s.M / s.rout, s.M / s.rin, kmax, xu, nullptr, nullptr);
    if (x.status < 0) return false;
    o.status = x.status;
    o.orders = 0;
    o.disk[0] = o.disk[1] = o.disk[2] = 0.0f;
    o.first_r = 0.0;
    for (int k = 0; k < x.n; ++k) {
        const double rc = s.M / xu[k];
        const float g = (float)doppler_g(rc, m.pt, m.pph, s.M, s.a);
        shade_disk((float)rc, g, s.qf, s.gain, o.disk);
        if (o.orders == 0) o.first_r = rc;
        o.orders++;
    }
    o.min_r = x.status == 1 ? s.r_plus : (x.u_turn > 0.0 ? s.M / x.u_turn : s.r_cam);
    return true;
}

// Long near-critical lists in a kernel of their own, one ray per thread.
// Inside the tracer the closed form runs under the FP32 loop's register cap
// (128) and spills, on the FP64 warps that the FP32 rays leave it; here it
// has its own budget (158 registers, no spills) and every warp of the GPU.
// A few dozen rays (a 1280x720x4 frame has 43) still go to the tracer,
// whose first warps take them while the FP32 rays run, so that one
// thread's latency (about 5 ms when this kernel ran them in front of the
// tracer) is hidden; a list of kCritKernelMin or more (critical-curve
// sampling: about 1 % of the rays) is solved here first.  The length is
// read on the device, so the launch needs no host synchronisation; solved
// rays get flag 2 and the tracer passes them over.
constexpr unsigned long long kCritKernelMin = 8192;

__global__ void __launch_bounds__(128)
critical_cf_kernel(const SceneDev s, InitSoA soa, float* __restrict__ srgb, float* __restrict__ rcross,
                   Counters* __restrict__ ctr, unsigned long long list_cap) {
    const unsigned long long Dl = min(ctr->deferred, list_cap);
    if (Dl < kCritKernelMin) return;
    const long long D = (long long)Dl;
    unsigned long long solved = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < D;
         i += (long long)gridDim.x * blockDim.x) {
        const long long item = soa.list[i];
        long long p; int sl, x, y; uint32_t sid;
        ray_coords(s, item, p, sl, x, y, sid);
        const CamDir dir = camera_dir(s, x, y, sid, false, 0.0, 0.0);
        CritCF o;
        if (!crit_cf_solve(s, camera_momentum(s, dir), o)) continue;
        float col[3];
        sample_colour(s, o.status == 1, o.orders, o.disk, (float)o.min_r, dir.cam_y, col);
        write_sample(s, srgb, rcross, p, sl, col, o.first_r);
        soa.flag[item] = 2;
        solved++;
    }
    for (int o = 16; o > 0; o >>= 1) solved += __shfl_down_sync(0xffffffffu, solved, o);
    if ((threadIdx.x & 31) == 0 && solved) {
        atomicAdd(&ctr->closed_form, solved);
        atomicAdd(&ctr->rays, solved);
    }
}

// Rays of the 7(8) path that entered the horizon band without a certificate
// of capture (status 3; listed after the near-critical rays): solved whole
// in closed form, one ray per thread, after the tracer.  At a = 0.998 the
// prograde photon orbit lies inside the band, and rays that wind there took
// hundreds of FP64 island steps each.  A ray outside the closed forms is
// traced whole in FP64 7(8) here instead.
__global__ void __launch_bounds__(128)
band_cf_kernel(const SceneDev s, InitSoA soa, float* __restrict__ srgb, float* __restrict__ rcross,
               Counters* __restrict__ ctr) {
    const long long D = (long long)ctr->deferred;
    const long long nb = (long long)ctr->band;
    unsigned long long steps = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nb;
         i += (long long)gridDim.x * blockDim.x) {
        const long long item = soa.list[D + i];
        long long p; int sl, x, y; uint32_t sid;
        ray_coords(s, item, p, sl, x, y, sid);
        const CamDir dir = camera_dir(s, x, y, sid, false, 0.0, 0.0);
        const Momentum m = camera_momentum(s, dir);
        float col[3];
        CritCF o;
        if (crit_cf_solve(s, m, o)) {
            sample_colour(s, o.status == 1, o.orders, o.disk, (float)o.min_r, dir.cam_y, col);
            write_sample(s, srgb, rcross, p, sl, col, o.first_r);
        } else {
            DRay78<false> R;
            dray78_start(R, s, -m.pt, m.pph, m.pr, m.pth);
            bool acc;
            while (!dray78_step(R, s, acc)) steps += acc ? 1 : 0;
            sample_colour(s, R.status == 1, R.orders, R.disk, (float)R.min_r, dir.cam_y, col);
            write_sample(s, srgb, rcross, p, sl, col, R.first_r);
        }
    }
    for (int o = 16; o > 0; o >>= 1) steps += __shfl_down_sync(0xffffffffu, steps, o);
    if ((threadIdx.x & 31) == 0 && steps) {
        atomicAdd(&ctr->steps, steps);
        atomicAdd(&ctr->fp64_steps, steps);
    }
}

// Near-critical rays from the deferred list, one per lane until the list is
// drained (rays taken four at a time from work2): solved in closed form
// (crit_cf_solve) when the scene asks for it and the ray is inside the
// closed forms, else traced whole in FP64.
template <int FAM>
__device__ __forceinline__ void trace_deferred(const SceneDev& s, const InitSoA& soa, float* __restrict__ srgb,
                                               float* __restrict__ rcross, Counters* __restrict__ ctr, long long D,
                                               unsigned long long& n_rays, unsigned long long& n_steps,
                                               unsigned long long& n_f64, unsigned long long& n_evals,
                                               unsigned long long& n_cf) {
    const unsigned FULL = 0xffffffffu;
    WarpQueue q{0, 0};
    bool drained = false, have = false;
    typename CritRay<FAM>::type R;
    long long item = 0, p = 0;
    int sl = 0;
    float cam_y = 0.0f;
    while (true) {
        unsigned need = __ballot_sync(FULL, !have);
        if (need && !drained) {
            long long idx = warp_take(q, need, &ctr->work2, D, 4);
            drained = q.base >= D;
            if (!have && idx >= 0 && soa.flag[soa.list[idx]] == 1) {
                item = soa.list[idx];
                int x, y; uint32_t sid;
                ray_coords(s, item, p, sl, x, y, sid);
                float4 a = soa.a[item], b = soa.b[item];
                cam_y = soa.cy[item];
                n_rays++;
                bool solved = false;
                if (s.crit_cf) {
                    // the Mino-time solution in closed form; the ray is
                    // integrated only when it is outside the closed forms
                    const CamDir dir = camera_dir(s, x, y, sid, false, 0.0, 0.0);
                    CritCF o;
                    solved = crit_cf_solve(s, camera_momentum(s, dir), o);
                    if (solved) {
                        float col[3];
                        sample_colour(s, o.status == 1, o.orders, o.disk, (float)o.min_r, cam_y, col);
                        write_sample(s, srgb, rcross, p, sl, col, o.first_r);
                        n_cf++;
                    }
                }
                if (!solved) {
                    if constexpr (FAM == kFam78df)
                        dray78df_start(R, s, HiLo{b.x, b.y}, HiLo{b.z, b.w}, HiLo{a.x, a.y}, HiLo{a.z, a.w});
                    else if constexpr (FAM == kFam78)
                        dray78_start(R, s, (double)b.x + (double)b.y, (double)b.z + (double)b.w,
                                     (double)a.x + (double)a.y, (double)a.z + (double)a.w);
                    else
                        dray_start(R, s, (double)b.x + (double)b.y, (double)b.z + (double)b.w,
                                   (double)a.x + (double)a.y, (double)a.z + (double)a.w);
                    have = true;
                }
            }
        }
        // rays solved in closed form leave their lanes free at once: the
        // warp stops only when its queue is drained as well
        if (!__any_sync(FULL, have)) {
            if (drained) break;
            continue;
        }
        if (have) {
            bool done;
            if constexpr (FAM == kFam78df) {
                bool acc;
                done = dray78df_step(R, s, acc);
                if (acc) { n_steps++; n_f64++; }
                n_evals += 13;
            } else if constexpr (FAM == kFam78) {
                bool acc;
                done = dray78_step(R, s, acc);
                if (acc) { n_steps++; n_f64++; }
                n_evals += 13;
            } else {
                done = dray_step(R, s);
                n_steps++; n_f64++; n_evals += 4;
            }
            if (done) {
                float col[3];
                sample_colour(s, R.status == 1, R.orders, R.disk, (float)R.min_r, cam_y, col);
                write_sample(s, srgb, rcross, p, sl, col, R.first_r);
                have = false;
            }
        }
    }
}

template <int MINB, int FAM>
__global__ void __launch_bounds__(kBlock, MINB)
render_mixed_kernel(const SceneDev s, const InitSoA soa, float* __restrict__ srgb, float* __restrict__ rcross,
                    float* __restrict__ inv3, Counters* __restrict__ ctr, int chunk) {
    const unsigned FULL = 0xffffffffu;
    const SpaceK k{(float)s.a, (float)(s.a * s.a), (float)s.M, (float)s.r_plus, (float)s.r_minus};
    unsigned long long n_rays = 0, n_steps = 0, n_f64 = 0, n_evals = 0, n_cf = 0;

    // ---- FP64 warps: near-critical rays.  Warp 0 of the first blocks starts
    // on them; every other warp joins once the FP32 queue is drained, so the
    // FP64 tail of a frame with many near-critical rays uses the whole grid.
    const long long D = (long long)ctr->deferred;
    const int nd = D > 0 ? (int)min((long long)gridDim.x, (D + 3) / 4) : 0;
    if ((threadIdx.x >> 5) == 0 && (int)blockIdx.x < nd)
        trace_deferred<FAM>(s, soa, srgb, rcross, ctr, D, n_rays, n_steps, n_f64, n_evals, n_cf);

    // ---- FP32 rays
    WarpQueue q{0, 0};
    bool drained = false, have = false;
    MRay<false> R;
    long long p = 0;
    int sl = 0;
    float cam_y = 0.0f;
    const int T = s.island_batch;
    while (true) {
        unsigned need = __ballot_sync(FULL, !have);
        if (need && !drained) {
            long long idx = warp_take(q, need, &ctr->work, s.total, chunk);
            drained = q.base >= s.total;
            if (!have && idx >= 0 && !soa.flag[idx]) {
                int x, y; uint32_t sid;
                ray_coords(s, idx, p, sl, x, y, sid);
                load_ray(soa, idx, R, cam_y);
                mray_start(R, s, k);
                if constexpr (FAM != kFamRk4) mray_set_k78(R, k);
                have = true;
                n_rays++;
                n_evals++;
            }
        }
        unsigned act = __ballot_sync(FULL, have && !R.pending);
        unsigned pend = __ballot_sync(FULL, have && R.pending);
        if (!(act | pend)) {
            if (drained) break;
            continue;
        }
        bool done = false;
        if (pend && ((int)__popc(pend) >= T || !act)) {
            if (have && R.pending) {
                if constexpr (FAM == kFam78df) {
                    int att;
                    done = mray_island78_df(R, s, k, att);
                    n_steps++; n_f64++; n_evals += 13 * att;
                } else if constexpr (FAM == kFam78) {
                    int att;
                    done = mray_island78(R, s, k, att);
                    n_steps++; n_f64++; n_evals += 13 * att;
                } else {
                    done = mray_island(R, s, k);
                    n_steps++; n_f64++; n_evals += 5;
                }
            }
        } else if (have && !R.pending) {
            // kStepsPerTurn FP32 steps (7(8): attempts) per pass of the
            // scheduling loop: the ballots and queue checks above are paid
            // once per pass; a lane that ends or parks early idles for the
            // rest of the pass
#pragma unroll 1
            for (int j = 0; j < kStepsPerTurn; ++j) {
                int r;
                if constexpr (FAM != kFamRk4) {
                    bool acc;
                    r = mray_step78(R, s, k, acc);
                    if (r != STEP_PARK) { n_steps += acc ? 1 : 0; n_evals += 13; }
                } else {
                    r = s.integrator == NP_INTEG_ADAPTIVE ? mray_step32_adaptive(R, s, k) : mray_step32(R, s, k);
                    if (r != STEP_PARK) { n_steps++; n_evals += s.integrator == NP_INTEG_ADAPTIVE ? 11 : 4; }
                }
                done = r == STEP_DONE;
                if (r != STEP_CONT) break;
            }
        }
        if (done) {
            if (FAM != kFamRk4 && R.status == 3) {
                // entered the horizon band: solved whole by band_cf_kernel
                const unsigned long long slot = atomicAdd(&ctr->band, 1ull);
                soa.list[D + (long long)slot] = (long long)sl * s.npix + p;
            } else {
                float col[3];
                sample_colour(s, R.status == 1, R.orders, R.disk, R.min_r, cam_y, col);
                write_sample(s, srgb, rcross, p, sl, col, R.first_r);
            }
            have = false;
        }
    }
    if (D > 0) trace_deferred<FAM>(s, soa, srgb, rcross, ctr, D, n_rays, n_steps, n_f64, n_evals, n_cf);
    flush_counters(ctr, n_rays, n_steps, n_f64, n_evals, n_cf);
}

// rgb[c][p] (+)= sum_s srgb[s][c][p], summed in sample order.
__global__ void resolve_kernel(const float* __restrict__ srgb, float* __restrict__ rgb,
                               long long npix, int spp, int accumulate) {
    long long n = 3 * npix;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        float acc = 0.0f;
        for (int sl = 0; sl < spp; ++sl) acc += srgb[(size_t)sl * n + i];
        rgb[i] = accumulate ? rgb[i] + acc : acc;
    }
}

// The first four equatorial crossings of a near-critical ray (any radius,
// up to the ray's end) in closed form, with their azimuths: the report of
// trace_rays_kernel for the rays the renderer solves in closed form.
__device__ __forceinline__ bool crit_cf_cross(const SceneDev& s, const Momentum& m, double* xr, double* xphi,
                                              int& ncross, int& st) {
    double l, q2, su, sm;
    if (!crit_constants(s, m, l, q2, su, sm)) return false;
    double xu[4], ph[4];
    int32_t xb[4];
    const double a = s.a / s.M, u0 = s.M / s.r_cam, uf = s.M / s.r_far;
    const gkcf::EqX x = gkcf::equator_crossings(a, l, q2, u0, s.cos_cam, su, sm, uf, 0.0, 1e300, 4, xu, nullptr, xb);
    if (x.status < 0) return false;
    if (x.n > 0) gkcf::crossing_phi(a, l, q2, u0, s.cos_cam, su, sm, uf, x.n, xu, xb, ph);
    for (int j = 0; j < x.n; ++j) { xr[j] = s.M / xu[j]; xphi[j] = s.ph_cam + ph[j]; }
    ncross = x.n;
    st = x.status;
    return true;
}

// Explicit rays (positions in continuous pixel coordinates), one per thread.
// The mixed path takes its island steps immediately (no batching) and
// traces near-critical rays with the FP64 Carter tracer, as the renderer does.
__global__ void trace_rays_kernel(const SceneDev s, int precision, int n, const double* __restrict__ px,
                                  const double* __restrict__ py, double* __restrict__ consts,
                                  double* __restrict__ cross, int32_t* __restrict__ status) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    CamDir dir = camera_dir(s, 0, 0, 0, true, px[i], py[i]);
    Momentum m = camera_momentum(s, dir);
    double E = -m.pt, L = m.pph;
    double Q = m.pth * m.pth + s.cos_cam * s.cos_cam * (L * L / (s.sin_cam * s.sin_cam) - s.a * s.a * E * E);
    if (consts) {
        consts[4 * i + 0] = m.pt; consts[4 * i + 1] = m.pph; consts[4 * i + 2] = m.pr; consts[4 * i + 3] = m.pth;
    }
    unsigned long long ev = 0;
    double xr[4] = {0, 0, 0, 0}, xphi[4] = {0, 0, 0, 0};
    int ncross, st;
    if (precision == NP_PREC_FP64) {
        RayFP64<true> R;
        fp64_init(s, m, R);
        if (s.integrator == NP_INTEG_RKF78) {
            while (!fp64_advance<kFp64Rkf78, false>(s, R, nullptr, ev)) {}
        } else {
            while (!fp64_advance<kFp64Rk4, false>(s, R, nullptr, ev)) {}
        }
        for (int j = 0; j < 4; ++j) { xr[j] = R.xr[j]; xphi[j] = R.xphi[j]; }
        ncross = R.crossings; st = R.status;
    } else if ((s.islands & kIslandCritical) && near_critical_screened(E, L, Q, s.a, s.M, s.r_plus, kCriticalDb) &&
               s.crit_cf && crit_cf_cross(s, m, xr, xphi, ncross, st)) {
        // solved in closed form
    } else if ((s.islands & kIslandCritical) && near_critical_screened(E, L, Q, s.a, s.M, s.r_plus, kCriticalDb)) {
        if (s.integrator == NP_INTEG_RKF78 && s.island_df) {
            DRay78df<true> R;
            dray78df_start(R, s, d_hl(E), d_hl(L), d_hl(m.pr), d_hl(m.pth));
            bool acc;
            while (!dray78df_step(R, s, acc)) {}
            for (int j = 0; j < 4; ++j) { xr[j] = R.xr[j]; xphi[j] = R.xphi[j]; }
            ncross = R.crossings; st = R.status;
        } else if (s.integrator == NP_INTEG_RKF78) {
            DRay78<true> R;
            dray78_start(R, s, E, L, m.pr, m.pth);
            bool acc;
            while (!dray78_step(R, s, acc)) {}
            for (int j = 0; j < 4; ++j) { xr[j] = R.xr[j]; xphi[j] = R.xphi[j]; }
            ncross = R.crossings; st = R.status;
        } else {
            DRay<true> R;
            dray_start(R, s, E, L, m.pr, m.pth);
            while (!dray_step(R, s)) {}
            for (int j = 0; j < 4; ++j) { xr[j] = R.xr[j]; xphi[j] = R.xphi[j]; }
            ncross = R.crossings; st = R.status;
        }
    } else if (s.integrator == NP_INTEG_RKF78) {
        const SpaceK k{(float)s.a, (float)(s.a * s.a), (float)s.M, (float)s.r_plus, (float)s.r_minus};
        MRay<true> R;
        R.pr = d_hl(m.pr); R.pth = d_hl(m.pth); R.E = d_hl(E); R.L = d_hl(L);
        mray_start(R, s, k);
        mray_set_k78(R, k);
        while (true) {
            bool acc;
            int r = mray_step78(R, s, k, acc);
            if (r == STEP_PARK) {
                int att;
                r = (s.island_df ? mray_island78_df(R, s, k, att) : mray_island78(R, s, k, att)) ? STEP_DONE : STEP_CONT;
            }
            if (r == STEP_DONE) break;
        }
        for (int j = 0; j < 4; ++j) { xr[j] = R.xr_d[j]; xphi[j] = R.xphi[j]; }
        ncross = R.crossings; st = R.status;
        if (st == 3) {
            // entered the horizon band: the whole ray in closed form, as the
            // renderer's band_cf_kernel (FP64 7(8) outside the closed forms)
            for (int j = 0; j < 4; ++j) { xr[j] = 0.0; xphi[j] = 0.0; }
            if (!crit_cf_cross(s, m, xr, xphi, ncross, st)) {
                DRay78<true> D;
                dray78_start(D, s, E, L, m.pr, m.pth);
                bool acc;
                while (!dray78_step(D, s, acc)) {}
                for (int j = 0; j < 4; ++j) { xr[j] = D.xr[j]; xphi[j] = D.xphi[j]; }
                ncross = D.crossings; st = D.status;
            }
        }
    } else {
        const SpaceK k{(float)s.a, (float)(s.a * s.a), (float)s.M, (float)s.r_plus, (float)s.r_minus};
        MRay<true> R;
        R.pr = d_hl(m.pr); R.pth = d_hl(m.pth); R.E = d_hl(E); R.L = d_hl(L);
        mray_start(R, s, k);
        while (true) {
            int r = s.integrator == NP_INTEG_ADAPTIVE ? mray_step32_adaptive(R, s, k) : mray_step32(R, s, k);
            if (r == STEP_PARK) r = mray_island(R, s, k) ? STEP_DONE : STEP_CONT;
            if (r == STEP_DONE) break;
        }
        for (int j = 0; j < 4; ++j) { xr[j] = R.xr_d[j]; xphi[j] = R.xphi[j]; }
        ncross = R.crossings; st = R.status;
    }
    if (cross) for (int j = 0; j < 4; ++j) { cross[8 * i + 2 * j] = xr[j]; cross[8 * i + 2 * j + 1] = xphi[j]; }
    if (status) status[i] = st + 16 * min(ncross, 15);
}

// Drift of H and Carter's Q along FP64 rays (explicit positions, one per thread).
__global__ void trace_invariants_kernel(const SceneDev s, int n, const double* __restrict__ px,
                                        const double* __restrict__ py, double* __restrict__ drift,
                                        int32_t* __restrict__ steps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    CamDir dir = camera_dir(s, 0, 0, 0, true, px[i], py[i]);
    Momentum m = camera_momentum(s, dir);
    unsigned long long ev = 0;
    RayFP64<false> R;
    fp64_init(s, m, R);
    if (s.integrator == NP_INTEG_RKF78) {
        while (!fp64_advance<kFp64Rkf78, true>(s, R, nullptr, ev)) {}
    } else {
        while (!fp64_advance<kFp64Rk4, true>(s, R, nullptr, ev)) {}
    }
    drift[2 * i] = R.dH;
    drift[2 * i + 1] = R.dQ;
    if (steps) steps[i] = R.step;
}

// Register-resident FMA throughput probe: 8 independent chains per thread.
template <typename T>
__global__ void fma_peak_kernel(T* out, int iters, T a, T b) {
    T x[8];
    for (int k = 0; k < 8; ++k) x[k] = (T)(threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = x[k] * a + b;
    }
    T s = 0;
    for (int k = 0; k < 8; ++k) s += x[k];
    if (s == (T)-1.2345) out[0] = s;   // keeps the loop live; never true for these inputs
}

// ---------------------------------------------------------------------------
// Per-(device, stream) scratch: per-sample colour planes, deferred list and
// counters.  Grows on demand; calls on the same stream reuse it in order.
struct Scratch {
    int device = -1;
    cudaStream_t stream = nullptr;
    float* srgb = nullptr; size_t srgb_n = 0;
    long long* list = nullptr; size_t list_n = 0;
    float4* soa_a = nullptr; float4* soa_b = nullptr; float* soa_cy = nullptr; unsigned char* soa_flag = nullptr;
    size_t soa_n = 0;
    Counters* ctr = nullptr;
    Counters* h_ctr = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
};
std::mutex g_scratch_mu;
std::vector<Scratch*> g_scratch;

int get_scratch(cudaStream_t stream, size_t srgb_n, size_t list_n, Scratch** out) {
    int dev = 0;
    NP_CU(cudaGetDevice(&dev), NP_ERR_NO_DEVICE);
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    Scratch* sc = nullptr;
    for (Scratch* s : g_scratch)
        if (s->device == dev && s->stream == stream) { sc = s; break; }
    if (!sc) {
        sc = new Scratch();
        sc->device = dev; sc->stream = stream;
        NP_CU(cudaMalloc(&sc->ctr, sizeof(Counters)), NP_ERR_ALLOC);
        NP_CU(cudaMallocHost(&sc->h_ctr, sizeof(Counters)), NP_ERR_ALLOC);
        NP_CU(cudaEventCreate(&sc->ev0), NP_ERR_KERNEL);
        NP_CU(cudaEventCreate(&sc->ev1), NP_ERR_KERNEL);
        NP_CU(cudaEventCreate(&sc->ev2), NP_ERR_KERNEL);
        g_scratch.push_back(sc);
    }
    if (sc->srgb_n < srgb_n) {
        if (sc->srgb) { cudaStreamSynchronize(stream); cudaFree(sc->srgb); sc->srgb = nullptr; sc->srgb_n = 0; }
        NP_CU(cudaMalloc(&sc->srgb, srgb_n * sizeof(float)), NP_ERR_ALLOC);
        sc->srgb_n = srgb_n;
    }
    if (sc->list_n < list_n) {
        if (sc->list) { cudaStreamSynchronize(stream); cudaFree(sc->list); sc->list = nullptr; sc->list_n = 0; }
        NP_CU(cudaMalloc(&sc->list, list_n * sizeof(long long)), NP_ERR_ALLOC);
        sc->list_n = list_n;
    }
    if (sc->soa_n < list_n && list_n > 1) {
        if (sc->soa_a) {
            cudaStreamSynchronize(stream);
            cudaFree(sc->soa_a); cudaFree(sc->soa_b); cudaFree(sc->soa_cy); cudaFree(sc->soa_flag);
            sc->soa_a = nullptr; sc->soa_b = nullptr; sc->soa_cy = nullptr; sc->soa_flag = nullptr; sc->soa_n = 0;
        }
        NP_CU(cudaMalloc(&sc->soa_a, list_n * sizeof(float4)), NP_ERR_ALLOC);
        NP_CU(cudaMalloc(&sc->soa_b, list_n * sizeof(float4)), NP_ERR_ALLOC);
        NP_CU(cudaMalloc(&sc->soa_cy, list_n * sizeof(float)), NP_ERR_ALLOC);
        NP_CU(cudaMalloc(&sc->soa_flag, list_n), NP_ERR_ALLOC);
        sc->soa_n = list_n;
    }
    *out = sc;
    return NP_OK;
}

int grid_for(const void* kernel) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, 0);
    if (per_sm < 1) per_sm = 1;
    return sms * per_sm;
}

// FP64 pass: one instantiation per integrator family, so the 7(8) pair's
// stage storage does not raise the register count of the RK4 kernel.
void launch_fp64(const SceneDev& s, float* srgb, float* rcross, float* inv3, Counters* ctr, cudaStream_t st) {
    if (s.integrator == NP_INTEG_RKF78) {
        render_fp64_kernel<kFp64Rkf78><<<grid_for((const void*)render_fp64_kernel<kFp64Rkf78>), kBlock, 0, st>>>(
            s, srgb, rcross, inv3, ctr);
    } else {
        render_fp64_kernel<kFp64Rk4><<<grid_for((const void*)render_fp64_kernel<kFp64Rk4>), kBlock, 0, st>>>(
            s, srgb, rcross, inv3, ctr);
    }
}

template <int MINB, int FAM>
void launch_mixed_t(const SceneDev& s, const InitSoA& soa, float* srgb, float* rc, float* inv3, Counters* ctr,
                    int chunk, cudaStream_t st) {
    render_mixed_kernel<MINB, FAM><<<grid_for((const void*)render_mixed_kernel<MINB, FAM>), kBlock, 0, st>>>(
        s, soa, srgb, rc, inv3, ctr, chunk);
}

// Register-cap variants of the mixed tracer (blocks of 128 threads per SM
// the compiler must fit: 3 -> 170 registers, 4 -> 128, 5 -> 102, 6 -> 85, 8 -> 64).
void launch_mixed(int minb, const SceneDev& s, const InitSoA& soa, float* srgb, float* rc, float* inv3,
                  Counters* ctr, int chunk, cudaStream_t st) {
    if (s.integrator == NP_INTEG_RKF78) {
        // the 7(8) loop holds about nine stage vectors: caps of 3 and 4 blocks only
        if (s.island_df) launch_mixed_t<4, kFam78df>(s, soa, srgb, rc, inv3, ctr, chunk, st);
        else if (g_tune.min_blocks78 == 4) launch_mixed_t<4, kFam78>(s, soa, srgb, rc, inv3, ctr, chunk, st);
        else launch_mixed_t<3, kFam78>(s, soa, srgb, rc, inv3, ctr, chunk, st);
        return;
    }
    switch (minb) {
        case 3: launch_mixed_t<3, kFamRk4>(s, soa, srgb, rc, inv3, ctr, chunk, st); break;
        case 5: launch_mixed_t<5, kFamRk4>(s, soa, srgb, rc, inv3, ctr, chunk, st); break;
        case 6: launch_mixed_t<6, kFamRk4>(s, soa, srgb, rc, inv3, ctr, chunk, st); break;
        case 8: launch_mixed_t<8, kFamRk4>(s, soa, srgb, rc, inv3, ctr, chunk, st); break;
        default: launch_mixed_t<4, kFamRk4>(s, soa, srgb, rc, inv3, ctr, chunk, st); break;
    }
}

// Long near-critical lists of a pass, in closed form before the tracer runs
// (the kernel returns at once for a short list).
void launch_critical(const SceneDev& s, const InitSoA& soa, float* srgb, float* rc, Counters* ctr,
                     unsigned long long list_cap, cudaStream_t st) {
    if (!(s.islands & kIslandCritical) || !s.crit_cf) return;
    critical_cf_kernel<<<np_device_sms() * 3, 128, 0, st>>>(s, soa, srgb, rc, ctr, list_cap);
}

// The horizon-band rays of a 7(8) pass, after the tracer.
void launch_band(const SceneDev& s, const InitSoA& soa, float* srgb, float* rc, Counters* ctr, cudaStream_t st) {
    if (!s.band_cf) return;
    band_cf_kernel<<<np_device_sms() * 3, 128, 0, st>>>(s, soa, srgb, rc, ctr);
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI.

extern "C" {

int np_abi_version(void) { return NP_ABI_VERSION; }

const char* np_last_error(void) { return g_last_error.c_str(); }

void np_scene_defaults(np_scene_t* s) {
    if (!s) return;
    std::memset(s, 0, sizeof(*s));
    s->width = 1280; s->height = 720; s->spp = 1; s->sample_offset = 0;
    s->mass = 10.0; s->spin = 0.0; s->r_cam = 50.0;
    s->theta_deg = 90.0; s->phi_deg = 0.0; s->fov_y_deg = 50.0;
    s->units = NP_UNITS_RS; s->camera = NP_CAMERA_STATIC;
    s->jitter = NP_JITTER_WANGHASH; s->seed = 0;
    s->integrator = NP_INTEG_RK4; s->max_steps = 10000;
    s->step_scale = 0.01; s->rtol = 1e-10; s->atol = 1e-12; s->escape_r = 0.0;
    s->disk_on = 1; s->disk_max_orders = 1; s->disk_rin = 0.0; s->disk_rout = 0.0;
    s->emissivity_q = 2.0; s->disk_gain = 1.0;
    s->crossing = NP_CROSS_LINEAR; s->background = NP_BG_GRADIENT;
    s->bg_sigma_deg = 1.0; s->bg_brightness = 3.0;
    s->check_invariants = 0; s->islands = NP_ISLANDS_DEFAULT;
}

int np_critical_curve(const np_scene_t* scene, float* rho) {
    if (!scene || !rho) return fail(NP_ERR_INVALID, "NULL argument");
    np_scene_t sc = *scene;
    sc.jitter = NP_JITTER_CRITICAL;
    SceneDev d;
    int rc = prepare_scene(sc, d);
    if (rc != NP_OK) return rc;
    for (int i = 0; i < kCritN; ++i) rho[i] = d.crit_rho[i];
    return NP_OK;
}

double np_isco_radius(double mass, double spin) {
    double a = spin;
    double z1 = 1.0 + std::cbrt(1.0 - a * a) * (std::cbrt(1.0 + a) + std::cbrt(1.0 - a));
    double z2 = std::sqrt(3.0 * a * a + z1 * z1);
    double sg = a >= 0.0 ? 1.0 : -1.0;
    return mass * (3.0 + z2 - sg * std::sqrt((3.0 - z1) * (3.0 + z1 + 2.0 * z2)));
}

void np_scene_benchmark(np_scene_t* s) {
    if (!s) return;
    np_scene_defaults(s);
    s->width = 1280; s->height = 720; s->spp = 4;
    s->mass = 1.0; s->spin = 0.9; s->r_cam = 50.0;
    s->theta_deg = 80.0; s->fov_y_deg = 55.0;
    s->units = NP_UNITS_M; s->jitter = NP_JITTER_STRATIFIED; s->seed = 0;
    s->max_steps = 4096; s->rtol = 1e-7; s->escape_r = 1000.0;
    s->disk_max_orders = 3; s->disk_rin = np_isco_radius(1.0, 0.9); s->disk_rout = 20.0;
    s->emissivity_q = 3.0; s->crossing = NP_CROSS_HERMITE;
}

int np_scene_validate(const np_scene_t* s) {
    if (!s) return fail(NP_ERR_INVALID, "scene is NULL");
    if (s->width <= 0 || s->height <= 0) return fail(NP_ERR_INVALID, "Invalid image dimensions.");
    if (s->spp <= 0) return fail(NP_ERR_INVALID, "Invalid samples per pixel.");
    if (s->sample_offset < 0) return fail(NP_ERR_INVALID, "Invalid sample offset.");
    if (!(s->mass > 0.0) || !(s->r_cam > 0.0) || !std::isfinite(s->mass) || !std::isfinite(s->r_cam))
        return fail(NP_ERR_INVALID, "Invalid mass or camera radius.");
    if (!(std::fabs(s->spin) < 1.0)) return fail(NP_ERR_INVALID, "Spin must satisfy |a/M| < 1.");
    if (!(s->fov_y_deg > 0.0 && s->fov_y_deg < 179.0))
        return fail(NP_ERR_INVALID, "Invalid FOV; expected (0, 179) degrees.");
    if (s->max_steps <= 0) return fail(NP_ERR_INVALID, "Invalid step cap.");
    if (!(s->step_scale > 0.0) || !std::isfinite(s->step_scale)) return fail(NP_ERR_INVALID, "Invalid step scale.");
    if (s->units != NP_UNITS_RS && s->units != NP_UNITS_M) return fail(NP_ERR_INVALID, "Invalid units.");
    if (s->jitter != NP_JITTER_WANGHASH && s->jitter != NP_JITTER_STRATIFIED && s->jitter != NP_JITTER_CRITICAL)
        return fail(NP_ERR_INVALID, "Invalid jitter mode.");
    if (s->integrator != NP_INTEG_RK4 && s->integrator != NP_INTEG_ADAPTIVE && s->integrator != NP_INTEG_RKF78)
        return fail(NP_ERR_INVALID, "Invalid integrator.");
    if (s->crossing != NP_CROSS_LINEAR && s->crossing != NP_CROSS_HERMITE && s->crossing != NP_CROSS_ROOT)
        return fail(NP_ERR_INVALID, "Invalid crossing mode.");
    if (!(s->inv_gate >= 0.0 && s->inv_gate < 1.0)) return fail(NP_ERR_INVALID, "Invalid invariant gate.");
    if (!(s->rtol_fp64 < 1.0) || !std::isfinite(s->rtol_fp64)) return fail(NP_ERR_INVALID, "Invalid FP64 tolerance.");
    if (s->island_arith != NP_ISLAND_ARITH_DF && s->island_arith != NP_ISLAND_ARITH_FP64)
        return fail(NP_ERR_INVALID, "Invalid island arithmetic.");
    if (s->critical_solver != NP_CRITICAL_CLOSED_FORM && s->critical_solver != NP_CRITICAL_INTEGRATE)
        return fail(NP_ERR_INVALID, "Invalid near-critical solver.");
    // non-finite values in any other field would only surface as NaN images
    auto fin = [](double v) { return std::isfinite(v); };
    if (!fin(s->theta_deg) || !fin(s->phi_deg)) return fail(NP_ERR_INVALID, "Invalid camera angle.");
    if (!(s->rtol > 0.0) || !(s->atol >= 0.0) || !fin(s->rtol) || !fin(s->atol))
        return fail(NP_ERR_INVALID, "Invalid tolerances.");
    if (!fin(s->escape_r)) return fail(NP_ERR_INVALID, "Invalid escape radius.");
    if (!fin(s->disk_rin) || !fin(s->disk_rout) || !fin(s->emissivity_q) || !fin(s->disk_gain))
        return fail(NP_ERR_INVALID, "Invalid disk parameters.");
    if (!fin(s->bg_sigma_deg) || !fin(s->bg_brightness)) return fail(NP_ERR_INVALID, "Invalid background parameters.");
    if ((long long)s->width * s->height > (1ll << 40) / std::max(1, s->spp))
        return fail(NP_ERR_INVALID, "Image too large.");
    return NP_OK;
}

// Root-found crossings on the mixed path exist for the embedded 7(8)
// integrator (Henon steps); the invariant gate exists on the FP64 path.
static int check_path(const np_scene_t& sc, int precision) {
    if (precision != NP_PREC_FP64 && precision != NP_PREC_MIXED) return fail(NP_ERR_INVALID, "Invalid precision.");
    if (precision == NP_PREC_MIXED && sc.crossing == NP_CROSS_ROOT && sc.integrator != NP_INTEG_RKF78)
        return fail(NP_ERR_INVALID, "Root crossings on precision mixed need the rkf78 integrator.");
    return NP_OK;
}

int np_render_device(const np_scene_t* scene, int precision, float* d_rgb, float* d_rcross, float* d_inv3,
                     int accumulate, void* stream_v, np_render_stats_t* stats) {
    if (!d_rgb || !scene) return fail(NP_ERR_INVALID, "NULL argument");
    if (int e = check_path(*scene, precision)) return e;
    SceneDev s;
    int rc = prepare_scene(*scene, s);
    if (rc != NP_OK) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return fail(NP_ERR_NO_DEVICE, "No CUDA devices found.");
    cudaStream_t st = (cudaStream_t)stream_v;
    Scratch* sc = nullptr;
    rc = get_scratch(st, (size_t)s.total * 3, precision == NP_PREC_MIXED ? (size_t)s.total : 1, &sc);
    if (rc != NP_OK) return rc;
    NP_CU(cudaMemsetAsync(sc->ctr, 0, sizeof(Counters), st), NP_ERR_KERNEL);
    if (stats) NP_CU(cudaEventRecord(sc->ev0, st), NP_ERR_KERNEL);
    if (precision == NP_PREC_FP64) {
        launch_fp64(s, sc->srgb, d_rcross, d_inv3, sc->ctr, st);
        NP_CU(cudaGetLastError(), NP_ERR_KERNEL);
        if (stats) NP_CU(cudaEventRecord(sc->ev1, st), NP_ERR_KERNEL);
    } else {
        InitSoA soa{sc->soa_a, sc->soa_b, sc->soa_cy, sc->soa_flag, sc->list};
        int ib = (int)std::min<long long>((s.total + 255) / 256, (long long)np_device_sms() * 8);
        ray_init_kernel<<<ib, 256, 0, st>>>(s, soa, sc->ctr);
        NP_CU(cudaGetLastError(), NP_ERR_KERNEL);
        if (stats) NP_CU(cudaEventRecord(sc->ev1, st), NP_ERR_KERNEL);
        launch_critical(s, soa, sc->srgb, d_rcross, sc->ctr, (unsigned long long)s.total, st);
        NP_CU(cudaGetLastError(), NP_ERR_KERNEL);
        launch_mixed(g_tune.min_blocks, s, soa, sc->srgb, d_rcross, d_inv3, sc->ctr, g_tune.chunk, st);
        NP_CU(cudaGetLastError(), NP_ERR_KERNEL);
        launch_band(s, soa, sc->srgb, d_rcross, sc->ctr, st);
        NP_CU(cudaGetLastError(), NP_ERR_KERNEL);
    }
    if (stats) NP_CU(cudaEventRecord(sc->ev2, st), NP_ERR_KERNEL);
    {
        long long n = 3 * s.npix;
        int blocks = (int)std::min<long long>((n + 255) / 256, (long long)np_device_sms() * 16);
        resolve_kernel<<<blocks, 256, 0, st>>>(sc->srgb, d_rgb, s.npix, s.spp, accumulate);
        NP_CU(cudaGetLastError(), NP_ERR_KERNEL);
    }
    if (stats) {
        NP_CU(cudaMemcpyAsync(sc->h_ctr, sc->ctr, sizeof(Counters), cudaMemcpyDeviceToHost, st), NP_ERR_KERNEL);
        NP_CU(cudaStreamSynchronize(st), NP_ERR_KERNEL);
        float ms = 0.0f, ms2 = 0.0f;
        if (precision == NP_PREC_FP64) {
            cudaEventElapsedTime(&ms, sc->ev0, sc->ev1);
        } else {   // ev0 -> ev1: ray init, ev1 -> ev2: tracer
            cudaEventElapsedTime(&ms2, sc->ev0, sc->ev1);
            cudaEventElapsedTime(&ms, sc->ev1, sc->ev2);
        }
        stats->rays = sc->h_ctr->rays;
        stats->steps = sc->h_ctr->steps;
        stats->fp64_steps = sc->h_ctr->fp64_steps;
        stats->rhs_evals = sc->h_ctr->evals;
        stats->deferred_rays = precision == NP_PREC_MIXED ? sc->h_ctr->deferred : 0;
        stats->closed_form_rays = sc->h_ctr->closed_form;
        stats->band_rays = sc->h_ctr->band;
        stats->kernel_ms = ms;
        stats->init_ms = ms2;
    }
    return NP_OK;
}

int np_render_host(const np_scene_t* scene, int precision, float* h_rgb, float* h_rcross, float* h_inv3,
                   np_render_stats_t* stats) {
    if (!scene || !h_rgb) return fail(NP_ERR_INVALID, "NULL argument");
    int rc = np_scene_validate(scene);
    if (rc != NP_OK) return rc;
    if (int e = check_path(*scene, precision)) return e;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return fail(NP_ERR_NO_DEVICE, "No CUDA devices found.");
    size_t npix = (size_t)scene->width * scene->height;
    // device staging buffers, cached per host thread and grown on demand
    thread_local float* d_buf = nullptr;
    thread_local size_t d_cap = 0;
    thread_local int d_dev = -1;
    int dev = 0;
    NP_CU(cudaGetDevice(&dev), NP_ERR_NO_DEVICE);
    size_t need = 4 * npix + 4;
    if (d_buf && (d_cap < need || d_dev != dev)) { cudaFree(d_buf); d_buf = nullptr; d_cap = 0; }
    if (!d_buf) {
        NP_CU(cudaMalloc(&d_buf, need * sizeof(float)), NP_ERR_ALLOC);
        d_cap = need; d_dev = dev;
    }
    float* d_rgb = d_buf;
    float* d_rc = h_rcross ? d_buf + 3 * npix : nullptr;
    float* d_inv = h_inv3 ? d_buf + 4 * npix : nullptr;
    cudaStream_t st = nullptr;
    if (h_inv3) NP_CU(cudaMemcpyAsync(d_inv, h_inv3, 3 * sizeof(float), cudaMemcpyHostToDevice, st), NP_ERR_KERNEL);
    rc = np_render_device(scene, precision, d_rgb, d_rc, d_inv, 0, st, stats);
    if (rc != NP_OK) return rc;
    NP_CU(cudaMemcpyAsync(h_rgb, d_rgb, 3 * npix * sizeof(float), cudaMemcpyDeviceToHost, st), NP_ERR_KERNEL);
    if (h_rcross) NP_CU(cudaMemcpyAsync(h_rcross, d_rc, npix * sizeof(float), cudaMemcpyDeviceToHost, st), NP_ERR_KERNEL);
    if (h_inv3) NP_CU(cudaMemcpyAsync(h_inv3, d_inv, 3 * sizeof(float), cudaMemcpyDeviceToHost, st), NP_ERR_KERNEL);
    NP_CU(cudaStreamSynchronize(st), NP_ERR_KERNEL);
    return NP_OK;
}

int np_trace_rays_device(const np_scene_t* scene, int precision, int n, const double* d_px, const double* d_py,
                         double* d_consts, double* d_cross, int32_t* d_status, void* stream_v) {
    if (n < 0 || (n > 0 && (!d_px || !d_py)) || !scene) return fail(NP_ERR_INVALID, "bad ray arrays");
    if (int e = check_path(*scene, precision)) return e;
    SceneDev s;
    int rc = prepare_scene(*scene, s);
    if (rc != NP_OK) return rc;
    if (n == 0) return NP_OK;
    cudaStream_t st = (cudaStream_t)stream_v;
    trace_rays_kernel<<<(n + 127) / 128, 128, 0, st>>>(s, precision, n, d_px, d_py, d_consts, d_cross, d_status);
    NP_CU(cudaGetLastError(), NP_ERR_KERNEL);
    return NP_OK;
}

int np_trace_invariants_device(const np_scene_t* scene, int n, const double* d_px, const double* d_py,
                               double* d_drift, int32_t* d_steps, void* stream_v) {
    if (n < 0 || (n > 0 && (!d_px || !d_py || !d_drift)) || !scene) return fail(NP_ERR_INVALID, "bad ray arrays");
    SceneDev s;
    int rc = prepare_scene(*scene, s);
    if (rc != NP_OK) return rc;
    if (n == 0) return NP_OK;
    cudaStream_t st = (cudaStream_t)stream_v;
    trace_invariants_kernel<<<(n + 127) / 128, 128, 0, st>>>(s, n, d_px, d_py, d_drift, d_steps);
    NP_CU(cudaGetLastError(), NP_ERR_KERNEL);
    return NP_OK;
}

int np_tune(int param, int value) {
    switch (param) {
        case NP_TUNE_CROSS_BATCH:
            if (value < 1 || value > 32) return fail(NP_ERR_INVALID, "crossing batch must be in [1, 32]");
            g_tune.cross_batch = value;
            return NP_OK;
        case NP_TUNE_ISLAND_BATCH:
            if (value < 1 || value > 32) return fail(NP_ERR_INVALID, "island batch must be in [1, 32]");
            g_tune.island_batch = value;
            return NP_OK;
        case NP_TUNE_MIN_BLOCKS:
            if (value != 3 && value != 4 && value != 5 && value != 6 && value != 8)
                return fail(NP_ERR_INVALID, "min blocks must be one of 3, 4, 5, 6, 8");
            g_tune.min_blocks = value;
            return NP_OK;
        case NP_TUNE_CHUNK:
            if (value < 1 || value > 4096) return fail(NP_ERR_INVALID, "chunk must be in [1, 4096]");
            g_tune.chunk = value;
            return NP_OK;
        case NP_TUNE_ISLAND_BATCH78:
            if (value < 1 || value > 32) return fail(NP_ERR_INVALID, "island batch must be in [1, 32]");
            g_tune.island_batch78 = value;
            return NP_OK;
        case NP_TUNE_MIN_BLOCKS78:
            if (value != 3 && value != 4) return fail(NP_ERR_INVALID, "min blocks of the 7(8) tracer must be 3 or 4");
            g_tune.min_blocks78 = value;
            return NP_OK;
        default:
            return fail(NP_ERR_INVALID, "unknown tuning parameter %d", param);
    }
}

int np_measure_fma_peak(int which, double* tflops) {
    if (!tflops || (which != 0 && which != 1)) return fail(NP_ERR_INVALID, "bad arguments");
    int dev = 0, sms = 0;
    NP_CU(cudaGetDevice(&dev), NP_ERR_NO_DEVICE);
    NP_CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), NP_ERR_NO_DEVICE);
    void* out = nullptr;
    NP_CU(cudaMalloc(&out, 16), NP_ERR_ALLOC);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0); cudaEventCreate(&e1);
    const int threads = 256, blocks = sms * 8;
    const int iters = which == 0 ? 1 << 16 : 1 << 11;
    double best = 0.0;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        if (which == 0) fma_peak_kernel<float><<<blocks, threads>>>((float*)out, iters, 0.999f, 0.001f);
        else fma_peak_kernel<double><<<blocks, threads>>>((double*)out, iters, 0.999, 0.001);
        cudaEventRecord(e1);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) { cudaFree(out); return fail(NP_ERR_KERNEL, "peak kernel: %s", cudaGetErrorString(e)); }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        double flops = 2.0 * 8.0 * (double)iters * threads * blocks;
        if (rep > 0) best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    cudaFree(out);
    *tflops = best;
    return NP_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free render pass.  Its scratch (counters, per-sample colours,
// ray-generation arrays, deferred list) lives in one file-scope device array
// sized for NP_NOALLOC_MAX_RAYS rays; each device's copy is looked up once
// with cudaGetSymbolAddress and reused.  Calls share the array.

namespace {

constexpr size_t na_align(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kNaRays = NP_NOALLOC_MAX_RAYS;
constexpr size_t kNaCtr = 0;
constexpr size_t kNaSrgb = kNaCtr + na_align(sizeof(Counters));
constexpr size_t kNaA = kNaSrgb + na_align(3 * kNaRays * sizeof(float));
constexpr size_t kNaB = kNaA + na_align(kNaRays * sizeof(float4));
constexpr size_t kNaCy = kNaB + na_align(kNaRays * sizeof(float4));
constexpr size_t kNaFlag = kNaCy + na_align(kNaRays * sizeof(float));
constexpr size_t kNaList = kNaFlag + na_align(kNaRays);
constexpr size_t kNaBytes = kNaList + na_align(kNaRays * sizeof(long long));

__device__ __align__(256) unsigned char g_na_scratch[kNaBytes];

constexpr int kNaMaxDevices = 64;
unsigned char* g_na_ptr[kNaMaxDevices] = {};
std::mutex g_na_mu;

}  // namespace

extern "C" int np_render_device_noalloc(const np_scene_t* scene, int precision, float* d_rgb, float* d_rcross,
                                        int accumulate, void* stream_v) {
    if (!scene || !d_rgb) return fail(NP_ERR_INVALID, "scene or rgb buffer is NULL");
    if (int e = check_path(*scene, precision)) return e;
    SceneDev s;
    int rc = prepare_scene(*scene, s);
    if (rc != NP_OK) return rc;
    if (s.total > (long long)kNaRays)
        return fail(NP_ERR_INVALID, "pass of %lld rays exceeds NP_NOALLOC_MAX_RAYS (%lld); split the samples "
                    "over several calls", s.total, (long long)kNaRays);
    int dev = 0;
    NP_CU(cudaGetDevice(&dev), NP_ERR_NO_DEVICE);
    if (dev < 0 || dev >= kNaMaxDevices) return fail(NP_ERR_INVALID, "device index %d out of range", dev);
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_na_mu);
        if (!g_na_ptr[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_na_scratch);
            if (e != cudaSuccess || !p)
                return fail(NP_ERR_NO_DEVICE, "cudaGetSymbolAddress of the scratch array failed: %s",
                            cudaGetErrorString(e));
            g_na_ptr[dev] = (unsigned char*)p;
        }
        base = g_na_ptr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream_v;
    Counters* ctr = (Counters*)(base + kNaCtr);
    float* srgb = (float*)(base + kNaSrgb);
    NP_CU(cudaMemsetAsync(ctr, 0, sizeof(Counters), st), NP_ERR_KERNEL);
    if (precision == NP_PREC_FP64) {
        launch_fp64(s, srgb, d_rcross, nullptr, ctr, st);
    } else {
        InitSoA soa{(float4*)(base + kNaA), (float4*)(base + kNaB), (float*)(base + kNaCy),
                    (unsigned char*)(base + kNaFlag), (long long*)(base + kNaList)};
        int ib = (int)std::min<long long>((s.total + 255) / 256, (long long)np_device_sms() * 8);
        ray_init_kernel<<<ib, 256, 0, st>>>(s, soa, ctr);
        NP_CU(cudaGetLastError(), NP_ERR_KERNEL);
        launch_critical(s, soa, srgb, d_rcross, ctr, (unsigned long long)s.total, st);
        NP_CU(cudaGetLastError(), NP_ERR_KERNEL);
        launch_mixed(g_tune.min_blocks, s, soa, srgb, d_rcross, nullptr, ctr, g_tune.chunk, st);
        NP_CU(cudaGetLastError(), NP_ERR_KERNEL);
        launch_band(s, soa, srgb, d_rcross, ctr, st);
    }
    NP_CU(cudaGetLastError(), NP_ERR_KERNEL);
    long long n = 3 * s.npix;
    int blocks = (int)std::min<long long>((n + 255) / 256, (long long)np_device_sms() * 16);
    resolve_kernel<<<blocks, 256, 0, st>>>(srgb, d_rgb, s.npix, s.spp, accumulate);
    NP_CU(cudaGetLastError(), NP_ERR_KERNEL);
    return NP_OK;
}

// ---------------------------------------------------------------------------
// Batched scenes: many scenes of uneven size, spin, inclination, spp and disk
// orders traced by one persistent launch of the mixed path over a single
// device-side ray queue.  Ray index i belongs to the scene s with
// ray_off[s] <= i < ray_off[s + 1]; lanes of one warp may hold rays of
// different scenes, so each lane keeps a pointer to its scene's constants
// (a few hundred bytes per scene, read through L1).  The sequence
// (counter reset, ray generation, tracing, resolve) is captured once into a
// CUDA graph and replayed.

namespace {

struct BatchDev {
    const SceneDev* __restrict__ scenes;
    const long long* __restrict__ ray_off;    // [n + 1]
    const long long* __restrict__ pix_off;    // [n + 1]
    int n;
    long long total, total_pix;
    unsigned long long list_cap;
    float* srgb;                   // scene s at 3 ray_off[s]: [spp][3][npix]
    float* rgb;                    // scene s at 3 pix_off[s]: [3][npix]
    float* rcross;                 // scene s at pix_off[s]
    unsigned* done;                // finished rays per scene
    unsigned long long* t_done;    // %globaltimer when a scene's last ray finished
    unsigned long long* t_start;   // %globaltimer at the start of ray generation
    InitSoA soa;
    Counters* ctr;
};

// Largest s in [0, n) with off[s] <= i.
__device__ __forceinline__ int find_seg(const long long* __restrict__ off, int n, long long i) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void batch_write(const BatchDev& B, int sc, const SceneDev& S, long long p, int sl,
                                            const float col[3], double first_r) {
    write_sample(S, B.srgb + 3 * B.ray_off[sc], B.rcross + B.pix_off[sc], p, sl, col, first_r);
    unsigned d = atomicAdd(&B.done[sc], 1u) + 1u;
    if ((long long)d == S.total) B.t_done[sc] = global_ns();
}

__global__ void __launch_bounds__(256) batch_init_kernel(const BatchDev B) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *B.t_start = global_ns();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < B.total;
         i += (long long)gridDim.x * blockDim.x) {
        const int sc = find_seg(B.ray_off, B.n, i);
        init_one(B.scenes[sc], i - B.ray_off[sc], i, B.soa, B.ctr, B.list_cap);
    }
}

template <int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) batch_mixed_kernel(const BatchDev B, int chunk, int T) {
    const unsigned FULL = 0xffffffffu;
    Counters* ctr = B.ctr;
    const InitSoA& soa = B.soa;
    unsigned long long n_rays = 0, n_steps = 0, n_f64 = 0, n_evals = 0, n_cf = 0;

    // ---- FP64 warps: near-critical rays of every scene
    const long long D = (long long)min(ctr->deferred, B.list_cap);
    const int nd = D > 0 ? (int)min((long long)gridDim.x, (D + 3) / 4) : 0;
    if ((threadIdx.x >> 5) == 0 && (int)blockIdx.x < nd) {
        WarpQueue q{0, 0};
        bool drained = false, have = false;
        DRay<false> R;
        const SceneDev* sp = B.scenes;
        int sc = 0;
        long long p = 0;
        int sl = 0;
        float cam_y = 0.0f;
        while (true) {
            unsigned need = __ballot_sync(FULL, !have);
            if (need && !drained) {
                long long idx = warp_take(q, need, &ctr->work2, D, 4);
                drained = q.base >= D;
                if (!have && idx >= 0) {
                    const long long item = soa.list[idx];
                    sc = find_seg(B.ray_off, B.n, item);
                    sp = B.scenes + sc;
                    int x, y; uint32_t sid;
                    ray_coords(*sp, item - B.ray_off[sc], p, sl, x, y, sid);
                    float4 a = soa.a[item], b = soa.b[item];
                    cam_y = soa.cy[item];
                    n_rays++;
                    bool solved = false;
                    if (sp->crit_cf) {
                        const CamDir dir = camera_dir(*sp, x, y, sid, false, 0.0, 0.0);
                        CritCF o;
                        solved = crit_cf_solve(*sp, camera_momentum(*sp, dir), o);
                        if (solved) {
                            float col[3];
                            sample_colour(*sp, o.status == 1, o.orders, o.disk, (float)o.min_r, cam_y, col);
                            batch_write(B, sc, *sp, p, sl, col, o.first_r);
                            n_cf++;
                        }
                    }
                    if (!solved) {
                        dray_start(R, *sp, (double)b.x + (double)b.y, (double)b.z + (double)b.w,
                                   (double)a.x + (double)a.y, (double)a.z + (double)a.w);
                        have = true;
                    }
                }
            }
            if (!__any_sync(FULL, have)) {
                if (drained) break;
                continue;
            }
            if (have) {
                bool done = dray_step(R, *sp);
                n_steps++; n_f64++; n_evals += 4;
                if (done) {
                    float col[3];
                    sample_colour(*sp, R.status == 1, R.orders, R.disk, (float)R.min_r, cam_y, col);
                    batch_write(B, sc, *sp, p, sl, col, R.first_r);
                    have = false;
                }
            }
        }
    }

    // ---- FP32 rays (the loop of render_mixed_kernel with a per-lane scene)
    WarpQueue q{0, 0};
    bool drained = false, have = false;
    MRay<false> R;
    const SceneDev* sp = B.scenes;
    SpaceK k{0.0f, 0.0f, 1.0f, 1.0f, 0.0f};
    int sc = 0;
    long long p = 0;
    int sl = 0;
    float cam_y = 0.0f;
    while (true) {
        unsigned need = __ballot_sync(FULL, !have);
        if (need && !drained) {
            long long idx = warp_take(q, need, &ctr->work, B.total, chunk);
            drained = q.base >= B.total;
            if (!have && idx >= 0 && !soa.flag[idx]) {
                sc = find_seg(B.ray_off, B.n, idx);
                sp = B.scenes + sc;
                const SceneDev& S = *sp;
                k = SpaceK{(float)S.a, (float)(S.a * S.a), (float)S.M, (float)S.r_plus, (float)S.r_minus};
                int x, y; uint32_t sid;
                ray_coords(S, idx - B.ray_off[sc], p, sl, x, y, sid);
                load_ray(soa, idx, R, cam_y);
                mray_start(R, S, k);
                have = true;
                n_rays++;
                n_evals++;
            }
        }
        unsigned act = __ballot_sync(FULL, have && !R.pending);
        unsigned pend = __ballot_sync(FULL, have && R.pending);
        if (!(act | pend)) {
            if (drained) break;
            continue;
        }
        bool done = false;
        const SceneDev& S = *sp;
        if (pend && ((int)__popc(pend) >= T || !act)) {
            if (have && R.pending) {
                done = mray_island(R, S, k);
                n_steps++; n_f64++; n_evals += 5;
            }
        } else if (have && !R.pending) {
#pragma unroll 1
            for (int j = 0; j < kStepsPerTurn; ++j) {
                int r = S.integrator == NP_INTEG_ADAPTIVE ? mray_step32_adaptive(R, S, k) : mray_step32(R, S, k);
                if (r != STEP_PARK) { n_steps++; n_evals += S.integrator == NP_INTEG_ADAPTIVE ? 11 : 4; }
                done = r == STEP_DONE;
                if (r != STEP_CONT) break;
            }
        }
        if (done) {
            float col[3];
            sample_colour(S, R.status == 1, R.orders, R.disk, R.min_r, cam_y, col);
            batch_write(B, sc, S, p, sl, col, R.first_r);
            have = false;
        }
    }
    flush_counters(ctr, n_rays, n_steps, n_f64, n_evals, n_cf);
}

__global__ void batch_resolve_kernel(const BatchDev B) {
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < B.total_pix;
         j += (long long)gridDim.x * blockDim.x) {
        const int sc = find_seg(B.pix_off, B.n, j);
        const SceneDev& S = B.scenes[sc];
        const long long p = j - B.pix_off[sc];
        const float* src = B.srgb + 3 * B.ray_off[sc];
        float* dst = B.rgb + 3 * B.pix_off[sc];
        for (int c = 0; c < 3; ++c) {
            float acc = 0.0f;
            for (int s = 0; s < S.spp; ++s) acc += src[((size_t)s * 3 + c) * S.npix + p];
            dst[(size_t)c * S.npix + p] = acc;
        }
    }
}

// Launch-shape variants the autotuner chooses from: threads per block and
// the blocks per SM the register allocation must allow.
struct BatchShape { int block, minb; };
constexpr BatchShape kBatchShapes[] = {{128, 4}, {64, 8}, {256, 2}, {128, 3}, {128, 5}};
constexpr int kNumBatchShapes = sizeof(kBatchShapes) / sizeof(kBatchShapes[0]);

struct BatchTune { int shape = 0, chunk = 64, island_batch = 8; };
BatchTune g_btune;
int g_btune_epoch = 0;

// Persistent grid of each shape: SMs x resident blocks (queried once per
// batch, before any graph capture).
template <int BLOCK, int MINB>
int batch_grid_t(int sms) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_mixed_kernel<BLOCK, MINB>, BLOCK, 0);
    return sms * std::max(1, per_sm);
}

int batch_grid(int shape, int sms) {
    switch (shape) {
        case 1: return batch_grid_t<64, 8>(sms);
        case 2: return batch_grid_t<256, 2>(sms);
        case 3: return batch_grid_t<128, 3>(sms);
        case 4: return batch_grid_t<128, 5>(sms);
        default: return batch_grid_t<128, 4>(sms);
    }
}

void batch_launch(const BatchDev& B, const BatchTune& t, int grid, cudaStream_t st) {
    switch (t.shape) {
        case 1: batch_mixed_kernel<64, 8><<<grid, 64, 0, st>>>(B, t.chunk, t.island_batch); break;
        case 2: batch_mixed_kernel<256, 2><<<grid, 256, 0, st>>>(B, t.chunk, t.island_batch); break;
        case 3: batch_mixed_kernel<128, 3><<<grid, 128, 0, st>>>(B, t.chunk, t.island_batch); break;
        case 4: batch_mixed_kernel<128, 5><<<grid, 128, 0, st>>>(B, t.chunk, t.island_batch); break;
        default: batch_mixed_kernel<128, 4><<<grid, 128, 0, st>>>(B, t.chunk, t.island_batch); break;
    }
}

}  // namespace

struct np_batch {
    int device = -1;
    int n = 0;
    cudaStream_t stream = nullptr;
    std::vector<long long> ray_off, pix_off;     // in queue order
    std::vector<long long> npix;                 // by caller index
    std::vector<int> pos;                        // caller index -> queue position
    BatchDev B{};
    void* mem = nullptr;
    Counters* h_ctr = nullptr;
    unsigned long long* h_times = nullptr;     // [n + 1]: t_done[0..n), t_start
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaGraphExec_t graph = nullptr;
    int graph_epoch = -1;
    BatchTune graph_tune{};
    int grid[8] = {};
};

namespace {

void batch_free(np_batch* b) {
    if (!b) return;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->mem) cudaFree(b->mem);
    if (b->h_ctr) cudaFreeHost(b->h_ctr);
    if (b->h_times) cudaFreeHost(b->h_times);
    if (b->e0) cudaEventDestroy(b->e0);
    if (b->e1) cudaEventDestroy(b->e1);
    delete b;
}

// Enqueues one batch pass (no host synchronisation).
int batch_enqueue(np_batch* b, const BatchTune& t, cudaStream_t st) {
    const BatchDev& B = b->B;
    NP_CU(cudaMemsetAsync(B.ctr, 0, sizeof(Counters), st), NP_ERR_KERNEL);
    NP_CU(cudaMemsetAsync(B.done, 0, (size_t)b->n * sizeof(unsigned), st), NP_ERR_KERNEL);
    const int ib = (int)std::min<long long>((B.total + 255) / 256, (long long)np_device_sms() * 8);
    batch_init_kernel<<<ib, 256, 0, st>>>(B);
    NP_CU(cudaGetLastError(), NP_ERR_KERNEL);
    batch_launch(B, t, b->grid[t.shape], st);
    NP_CU(cudaGetLastError(), NP_ERR_KERNEL);
    const int rb = (int)std::min<long long>((B.total_pix + 255) / 256, (long long)np_device_sms() * 16);
    batch_resolve_kernel<<<rb, 256, 0, st>>>(B);
    NP_CU(cudaGetLastError(), NP_ERR_KERNEL);
    return NP_OK;
}

}  // namespace

extern "C" {

np_batch_t* np_batch_create(const np_scene_t* scenes, int n, int precision, void* stream) {
    if (!scenes || n < 1) { fail(NP_ERR_INVALID, "scenes is NULL or n < 1"); return nullptr; }
    if (precision != NP_PREC_MIXED) {
        fail(NP_ERR_INVALID, "batched scenes run the mixed-precision path");
        return nullptr;
    }
    std::vector<SceneDev> byidx((size_t)n), devs((size_t)n);
    np_batch* b = new np_batch();
    b->n = n;
    b->stream = (cudaStream_t)stream;
    b->ray_off.assign((size_t)n + 1, 0);
    b->pix_off.assign((size_t)n + 1, 0);
    for (int i = 0; i < n; ++i) {
        int rc = check_path(scenes[i], NP_PREC_MIXED);
        if (rc == NP_OK && scenes[i].integrator == NP_INTEG_RKF78)
            rc = fail(NP_ERR_INVALID, "the 7(8) integrator runs one scene per launch (np_render_device)");
        if (rc == NP_OK) rc = prepare_scene(scenes[i], byidx[(size_t)i]);
        if (rc != NP_OK) {
            std::string msg = g_last_error;
            batch_free(b);
            fail(rc, "scene %d: %s", i, msg.c_str());
            return nullptr;
        }
        b->npix.push_back(byidx[(size_t)i].npix);
    }
    // Queue order: fewest rays first (shortest job first), which minimises
    // the mean scene completion time of a FIFO ray queue; ties keep caller order.
    std::vector<int> order((size_t)n);
    for (int i = 0; i < n; ++i) order[(size_t)i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int x, int y) { return byidx[(size_t)x].total < byidx[(size_t)y].total; });
    b->pos.assign((size_t)n, 0);
    for (int q = 0; q < n; ++q) {
        const SceneDev& d = byidx[(size_t)order[(size_t)q]];
        devs[(size_t)q] = d;
        b->pos[(size_t)order[(size_t)q]] = q;
        b->ray_off[(size_t)q + 1] = b->ray_off[(size_t)q] + d.total;
        b->pix_off[(size_t)q + 1] = b->pix_off[(size_t)q] + d.npix;
    }
    const long long total = b->ray_off[(size_t)n], total_pix = b->pix_off[(size_t)n];
    const unsigned long long list_cap = (unsigned long long)std::max<long long>(1024, total / 64);
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    size_t off = 0;
    const size_t o_scenes = off; off += al(sizeof(SceneDev) * (size_t)n);
    const size_t o_roff = off; off += al(sizeof(long long) * ((size_t)n + 1));
    const size_t o_poff = off; off += al(sizeof(long long) * ((size_t)n + 1));
    const size_t o_srgb = off; off += al(sizeof(float) * 3 * (size_t)total);
    const size_t o_rgb = off; off += al(sizeof(float) * 3 * (size_t)total_pix);
    const size_t o_rc = off; off += al(sizeof(float) * (size_t)total_pix);
    const size_t o_done = off; off += al(sizeof(unsigned) * (size_t)n);
    const size_t o_tdone = off; off += al(sizeof(unsigned long long) * ((size_t)n + 1));
    const size_t o_a = off; off += al(sizeof(float4) * (size_t)total);
    const size_t o_b = off; off += al(sizeof(float4) * (size_t)total);
    const size_t o_cy = off; off += al(sizeof(float) * (size_t)total);
    const size_t o_flag = off; off += al((size_t)total);
    const size_t o_list = off; off += al(sizeof(long long) * (size_t)list_cap);
    const size_t o_ctr = off; off += al(sizeof(Counters));
    if (cudaGetDevice(&b->device) != cudaSuccess || cudaMalloc(&b->mem, off) != cudaSuccess ||
        cudaMallocHost(&b->h_ctr, sizeof(Counters)) != cudaSuccess ||
        cudaMallocHost(&b->h_times, sizeof(unsigned long long) * ((size_t)n + 1)) != cudaSuccess ||
        cudaEventCreate(&b->e0) != cudaSuccess || cudaEventCreate(&b->e1) != cudaSuccess) {
        cudaGetLastError();
        batch_free(b);
        fail(NP_ERR_ALLOC, "device allocation of %zu bytes for %d scenes failed", off, n);
        return nullptr;
    }
    unsigned char* m = (unsigned char*)b->mem;
    BatchDev& B = b->B;
    B.scenes = (const SceneDev*)(m + o_scenes);
    B.ray_off = (const long long*)(m + o_roff);
    B.pix_off = (const long long*)(m + o_poff);
    B.n = n; B.total = total; B.total_pix = total_pix; B.list_cap = list_cap;
    B.srgb = (float*)(m + o_srgb); B.rgb = (float*)(m + o_rgb); B.rcross = (float*)(m + o_rc);
    B.done = (unsigned*)(m + o_done);
    B.t_done = (unsigned long long*)(m + o_tdone);
    B.t_start = B.t_done + n;
    B.soa = InitSoA{(float4*)(m + o_a), (float4*)(m + o_b), (float*)(m + o_cy), (unsigned char*)(m + o_flag),
                    (long long*)(m + o_list)};
    B.ctr = (Counters*)(m + o_ctr);
    if (cudaMemcpy((void*)B.scenes, devs.data(), sizeof(SceneDev) * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy((void*)B.ray_off, b->ray_off.data(), sizeof(long long) * ((size_t)n + 1),
                   cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy((void*)B.pix_off, b->pix_off.data(), sizeof(long long) * ((size_t)n + 1),
                   cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(B.rcross, 0, sizeof(float) * (size_t)total_pix) != cudaSuccess) {
        cudaGetLastError();
        batch_free(b);
        fail(NP_ERR_KERNEL, "upload of the scene table failed");
        return nullptr;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    for (int i = 0; i < kNumBatchShapes; ++i) b->grid[i] = batch_grid(i, std::max(1, sms));
    return b;
}

void np_batch_destroy(np_batch_t* b) {
    if (b) cudaStreamSynchronize(b->stream);
    batch_free(b);
}

int np_batch_run(np_batch_t* b, int use_graph, np_batch_stats_t* stats) {
    if (!b) return fail(NP_ERR_INVALID, "batch is NULL");
    int dev = 0;
    NP_CU(cudaGetDevice(&dev), NP_ERR_NO_DEVICE);
    if (dev != b->device) return fail(NP_ERR_INVALID, "batch was created on device %d, current is %d", b->device, dev);
    cudaStream_t st = b->stream;
    const BatchTune t = g_btune;
    NP_CU(cudaEventRecord(b->e0, st), NP_ERR_KERNEL);
    if (use_graph) {
        if (!b->graph || b->graph_epoch != g_btune_epoch) {
            if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
            cudaStream_t cap = nullptr;
            NP_CU(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), NP_ERR_KERNEL);
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
            int rc = e == cudaSuccess ? batch_enqueue(b, t, cap) : NP_ERR_KERNEL;
            cudaError_t e2 = cudaStreamEndCapture(cap, &g);
            cudaStreamDestroy(cap);
            if (e != cudaSuccess || rc != NP_OK || e2 != cudaSuccess || !g) {
                if (g) cudaGraphDestroy(g);
                cudaGetLastError();
                return fail(NP_ERR_KERNEL, "capture of the batch graph failed");
            }
            e = cudaGraphInstantiate(&b->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { b->graph = nullptr; return fail(NP_ERR_KERNEL, "graph instantiation: %s", cudaGetErrorString(e)); }
            b->graph_epoch = g_btune_epoch;
            b->graph_tune = t;
        }
        NP_CU(cudaGraphLaunch(b->graph, st), NP_ERR_KERNEL);
    } else {
        int rc = batch_enqueue(b, t, st);
        if (rc != NP_OK) return rc;
    }
    NP_CU(cudaEventRecord(b->e1, st), NP_ERR_KERNEL);
    if (stats) {
        NP_CU(cudaMemcpyAsync(b->h_ctr, b->B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, st), NP_ERR_KERNEL);
        NP_CU(cudaMemcpyAsync(b->h_times, b->B.t_done, sizeof(unsigned long long) * ((size_t)b->n + 1),
                              cudaMemcpyDeviceToHost, st), NP_ERR_KERNEL);
        NP_CU(cudaStreamSynchronize(st), NP_ERR_KERNEL);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, b->e0, b->e1);
        std::vector<double> lat((size_t)b->n);
        const unsigned long long t0 = b->h_times[b->n];
        for (int i = 0; i < b->n; ++i) lat[(size_t)i] = (double)(b->h_times[i] - t0) * 1e-6;
        std::vector<double> sorted = lat;
        std::sort(sorted.begin(), sorted.end());
        auto q = [&](double f) { return sorted[(size_t)std::min<double>((double)b->n - 1, std::floor(f * (b->n - 1) + 0.5))]; };
        stats->scenes = b->n;
        stats->rays = b->h_ctr->rays;
        stats->steps = b->h_ctr->steps;
        stats->fp64_steps = b->h_ctr->fp64_steps;
        stats->deferred_rays = std::min<unsigned long long>(b->h_ctr->deferred, b->B.list_cap);
        stats->closed_form_rays = b->h_ctr->closed_form;
        stats->total_ms = ms;
        stats->scene_ms_p50 = q(0.5);
        stats->scene_ms_p99 = q(0.99);
        stats->scene_ms_max = sorted.back();
        stats->block = kBatchShapes[t.shape].block;
        stats->min_blocks = kBatchShapes[t.shape].minb;
        stats->chunk = t.chunk;
        stats->island_batch = t.island_batch;
    }
    return NP_OK;
}

int np_batch_scene_output(np_batch_t* b, int i, float** d_rgb, float** d_rcross) {
    if (!b || i < 0 || i >= b->n) return fail(NP_ERR_INVALID, "bad batch or scene index");
    const long long po = b->pix_off[(size_t)b->pos[(size_t)i]];
    if (d_rgb) *d_rgb = b->B.rgb + 3 * po;
    if (d_rcross) *d_rcross = b->B.rcross + po;
    return NP_OK;
}

int np_batch_copy_output(np_batch_t* b, int i, float* d_rgb, float* d_rcross) {
    if (!b || i < 0 || i >= b->n) return fail(NP_ERR_INVALID, "bad batch or scene index");
    const size_t np_ = (size_t)b->npix[(size_t)i];
    const long long po = b->pix_off[(size_t)b->pos[(size_t)i]];
    if (d_rgb)
        NP_CU(cudaMemcpyAsync(d_rgb, b->B.rgb + 3 * po, 3 * np_ * sizeof(float), cudaMemcpyDeviceToDevice,
                              b->stream), NP_ERR_KERNEL);
    if (d_rcross)
        NP_CU(cudaMemcpyAsync(d_rcross, b->B.rcross + po, np_ * sizeof(float), cudaMemcpyDeviceToDevice,
                              b->stream), NP_ERR_KERNEL);
    return NP_OK;
}

int np_batch_scene_latency(np_batch_t* b, double* ms) {
    if (!b || !ms) return fail(NP_ERR_INVALID, "NULL argument");
    NP_CU(cudaStreamSynchronize(b->stream), NP_ERR_KERNEL);
    NP_CU(cudaMemcpy(b->h_times, b->B.t_done, sizeof(unsigned long long) * ((size_t)b->n + 1), cudaMemcpyDeviceToHost),
          NP_ERR_KERNEL);
    for (int i = 0; i < b->n; ++i) ms[i] = (double)(b->h_times[b->pos[(size_t)i]] - b->h_times[b->n]) * 1e-6;
    return NP_OK;
}

int np_batch_set_tuning(int shape, int chunk, int island_batch) {
    if (shape < 0 || shape >= kNumBatchShapes) return fail(NP_ERR_INVALID, "shape must be in [0, %d)", kNumBatchShapes);
    if (chunk < 1 || chunk > 4096) return fail(NP_ERR_INVALID, "chunk must be in [1, 4096]");
    if (island_batch < 1 || island_batch > 32) return fail(NP_ERR_INVALID, "island batch must be in [1, 32]");
    g_btune.shape = shape; g_btune.chunk = chunk; g_btune.island_batch = island_batch;
    ++g_btune_epoch;
    return NP_OK;
}

int np_batch_shape(int shape, int* block, int* min_blocks) {
    if (shape < 0 || shape >= kNumBatchShapes) return fail(NP_ERR_INVALID, "shape must be in [0, %d)", kNumBatchShapes);
    if (block) *block = kBatchShapes[shape].block;
    if (min_blocks) *min_blocks = kBatchShapes[shape].minb;
    return NP_OK;
}

// Coordinate descent over launch shape, queue chunk and island batch on the
// given (sub-)batch: each trial is one timed pass after one untimed pass of
// the first trial; the best setting is installed and returned.
int np_batch_autotune(np_batch_t* b, np_batch_tune_t* out) {
    if (!b) return fail(NP_ERR_INVALID, "batch is NULL");
    BatchTune best = g_btune;
    auto trial = [&](const BatchTune& t, double& ms) -> int {
        BatchTune saved = g_btune;
        g_btune = t;
        np_batch_stats_t s{};
        int rc = np_batch_run(b, 0, &s);
        g_btune = saved;
        ms = s.total_ms;
        return rc;
    };
    double best_ms = 0.0;
    int rc = trial(best, best_ms);                  // warm-up
    if (rc != NP_OK) return rc;
    rc = trial(best, best_ms);
    if (rc != NP_OK) return rc;
    int trials = 2;
    for (int s = 0; s < kNumBatchShapes; ++s) {
        if (s == best.shape) continue;
        BatchTune t = best; t.shape = s;
        double ms; if ((rc = trial(t, ms)) != NP_OK) return rc;
        ++trials;
        if (ms < best_ms) { best_ms = ms; best = t; }
    }
    const int chunks[] = {16, 32, 64, 128, 256};
    const BatchTune base_c = best;
    for (int c : chunks) {
        if (c == base_c.chunk) continue;
        BatchTune t = base_c; t.chunk = c;
        double ms; if ((rc = trial(t, ms)) != NP_OK) return rc;
        ++trials;
        if (ms < best_ms) { best_ms = ms; best = t; }
    }
    const int batches[] = {4, 8, 12, 16};
    const BatchTune base_i = best;
    for (int ib : batches) {
        if (ib == base_i.island_batch) continue;
        BatchTune t = base_i; t.island_batch = ib;
        double ms; if ((rc = trial(t, ms)) != NP_OK) return rc;
        ++trials;
        if (ms < best_ms) { best_ms = ms; best = t; }
    }
    g_btune = best;
    ++g_btune_epoch;
    if (out) {
        out->shape = best.shape;
        out->block = kBatchShapes[best.shape].block;
        out->min_blocks = kBatchShapes[best.shape].minb;
        out->chunk = best.chunk;
        out->island_batch = best.island_batch;
        out->best_ms = best_ms;
        out->trials = trials;
    }
    return NP_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Progressive frames: per-pixel colour sums accumulated on the device over
// passes of `samples` spp, then exposure, optional Reinhard tone map, display
// gamma and 8-bit quantisation on the device (render.cu:523-620).

namespace {

// sum[c][p] / spp -> interleaved 8-bit RGB, with the reference's output
// mapping: scale 2^EV, x / (1 + x) when tonemap, x^(1/gamma) unless gamma is
// 1, clamp to [0, 1], truncation of 255 x (render.cu:577-601).
__global__ void tonemap_kernel(const float* __restrict__ sum, long long npix, float inv_spp, float scale, int reinhard,
                               float gamma, unsigned char* __restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npix;
         i += (long long)gridDim.x * blockDim.x) {
        for (int c = 0; c < 3; ++c) {
            float v = sum[(size_t)c * npix + i] * inv_spp;
            v *= scale;
            if (reinhard) v = v / (1.0f + v);
            if (fabsf(gamma - 1.0f) > 1e-6f) v = powf(fmaxf(v, 0.0f), 1.0f / fmaxf(1e-6f, gamma));
            v = fminf(fmaxf(v, 0.0f), 1.0f);
            out[3 * i + c] = (unsigned char)(255.0f * v);
        }
    }
}

__global__ void scale_kernel(const float* __restrict__ in, float* __restrict__ out, long long n, float s) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = in[i] * s;
}

}  // namespace

struct np_frame {
    int device = -1;
    int W = 0, H = 0;
    int spp_done = 0;
    cudaStream_t stream = nullptr;
    float* d_sum = nullptr;        // [3][H][W] colour sums
    float* d_rc = nullptr;         // [H][W] first-crossing radius of sample 0
    float* d_inv = nullptr;        // [3] invariant maxima
    unsigned char* d_u8 = nullptr;
    float* d_tmp = nullptr;
};

extern "C" {

np_frame_t* np_frame_create(int width, int height, void* stream) {
    if (width <= 0 || height <= 0) { fail(NP_ERR_INVALID, "Invalid image dimensions."); return nullptr; }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        fail(NP_ERR_NO_DEVICE, "No CUDA devices found.");
        return nullptr;
    }
    np_frame* f = new np_frame();
    f->W = width; f->H = height; f->stream = (cudaStream_t)stream;
    const size_t np_ = (size_t)width * height;
    if (cudaGetDevice(&f->device) != cudaSuccess || cudaMalloc(&f->d_sum, 3 * np_ * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&f->d_rc, np_ * sizeof(float)) != cudaSuccess || cudaMalloc(&f->d_inv, 4 * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&f->d_u8, 3 * np_) != cudaSuccess || cudaMalloc(&f->d_tmp, 3 * np_ * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        np_frame_destroy(f);
        fail(NP_ERR_ALLOC, "device allocation for a %dx%d frame failed", width, height);
        return nullptr;
    }
    np_frame_reset(f);
    return f;
}

void np_frame_destroy(np_frame_t* f) {
    if (!f) return;
    cudaStreamSynchronize(f->stream);
    cudaFree(f->d_sum); cudaFree(f->d_rc); cudaFree(f->d_inv); cudaFree(f->d_u8); cudaFree(f->d_tmp);
    delete f;
}

int np_frame_reset(np_frame_t* f) {
    if (!f) return fail(NP_ERR_INVALID, "frame is NULL");
    const size_t np_ = (size_t)f->W * f->H;
    NP_CU(cudaMemsetAsync(f->d_sum, 0, 3 * np_ * sizeof(float), f->stream), NP_ERR_KERNEL);
    NP_CU(cudaMemsetAsync(f->d_rc, 0, np_ * sizeof(float), f->stream), NP_ERR_KERNEL);
    NP_CU(cudaMemsetAsync(f->d_inv, 0, 4 * sizeof(float), f->stream), NP_ERR_KERNEL);
    f->spp_done = 0;
    return NP_OK;
}

int np_frame_add_pass(np_frame_t* f, const np_scene_t* scene, int precision, np_render_stats_t* stats) {
    if (!f || !scene) return fail(NP_ERR_INVALID, "NULL argument");
    if (scene->width != f->W || scene->height != f->H) return fail(NP_ERR_INVALID, "scene size differs from the frame");
    np_scene_t s = *scene;
    s.sample_offset = scene->sample_offset + f->spp_done;
    int rc = np_render_device(&s, precision, f->d_sum, f->spp_done == 0 ? f->d_rc : nullptr,
                              scene->check_invariants ? f->d_inv : nullptr, f->spp_done > 0 ? 1 : 0, f->stream, stats);
    if (rc != NP_OK) return rc;
    f->spp_done += scene->spp;
    return NP_OK;
}

int np_frame_spp(const np_frame_t* f) { return f ? f->spp_done : 0; }

int np_frame_tonemap(np_frame_t* f, float exposure_ev, float gamma, int reinhard, unsigned char* h_rgb8) {
    if (!f || !h_rgb8) return fail(NP_ERR_INVALID, "NULL argument");
    if (f->spp_done <= 0) return fail(NP_ERR_INVALID, "no pass rendered");
    const long long np_ = (long long)f->W * f->H;
    const float g = gamma <= 0.0f ? 1.0f : gamma;
    const int blocks = (int)std::min<long long>((np_ + 255) / 256, (long long)np_device_sms() * 16);
    tonemap_kernel<<<blocks, 256, 0, f->stream>>>(f->d_sum, np_, 1.0f / (float)f->spp_done, powf(2.0f, exposure_ev),
                                                  reinhard ? 1 : 0, g, f->d_u8);
    NP_CU(cudaGetLastError(), NP_ERR_KERNEL);
    NP_CU(cudaMemcpyAsync(h_rgb8, f->d_u8, 3 * (size_t)np_, cudaMemcpyDeviceToHost, f->stream), NP_ERR_KERNEL);
    NP_CU(cudaStreamSynchronize(f->stream), NP_ERR_KERNEL);
    return NP_OK;
}

int np_frame_save(np_frame_t* f, float* h_sum, float* h_rcross, float* h_inv3, int* spp) {
    if (!f || !h_sum || !spp) return fail(NP_ERR_INVALID, "NULL argument");
    const size_t np_ = (size_t)f->W * f->H;
    NP_CU(cudaMemcpyAsync(h_sum, f->d_sum, 3 * np_ * sizeof(float), cudaMemcpyDeviceToHost, f->stream),
          NP_ERR_KERNEL);
    if (h_rcross)
        NP_CU(cudaMemcpyAsync(h_rcross, f->d_rc, np_ * sizeof(float), cudaMemcpyDeviceToHost, f->stream),
              NP_ERR_KERNEL);
    if (h_inv3)
        NP_CU(cudaMemcpyAsync(h_inv3, f->d_inv, 3 * sizeof(float), cudaMemcpyDeviceToHost, f->stream), NP_ERR_KERNEL);
    NP_CU(cudaStreamSynchronize(f->stream), NP_ERR_KERNEL);
    *spp = f->spp_done;
    return NP_OK;
}

int np_frame_load(np_frame_t* f, const float* h_sum, const float* h_rcross, const float* h_inv3, int spp) {
    if (!f || !h_sum) return fail(NP_ERR_INVALID, "NULL argument");
    if (spp < 0) return fail(NP_ERR_INVALID, "negative sample count");
    const size_t np_ = (size_t)f->W * f->H;
    NP_CU(cudaMemcpyAsync(f->d_sum, h_sum, 3 * np_ * sizeof(float), cudaMemcpyHostToDevice, f->stream),
          NP_ERR_KERNEL);
    if (h_rcross)
        NP_CU(cudaMemcpyAsync(f->d_rc, h_rcross, np_ * sizeof(float), cudaMemcpyHostToDevice, f->stream),
              NP_ERR_KERNEL);
    else
        NP_CU(cudaMemsetAsync(f->d_rc, 0, np_ * sizeof(float), f->stream), NP_ERR_KERNEL);
    if (h_inv3)
        NP_CU(cudaMemcpyAsync(f->d_inv, h_inv3, 3 * sizeof(float), cudaMemcpyHostToDevice, f->stream), NP_ERR_KERNEL);
    else
        NP_CU(cudaMemsetAsync(f->d_inv, 0, 4 * sizeof(float), f->stream), NP_ERR_KERNEL);
    NP_CU(cudaStreamSynchronize(f->stream), NP_ERR_KERNEL);
    f->spp_done = spp;
    return NP_OK;
}

int np_frame_read(np_frame_t* f, float* h_rgb_mean, float* h_rcross, float* h_inv3) {
    if (!f) return fail(NP_ERR_INVALID, "frame is NULL");
    if (f->spp_done <= 0) return fail(NP_ERR_INVALID, "no pass rendered");
    const long long np_ = (long long)f->W * f->H;
    if (h_rgb_mean) {
        const int blocks = (int)std::min<long long>((3 * np_ + 255) / 256, (long long)np_device_sms() * 16);
        scale_kernel<<<blocks, 256, 0, f->stream>>>(f->d_sum, f->d_tmp, 3 * np_, 1.0f / (float)f->spp_done);
        NP_CU(cudaGetLastError(), NP_ERR_KERNEL);
        NP_CU(cudaMemcpyAsync(h_rgb_mean, f->d_tmp, 3 * (size_t)np_ * sizeof(float), cudaMemcpyDeviceToHost, f->stream),
              NP_ERR_KERNEL);
    }
    if (h_rcross)
        NP_CU(cudaMemcpyAsync(h_rcross, f->d_rc, (size_t)np_ * sizeof(float), cudaMemcpyDeviceToHost, f->stream),
              NP_ERR_KERNEL);
    if (h_inv3)
        NP_CU(cudaMemcpyAsync(h_inv3, f->d_inv, 3 * sizeof(float), cudaMemcpyDeviceToHost, f->stream), NP_ERR_KERNEL);
    NP_CU(cudaStreamSynchronize(f->stream), NP_ERR_KERNEL);
    return NP_OK;
}

}  // extern "C"
