/*
 * np_render.h -- C ABI of the GB300 Kerr null-geodesic renderer.
 *
 * This is the drop-in boundary for the reference renderer's hot path
 * (`renderKernel` + `render_one`, render.cu:118-364 and render.cu:523-620).
 * Everything crosses as plain pointers, sizes and a POD scene description;
 * no C++ or torch types appear in any signature.
 *
 * Units.  With `units == NP_UNITS_RS` the scene follows render.cu exactly:
 * `mass` is M, `r_cam` is in Schwarzschild radii (render.cu:21,131-135),
 * and the camera angles / mass / radius pass through float exactly as the
 * reference kernel arguments do (render.cu:118-123, 483-485).  With
 * `units == NP_UNITS_M` every length is in units of M and all scene
 * quantities stay double.
 *
 * Output layout (planar, structure of arrays, row-major, y = 0 is the top
 * row as in render.cu:128,148-151):
 *   rgb    float[3][height][width]  sum over this call's samples of the
 *                                   per-sample linear radiance (render.cu:361-363)
 *   rcross float[height][width]     first disk-crossing radius of sample 0
 *                                   of this call (0 when sample 0 missed the disk)
 *   inv3   float[3]                 max |H|, |dE/E|, |dL/L| (render.cu:233-244,
 *                                   327-345); may be NULL
 *
 * Error handling: every entry point returns an np_status code; the message
 * of the last failure on the calling thread is available from
 * np_last_error().  Nothing aborts the process.
 */
#ifndef NP_RENDER_H
#define NP_RENDER_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NP_ABI_VERSION 4

typedef enum np_status {
    NP_OK = 0,
    NP_ERR_INVALID = -1,     /* bad argument (mirrors geokerr_stream.cu:163-165 "-1") */
    NP_ERR_ALLOC = -2,       /* device allocation failed ("-2") */
    NP_ERR_KERNEL = -3,      /* launch or execution failure ("-3") */
    NP_ERR_NO_DEVICE = -4,   /* no CUDA device visible */
    NP_ERR_TIMEOUT = -5      /* a bounded device wait gave up */
} np_status;

typedef enum np_units { NP_UNITS_RS = 0, NP_UNITS_M = 1 } np_units;
/* NP_JITTER_CRITICAL: stratified jitter, and every odd sample moved along its
 * position angle in the camera's tangent plane to within +-2 % of the
 * critical curve's radius there (seeded by `seed`), so that half the rays of
 * a pass are near-critical (importance sampling of the photon ring). */
typedef enum np_jitter { NP_JITTER_WANGHASH = 0, NP_JITTER_STRATIFIED = 1, NP_JITTER_CRITICAL = 2 } np_jitter;
typedef enum np_camera { NP_CAMERA_STATIC = 0, NP_CAMERA_ZAMO = 1 } np_camera;
/* NP_INTEG_RKF78: Fehlberg's embedded 7(8) pair, the 8th-order solution
 * propagated, one attempt per scheduling pass of a lane.
 *   NP_PREC_FP64   research mode: error control on (r, theta, phi, p_r,
 *                  p_theta, p_phi) with the scene's rtol/atol, and, when
 *                  inv_gate > 0, invariant-gated acceptance: a step is also
 *                  rejected (h halved) when its change of the Hamiltonian,
 *                  relative to the sum of the Hamiltonian's absolute terms,
 *                  or its change of Carter's constant Q, relative to
 *                  max(|Q0|, (E M)^2), exceeds inv_gate.
 *   NP_PREC_MIXED  the Carter-form system in compensated FP32, error control
 *                  on (r, theta, p_r, p_theta) with rtol and atol (atol at
 *                  least 1e-9 M); FP64 islands take 7(8) steps at rtol,
 *                  near-critical rays are solved in FP64 closed form (or
 *                  traced whole in FP64 at rtol_fp64, critical_solver),
 *                  and a ray inside the horizon band that provably falls
 *                  in (no radial turning point left) ends there; any other
 *                  ray that enters the band is solved in closed form too.
 *                  inv_gate is not used.  With NP_CROSS_ROOT a
 *                  crossing is landed on the equator by one more 7(8) step
 *                  in theta (Henon's method). */
typedef enum np_integrator { NP_INTEG_RK4 = 0, NP_INTEG_ADAPTIVE = 1, NP_INTEG_RKF78 = 2 } np_integrator;
/* NP_CROSS_ROOT: the crossing is as accurate as the integrator itself (no
 * interpolant error).  FP64 path: theta = pi/2 located by bracketed root
 * finding on re-integrations of the crossing step from its start.  Mixed
 * path (NP_INTEG_RKF78 only): one 7(8) step from the crossing step's start
 * with theta as the independent variable lands on theta = pi/2 exactly
 * (M. Henon, Physica D 5, 1982). */
typedef enum np_crossing { NP_CROSS_LINEAR = 0, NP_CROSS_HERMITE = 1, NP_CROSS_ROOT = 2 } np_crossing;
typedef enum np_background { NP_BG_GRADIENT = 0, NP_BG_POINT = 1 } np_background;

/* Arithmetic of the geodesic integration.
 *   NP_PREC_FP64   the reference's FP64 Hamiltonian RK4 (render.cu:161-251),
 *                  all eight phase-space components, compensated sums.
 *   NP_PREC_MIXED  FP32 bulk integration of (r, theta, p_r, p_theta) with a
 *                  compensated (hi+lo) state, FP64 steps near the horizon, at
 *                  turning points and for near-critical impact parameters. */
typedef enum np_precision { NP_PREC_FP64 = 0, NP_PREC_MIXED = 1 } np_precision;

/* Arithmetic of the island steps and near-critical rays of the mixed 7(8)
 * path (np_scene_t.island_arith; the RK4 and step-doubling mixed paths use
 * native FP64).
 *   NP_ISLAND_ARITH_FP64  native FP64 (default)
 *   NP_ISLAND_ARITH_DF    double-float: unevaluated pairs of FP32 values, a
 *                         48-bit significand, on the FP32 pipes (a double-
 *                         float addition costs 20 FP32 operations, a product
 *                         8).  On GB300 it measured slower than native FP64
 *                         despite FP64's 1/64 rate: its long dependent
 *                         operation chains leave the few island warps
 *                         latency-bound. */
typedef enum np_island_arith { NP_ISLAND_ARITH_FP64 = 0, NP_ISLAND_ARITH_DF = 1 } np_island_arith;

/* Near-critical rays of NP_PREC_MIXED (np_scene_t.critical_solver; used
 * when NP_ISLAND_CRITICAL is set).
 *   NP_CRITICAL_CLOSED_FORM  the FP64 Mino-time solution (default): the
 *                            Mino time of each equatorial crossing from the
 *                            polar motion mu = mu+ cn(omega lambda + w0 | k),
 *                            its radius from one Jacobi amplitude of the
 *                            radial motion (Carlson's R_F), capture or escape
 *                            from the roots of the radial potential; no
 *                            integration steps.  Rays outside the closed
 *                            forms (a = 0, Carter's Q = 0, a camera inside
 *                            the photon region or beyond the escape radius)
 *                            are integrated as below.  On the 7(8) path
 *                            with NP_ISLAND_HORIZON (and the disk outside
 *                            the horizon band), a ray that enters the band
 *                            without a certificate of capture is solved the
 *                            same way, whole, instead of taking FP64 island
 *                            steps there.
 *   NP_CRITICAL_INTEGRATE    traced whole in FP64 (island_arith) by the
 *                            integrator family of the scene: 7(8) at
 *                            rtol_fp64, RK4 with the reference step law. */
typedef enum np_critical_solver { NP_CRITICAL_CLOSED_FORM = 0, NP_CRITICAL_INTEGRATE = 1 } np_critical_solver;

/* FP64 islands of NP_PREC_MIXED (bit mask, np_scene_t.islands). */
#define NP_ISLAND_HORIZON 1   /* steps within 0.1 M of the outer horizon */
#define NP_ISLAND_TURNING 2   /* steps across a radial or polar turning point */
#define NP_ISLAND_CRITICAL 4  /* whole rays with |b - b_crit| < 1e-3 M */
#define NP_ISLANDS_ALL 7
/* Default mask: horizon and near-critical islands.  Turning-point islands
 * changed neither the frame agreement with NP_PREC_FP64 nor the crossing
 * error against the Mino-time solver on the 1280x720x4 benchmark frame and
 * cost a fifth of its kernel time; they stay available as an option, and
 * NP_INTEG_ADAPTIVE always takes its turning-point steps in FP64. */
#define NP_ISLANDS_DEFAULT (NP_ISLAND_HORIZON | NP_ISLAND_CRITICAL)

typedef struct np_scene {
    int32_t width, height;        /* render.cu:16-17 */
    int32_t spp;                  /* samples traced by this call (render.cu:23) */
    int32_t sample_offset;        /* first sample index (spp_done, render.cu:545) */
    double mass;                  /* M (render.cu:20) */
    double spin;                  /* a/M, |spin| < 1 (render.cu:29) */
    double r_cam;                 /* camera radius (Rs or M, see units) */
    double theta_deg;             /* camera polar angle (render.cu:19) */
    double phi_deg;               /* camera azimuth (render.cu:27,632) */
    double fov_y_deg;             /* vertical field of view (render.cu:18) */
    int32_t units;                /* np_units */
    int32_t camera;               /* np_camera; static falls back to ZAMO inside the ergosphere */
    int32_t jitter;               /* np_jitter */
    uint32_t seed;                /* seed of NP_JITTER_STRATIFIED */
    int32_t integrator;           /* np_integrator */
    int32_t max_steps;            /* step cap (MAX_INTEGRATION_STEPS, bh_common.h:203) */
    double step_scale;            /* h = step_scale * clamp(r/M, 1, 100) (render.cu:185,207) */
    double rtol, atol;            /* adaptive tolerances (bh_common.h:221,228) */
    double escape_r;              /* absolute escape radius; <= 0 means r_cam + 10 Rs (render.cu:182) */
    int32_t disk_on;              /* render.cu:43 */
    int32_t disk_max_orders;      /* render.cu:45 */
    double disk_rin, disk_rout;   /* absolute radii; <= 0 means 3 Rs / 20 Rs (render.cu:179-180) */
    double emissivity_q;          /* j ~ r^-q (render.cu:67 uses q = 2) */
    double disk_gain;             /* render.cu:44 */
    int32_t crossing;             /* np_crossing; linear is render.cu:218-220 */
    int32_t background;           /* np_background (render.cu:39) */
    double bg_sigma_deg;          /* render.cu:40 */
    double bg_brightness;         /* render.cu:41 */
    int32_t check_invariants;     /* render.cu:32 */
    int32_t islands;              /* NP_ISLAND_* mask of the mixed path */
    double inv_gate;              /* NP_INTEG_RKF78 invariant gate; <= 0 disables */
    double rtol_fp64;             /* rtol of the near-critical rays the mixed 7(8) path traces
                                     whole in FP64 (NP_CRITICAL_INTEGRATE); <= 0 means rtol */
    int32_t island_arith;         /* np_island_arith: arithmetic of the FP64-class steps of the
                                     mixed 7(8) path */
    int32_t critical_solver;      /* np_critical_solver: near-critical rays of the mixed path */
} np_scene_t;

/* Per-call statistics, filled when the pointer is non-NULL. */
typedef struct np_render_stats {
    uint64_t rays;                /* rays traced */
    uint64_t steps;               /* accepted integration steps */
    uint64_t fp64_steps;          /* steps taken in FP64 by the mixed path */
    uint64_t rhs_evals;           /* right-hand-side evaluations */
    uint64_t deferred_rays;       /* near-critical rays (mixed path) */
    double kernel_ms;             /* device time of the tracer kernel */
    double init_ms;               /* device time of the ray-generation kernel (mixed path) */
    uint64_t closed_form_rays;    /* near-critical rays solved in closed form (mixed path) */
    uint64_t band_rays;           /* 7(8) rays handed from the horizon band to the closed form */
} np_render_stats_t;

/* ABI version compiled into the library. */
int np_abi_version(void);

/* Message of the last failure on this thread ("" when none). */
const char* np_last_error(void);

/* Reference defaults of render.cu:15-46 (1280x720, M=10, r_cam=50 Rs, ...). */
void np_scene_defaults(np_scene_t* scene);

/* The 1280x720 a=0.9 benchmark scene: M=1, r_cam=50 M, theta=80 deg,
 * fov 55 deg, 4 spp stratified from seed 0, disk from the prograde ISCO to
 * 20 M with j ~ r^-3, 3 crossing orders, step cap 4096, escape at 1000 M. */
void np_scene_benchmark(np_scene_t* scene);

/* Prograde ISCO radius (Bardeen, Press & Teukolsky 1972) for mass M, spin a/M. */
double np_isco_radius(double mass, double spin);
/* Tangent-plane radius of the critical curve of `scene`'s camera at 256
 * position angles psi_i = -pi + 2 pi i / 256 (the table NP_JITTER_CRITICAL
 * samples around); host computation, no GPU needed. */
int np_critical_curve(const np_scene_t* scene, float* rho);

/* Validates a scene the way render.cu:431-465 validates its flags. */
int np_scene_validate(const np_scene_t* scene);

/* Renders one pass into DEVICE buffers on `stream` (a cudaStream_t, NULL =
 * legacy default stream).  When `accumulate` is non-zero the pass is added
 * to rgb (progressive spp), otherwise rgb is overwritten.  rcross is
 * written when non-NULL; inv3 is max-updated when non-NULL.  Returns after
 * the launch; the caller synchronises the stream. */
int np_render_device(const np_scene_t* scene, int precision,
                     float* d_rgb, float* d_rcross, float* d_inv3,
                     int accumulate, void* stream, np_render_stats_t* stats);

/* Same pass with HOST buffers: the library copies to and from the device
 * inside the call and returns when the results are in host memory. */
int np_render_host(const np_scene_t* scene, int precision,
                   float* h_rgb, float* h_rcross, float* h_inv3,
                   np_render_stats_t* stats);

/* Traces explicit rays and reports per-ray events; used for accuracy
 * studies against the semi-analytic solver.  Ray i starts at pixel
 * coordinates (px[i], py[i]) (continuous, 0..width, 0..height).  Outputs
 * per ray (device pointers):
 *   consts[4*i+0..3] = p_t, p_phi, p_r, p_theta at the camera
 *   cross[8*i + 2k], cross[8*i + 2k + 1] = r and phi of the k-th equatorial
 *       crossing (k < 4), 0 when absent
 *   status[i] = 0 escaped, 1 captured, 2 step cap; plus 16 * (crossings) */
int np_trace_rays_device(const np_scene_t* scene, int precision, int n,
                         const double* d_px, const double* d_py,
                         double* d_consts, double* d_cross, int32_t* d_status,
                         void* stream);

/* Conserved-quantity drift of explicit rays on the FP64 path (any FP64
 * integrator): per ray i, drift[2*i] = max |H| / E^2 and drift[2*i+1] =
 * max |Q - Q0| / max(|Q0|, (E M)^2) over its accepted steps (H the
 * Hamiltonian, Q Carter's constant, E = -p_t; E and L = p_phi are exact
 * constants of this formulation), steps[i] = accepted steps.  Ray
 * positions as np_trace_rays_device; device pointers. */
int np_trace_invariants_device(const np_scene_t* scene, int n, const double* d_px, const double* d_py,
                               double* d_drift, int32_t* d_steps, void* stream);

/* ------------------------------------------------------------------------
 * Differentiable render (adjoint).  The image is the mean over samples of
 * the scene's colours; gradients are taken with respect to (spin a/M,
 * camera inclination theta in radians, disk gain, emissivity index q) by a
 * reverse sweep through the RK4 steps with checkpoints every K steps.  The
 * scene must use lengths in M, fixed-step RK4, Hermite crossings and the
 * gradient sky.  Event changes (disk edges, capture, escape) are not
 * differentiated. */
typedef struct np_adjoint np_adjoint_t;

typedef struct np_adjoint_stats {
    double forward_ms;                 /* device time of the forward pass */
    double backward_ms;                /* device time of the reverse sweep */
    uint64_t workspace_bytes;          /* device bytes held by the handle */
    uint64_t checkpoint_bytes_per_ray; /* checkpoint storage per ray */
} np_adjoint_stats_t;

np_adjoint_t* np_adjoint_create(void);
void np_adjoint_destroy(np_adjoint_t* handle);

/* Forward pass: renders the mean image d_img [3][H][W] and keeps the
 * checkpoints in the handle.  d_sample_rgb [spp][3][H][W] and d_sample_sig
 * [spp][H][W] (status + 4 * disk hits per sample) are written when non-NULL.
 * precision: NP_PREC_MIXED integrates in FP32, NP_PREC_FP64 in FP64. */
int np_adjoint_forward(np_adjoint_t* handle, const np_scene_t* scene, int precision, int K, float* d_img,
                       float* d_sample_rgb, int32_t* d_sample_sig, void* stream, np_adjoint_stats_t* stats);

/* Reverse sweep for the upstream gradient d_grad_img = dLoss/d_img
 * [3][H][W]; writes dLoss/d(spin, theta_rad, gain, q) to h_grad4 (host) and,
 * when d_sample_grad is non-NULL, each sample's contribution to it
 * ([spp][H][W][4], device).  Synchronises the stream. */
int np_adjoint_backward(np_adjoint_t* handle, const float* d_grad_img, double* h_grad4, double* d_sample_grad,
                        void* stream, np_adjoint_stats_t* stats);

/* Largest pass (width * height * spp rays) np_render_device_noalloc accepts. */
#define NP_NOALLOC_MAX_RAYS 262144

/* No counterpart in the reference: an entry point for callers that cannot
 * allocate device memory.  Some hosts own the whole GPU through their own
 * allocator (an engine or framework that reserves device memory up front)
 * or forbid allocation inside their frame loop; for them this renders one
 * pass like np_render_device but uses, instead of library-allocated scratch,
 * a fixed scratch array compiled into the library (about 15 MB, held on
 * every GPU that loads the library until the process exits).  Limits and
 * rules:
 *   - at most NP_NOALLOC_MAX_RAYS rays per call; larger passes are rejected
 *     with NP_ERR_INVALID (split the samples over several calls with
 *     sample_offset and accumulate = 1);
 *   - d_rcross may be NULL.  Each call writes the first-crossing radius of
 *     its own first sample, so when a pass is split over several calls pass
 *     d_rcross to the first call only;
 *   - the first call on each device looks up the array's device address;
 *     make that first call before any stream capture.  The address is kept
 *     for the life of the process: resetting the device (cudaDeviceReset)
 *     after that first call is not supported;
 *   - every call shares the one array, so calls whose work overlaps on the
 *     GPU (different streams, or different host threads) race; serialise
 *     them;
 *   - no statistics are returned and nothing is allocated or freed.
 * Buffers are device pointers as for np_render_device. */
int np_render_device_noalloc(const np_scene_t* scene, int precision,
                             float* d_rgb, float* d_rcross, int accumulate, void* stream);

/* Launch tunables of the mixed path (process-wide; the autotuner sets them).
 *   NP_TUNE_ISLAND_BATCH  parked lanes of a warp that trigger a batched FP64
 *                         island step (1..32, default 8)
 *   NP_TUNE_MIN_BLOCKS    register cap of the tracer as resident 128-thread
 *                         blocks per SM (3, 4, 5, 6 or 8; default 4)
 *   NP_TUNE_CHUNK         ray indices a warp takes per atomic (default 64)
 *   NP_TUNE_CROSS_BATCH   lanes of a warp with a pending root-found crossing
 *                         (NP_CROSS_ROOT, FP64 path) that trigger the search
 *                         of all of them (1-32, default 12; 1 = at once)
 *   NP_TUNE_MIN_BLOCKS78  register cap of the mixed 7(8) tracer (3 or 4,
 *                         default 4)
 *   NP_TUNE_ISLAND_BATCH78 NP_TUNE_ISLAND_BATCH of the mixed 7(8) tracer
 *                         (1..32, default 32) */
#define NP_TUNE_ISLAND_BATCH 1
#define NP_TUNE_MIN_BLOCKS 2
#define NP_TUNE_CHUNK 3
#define NP_TUNE_CROSS_BATCH 4
#define NP_TUNE_MIN_BLOCKS78 5
#define NP_TUNE_ISLAND_BATCH78 6
int np_tune(int param, int value);

/* Measures the sustained FMA throughput of this GPU's SIMT pipes with a
 * register-resident FMA loop: which = 0 for FP32, 1 for FP64.  Writes
 * TFLOP/s (an FMA counts as two flops).  Synchronous. */
int np_measure_fma_peak(int which, double* tflops);

/* ------------------------------------------------------------------------
 * Batched scenes (no counterpart in the reference, whose renderer takes one
 * scene per process): n scenes of any size, spin, inclination, spp and disk
 * orders traced by one persistent launch of the mixed path over one device
 * ray queue; the pass (counter reset, ray generation, tracing, resolve) is
 * captured into a CUDA graph on the first np_batch_run with use_graph = 1
 * and replayed afterwards.  Only NP_PREC_MIXED with the RK4 and step-doubling
 * integrators is accepted (NP_INTEG_RKF78 scenes are refused: the embedded
 * 7(8) tracer runs one scene per launch); near-critical rays follow each
 * scene's critical_solver.  Outputs stay in
 * the batch: np_batch_scene_output returns device pointers to scene i's
 * planar [3][H][W] image and [H][W] first-crossing radii. */
typedef struct np_batch np_batch_t;

typedef struct np_batch_stats {
    int32_t scenes;
    uint64_t rays, steps, fp64_steps, deferred_rays;
    double total_ms;            /* CUDA-event time of the whole pass */
    double scene_ms_p50, scene_ms_p99, scene_ms_max;   /* scene completion after ray generation starts */
    int32_t block, min_blocks, chunk, island_batch;    /* launch setting used */
    uint64_t closed_form_rays;  /* near-critical rays solved in closed form */
} np_batch_stats_t;

typedef struct np_batch_tune {
    int32_t shape, block, min_blocks, chunk, island_batch, trials;
    double best_ms;
} np_batch_tune_t;

/* NULL on failure (np_last_error). `stream` is the CUDA stream of the batch. */
np_batch_t* np_batch_create(const np_scene_t* scenes, int n, int precision, void* stream);
void np_batch_destroy(np_batch_t* b);
/* One pass; with stats non-NULL the call waits for the pass and fills them. */
int np_batch_run(np_batch_t* b, int use_graph, np_batch_stats_t* stats);
int np_batch_scene_output(np_batch_t* b, int i, float** d_rgb, float** d_rcross);
/* Copies scene i's image and radii of the last pass into caller device
 * buffers (ordered on the batch stream; either pointer may be NULL). */
int np_batch_copy_output(np_batch_t* b, int i, float* d_rgb, float* d_rcross);
/* Per-scene completion times (ms after ray generation started) of the last pass. */
int np_batch_scene_latency(np_batch_t* b, double* ms);
/* Launch setting of later passes: shape index (np_batch_shape gives its
 * threads per block and resident blocks per SM), rays a warp takes from the
 * queue at once, and parked lanes that trigger a batched FP64 island step. */
int np_batch_set_tuning(int shape, int chunk, int island_batch);
int np_batch_shape(int shape, int* block, int* min_blocks);
/* Coordinate-descent autotuner over shape, chunk and island batch on batch b
 * (typically a sub-batch of the production scenes); installs the best. */
int np_batch_autotune(np_batch_t* b, np_batch_tune_t* out);

/* ------------------------------------------------------------------------
 * The physics-header API (include/np_kerr.h, the reference's bh_kerr.h
 * names) driven from C: ray i starts at a static observer (zamo = 0; a ZAMO
 * when 1) at cam[6i..6i+2] = (r, theta, phi) with local direction
 * cam[6i+3..6i+5] = (n_r, n_theta, n_phi) (init_ray_from_camera_general_d /
 * init_ray_from_camera_zamo_d, bh_kerr.h:781-826, 910-967) and takes up to
 * `steps` integrateGeodesicKerrD steps of h = h_scale r (bh_kerr.h:734-774),
 * stopping when a step returns false.  states[8i..8i+7] = (t, r, theta, phi,
 * p_t, p_r, p_theta, p_phi); alive[i] = the last step's result.  The device
 * entry takes device pointers and is ordered on `stream`; the host entry runs
 * the same header code on the CPU. */
int np_kerr_integrate_device(int n, double M, double a, const double* d_cam, int steps, double h_scale, int zamo,
                             double* d_states, int* d_alive, void* stream);
int np_kerr_integrate_host(int n, double M, double a, const double* cam, int steps, double h_scale, int zamo,
                           double* states, int* alive);

/* ------------------------------------------------------------------------
 * Progressive frames (render.cu:523-620 with the accumulation and output
 * mapping on the device): passes of scene.spp samples add their colour sums
 * into a device buffer (sample offsets continue across passes), and
 * np_frame_tonemap maps sum / spp to interleaved 8-bit RGB with exposure
 * 2^EV, optional Reinhard x/(1+x), display gamma (none when gamma is 1 or
 * <= 0 means 1) and truncation of 255 x, exactly as the reference's host
 * loop.  np_frame_read returns the mean colour [3][H][W], the first-crossing
 * radius of sample 0 and the invariant maxima (when the scene asks for them). */
typedef struct np_frame np_frame_t;
np_frame_t* np_frame_create(int width, int height, void* stream);
void np_frame_destroy(np_frame_t* f);
int np_frame_reset(np_frame_t* f);
int np_frame_add_pass(np_frame_t* f, const np_scene_t* scene, int precision, np_render_stats_t* stats);
int np_frame_spp(const np_frame_t* f);
int np_frame_tonemap(np_frame_t* f, float exposure_ev, float gamma, int reinhard, unsigned char* h_rgb8);
int np_frame_read(np_frame_t* f, float* h_rgb_mean, float* h_rcross, float* h_inv3);
/* Accumulator state for checkpoint/resume (host buffers): colour sums
 * [3][H][W] (not means), the first-crossing radius [H][W], the invariant
 * maxima [3] and the samples accumulated.  A frame loaded with a saved
 * state and given the same further passes ends bit-identical to one that
 * was never interrupted (the passes' sample indices continue from spp).
 * h_rcross and h_inv3 may be NULL (load: zeros). */
int np_frame_save(np_frame_t* f, float* h_sum, float* h_rcross, float* h_inv3, int* spp);
int np_frame_load(np_frame_t* f, const float* h_sum, const float* h_rcross, const float* h_inv3, int spp);

/* ------------------------------------------------------------------------
 * Schwarzschild deflection table (schwarzschild_blackhole.cu:44-266):
 * equatorial photons from r_start with impact parameter b[i] (lengths in the
 * units of `mass`), FP32 RK4 of bh_schwarzschild.h; deflection[i] = total
 * phi swept, rmin[i] = closest approach (the analytic root for escaping
 * rays), status[i] = 0 escaped, 1 captured, 2 near the photon sphere, 3 step
 * budget spent.  np_schwarzschild_precompute is the reference's
 * precomputeGeodesics with host arrays (b filled log-spaced, bending = deflection
 * - pi for escaped rays, NaN otherwise). */
int np_schwarzschild_deflection_device(float mass, float r_start, int n, const float* d_b, float* d_deflection,
                                       float* d_rmin, int32_t* d_status, void* stream);
int np_schwarzschild_deflection_host(float mass, float r_start, int n, const float* b, float* deflection, float* rmin,
                                     int32_t* status);
int np_schwarzschild_precompute(float mass, int n, float* b, float* deflection, float* bending, float* rmin,
                                int32_t* status);

#ifdef __cplusplus
}
#endif

#endif /* NP_RENDER_H */
