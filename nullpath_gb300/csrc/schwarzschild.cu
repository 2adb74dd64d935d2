// schwarzschild.cu -- deflection table of equatorial Schwarzschild photons
// (schwarzschild_blackhole.cu:44-266): one ray per thread from r_start with
// impact parameter b, FP32 RK4 of the Schwarzschild Hamiltonian
// (include/np_kerr.h, bh_schwarzschild.h:124-295) with the radius-scaled step
// h = 0.01 clamp(r / (Rs/2), 1, 100); total phi swept, closest approach
// (turning point interpolated on p_r, replaced by the analytic root for
// escaping rays) and the outcome 0 escaped, 1 captured, 2 near the photon
// sphere, 3 step budget spent.  The host wrapper builds the reference's
// log-spaced b grid and bending angles.
#include <cmath>
#include <cstdlib>
#include <vector>

#include <cuda_runtime.h>

#include "np_kerr.h"
#include "np_render.h"

// Streaming multiprocessors of the current device (1 if it cannot be read).
static int device_sms() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        n <= 0)
        return 1;
    return n;
}

void np_record_error(const char* msg);

namespace {

constexpr int kMaxSteps = 10000;      // MAX_INTEGRATION_STEPS (bh_common.h:203)
constexpr float kStep = 0.01f;        // INTEGRATION_STEP_SIZE (bh_common.h:213)

NP_HD inline void deflect_one(float mass, float r_start, float b, float* defl, float* rmin, int* status) {
    const SchwarzschildMetric metric(mass);
    GeodesicState s;
    s.r = r_start;
    s.theta = BH_PI * 0.5f;
    s.pt = -1.0f;
    s.pphi = b;
    const float A = 1.0f - metric.Rs / s.r;
    const float pr2 = 1.0f / (A * A) - b * b / (A * s.r * s.r);
    s.pr = -sqrtf(fmaxf(0.0f, pr2));
    float min_r = s.r, total = 0.0f, prev_phi = 0.0f, prev_r = s.r, prev_pr = s.pr;
    bool escaped = false;
    for (int k = 0; k < kMaxSteps; ++k) {
        const float h = kStep * fminf(100.0f, fmaxf(1.0f, s.r / (0.5f * metric.Rs)));
        if (!integrateGeodesic(s, metric, h)) break;
        min_r = fminf(min_r, s.r);
        if (prev_pr < 0.0f && s.pr > 0.0f) {          // refine at the turning point
            const float den = s.pr - prev_pr;
            if (fabsf(den) > 1e-12f) {
                const float al = fminf(fmaxf(-prev_pr / den, 0.0f), 1.0f);
                min_r = fminf(min_r, prev_r + al * (s.r - prev_r));
            }
        }
        prev_r = s.r;
        prev_pr = s.pr;
        float dphi = s.phi - prev_phi;
        if (dphi > BH_PI) dphi -= 2.0f * BH_PI;
        if (dphi < -BH_PI) dphi += 2.0f * BH_PI;
        total += dphi;
        prev_phi = s.phi;
        if (s.r > r_start + 1.0f && s.pr > 0.0f) { escaped = true; break; }
    }
    *defl = total;
    float r_an = 0.0f;
    *rmin = (escaped && schwarzschild_rmin_analytic(metric.Rs, b, &r_an)) ? r_an : min_r;
    if (escaped) *status = 0;
    else if (s.r <= metric.Rs + 0.01f) *status = 1;
    else if (fabsf(min_r - BH_PHOTON_SPHERE_MULTIPLIER * metric.Rs) < 0.01f * metric.Rs) *status = 2;
    else *status = 3;
}

__global__ void deflection_kernel(float mass, float r_start, int n, const float* __restrict__ b,
                                  float* __restrict__ defl, float* __restrict__ rmin, int* __restrict__ status) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        deflect_one(mass, r_start, b[i], defl + i, rmin + i, status + i);
}

}  // namespace

extern "C" {

int np_schwarzschild_deflection_device(float mass, float r_start, int n, const float* d_b, float* d_deflection,
                                       float* d_rmin, int32_t* d_status, void* stream) {
    if (n < 0 || !(mass > 0.0f) || (n > 0 && (!d_b || !d_deflection || !d_rmin || !d_status))) {
        np_record_error("np_schwarzschild_deflection_device: bad arguments");
        return NP_ERR_INVALID;
    }
    if (n == 0) return NP_OK;
    const int threads = 128;
    const int cap = device_sms() * 16;
    const int blocks = (n + threads - 1) / threads < cap ? (n + threads - 1) / threads : cap;
    deflection_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(mass, r_start, n, d_b, d_deflection, d_rmin,
                                                                   (int*)d_status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        np_record_error(cudaGetErrorString(e));
        return NP_ERR_KERNEL;
    }
    return NP_OK;
}

int np_schwarzschild_deflection_host(float mass, float r_start, int n, const float* b, float* deflection, float* rmin,
                                     int32_t* status) {
    if (n < 0 || !(mass > 0.0f) || (n > 0 && (!b || !deflection || !rmin || !status))) {
        np_record_error("np_schwarzschild_deflection_host: bad arguments");
        return NP_ERR_INVALID;
    }
    for (int i = 0; i < n; ++i) deflect_one(mass, r_start, b[i], deflection + i, rmin + i, (int*)status + i);
    return NP_OK;
}

// The reference's table builder (schwarzschild_blackhole.cu:140-266): b from
// 0.3 to 20 b_crit(Rs), log-spaced (BH_B_MIN_RS / BH_B_MAX_RS override the
// ends in units of Rs), r_start = max(1000, 1.2 b_max), bending = deflection
// - pi for escaped rays and NaN otherwise.  Host arrays of n >= 2 entries.
int np_schwarzschild_precompute(float mass, int n, float* b, float* deflection, float* bending, float* rmin,
                                int32_t* status) {
    if (n < 2 || !(mass > 0.0f) || !b || !deflection || !bending || !rmin || !status) {
        np_record_error("num_rays must be >= 2 and all buffers non-NULL");
        return NP_ERR_INVALID;
    }
    const float Rs = BH_SCHWARZSCHILD_MULTIPLIER * mass;
    const float bc = bh_bcrit_from_Rs(Rs);
    float b_min = 0.30f * bc, b_max = 20.0f * bc;
    if (const char* e = std::getenv("BH_B_MIN_RS")) { float v = std::strtof(e, nullptr); if (v > 0.f) b_min = v * Rs; }
    if (const char* e = std::getenv("BH_B_MAX_RS")) { float v = std::strtof(e, nullptr); if (v > 0.f) b_max = v * Rs; }
    if (b_min >= b_max) { b_min = Rs; b_max = 50.0f * Rs; }
    for (int i = 0; i < n; ++i) b[i] = b_min * powf(b_max / b_min, (float)i / (float)(n - 1));
    const float r_start = fmaxf(1000.0f, 1.2f * b_max);
    float *d = nullptr;
    if (cudaMalloc(&d, (size_t)n * 4 * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        np_record_error("device allocation failed");
        return NP_ERR_ALLOC;
    }
    float* d_b = d;
    float* d_def = d + n;
    float* d_rm = d + 2 * n;
    int32_t* d_st = (int32_t*)(d + 3 * n);
    int rc = NP_OK;
    if (cudaMemcpy(d_b, b, (size_t)n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) rc = NP_ERR_KERNEL;
    if (rc == NP_OK) rc = np_schwarzschild_deflection_device(mass, r_start, n, d_b, d_def, d_rm, d_st, nullptr);
    if (rc == NP_OK && (cudaMemcpy(deflection, d_def, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess ||
                        cudaMemcpy(rmin, d_rm, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess ||
                        cudaMemcpy(status, d_st, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess))
        rc = NP_ERR_KERNEL;
    cudaFree(d);
    if (rc != NP_OK) { cudaGetLastError(); return rc; }
    for (int i = 0; i < n; ++i) bending[i] = status[i] == 0 ? deflection[i] - BH_PI : NAN;
    return NP_OK;
}

}  // extern "C"
