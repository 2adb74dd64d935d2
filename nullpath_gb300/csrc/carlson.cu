// carlson.cu -- batched Carlson elliptic integrals on sm_103a (the batch
// kernel of geokerr_port/cuda/carlson_elliptic.cu:351-382, with its
// two-character case codes "RF", "RC", "RD", "RJ"), its host twin, and the
// reference's host entry points validate_carlson_cuda / test_carlson_cuda
// (carlson_elliptic.cu:387, 398) with working bodies.
#include <cmath>
#include <cstdio>

#include <cuda_runtime.h>

#include "carlson.cuh"
#include "mino_carlson.cuh"
#include "geokerr_c_api.h"

// Streaming multiprocessors of the current device (1 if it cannot be read).
static int device_sms() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        n <= 0)
        return 1;
    return n;
}
#include "np_render.h"

void np_record_error(const char* msg);

namespace {

NP_CARLSON_HD double carlson_case(char a, char b, double x, double y, double z, double p) {
    if (a != 'R') return np::carlson::nan_();
    switch (b) {
        case 'F': return np::carlson::rf(x, y, z);
        case 'C': return np::carlson::rc(x, y);
        case 'D': return np::carlson::rd(x, y, z);
        case 'J': return np::carlson::rj(x, y, z, p);
        default: return np::carlson::nan_();
    }
}

__global__ void carlson_batch_kernel(int n, const char* __restrict__ types, const double* __restrict__ x,
                                     const double* __restrict__ y, const double* __restrict__ z,
                                     const double* __restrict__ p, double* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = carlson_case(types[2 * i], types[2 * i + 1], x[i], y[i], z[i], p ? p[i] : 0.0);
}

__global__ void mino_times_kernel(int n, double a, const double* __restrict__ ua, const double* __restrict__ ub,
                                  const double* __restrict__ mua, const double* __restrict__ mub,
                                  const double* __restrict__ l, const double* __restrict__ q2,
                                  double* __restrict__ lam_u, double* __restrict__ lam_mu) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        lam_u[i] = np::mino::mino_u(a, l[i], q2[i], ua[i], ub[i]);
        lam_mu[i] = np::mino::mino_mu(a, l[i], q2[i], mua[i], mub[i]);
    }
}

__global__ void mu_of_lambda_kernel(int n, double a, const double* __restrict__ l, const double* __restrict__ q2,
                                    const double* __restrict__ mu0, const double* __restrict__ sm,
                                    const double* __restrict__ lam, double* __restrict__ mu) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        mu[i] = np::mino::mu_of_lambda(a, l[i], q2[i], mu0[i], sm[i], lam[i]);
}

__global__ void crossings_cf_kernel(int n, double a, const double* __restrict__ u0, const double* __restrict__ mu0,
                                    const double* __restrict__ l, const double* __restrict__ q2,
                                    const double* __restrict__ su, const double* __restrict__ sm, double u_end, int K,
                                    double* __restrict__ xu, int32_t* __restrict__ nx) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double* x = xu + (size_t)i * K;
        for (int k = 0; k < K; ++k) x[k] = 0.0;
        nx[i] = np::mino::equator_crossings_cf(a, u0[i], mu0[i], l[i], q2[i], su[i], sm[i], u_end, K, x);
    }
}

}  // namespace

extern "C" {

int np_geokerr_equator_crossings_cf_device(int n, double a, const double* d_u0, const double* d_mu0, const double* d_l,
                                           const double* d_q2, const double* d_su, const double* d_sm, double u_end,
                                           int K, double* d_xu, int32_t* d_nx, void* stream) {
    if (n < 0 || K < 1 || (n > 0 && (!d_u0 || !d_mu0 || !d_l || !d_q2 || !d_su || !d_sm || !d_xu || !d_nx))) {
        np_record_error("np_geokerr_equator_crossings_cf_device: bad arguments");
        return NP_ERR_INVALID;
    }
    if (n == 0) return NP_OK;
    const int threads = 128;
    const int cap = device_sms() * 16;
    const int blocks = (n + threads - 1) / threads < cap ? (n + threads - 1) / threads : cap;
    crossings_cf_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(n, a, d_u0, d_mu0, d_l, d_q2, d_su, d_sm, u_end, K,
                                                                     d_xu, d_nx);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        np_record_error(cudaGetErrorString(e));
        return NP_ERR_KERNEL;
    }
    return NP_OK;
}

int np_geokerr_equator_crossings_cf_host(int n, double a, const double* u0, const double* mu0, const double* l,
                                         const double* q2, const double* su, const double* sm, double u_end, int K,
                                         double* xu, int32_t* nx) {
    if (n < 0 || K < 1 || (n > 0 && (!u0 || !mu0 || !l || !q2 || !su || !sm || !xu || !nx))) {
        np_record_error("np_geokerr_equator_crossings_cf_host: bad arguments");
        return NP_ERR_INVALID;
    }
    for (int i = 0; i < n; ++i) {
        double* x = xu + (size_t)i * K;
        for (int k = 0; k < K; ++k) x[k] = 0.0;
        nx[i] = np::mino::equator_crossings_cf(a, u0[i], mu0[i], l[i], q2[i], su[i], sm[i], u_end, K, x);
    }
    return NP_OK;
}

int np_geokerr_mu_of_lambda_device(int n, double a, const double* d_l, const double* d_q2, const double* d_mu0,
                                   const double* d_sm, const double* d_lam, double* d_mu, void* stream) {
    if (n < 0 || (n > 0 && (!d_l || !d_q2 || !d_mu0 || !d_sm || !d_lam || !d_mu))) {
        np_record_error("np_geokerr_mu_of_lambda_device: NULL buffer or negative count");
        return NP_ERR_INVALID;
    }
    if (n == 0) return NP_OK;
    const int threads = 128;
    const int cap = device_sms() * 16;
    const int blocks = (n + threads - 1) / threads < cap ? (n + threads - 1) / threads : cap;
    mu_of_lambda_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(n, a, d_l, d_q2, d_mu0, d_sm, d_lam, d_mu);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        np_record_error(cudaGetErrorString(e));
        return NP_ERR_KERNEL;
    }
    return NP_OK;
}

int np_geokerr_mu_of_lambda_host(int n, double a, const double* l, const double* q2, const double* mu0,
                                 const double* sm, const double* lam, double* mu) {
    if (n < 0 || (n > 0 && (!l || !q2 || !mu0 || !sm || !lam || !mu))) {
        np_record_error("np_geokerr_mu_of_lambda_host: NULL buffer or negative count");
        return NP_ERR_INVALID;
    }
    for (int i = 0; i < n; ++i) mu[i] = np::mino::mu_of_lambda(a, l[i], q2[i], mu0[i], sm[i], lam[i]);
    return NP_OK;
}

int np_jacobi_host(int n, const double* u, const double* m, double* sn, double* cn, double* dn) {
    if (n < 0 || (n > 0 && (!u || !m || !sn || !cn || !dn))) {
        np_record_error("np_jacobi_host: NULL buffer or negative count");
        return NP_ERR_INVALID;
    }
    for (int i = 0; i < n; ++i) np::mino::jacobi_sncndn(u[i], m[i], sn[i], cn[i], dn[i]);
    return NP_OK;
}

int np_geokerr_mino_times_device(int n, double a, const double* d_ua, const double* d_ub, const double* d_mua,
                                 const double* d_mub, const double* d_l, const double* d_q2, double* d_lam_u,
                                 double* d_lam_mu, void* stream) {
    if (n < 0 || (n > 0 && (!d_ua || !d_ub || !d_mua || !d_mub || !d_l || !d_q2 || !d_lam_u || !d_lam_mu))) {
        np_record_error("np_geokerr_mino_times_device: NULL buffer or negative count");
        return NP_ERR_INVALID;
    }
    if (n == 0) return NP_OK;
    const int threads = 128;
    const int cap = device_sms() * 16;
    const int blocks = (n + threads - 1) / threads < cap ? (n + threads - 1) / threads : cap;
    mino_times_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(n, a, d_ua, d_ub, d_mua, d_mub, d_l, d_q2, d_lam_u,
                                                                   d_lam_mu);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        np_record_error(cudaGetErrorString(e));
        return NP_ERR_KERNEL;
    }
    return NP_OK;
}

int np_geokerr_mino_times_host(int n, double a, const double* ua, const double* ub, const double* mua,
                               const double* mub, const double* l, const double* q2, double* lam_u, double* lam_mu) {
    if (n < 0 || (n > 0 && (!ua || !ub || !mua || !mub || !l || !q2 || !lam_u || !lam_mu))) {
        np_record_error("np_geokerr_mino_times_host: NULL buffer or negative count");
        return NP_ERR_INVALID;
    }
    for (int i = 0; i < n; ++i) {
        lam_u[i] = np::mino::mino_u(a, l[i], q2[i], ua[i], ub[i]);
        lam_mu[i] = np::mino::mino_mu(a, l[i], q2[i], mua[i], mub[i]);
    }
    return NP_OK;
}

int np_carlson_batch_device(int n, const char* d_types, const double* d_x, const double* d_y, const double* d_z,
                            const double* d_p, double* d_out, void* stream) {
    if (n < 0 || (n > 0 && (!d_types || !d_x || !d_y || !d_z || !d_out))) {
        np_record_error("np_carlson_batch_device: NULL buffer or negative count");
        return NP_ERR_INVALID;
    }
    if (n == 0) return NP_OK;
    const int threads = 256;
    const int cap = device_sms() * 16;
    const int blocks = (n + threads - 1) / threads < cap ? (n + threads - 1) / threads : cap;
    carlson_batch_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(n, d_types, d_x, d_y, d_z, d_p, d_out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        np_record_error(cudaGetErrorString(e));
        return NP_ERR_KERNEL;
    }
    return NP_OK;
}

int np_carlson_batch_host(int n, const char* types, const double* x, const double* y, const double* z,
                          const double* p, double* out) {
    if (n < 0 || (n > 0 && (!types || !x || !y || !z || !out))) {
        np_record_error("np_carlson_batch_host: NULL buffer or negative count");
        return NP_ERR_INVALID;
    }
    for (int i = 0; i < n; ++i) out[i] = carlson_case(types[2 * i], types[2 * i + 1], x[i], y[i], z[i], p ? p[i] : 0.0);
    return NP_OK;
}

// Known values (closed forms): R_F(0,1,2) = K(1/sqrt 2)/sqrt 2 ... are
// checked against the host evaluation of the same cases; prints one line per
// function with the largest device/host relative difference.
void validate_carlson_cuda(void) {
    const int n = 8;
    const char types[] = "RFRFRCRCRDRDRJRJ";
    const double x[n] = {1.0, 0.5, 0.0, 2.0, 0.0, 1.5, 0.5, 2.0};
    const double y[n] = {2.0, 1.0, 0.25, -1.0, 2.0, 0.2, 1.0, 3.0};
    const double z[n] = {0.0, 3.0, 0.0, 0.0, 1.0, 4.0, 3.0, 4.0};
    const double p[n] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 2.0, -0.5};
    double host[n], dev[n];
    np_carlson_batch_host(n, types, x, y, z, p, host);
    char* dt = nullptr;
    double *dx = nullptr, *dy = nullptr, *dz = nullptr, *dp = nullptr, *dout = nullptr;
    bool ok = cudaMalloc(&dt, sizeof(types)) == cudaSuccess && cudaMalloc(&dx, sizeof(x)) == cudaSuccess &&
              cudaMalloc(&dy, sizeof(y)) == cudaSuccess && cudaMalloc(&dz, sizeof(z)) == cudaSuccess &&
              cudaMalloc(&dp, sizeof(p)) == cudaSuccess && cudaMalloc(&dout, sizeof(dev)) == cudaSuccess;
    if (ok) {
        cudaMemcpy(dt, types, sizeof(types), cudaMemcpyHostToDevice);
        cudaMemcpy(dx, x, sizeof(x), cudaMemcpyHostToDevice);
        cudaMemcpy(dy, y, sizeof(y), cudaMemcpyHostToDevice);
        cudaMemcpy(dz, z, sizeof(z), cudaMemcpyHostToDevice);
        cudaMemcpy(dp, p, sizeof(p), cudaMemcpyHostToDevice);
        ok = np_carlson_batch_device(n, dt, dx, dy, dz, dp, dout, nullptr) == NP_OK &&
             cudaMemcpy(dev, dout, sizeof(dev), cudaMemcpyDeviceToHost) == cudaSuccess;
    }
    std::printf("CUDA Carlson elliptic integral validation (device vs host)\n");
    if (!ok) {
        std::printf("  device run failed: %s\n", cudaGetErrorString(cudaGetLastError()));
    } else {
        for (int f = 0; f < 4; ++f) {
            double worst = 0.0;
            for (int i = 2 * f; i < 2 * f + 2; ++i) worst = std::fmax(worst, std::fabs(dev[i] - host[i]) / std::fabs(host[i]));
            std::printf("  R%c: max relative difference %.3e\n", types[4 * f + 1], worst);
        }
    }
    cudaFree(dt); cudaFree(dx); cudaFree(dy); cudaFree(dz); cudaFree(dp); cudaFree(dout);
}

// R_F(1, 2, 0) on the device (carlson_elliptic.cu:398-403 test case).
void test_carlson_cuda(void) {
    const char t[2] = {'R', 'F'};
    const double x = 1.0, y = 2.0, z = 0.0, p = 0.0;
    double r = std::nan("");
    char* dt = nullptr;
    double* d = nullptr;
    if (cudaMalloc(&dt, 2) == cudaSuccess && cudaMalloc(&d, 5 * sizeof(double)) == cudaSuccess) {
        const double in[4] = {x, y, z, p};
        cudaMemcpy(dt, t, 2, cudaMemcpyHostToDevice);
        cudaMemcpy(d, in, 4 * sizeof(double), cudaMemcpyHostToDevice);
        if (np_carlson_batch_device(1, dt, d, d + 1, d + 2, d + 3, d + 4, nullptr) == NP_OK)
            cudaMemcpy(&r, d + 4, sizeof(double), cudaMemcpyDeviceToHost);
    }
    std::printf("RF(1, 2, 0) = %.16f\n", r);
    cudaFree(dt);
    cudaFree(d);
}

}  // extern "C"
