// kerr_api.cu -- C-ABI access to the physics-header API (include/np_kerr.h)
// on the device and, with the same header code, on the host: camera rays of
// a static observer (or ZAMO) followed by fixed FP64 RK4 steps, one ray per
// thread.  It lets callers of the reference's bh_kerr.h building blocks
// (bh_kerr.h:734-967) drive them from C, ctypes or cgo, and it checks that
// the header compiles and agrees between sm_103a and the host.
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

NP_HD inline int kerr_one(double M, double a, const double* cam, int steps, double h_scale, int zamo, double* st) {
    const double r = cam[0], th = cam[1], ph = cam[2];
    GeodesicStateD s = zamo ? init_ray_from_camera_zamo_d(M, a, r, th, ph, cam[3], cam[4], cam[5])
                            : init_ray_from_camera_general_d(M, a, r, th, ph, cam[3], cam[4], cam[5]);
    bool alive = true;
    for (int k = 0; k < steps && alive; ++k) alive = integrateGeodesicKerrD(s, M, a, h_scale * s.r);
    st[0] = s.t; st[1] = s.r; st[2] = s.theta; st[3] = s.phi;
    st[4] = s.pt; st[5] = s.pr; st[6] = s.ptheta; st[7] = s.pphi;
    return alive ? 1 : 0;
}

__global__ void kerr_integrate_kernel(int n, double M, double a, const double* __restrict__ cam, int steps,
                                      double h_scale, int zamo, double* __restrict__ states, int* __restrict__ alive) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        alive[i] = kerr_one(M, a, cam + 6 * (size_t)i, steps, h_scale, zamo, states + 8 * (size_t)i);
}

int check_args(int n, double M, double a, const double* cam, int steps, double* states, int* alive) {
    if (n < 0 || !cam || !states || !alive || steps < 0) {
        np_record_error("np_kerr_integrate: NULL buffer or negative count");
        return NP_ERR_INVALID;
    }
    if (!(M > 0.0) || !(a * a < M * M)) {
        np_record_error("np_kerr_integrate: need M > 0 and |a| < M");
        return NP_ERR_INVALID;
    }
    return NP_OK;
}

}  // namespace

extern "C" {

int np_kerr_integrate_device(int n, double M, double a, const double* d_cam, int steps, double h_scale, int zamo,
                             double* d_states, int* d_alive, void* stream) {
    int rc = check_args(n, M, a, d_cam, steps, d_states, d_alive);
    if (rc != NP_OK || n == 0) return rc;
    const int threads = 128, cap = device_sms() * 16;
    const int blocks = (int)((n + threads - 1) / threads < cap ? (n + threads - 1) / threads : cap);
    kerr_integrate_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(n, M, a, d_cam, steps, h_scale, zamo, d_states,
                                                                       d_alive);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        np_record_error(cudaGetErrorString(e));
        return NP_ERR_KERNEL;
    }
    return NP_OK;
}

int np_kerr_integrate_host(int n, double M, double a, const double* cam, int steps, double h_scale, int zamo,
                           double* states, int* alive) {
    int rc = check_args(n, M, a, cam, steps, states, alive);
    if (rc != NP_OK) return rc;
    for (int i = 0; i < n; ++i) alive[i] = kerr_one(M, a, cam + 6 * (size_t)i, steps, h_scale, zamo, states + 8 * (size_t)i);
    return NP_OK;
}

}  // extern "C"
