"""The physics-header API (include/np_kerr.h) from Python: camera rays plus
fixed FP64 RK4 steps, on the device or on the host (np_kerr_integrate_*)."""
import ctypes as C

import numpy as np

from ._lib import load, check

_PROTOS = {
    "np_kerr_integrate_device": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_void_p, C.c_int, C.c_double, C.c_int,
                                           C.c_void_p, C.c_void_p, C.c_void_p]),
    "np_kerr_integrate_host": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_void_p, C.c_int, C.c_double, C.c_int,
                                         C.c_void_p, C.c_void_p]),
}


def _lib():
    lib = load()
    if not getattr(lib, "_kerr_ready", False):
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib._kerr_ready = True
    return lib


def integrate(M, a, cam, steps, h_scale=0.01, zamo=False, device=True):
    """cam: [n, 6] array of (r, theta, phi, n_r, n_theta, n_phi).  Returns
    (states [n, 8] = (t, r, theta, phi, p_t, p_r, p_theta, p_phi), alive [n])
    as numpy arrays."""
    cam = np.ascontiguousarray(cam, dtype=np.float64)
    n = cam.shape[0]
    lib = _lib()
    if device:
        import torch
        dc = torch.from_numpy(cam).cuda()
        ds = torch.empty((n, 8), dtype=torch.float64, device="cuda")
        da = torch.empty((n,), dtype=torch.int32, device="cuda")
        check(lib.np_kerr_integrate_device(n, M, a, C.c_void_p(dc.data_ptr()), steps, h_scale, int(zamo),
                                           C.c_void_p(ds.data_ptr()), C.c_void_p(da.data_ptr()),
                                           C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        torch.cuda.synchronize()
        return ds.cpu().numpy(), da.cpu().numpy()
    st = np.empty((n, 8), dtype=np.float64)
    al = np.empty((n,), dtype=np.int32)
    check(lib.np_kerr_integrate_host(n, M, a, cam.ctypes.data, steps, h_scale, int(zamo), st.ctypes.data,
                                     al.ctypes.data))
    return st, al
