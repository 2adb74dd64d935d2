"""Schwarzschild deflection table (np_schwarzschild_* of include/np_render.h)."""
import ctypes as C

import numpy as np

from ._lib import load, check

_PROTOS = {
    "np_schwarzschild_deflection_device": (C.c_int, [C.c_float, C.c_float, C.c_int] + [C.c_void_p] * 5),
    "np_schwarzschild_deflection_host": (C.c_int, [C.c_float, C.c_float, C.c_int] + [C.c_void_p] * 4),
    "np_schwarzschild_precompute": (C.c_int, [C.c_float, C.c_int] + [C.c_void_p] * 5),
}


def _lib():
    lib = load()
    if not getattr(lib, "_schw_ready", False):
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib._schw_ready = True
    return lib


def deflection(mass, b, r_start=1000.0, device=True):
    """(deflection, r_min, status) of equatorial photons with impact parameters b."""
    b = np.ascontiguousarray(b, dtype=np.float32)
    n = b.size
    lib = _lib()
    if not device:
        d, r, s = np.empty(n, np.float32), np.empty(n, np.float32), np.empty(n, np.int32)
        check(lib.np_schwarzschild_deflection_host(mass, r_start, n, b.ctypes.data, d.ctypes.data, r.ctypes.data,
                                                   s.ctypes.data))
        return d, r, s
    import torch
    db = torch.from_numpy(b).cuda()
    d = torch.empty(n, dtype=torch.float32, device="cuda")
    r = torch.empty(n, dtype=torch.float32, device="cuda")
    s = torch.empty(n, dtype=torch.int32, device="cuda")
    check(lib.np_schwarzschild_deflection_device(mass, r_start, n, C.c_void_p(db.data_ptr()), C.c_void_p(d.data_ptr()),
                                                 C.c_void_p(r.data_ptr()), C.c_void_p(s.data_ptr()),
                                                 C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    return d.cpu().numpy(), r.cpu().numpy(), s.cpu().numpy()


def precompute(mass, n):
    """The reference's precomputeGeodesics: dict of b, deflection, bending, r_min, status."""
    out = {k: np.empty(n, np.float32) for k in ("b", "deflection", "bending", "rmin")}
    out["status"] = np.empty(n, np.int32)
    check(_lib().np_schwarzschild_precompute(mass, n, *[out[k].ctypes.data for k in
                                                         ("b", "deflection", "bending", "rmin", "status")]))
    return out
