"""Carlson symmetric elliptic integrals over the np_carlson_batch_* C ABI
(include/geokerr_c_api.h)."""
import ctypes as C

import numpy as np

from ._lib import load, check

_PROTOS = {
    "np_carlson_batch_device": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_void_p]),
    "np_carlson_batch_host": (C.c_int, [C.c_int, C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p]),
}


def _lib():
    lib = load()
    if not getattr(lib, "_carlson_ready", False):
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib._carlson_ready = True
    return lib


def evaluate(kinds, x, y, z=None, p=None, device=True):
    """kinds: sequence of "RF"/"RC"/"RD"/"RJ"; returns a float64 numpy array."""
    n = len(kinds)
    types = "".join(kinds).encode()
    assert len(types) == 2 * n
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    z = np.ascontiguousarray(np.zeros(n) if z is None else z, dtype=np.float64)
    p = np.ascontiguousarray(np.zeros(n) if p is None else p, dtype=np.float64)
    lib = _lib()
    if not device:
        out = np.empty(n)
        check(lib.np_carlson_batch_host(n, types, x.ctypes.data, y.ctypes.data, z.ctypes.data, p.ctypes.data,
                                        out.ctypes.data))
        return out
    import torch
    dt = torch.frombuffer(bytearray(types), dtype=torch.uint8).cuda()
    dx, dy, dz, dp = (torch.from_numpy(v).cuda() for v in (x, y, z, p))
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    check(lib.np_carlson_batch_device(n, C.c_void_p(dt.data_ptr()), C.c_void_p(dx.data_ptr()),
                                      C.c_void_p(dy.data_ptr()), C.c_void_p(dz.data_ptr()), C.c_void_p(dp.data_ptr()),
                                      C.c_void_p(out.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    return out.cpu().numpy()
