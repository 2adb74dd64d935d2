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


_MINO = {
    "np_geokerr_mino_times_device": (C.c_int, [C.c_int, C.c_double] + [C.c_void_p] * 8 + [C.c_void_p]),
    "np_geokerr_mino_times_host": (C.c_int, [C.c_int, C.c_double] + [C.c_void_p] * 8),
}


def mino_times(a, ua, ub, mua, mub, l, q2, device=True):
    """Semi-analytic Mino times (lam_u, lam_mu) of monotonic radial and polar
    segments with Carlson's R_F (np_geokerr_mino_times_*)."""
    lib = _lib()
    if not getattr(lib, "_mino_ready", False):
        for name, (res, args) in _MINO.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib._mino_ready = True
    ins = [np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), np.shape(ua)))
           for v in (ua, ub, mua, mub, l, q2)]
    n = ins[0].size
    if not device:
        lu, lm = np.empty(n), np.empty(n)
        check(lib.np_geokerr_mino_times_host(n, a, *[v.ctypes.data for v in ins], lu.ctypes.data, lm.ctypes.data))
        return lu, lm
    import torch
    d = [torch.from_numpy(v.ravel().copy()).cuda() for v in ins]
    lu = torch.empty(n, dtype=torch.float64, device="cuda")
    lm = torch.empty(n, dtype=torch.float64, device="cuda")
    check(lib.np_geokerr_mino_times_device(n, a, *[C.c_void_p(t.data_ptr()) for t in d], C.c_void_p(lu.data_ptr()),
                                           C.c_void_p(lm.data_ptr()),
                                           C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    return lu.cpu().numpy(), lm.cpu().numpy()


_POLAR = {
    "np_geokerr_mu_of_lambda_host": (C.c_int, [C.c_int, C.c_double] + [C.c_void_p] * 6),
    "np_geokerr_mu_of_lambda_device": (C.c_int, [C.c_int, C.c_double] + [C.c_void_p] * 6 + [C.c_void_p]),
    "np_jacobi_host": (C.c_int, [C.c_int] + [C.c_void_p] * 5),
}


def _polar_lib():
    lib = _lib()
    if not getattr(lib, "_polar_ready", False):
        for name, (res, args) in _POLAR.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib._polar_ready = True
    return lib


def jacobi(u, m):
    """(sn, cn, dn)(u | m) on the host."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    m = np.ascontiguousarray(np.broadcast_to(np.asarray(m, dtype=np.float64), u.shape))
    out = [np.empty(u.size) for _ in range(3)]
    check(_polar_lib().np_jacobi_host(u.size, u.ctypes.data, m.ctypes.data, *[o.ctypes.data for o in out]))
    return tuple(out)


def mu_of_lambda(a, l, q2, mu0, sm, lam, device=True):
    """Closed-form polar motion mu(lambda) (np_geokerr_mu_of_lambda_*)."""
    lam = np.ascontiguousarray(lam, dtype=np.float64)
    ins = [np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), lam.shape)) for v in (l, q2, mu0, sm)]
    n = lam.size
    lib = _polar_lib()
    if not device:
        out = np.empty(n)
        check(lib.np_geokerr_mu_of_lambda_host(n, a, *[v.ctypes.data for v in ins], lam.ctypes.data, out.ctypes.data))
        return out
    import torch
    d = [torch.from_numpy(v.ravel().copy()).cuda() for v in ins + [lam]]
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    check(lib.np_geokerr_mu_of_lambda_device(n, a, *[C.c_void_p(t.data_ptr()) for t in d], C.c_void_p(out.data_ptr()),
                                             C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    return out.cpu().numpy()


def equator_crossings_cf(a, u0, mu0, l, q2, su, sm, u_end=1e-3, K=4, device=False):
    """Closed-form equatorial crossings (np_geokerr_equator_crossings_cf_*):
    (xu [n, K], nx [n])."""
    lib = _lib()
    if not getattr(lib, "_cf_ready", False):
        lib.np_geokerr_equator_crossings_cf_host.restype = C.c_int
        lib.np_geokerr_equator_crossings_cf_host.argtypes = [C.c_int, C.c_double] + [C.c_void_p] * 6 + \
            [C.c_double, C.c_int, C.c_void_p, C.c_void_p]
        lib.np_geokerr_equator_crossings_cf_device.restype = C.c_int
        lib.np_geokerr_equator_crossings_cf_device.argtypes = [C.c_int, C.c_double] + [C.c_void_p] * 6 + \
            [C.c_double, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        lib._cf_ready = True
    ins = [np.ascontiguousarray(np.atleast_1d(np.asarray(v, dtype=np.float64))) for v in (u0, mu0, l, q2, su, sm)]
    n = max(v.size for v in ins)
    ins = [np.ascontiguousarray(np.broadcast_to(v, (n,))) for v in ins]
    if not device:
        xu = np.zeros((n, K))
        nx = np.zeros(n, np.int32)
        check(lib.np_geokerr_equator_crossings_cf_host(n, a, *[v.ctypes.data for v in ins], u_end, K, xu.ctypes.data,
                                                       nx.ctypes.data))
        return xu, nx
    import torch
    d = [torch.from_numpy(v.copy()).cuda() for v in ins]
    xu = torch.zeros((n, K), dtype=torch.float64, device="cuda")
    nx = torch.zeros(n, dtype=torch.int32, device="cuda")
    check(lib.np_geokerr_equator_crossings_cf_device(n, a, *[C.c_void_p(t.data_ptr()) for t in d], u_end, K,
                                                     C.c_void_p(xu.data_ptr()), C.c_void_p(nx.data_ptr()),
                                                     C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    return xu.cpu().numpy(), nx.cpu().numpy()
