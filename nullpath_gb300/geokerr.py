"""Python entry points of the GEOKERR-equivalent solver (include/geokerr_c_api.h).

The f90-compatible functions take and return host numpy arrays; the batched
functions take torch CUDA tensors and run one geodesic per GPU thread.
"""
import ctypes as C

import numpy as np

from ._lib import load, check

D, I, V = C.c_double, C.c_int, C.c_void_p
_PROTOS = {
    "geokerr_eval_lambda": (None, [D] * 9 + [I] + [V] * 5 + [C.POINTER(I)] * 3),
    "geokerr_estimate_periods": (None, [D] * 5 + [C.POINTER(D), C.POINTER(D), C.POINTER(I)]),
    "geokerr_phi_omega": (D, [D] * 5),
    "geokerr_stream_cuda": (I, [D] * 8 + [I] + [V] * 5),
    "geokerr_complete_stream_cuda": (I, [D] * 8 + [I] + [V] * 5),
    "compute_geokerr_complete_cuda": (None, [V] * 12 + [I]),
    "np_geokerr_points_device": (I, [I, D] + [V] * 7 + [I, I, D] + [V] * 8 + [V]),
    "np_geokerr_points_taylor_device": (I, [I, D] + [V] * 7 + [I, I, D] + [V] * 8 + [V]),
    "np_geokerr_points_host": (I, [I, D] + [V] * 7 + [I, I, D] + [V] * 8 + [V]),
    "np_geokerr_eval_lambda_device": (I, [I, D] + [V] * 8 + [I] + [V] * 8 + [V, V]),
    "np_geokerr_eval_lambda_work_bytes": (C.c_size_t, [I, I]),
    "np_geokerr_equator_crossings_device": (I, [I, D] + [V] * 6 + [D, I] + [V] * 3 + [V]),
    "np_geokerr_final_state_host": (I, [I] + [V] * 13),
    "geokerr_cuda_batch": (None, [V] * 10 + [I, I, D]),
    "geokerr_improved_batch": (None, [V] * 10 + [I, I, D]),
    "compute_mino_time_batch_cuda": (None, [V] * 14 + [I]),
    "geokerr_single_case_": (None, [V] * 13),
    "np_geokerr_camera_grid_device": (I, [D, D, I, I, D, D, D, D, D] + [V] * 6 + [V]),
    "np_geokerr_camera_grid_host": (I, [D, D, I, I, D, D, D, D, D] + [V] * 6),
    "np_geokerr_disk_crossings_device": (I, [I, D] + [V] * 6 + [D, D, D, I] + [V] * 4 + [V]),
    "np_geokerr_disk_crossings_host": (I, [I, D] + [V] * 6 + [D, D, D, I] + [V] * 4),
}


def _lib():
    lib = load()
    if not getattr(lib, "_gk_ready", False):
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib._gk_ready = True
    return lib


def _vp(a):
    return a.ctypes.data_as(V)


def eval_lambda(u0, mu0, uf, a, Lz, Q2, t0, lam0, dlam, S):
    """geokerr_eval_lambda on the GPU; returns a dict of numpy arrays."""
    lib = _lib()
    arrs = [np.zeros(S) for _ in range(5)]
    tpmi, tpri, info = I(), I(), I()
    lib.geokerr_eval_lambda(u0, mu0, uf, a, Lz, Q2, t0, lam0, dlam, S, *[_vp(x) for x in arrs],
                            C.byref(tpmi), C.byref(tpri), C.byref(info))
    return dict(u=arrs[0], mu=arrs[1], t=arrs[2], phi=arrs[3], affine=arrs[4],
                tpmi=tpmi.value, tpri=tpri.value, info=info.value)


def estimate_periods(u0, mu0, a, Lz, Q2):
    lib = _lib()
    tr, tt, info = D(), D(), I()
    lib.geokerr_estimate_periods(u0, mu0, a, Lz, Q2, C.byref(tr), C.byref(tt), C.byref(info))
    return tr.value, tt.value, info.value


def phi_omega(u0, mu0, a, Lz, Q2):
    return _lib().geokerr_phi_omega(u0, mu0, a, Lz, Q2)


def stream(u0, uf, mu0, a, L, Q2, lam0, dlam, S, complete=False):
    lib = _lib()
    arrs = [np.zeros(S) for _ in range(5)]
    fn = lib.geokerr_complete_stream_cuda if complete else lib.geokerr_stream_cuda
    rc = fn(u0, uf, mu0, a, L, Q2, lam0, dlam, S, *[_vp(x) for x in arrs])
    return rc, dict(u=arrs[0], mu=arrs[1], t=arrs[2], phi=arrs[3], affine=arrs[4])


def complete(u0, uf, mu0, a, l, q2, su, sm):
    lib = _lib()
    n = len(u0)
    f = lambda x: np.ascontiguousarray(x, np.float64)
    i = lambda x: np.ascontiguousarray(x, np.int32)
    ins = [f(u0), f(uf), f(mu0), f(a), f(l), f(q2), i(su), i(sm)]
    lam, muf = np.zeros(n), np.zeros(n)
    nc, valid = np.zeros(n, np.int32), np.zeros(n, np.int8)
    lib.compute_geokerr_complete_cuda(*[_vp(x) for x in ins], _vp(lam), _vp(muf), _vp(nc), _vp(valid), n)
    return lam, muf, nc, valid


def final_state(a, u0, mu0, l, q2, su, sm, lam):
    """np_geokerr_final_state_host: (u, mu, t, phi, valid) at Mino time lam per ray."""
    lib = _lib()
    f = lambda x: np.ascontiguousarray(np.broadcast_to(np.asarray(x, np.float64), np.shape(u0)), np.float64)
    ins = [f(v) for v in (a, u0, mu0, l, q2, su, sm, lam)]
    n = ins[1].size
    outs = [np.zeros(n) for _ in range(4)]
    valid = np.zeros(n, np.int8)
    check(lib.np_geokerr_final_state_host(n, *[_vp(x) for x in ins], *[_vp(x) for x in outs], _vp(valid)))
    return (*outs, valid)


def cuda_batch(a, r0, mu0, E, L, Q2, lambda_max, n_steps=1000, improved=False):
    """geokerr_cuda_batch / geokerr_improved_batch: final (r, mu, phi, t) per ray."""
    lib = _lib()
    f = lambda x: np.ascontiguousarray(x, np.float64)
    ins = [f(v) for v in (a, r0, mu0, E, L, Q2)]
    n = ins[0].size
    outs = [np.zeros(n) for _ in range(4)]
    fn = lib.geokerr_improved_batch if improved else lib.geokerr_cuda_batch
    fn(*[_vp(x) for x in ins], *[_vp(x) for x in outs], n, n_steps, lambda_max)
    return tuple(outs)


def mino_time_batch(u0, uf, mu0, muf, a, l, q2, tpm, tpr, su, sm, ncase):
    """compute_mino_time_batch_cuda: (lambda, valid) per case."""
    lib = _lib()
    f = lambda x: np.ascontiguousarray(x, np.float64)
    i = lambda x: np.ascontiguousarray(x, np.int32)
    ins = [f(u0), f(uf), f(mu0), f(muf), f(a), f(l), f(q2), i(tpm), i(tpr), i(su), i(sm), i(ncase)]
    n = ins[0].size
    lam, valid = np.zeros(n), np.zeros(n, np.int8)
    lib.compute_mino_time_batch_cuda(*[_vp(x) for x in ins], _vp(lam), _vp(valid), n)
    return lam, valid


def single_case(u0, uf, mu0, a, l, q2, su, sm, muf=0.0):
    """geokerr_single_case_ (by-reference arguments): (lambda, muf, ncase, valid)."""
    lib = _lib()
    d = [C.c_double(v) for v in (u0, uf, mu0, muf, a, l, q2)]
    iv = [C.c_int(int(su)), C.c_int(int(sm))]
    lam, mo, nc, ok = C.c_double(), C.c_double(), C.c_int(), C.c_int()
    lib.geokerr_single_case_(*[C.byref(x) for x in d], *[C.byref(x) for x in iv], C.byref(lam), C.byref(mo),
                             C.byref(nc), C.byref(ok))
    return lam.value, mo.value, nc.value, ok.value


def _t(x):
    return C.c_void_p(x.data_ptr()) if x is not None else None


def points(a, u0, uf, mu0, l, q2, su, sm, tpr=1, nup=32, offset=0.5, method="closed_form"):
    """Batched GEOKERR sampler on CUDA tensors; returns a dict of [n, nup]
    tensors.  method "closed_form" evaluates every point on its own thread
    (rays outside the closed forms on the Taylor solver); "taylor" integrates
    every ray with the order-24 Taylor solver."""
    import torch
    lib = _lib()
    dev = torch.device("cuda")
    cv = lambda x: torch.as_tensor(x, dtype=torch.float64, device=dev).contiguous()
    ins = [cv(x) for x in (u0, uf, mu0, l, q2, su, sm)]
    n = ins[0].numel()
    out = {k: torch.zeros((n, nup), dtype=torch.float64, device=dev) for k in ("u", "mu", "dt", "dphi", "lam")}
    out["tpm"] = torch.zeros((n, nup), dtype=torch.int32, device=dev)
    out["tpr"] = torch.zeros((n, nup), dtype=torch.int32, device=dev)
    out["n"] = torch.zeros(n, dtype=torch.int32, device=dev)
    if method not in ("closed_form", "taylor"):
        raise ValueError("method must be 'closed_form' or 'taylor'")
    fn = lib.np_geokerr_points_device if method == "closed_form" else lib.np_geokerr_points_taylor_device
    check(fn(n, a, *[_t(x) for x in ins], tpr, nup, offset,
             *[_t(out[k]) for k in ("u", "mu", "dt", "dphi", "lam", "tpm", "tpr", "n")],
             C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return out


def points_host(a, u0, uf, mu0, l, q2, su, sm, tpr=1, nup=32, offset=0.5):
    """The closed-form sampler run on the host (the device code's arithmetic,
    the same bits); numpy in and out, plus method[n] (1: four real radial
    roots, 2: two real roots and a complex pair around the motion, 3: two
    real roots below it and a complex pair, 4: two complex pairs, 0: Taylor
    solver or no points)."""
    lib = _lib()
    cv = lambda x: np.ascontiguousarray(np.broadcast_to(np.asarray(x, dtype=np.float64), np.shape(l)))
    ins = [cv(x) for x in (u0, uf, mu0, l, q2, su, sm)]
    n = ins[0].size
    out = {k: np.zeros((n, nup), dtype=np.float64) for k in ("u", "mu", "dt", "dphi", "lam")}
    out["tpm"] = np.zeros((n, nup), dtype=np.int32)
    out["tpr"] = np.zeros((n, nup), dtype=np.int32)
    out["n"] = np.zeros(n, dtype=np.int32)
    out["method"] = np.zeros(n, dtype=np.int32)
    check(lib.np_geokerr_points_host(n, a, *[x.ctypes.data for x in ins], tpr, nup, offset,
                                     *[out[k].ctypes.data for k in ("u", "mu", "dt", "dphi", "lam", "tpm", "tpr", "n",
                                                                    "method")]))
    return out


def disk_crossings(a, u0, mu0, l, q2, su, sm, u_far, u_lo=0.0, u_hi=float("inf"), K=4, device=False, phi=True):
    """Equatorial crossings by Jacobi amplitude (np_geokerr_disk_crossings_*):
    the first K crossings with u in [u_lo, u_hi] up to the ray's end (the
    horizon, or u_far after its turning point).  Returns dict xu[n][K],
    xphi[n][K] (azimuth change from the start; when phi), nx[n] and
    status[n] (0 leaves, 1 captured, -1 outside the closed forms), numpy
    arrays on the host, CUDA tensors with device=True."""
    lib = _lib()
    if device:
        import torch
        dev = torch.device("cuda")
        cv = lambda x: torch.as_tensor(np.broadcast_to(np.asarray(x, dtype=np.float64), np.shape(l)).copy(),
                                       device=dev).contiguous()
        ins = [cv(x) for x in (u0, mu0, l, q2, su, sm)]
        n = ins[0].numel()
        out = {"xu": torch.zeros((n, K), dtype=torch.float64, device=dev),
               "nx": torch.zeros(n, dtype=torch.int32, device=dev),
               "status": torch.zeros(n, dtype=torch.int32, device=dev)}
        if phi:
            out["xphi"] = torch.zeros((n, K), dtype=torch.float64, device=dev)
        ptr = lambda t: V(t.data_ptr()) if t is not None else None
        check(lib.np_geokerr_disk_crossings_device(n, a, *[ptr(x) for x in ins], u_far, u_lo, u_hi, K,
                                                   ptr(out["xu"]), ptr(out.get("xphi")), ptr(out["nx"]),
                                                   ptr(out["status"]), V(torch.cuda.current_stream().cuda_stream)))
        return out
    cv = lambda x: np.ascontiguousarray(np.broadcast_to(np.asarray(x, dtype=np.float64), np.shape(l)))
    ins = [cv(x) for x in (u0, mu0, l, q2, su, sm)]
    n = ins[0].size
    out = {"xu": np.zeros((n, K)), "nx": np.zeros(n, dtype=np.int32), "status": np.zeros(n, dtype=np.int32)}
    if phi:
        out["xphi"] = np.zeros((n, K))
    check(lib.np_geokerr_disk_crossings_host(n, a, *[x.ctypes.data for x in ins], u_far, u_lo, u_hi, K,
                                             out["xu"].ctypes.data, out["xphi"].ctypes.data if phi else None,
                                             out["nx"].ctypes.data, out["status"].ctypes.data))
    return out


def eval_lambda_batch(a, u0, mu0, uf, Lz, Q2, t0, lam0, dlam, S):
    """Batched geokerr_eval_lambda on CUDA tensors."""
    import torch
    lib = _lib()
    dev = torch.device("cuda")
    cv = lambda x: torch.as_tensor(x, dtype=torch.float64, device=dev).contiguous()
    ins = [cv(x) for x in (u0, mu0, uf, Lz, Q2, t0, lam0, dlam)]
    n = ins[0].numel()
    out = {k: torch.zeros((n, S), dtype=torch.float64, device=dev) for k in ("u", "mu", "t", "phi", "affine")}
    for k in ("tpmi", "tpri", "info"):
        out[k] = torch.zeros(n, dtype=torch.int32, device=dev)
    work = torch.empty(lib.np_geokerr_eval_lambda_work_bytes(n, S), dtype=torch.uint8, device=dev)
    check(lib.np_geokerr_eval_lambda_device(n, a, *[_t(x) for x in ins], S,
                                            *[_t(out[k]) for k in ("u", "mu", "t", "phi", "affine", "tpmi", "tpri",
                                                                   "info")],
                                            _t(work), C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return out


def equator_crossings(a, u0, mu0, l, q2, su, sm, u_end=1e-3, K=4):
    """First K equatorial crossings (u, phi) per ray on CUDA tensors."""
    import torch
    lib = _lib()
    dev = torch.device("cuda")
    cv = lambda x: torch.as_tensor(x, dtype=torch.float64, device=dev).contiguous()
    ins = [cv(x) for x in (u0, mu0, l, q2, su, sm)]
    n = ins[0].numel()
    xu = torch.zeros((n, K), dtype=torch.float64, device=dev)
    xphi = torch.zeros((n, K), dtype=torch.float64, device=dev)
    nx = torch.zeros(n, dtype=torch.int32, device=dev)
    check(lib.np_geokerr_equator_crossings_device(n, a, *[_t(x) for x in ins], u_end, K, _t(xu), _t(xphi), _t(nx),
                                                  C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return xu, xphi, nx


def render_ray_constants(consts, scene):
    """GEOKERR inputs (u0, mu0, l, q2, su, sm) of render rays from their camera
    momenta (p_t, p_phi, p_r, p_theta) as returned by trace_rays: E = -p_t,
    l = p_phi/(E M), q2 = Q/(E M)^2 with Carter's Q = p_theta^2 +
    cos^2(theta) (L^2/sin^2(theta) - a^2 E^2); su = +1 for ingoing rays
    (p_r < 0) and sm = -sign(p_theta), since mu = cos(theta)."""
    import math
    c = np.asarray(consts)
    E, L, pr, pth = -c[:, 0], c[:, 1], c[:, 2], c[:, 3]
    M = scene.mass
    lunit = M if scene.units == 1 else 2.0 * M
    r_cam = scene.r_cam * lunit
    th = math.radians(scene.theta_deg)
    a = scene.spin * M
    Q = pth * pth + math.cos(th) ** 2 * (L * L / math.sin(th) ** 2 - a * a * E * E)
    n = len(E)
    u0 = np.full(n, M / r_cam)
    mu0 = np.full(n, math.cos(th))
    su = np.where(pr < 0, 1.0, -1.0)
    sm = np.where(pth > 0, -1.0, 1.0)
    return u0, mu0, L / (E * M), Q / (E * E * M * M), su, sm


_GRID_KEYS = ("alpha", "beta", "l", "q2", "su", "sm")


def camera_grid(a, mu0, n_alpha, n_beta, a1=-12.0, a2=12.0, b1=-12.0, b2=12.0, input_limit=1e-5, device=True):
    """GEOKERR's standard camera grid (geokerr_original.f:183-220): dict of
    alpha, beta, l, q2, su, sm over n_alpha x n_beta cell-centred positions
    (ray i n_beta + j), as CUDA float64 tensors (device=True, filled by a
    kernel) or numpy arrays (the host entry point)."""
    lib = _lib()
    n = n_alpha * n_beta
    if device:
        import torch
        out = {k: torch.empty(n, dtype=torch.float64, device="cuda") for k in _GRID_KEYS}
        check(lib.np_geokerr_camera_grid_device(a, mu0, n_alpha, n_beta, a1, a2, b1, b2, input_limit,
                                                *[V(out[k].data_ptr()) for k in _GRID_KEYS],
                                                V(torch.cuda.current_stream().cuda_stream)))
        return out
    out = {k: np.empty(n) for k in _GRID_KEYS}
    check(lib.np_geokerr_camera_grid_host(a, mu0, n_alpha, n_beta, a1, a2, b1, b2, input_limit,
                                          *[_vp(out[k]) for k in _GRID_KEYS]))
    return out
