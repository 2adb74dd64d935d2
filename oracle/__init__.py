"""ctypes access to the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import
this package; the product library never calls it.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_O = None
_R = None


def _scene_type():
    from nullpath_gb300._abi import Scene
    return Scene


def load():
    global _O
    if _O is None:
        p = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(p):
            raise RuntimeError("oracle/liboracle.so not built; run `make -C oracle`")
        lib = C.CDLL(p)
        S = C.POINTER(_scene_type())
        lib.npo_render.argtypes = [S, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        lib.npo_render.restype = C.c_int
        lib.npo_trace_rays.argtypes = [S, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_int]
        lib.npo_trace_rays.restype = C.c_int
        lib.npo_trace_invariants.argtypes = [S, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        lib.npo_trace_invariants.restype = C.c_int
        lib.npo_rkf78_tableau.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        lib.npo_rkf78_tableau.restype = None
        lib.npo_frame_rays.argtypes = [S, C.c_int, C.c_int, C.c_void_p]
        lib.npo_frame_rays.restype = C.c_int
        lib.npo_critical_curve.argtypes = [S, C.c_void_p]
        lib.npo_critical_curve.restype = C.c_int
        lib.npo_metric_inv.argtypes = [C.c_double] * 4 + [C.c_void_p]
        lib.npo_metric_inv.restype = None
        lib.npo_metric_inv_derivs.argtypes = [C.c_double] * 4 + [C.c_void_p, C.c_void_p]
        lib.npo_metric_inv_derivs.restype = None
        _O = lib
    return _O


def load_ref():
    """The reference's own headers compiled here (oracle/_ref); None when absent."""
    global _R
    if _R is None:
        p = os.path.join(HERE, "_ref", "libnpref.so")
        if not os.path.exists(p):
            return None
        lib = C.CDLL(p)
        S = C.POINTER(_scene_type())
        lib.npref_render.argtypes = [S, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        lib.npref_render.restype = C.c_int
        lib.npref_metric_inv.argtypes = [C.c_double] * 4 + [C.c_void_p]
        lib.npref_metric_inv_derivs.argtypes = [C.c_double] * 4 + [C.c_void_p, C.c_void_p]
        _R = lib
    return _R


def _vp(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def render(scene, y0=0, y1=None, threads=0, with_inv=False):
    """Oracle render of rows [y0, y1): returns (rgb[3,H,W], rcross[H,W][, inv3])."""
    lib = load()
    H, W = scene.height, scene.width
    y1 = H if y1 is None else y1
    rgb = np.zeros((3, H, W), np.float32)
    rc = np.zeros((H, W), np.float32)
    inv = np.zeros(3, np.float32) if with_inv else None
    rc_ = lib.npo_render(C.byref(scene), y0, y1, _vp(rgb), _vp(rc), _vp(inv), threads)
    if rc_ != 0:
        raise RuntimeError("oracle render failed: %d" % rc_)
    return (rgb, rc, inv) if with_inv else (rgb, rc)


def render_ref(scene, y0=0, y1=None):
    lib = load_ref()
    if lib is None:
        return None
    H, W = scene.height, scene.width
    y1 = H if y1 is None else y1
    rgb = np.zeros((3, H, W), np.float32)
    rc = np.zeros((H, W), np.float32)
    if lib.npref_render(C.byref(scene), y0, y1, _vp(rgb), _vp(rc)) != 0:
        raise RuntimeError("reference render failed")
    return rgb, rc


def trace_rays(scene, px, py, threads=0):
    lib = load()
    px = np.ascontiguousarray(px, np.float64)
    py = np.ascontiguousarray(py, np.float64)
    n = px.size
    consts = np.zeros((n, 4), np.float64)
    cross = np.zeros((n, 4, 2), np.float64)
    status = np.zeros(n, np.int32)
    steps = np.zeros(n, np.int32)
    if lib.npo_trace_rays(C.byref(scene), n, _vp(px), _vp(py), _vp(consts), _vp(cross), _vp(status),
                          _vp(steps), threads) != 0:
        raise RuntimeError("oracle trace failed")
    return {"consts": consts, "cross": cross, "status": status, "steps": steps}


def frame_rays(scene, y0, y1):
    """Camera momenta (p_t, p_phi, p_r, p_theta) of sample `sample_offset` of
    every pixel of rows [y0, y1): array [y1 - y0, width, 4]."""
    out = np.zeros((y1 - y0, scene.width, 4), np.float64)
    if load().npo_frame_rays(C.byref(scene), y0, y1, _vp(out)) != 0:
        raise RuntimeError("npo_frame_rays failed")
    return out


def frame_crossings(scene, y0, y1, K=4, threads=None):
    """Equatorial crossing radii (Mino-time solver, GEOR with mu_f = 0) of
    the rays of frame_rays(scene, y0, y1): array [y1 - y0, width, K], 0
    where a ray has fewer crossings.  The solver stops at u = M / escape_r."""
    import math
    from concurrent.futures import ThreadPoolExecutor
    c = frame_rays(scene, y0, y1).reshape(-1, 4)
    M = scene.mass
    lunit = M if scene.units == 1 else 2.0 * M
    r_cam = scene.r_cam * lunit
    th = math.radians(scene.theta_deg)
    a = scene.spin * M
    E, L, pr, pth = -c[:, 0], c[:, 1], c[:, 2], c[:, 3]
    Q = pth * pth + math.cos(th) ** 2 * (L * L / math.sin(th) ** 2 - a * a * E * E)
    l, q2 = L / (E * M), Q / (E * E * M * M)
    su = np.where(pr < 0, 1.0, -1.0)
    sm = np.where(pth > 0, -1.0, 1.0)
    r_far = scene.escape_r if scene.escape_r > 0 else (scene.r_cam + 20.0) * lunit

    def one(i):
        n, xu, _ = geokerr_crossings(M / r_cam, math.cos(th), scene.spin, l[i], q2[i], su[i], sm[i], M / r_far, K)
        return np.where(xu > 0, M / np.maximum(xu, 1e-300), 0.0)
    with ThreadPoolExecutor(max_workers=threads or os.cpu_count()) as ex:
        xr = list(ex.map(one, range(len(E))))
    return np.array(xr).reshape(y1 - y0, scene.width, K)


def trace_invariants(scene, px, py, threads=0):
    """Per-ray (max |H|/E^2, max |dQ|/Q scale) and step counts, as np_trace_invariants_device."""
    lib = load()
    px = np.ascontiguousarray(px, np.float64)
    py = np.ascontiguousarray(py, np.float64)
    n = px.size
    drift = np.zeros((n, 2), np.float64)
    steps = np.zeros(n, np.int32)
    if lib.npo_trace_invariants(C.byref(scene), n, _vp(px), _vp(py), _vp(drift), _vp(steps), threads) != 0:
        raise RuntimeError("oracle trace_invariants failed")
    return drift, steps


def rkf78_tableau():
    """(A[13,13], b8[13], err[13]) of the oracle's Fehlberg 7(8) pair."""
    A = np.zeros((13, 13))
    b = np.zeros(13)
    e = np.zeros(13)
    load().npo_rkf78_tableau(_vp(A), _vp(b), _vp(e))
    return A, b, e


def metric_inv(lib, M, a, r, th):
    g = np.zeros(5)
    fn = lib.npo_metric_inv if hasattr(lib, "npo_metric_inv") else lib.npref_metric_inv
    fn(M, a, r, th, _vp(g))
    return g


def metric_inv_derivs(lib, M, a, r, th):
    dr = np.zeros(5)
    dt = np.zeros(5)
    fn = lib.npo_metric_inv_derivs if hasattr(lib, "npo_metric_inv_derivs") else lib.npref_metric_inv_derivs
    fn(M, a, r, th, _vp(dr), _vp(dt))
    return dr, dt


# ---------------------------------------------------------------------------
# GEOKERR restatement (geokerr_oracle.cpp)

def _geo_protos(lib):
    if getattr(lib, "_geo_ready", False):
        return
    D, I, V = C.c_double, C.c_int, C.c_void_p
    lib.npo_geokerr.argtypes = [D] * 8 + [I, I, D] + [V] * 7
    lib.npo_geokerr.restype = I
    lib.npo_geokerr_eval_lambda.argtypes = [D] * 9 + [I] + [V] * 5 + [C.POINTER(I)] * 3
    lib.npo_geokerr_eval_lambda.restype = None
    lib.npo_geokerr_estimate_periods.argtypes = [D] * 5 + [C.POINTER(D), C.POINTER(D), C.POINTER(I)]
    lib.npo_geokerr_estimate_periods.restype = None
    lib.npo_geokerr_phi_omega.argtypes = [D] * 5
    lib.npo_geokerr_phi_omega.restype = D
    lib.npo_geokerr_stream.argtypes = [D] * 8 + [I] + [V] * 5
    lib.npo_geokerr_stream.restype = I
    lib.npo_geokerr_crossings.argtypes = [D] * 8 + [I, V, V]
    lib.npo_geokerr_crossings.restype = I
    lib.npo_geokerr_final.argtypes = [D] * 8 + [V]
    lib.npo_geokerr_final.restype = I
    lib.npo_geokerr_mino_time.argtypes = [D] * 8 + [I, C.POINTER(D)]
    lib.npo_geokerr_mino_time.restype = I
    lib._geo_ready = True


def geokerr_points(u0, uf, mu0, a, l, q2, su, sm, tpr=1, nup=32, offset=0.5):
    """GEOKERR sampler: dict of u, mu, dt, dphi, lam, tpm, tpr arrays and n."""
    lib = load()
    _geo_protos(lib)
    out = {k: np.zeros(nup) for k in ("u", "mu", "dt", "dphi", "lam")}
    out["tpm"] = np.zeros(nup, np.int32)
    out["tpr"] = np.zeros(nup, np.int32)
    n = lib.npo_geokerr(u0, uf, mu0, a, l, q2, su, sm, tpr, nup, offset,
                        *[_vp(out[k]) for k in ("u", "mu", "dt", "dphi", "lam", "tpm", "tpr")])
    out["n"] = n
    return out


def geokerr_eval_lambda(u0, mu0, uf, a, Lz, Q2, t0, lam0, dlam, S):
    lib = load()
    _geo_protos(lib)
    arrs = [np.zeros(S) for _ in range(5)]
    tpmi, tpri, info = C.c_int(), C.c_int(), C.c_int()
    lib.npo_geokerr_eval_lambda(u0, mu0, uf, a, Lz, Q2, t0, lam0, dlam, S, *[_vp(x) for x in arrs],
                                C.byref(tpmi), C.byref(tpri), C.byref(info))
    return dict(u=arrs[0], mu=arrs[1], t=arrs[2], phi=arrs[3], affine=arrs[4],
                tpmi=tpmi.value, tpri=tpri.value, info=info.value)


def geokerr_estimate_periods(u0, mu0, a, Lz, Q2):
    lib = load()
    _geo_protos(lib)
    tr, tt, info = C.c_double(), C.c_double(), C.c_int()
    lib.npo_geokerr_estimate_periods(u0, mu0, a, Lz, Q2, C.byref(tr), C.byref(tt), C.byref(info))
    return tr.value, tt.value, info.value


def geokerr_stream(u0, uf, mu0, a, L, Q2, lam0, dlam, S):
    lib = load()
    _geo_protos(lib)
    arrs = [np.zeros(S) for _ in range(5)]
    rc = lib.npo_geokerr_stream(u0, uf, mu0, a, L, Q2, lam0, dlam, S, *[_vp(x) for x in arrs])
    return rc, dict(u=arrs[0], mu=arrs[1], t=arrs[2], phi=arrs[3], affine=arrs[4])


def geokerr_camera_grid(a, mu0, n_alpha, n_beta, a1=-12.0, a2=12.0, b1=-12.0, b2=12.0, input_limit=1e-5):
    """Constants of GEOKERR's standard rectangular camera grid
    (geokerr_original.f:255-290): cell-centred alpha, beta; l, q2, su, sm."""
    i = np.arange(n_alpha)
    j = np.arange(n_beta)
    al = a1 + (a2 - a1) * (i + 0.5) / n_alpha
    be = b1 + (b2 - b1) * (j + 0.5) / n_beta
    AL, BE = np.meshgrid(al, be, indexing="ij")
    AL, BE = AL.ravel(), BE.ravel()
    l = -AL * np.sqrt(1.0 - mu0 * mu0)
    q2 = BE * BE - (a * a - AL * AL) * mu0 * mu0
    q2 = np.where(np.abs(q2) < input_limit ** 2, 0.0, q2)
    l = np.where(np.abs(l) < input_limit, 0.0, l)
    sm = np.where((BE > 0) & (mu0 < 1.0), 1.0, -1.0)
    su = np.ones_like(l)
    return dict(alpha=AL, beta=BE, l=l, q2=q2, su=su, sm=sm)


def geokerr_crossings(u0, mu0, a, l, q2, su, sm, u_end=1e-3, K=4):
    lib = load()
    _geo_protos(lib)
    xu, xphi = np.zeros(K), np.zeros(K)
    n = lib.npo_geokerr_crossings(u0, mu0, a, l, q2, su, sm, u_end, K, _vp(xu), _vp(xphi))
    return n, xu, xphi


def geokerr_final(u0, mu0, a, l, q2, su, sm, lam):
    """(valid, [u, mu, t, phi]) at Mino time lam of the ray leaving (u0, mu0)."""
    lib = load()
    _geo_protos(lib)
    out = np.zeros(4)
    ok = lib.npo_geokerr_final(u0, mu0, a, l, q2, su, sm, lam, _vp(out))
    return ok, out


def geokerr_mino_time(u0, uf, mu0, a, l, q2, su, sm, after_tp=False):
    """(valid, lambda): Mino time from u0 to uf, directly or after the radial turning point."""
    lib = load()
    _geo_protos(lib)
    lam = C.c_double()
    ok = lib.npo_geokerr_mino_time(u0, uf, mu0, a, l, q2, su, sm, int(bool(after_tp)), C.byref(lam))
    return ok, lam.value


def critical_curve(scene):
    """The oracle's critical-curve table (256 tangent-plane radii) of `scene`."""
    rho = np.zeros(256, dtype=np.float32)
    if load().npo_critical_curve(C.byref(scene), rho.ctypes.data) != 0:
        raise RuntimeError("npo_critical_curve failed")
    return rho


# ---------------------------------------------------------------------------
# GEOKERR validation harness core (gkval_core.cpp) and the gkval binary

GKVAL_BIN = os.path.join(HERE, "gkval")


def gkval():
    """liboracle.so with the gkv_* prototypes set."""
    lib = load()
    if not getattr(lib, "_gkv_ready", False):
        D, U64, I, V, SZ = C.c_double, C.c_uint64, C.c_int, C.c_void_p, C.c_size_t
        protos = {
            "gkv_field_name": ([I], C.c_char_p),
            "gkv_field_index": ([C.c_char_p], I),
            "gkv_sha256": ([V, SZ, V], None),
            "gkv_placeholder_hash": ([V, SZ, V], None),
            "gkv_ulp_distance": ([D, D], U64),
            "gkv_accept_sample": ([D, D, D, D, U64], I),
            "gkv_first_fail": ([V, V, SZ, D, D, U64], C.c_int64),
            "gkv_unwrap": ([V, SZ], None),
            "gkv_quantize": ([D, I, C.POINTER(U64)], I),
            "gkv_hash_leaf": ([I, C.c_char_p, U64, I, U64, U64, V, SZ, V], None),
            "gkv_hash_node": ([I, V, V, V], None),
            "gkv_merkle": ([I, V, SZ, V], None),
            "gkv_save_fail_window": ([C.c_char_p, U64, I, U64, U64, V, V], I),
            "gkv_load_fail_window": ([C.c_char_p, U64, I, U64, U64, V, V], I),
            "gkv_fail_window_bounds": ([U64, U64, U64, U64, C.POINTER(U64), C.POINTER(U64)], None),
            "gkv_adaptive_grid": ([D] * 6 + [U64, D, C.POINTER(D), C.POINTER(D)], I),
            "gkv_check_fp_env": ([I], I),
        }
        for name, (args, res) in protos.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        lib._gkv_ready = True
    return lib
