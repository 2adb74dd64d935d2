"""Loader of the CUDA library and ctypes prototypes of its C ABI.

The library is loaded from nullpath_gb300/lib in this tree; there is no
fallback: a missing or unloadable library raises.
"""
import ctypes as C
import os

from ._abi import Scene, RenderStats

_LIB = None


def lib_path():
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libnullpath_gb300.so")


# exported symbol -> (restype, argtypes); the list mirrors include/*.h
PROTOTYPES = {
    "np_abi_version": (C.c_int, []),
    "np_last_error": (C.c_char_p, []),
    "np_scene_defaults": (None, [C.POINTER(Scene)]),
    "np_scene_benchmark": (None, [C.POINTER(Scene)]),
    "np_isco_radius": (C.c_double, [C.c_double, C.c_double]),
    "np_critical_curve": (C.c_int, [C.POINTER(Scene), C.c_void_p]),
    "np_scene_validate": (C.c_int, [C.POINTER(Scene)]),
    "np_render_device": (C.c_int, [C.POINTER(Scene), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_int, C.c_void_p, C.POINTER(RenderStats)]),
    "np_render_host": (C.c_int, [C.POINTER(Scene), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.POINTER(RenderStats)]),
    "np_trace_rays_device": (C.c_int, [C.POINTER(Scene), C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "np_trace_invariants_device": (C.c_int, [C.POINTER(Scene), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.c_void_p]),
    "np_measure_fma_peak": (C.c_int, [C.c_int, C.POINTER(C.c_double)]),
    "np_tune": (C.c_int, [C.c_int, C.c_int]),
    "np_render_device_noalloc": (C.c_int, [C.POINTER(Scene), C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                           C.c_void_p]),
}


def load(path=None):
    """Loads (once) and returns the ctypes handle of libnullpath_gb300.so."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or lib_path()
    if not os.path.exists(p):
        raise RuntimeError("libnullpath_gb300.so not built (%s); run __graft_entry__.build()" % p)
    lib = C.CDLL(p)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


class NullPathError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("nullpath error %d: %s" % (code, msg))
        self.code = code


def check(rc):
    if rc != 0:
        msg = load().np_last_error()
        raise NullPathError(rc, msg.decode() if msg else "")
    return rc
