"""Python entry points over the C ABI (include/np_render.h).

PyTorch supplies device memory and streams; every computation runs in the
CUDA library.  There is no CPU path here: without the library or a GPU the
calls raise.
"""
import ctypes as C

import numpy as np

from ._abi import Scene, RenderStats, NP_PREC_FP64, NP_PREC_MIXED
from ._lib import load, check

_PREC = {"fp64": NP_PREC_FP64, "mixed": NP_PREC_MIXED, NP_PREC_FP64: NP_PREC_FP64, NP_PREC_MIXED: NP_PREC_MIXED}


def precision_code(precision):
    try:
        return _PREC[precision]
    except KeyError:
        raise ValueError("precision must be 'fp64' or 'mixed', got %r" % (precision,))


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def render(scene, precision="mixed", rgb=None, rcross=None, inv3=None, accumulate=False,
           stream=None, stats=False):
    """Renders one pass of `scene` on the current CUDA device.

    Returns (rgb[3, H, W], rcross[H, W]) float32 CUDA tensors (and a
    RenderStats when stats=True, which synchronises the stream).
    """
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("render() needs a CUDA device")
    lib = load()
    H, W = scene.height, scene.width
    dev = torch.device("cuda", torch.cuda.current_device())
    if rgb is None:
        rgb = torch.zeros((3, H, W), dtype=torch.float32, device=dev)
    if rcross is None:
        rcross = torch.zeros((H, W), dtype=torch.float32, device=dev)
    if stream is None:
        stream = torch.cuda.current_stream()
    st = RenderStats() if stats else None
    check(lib.np_render_device(C.byref(scene), precision_code(precision), _ptr(rgb), _ptr(rcross),
                               _ptr(inv3), 1 if accumulate else 0, C.c_void_p(stream.cuda_stream),
                               C.byref(st) if st is not None else None))
    if stats:
        return rgb, rcross, st
    return rgb, rcross


def render_host(scene, precision="mixed", with_inv=False):
    """Renders with host (numpy) buffers; copies happen inside the library call."""
    lib = load()
    H, W = scene.height, scene.width
    rgb = np.zeros((3, H, W), np.float32)
    rc = np.zeros((H, W), np.float32)
    inv = np.zeros(3, np.float32) if with_inv else None
    st = RenderStats()
    check(lib.np_render_host(C.byref(scene), precision_code(precision),
                             rgb.ctypes.data_as(C.c_void_p), rc.ctypes.data_as(C.c_void_p),
                             inv.ctypes.data_as(C.c_void_p) if inv is not None else None, C.byref(st)))
    return (rgb, rc, inv, st) if with_inv else (rgb, rc, st)


def trace_rays(scene, px, py, precision="mixed"):
    """Traces rays through continuous image positions (px, py); returns a dict
    of CUDA tensors: consts[n,4] (p_t, p_phi, p_r, p_theta), cross[n,4,2]
    (r, phi of the first four equatorial crossings), status[n]."""
    import torch
    lib = load()
    px = torch.as_tensor(px, dtype=torch.float64, device="cuda").contiguous()
    py = torch.as_tensor(py, dtype=torch.float64, device="cuda").contiguous()
    n = px.numel()
    consts = torch.zeros((n, 4), dtype=torch.float64, device="cuda")
    cross = torch.zeros((n, 4, 2), dtype=torch.float64, device="cuda")
    status = torch.zeros((n,), dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    check(lib.np_trace_rays_device(C.byref(scene), precision_code(precision), n, _ptr(px), _ptr(py),
                                   _ptr(consts), _ptr(cross), _ptr(status), C.c_void_p(stream.cuda_stream)))
    return {"consts": consts, "cross": cross, "status": status}


def trace_invariants(scene, px, py):
    """FP64 rays through image positions (px, py): returns (drift[n, 2], steps[n])
    as CUDA tensors, drift = (max |H| / E^2, max |Q - Q0| / max(|Q0|, (E M)^2))
    over each ray's accepted steps (Q is Carter's constant)."""
    import torch
    lib = load()
    px = torch.as_tensor(px, dtype=torch.float64, device="cuda").contiguous()
    py = torch.as_tensor(py, dtype=torch.float64, device="cuda").contiguous()
    n = px.numel()
    drift = torch.zeros((n, 2), dtype=torch.float64, device="cuda")
    steps = torch.zeros((n,), dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    check(lib.np_trace_invariants_device(C.byref(scene), n, _ptr(px), _ptr(py), _ptr(drift), _ptr(steps),
                                         C.c_void_p(stream.cuda_stream)))
    return drift, steps
