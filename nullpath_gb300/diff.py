"""Differentiable Kerr render over the adjoint C ABI (include/np_render.h).

    img = render_diff(params, scene)   # params = tensor [spin, theta_rad, gain, q]
    loss = ((img - target) ** 2).sum(); loss.backward()

The backward pass is the hand-written reverse sweep of adjoint.cu with
checkpoints every K steps.  `fd_gradient` is the checker: central finite
differences of the same loss with each sample's event structure held fixed
(samples whose disk hits or capture change between the +-h renders fall back
to one-sided differences), which is what the adjoint differentiates.
"""
import ctypes as C
import math

import numpy as np

from ._abi import Scene, NP_PREC_FP64, NP_PREC_MIXED
from ._lib import load, check


class AdjointStats(C.Structure):
    _fields_ = [("forward_ms", C.c_double), ("backward_ms", C.c_double),
                ("workspace_bytes", C.c_uint64), ("checkpoint_bytes_per_ray", C.c_uint64)]


_PROTOS = {
    "np_adjoint_create": (C.c_void_p, []),
    "np_adjoint_destroy": (None, [C.c_void_p]),
    "np_adjoint_forward": (C.c_int, [C.c_void_p, C.POINTER(Scene), C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.POINTER(AdjointStats)]),
    "np_adjoint_backward": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_double), C.c_void_p, C.c_void_p,
                                      C.POINTER(AdjointStats)]),
}


def _lib():
    lib = load()
    if not getattr(lib, "_adj_ready", False):
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib._adj_ready = True
    return lib


def scene_with(scene, spin, theta_rad, gain, q):
    return scene.replace(spin=float(spin), theta_deg=float(theta_rad) * 180.0 / math.pi,
                         disk_gain=float(gain), emissivity_q=float(q))


class Adjoint:
    """Owns a device workspace (checkpoints) between a forward and its backward."""

    def __init__(self):
        self.lib = _lib()
        self.h = self.lib.np_adjoint_create()

    def close(self):
        if self.h:
            self.lib.np_adjoint_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, scene, precision="mixed", K=16, samples=False, stats=None):
        import torch
        prec = NP_PREC_MIXED if precision == "mixed" else NP_PREC_FP64
        H, W, S = scene.height, scene.width, scene.spp
        img = torch.zeros((3, H, W), dtype=torch.float32, device="cuda")
        srgb = torch.zeros((S, 3, H, W), dtype=torch.float32, device="cuda") if samples else None
        sig = torch.zeros((S, H, W), dtype=torch.int32, device="cuda") if samples else None
        st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        check(self.lib.np_adjoint_forward(self.h, C.byref(scene), prec, K, C.c_void_p(img.data_ptr()),
                                          C.c_void_p(srgb.data_ptr()) if samples else None,
                                          C.c_void_p(sig.data_ptr()) if samples else None, st,
                                          C.byref(stats) if stats is not None else None))
        return (img, srgb, sig) if samples else img

    def backward(self, grad_img, stats=None, per_sample=None):
        """Returns dLoss/d[spin, theta_rad, gain, q]; per_sample, when given, is a
        CUDA float64 tensor [spp, H, W, 4] that receives each sample's share."""
        import torch
        g = grad_img.detach().to(device="cuda", dtype=torch.float32).contiguous()
        out = (C.c_double * 4)()
        check(self.lib.np_adjoint_backward(self.h, C.c_void_p(g.data_ptr()), out,
                                           C.c_void_p(per_sample.data_ptr()) if per_sample is not None else None,
                                           C.c_void_p(torch.cuda.current_stream().cuda_stream),
                                           C.byref(stats) if stats is not None else None))
        return np.array(out[:], dtype=np.float64)


def _make_fn():
    import torch

    class KerrRenderFn(torch.autograd.Function):
        """params = [spin, theta_rad, gain, q] -> mean image [3, H, W]."""

        @staticmethod
        def forward(ctx, params, scene, precision, K):
            p = params.detach().cpu().double().numpy()
            adj = Adjoint()
            img = adj.forward(scene_with(scene, *p), precision, K)
            ctx.adj = adj
            ctx.dtype, ctx.device = params.dtype, params.device
            return img

        @staticmethod
        def backward(ctx, grad_img):
            g = ctx.adj.backward(grad_img)
            ctx.adj.close()
            return torch.as_tensor(g, dtype=ctx.dtype, device=ctx.device), None, None, None

    return KerrRenderFn


_FN = None


def render_diff(params, scene, precision="mixed", K=16):
    """Differentiable render; params is a 4-element tensor [spin, theta_rad, gain, q]."""
    global _FN
    if _FN is None:
        _FN = _make_fn()
    return _FN.apply(params, scene, precision, K)


def fd_gradient(scene, params, target, h=1e-4, precision="fp64", per_sample=False):
    """Central-difference gradient of sum((img - target)^2) with respect to
    [spin, theta_rad, gain, q], every sample's event structure held fixed.

    With per_sample=True also returns the per-sample contributions
    [spp, H, W, 4] and a mask of the samples whose difference quotient is
    resolved: the central differences at h and h/16 agree to 1 % beyond the
    rounding of the FP32 sample colours.  The differentiable render's step law
    shrinks near the polar axis, so that rays with L close to 0, which turn
    within a few times their closest approach to the pole, are resolved and
    the discrete map stays smooth at the scale h; the resolved mask then
    leaves out only samples near rounding or interpolant switches."""
    import torch
    adj = Adjoint()
    p0 = np.asarray(params, dtype=np.float64)
    img0, c0, s0 = adj.forward(scene_with(scene, *p0), precision, 16, samples=True)
    img0 = img0.double()
    c0d = c0.double()
    resid = 2.0 * (img0 - target.double())          # dL/dimg at p0
    S = scene.spp
    ulp = 2.0 ** -24

    def per_sample_fd(i, step):
        pp, pm = p0.copy(), p0.copy()
        pp[i] += step
        pm[i] -= step
        _, cp, sp = adj.forward(scene_with(scene, *pp), precision, 16, samples=True)
        _, cm, sm = adj.forward(scene_with(scene, *pm), precision, 16, samples=True)
        cp, cm = cp.double(), cm.double()
        same_p = (sp == s0).unsqueeze(1)
        same_m = (sm == s0).unsqueeze(1)
        zero = torch.zeros_like(cp)
        d = torch.where(same_p & same_m, (cp - cm) / (2 * step),
                        torch.where(same_p, (cp - c0d) / step, torch.where(same_m, (c0d - cm) / step, zero)))
        # rounding of the FP32 colours, propagated through the quotient
        nz = torch.where(same_p & same_m, ulp * (cp.abs() + cm.abs()) / (2 * step),
                         torch.where(same_p, ulp * (cp.abs() + c0d.abs()) / step,
                                     torch.where(same_m, ulp * (c0d.abs() + cm.abs()) / step, zero)))
        w = resid.unsqueeze(0) / S
        return (w * d).sum(dim=1), (w.abs() * nz).sum(dim=1), ((sp == s0) & (sm == s0))

    grad = np.zeros(4)
    ps, ok = [], []
    for i in range(4):
        contrib, noise, same = per_sample_fd(i, h)
        grad[i] = float(contrib.sum())
        if per_sample:
            fine, noise_f, same_f = per_sample_fd(i, h / 16.0)
            tol = 1e-2 * torch.maximum(contrib.abs(), fine.abs()) + 2.0 * (noise + noise_f)
            ps.append(contrib)
            ok.append(same & same_f & ((contrib - fine).abs() <= tol))
    adj.close()
    if per_sample:
        return grad, torch.stack(ps, dim=-1), torch.stack(ok, dim=-1), s0
    return grad


def gradient_check(scene, params, target, precision="mixed", K=16, h=1e-4, fd=None):
    """Adjoint against the event-masked FD: over every sample (rel_err_all)
    and over the FD-resolved samples (rel_err_resolved).
    `fd` may carry a previous fd_gradient(..., per_sample=True) result for the
    same scene, params and target.  Returns a dict with both gradients, the
    relative error per component and the share of samples (and of |gradient|)
    left out as unresolved."""
    import torch
    if fd is None:
        fd = fd_gradient(scene, params, target, h=h, precision="fp64", per_sample=True)
    fd, fd_ps, resolved, sig = fd
    adj = Adjoint()
    img = adj.forward(scene_with(scene, *params), precision, K)
    ps = torch.zeros((scene.spp, scene.height, scene.width, 4), dtype=torch.float64, device="cuda")
    g_all = adj.backward(2.0 * (img.double() - target.double()), per_sample=ps)
    adj.close()
    g_res = (ps * resolved).sum(dim=(0, 1, 2)).cpu().numpy()
    f_res = (fd_ps * resolved).sum(dim=(0, 1, 2)).cpu().numpy()
    rel = np.abs(g_res - f_res) / np.maximum(np.abs(f_res), 1e-12)
    rel_all = np.abs(np.asarray(g_all) - np.asarray(fd)) / np.maximum(np.abs(np.asarray(fd)), 1e-12)
    excl = (~resolved).float().mean(dim=(0, 1, 2)).cpu().numpy()
    excl_share = ((ps.abs() * (~resolved)).sum(dim=(0, 1, 2)) / ps.abs().sum(dim=(0, 1, 2)).clamp_min(1e-300))
    return {"adjoint": g_all.tolist(), "fd": fd.tolist(), "adjoint_resolved": g_res.tolist(),
            "fd_resolved": f_res.tolist(), "rel_err_resolved": rel.tolist(), "rel_err_all": rel_all.tolist(),
            "excluded_sample_frac": excl.tolist(), "excluded_abs_grad_share": excl_share.cpu().numpy().tolist()}


def autotune_K(scene, precision="mixed", Ks=(16, 32, 64, 128, 256), mem_cap=None, reps=2):
    """Chooses the adjoint's checkpoint interval K by measured time under a
    memory cap.  For each K of `Ks` it runs forward + backward `reps` times on
    `scene` (with a unit image gradient) and records the best CUDA-event time
    and the workspace; the fastest K whose workspace fits `mem_cap` bytes
    (default: half of the device's free memory) wins.  Small K stores more
    checkpoints; large K recomputes longer segments and holds a longer
    segment buffer per reverse-sweep thread.  Returns a dict with the chosen
    K and the per-K measurements."""
    import torch
    if mem_cap is None:
        mem_cap = torch.cuda.mem_get_info()[0] // 2
    rows = {}
    ones = torch.ones((3, scene.height, scene.width), dtype=torch.float32, device="cuda")
    for K in Ks:
        best = None
        ws = 0
        for _ in range(reps):
            adj = Adjoint()
            st = AdjointStats()
            try:
                adj.forward(scene, precision, K, stats=st)
                adj.backward(ones, stats=st)
            finally:
                adj.close()
            t = st.forward_ms + st.backward_ms
            ws = int(st.workspace_bytes)
            best = t if best is None else min(best, t)
        rows[K] = {"ms": best, "workspace_bytes": ws, "fits": ws <= mem_cap}
    ok = [K for K in Ks if rows[K]["fits"]]
    if not ok:
        raise RuntimeError("no checkpoint interval fits %d bytes" % mem_cap)
    K = min(ok, key=lambda k: rows[k]["ms"])
    return {"K": K, "mem_cap_bytes": int(mem_cap), "per_K": {str(k): v for k, v in rows.items()}}
