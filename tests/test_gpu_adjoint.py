"""Adjoint of the differentiable render against central finite differences
(FP64, h = 1e-4, event structure held fixed) on the target/current pair of the
differentiable-render configuration: target (a=0.7, theta=60 deg, gain=1,
q=3), current (0.5, 50 deg, 0.8, 2.5), L2 loss, seed 2 (smaller image)."""
import math

import numpy as np
import pytest

import nullpath_gb300 as npx
from nullpath_gb300 import diff

pytestmark = pytest.mark.gpu


def _scene(w=48, h=48, spp=2):
    return npx.benchmark_scene(width=w, height=h, spp=spp, spin=0.5, seed=2)


def _setup(prec, w=48, h=48, spp=2):
    import torch
    sc = _scene(w, h, spp)
    target = diff.Adjoint().forward(diff.scene_with(sc, 0.7, math.radians(60.0), 1.0, 3.0), "fp64", 16)
    params = torch.tensor([0.5, math.radians(50.0), 0.8, 2.5], dtype=torch.float64, requires_grad=True)
    return sc, target, params


def test_per_sample_adjoint_matches_complex_step(cuda):
    """FP64 per-sample gradients against the complex-step derivative of the
    same discrete map (oracle/adjoint_cs.py) on 24 random disk samples.  The
    oracle skips samples whose own complex step and central difference at
    1e-7 disagree (maps that change faster than rounding can follow)."""
    import torch
    from oracle import adjoint_cs as cs
    sc = diff.scene_with(_scene(64, 64, 2), 0.5, math.radians(50.0), 0.8, 2.5)
    d = cs.scene_dict(sc)
    adj = diff.Adjoint()
    _, _, sig = adj.forward(sc, "fp64", 16, samples=True)
    ps = torch.zeros((2, 64, 64, 4), dtype=torch.float64, device="cuda")
    adj.backward(torch.ones((3, 64, 64), dtype=torch.float32, device="cuda"), per_sample=ps)
    adj.close()
    sig = sig.flatten().cpu().numpy()
    ps = ps.reshape(-1, 4).cpu().numpy()
    hits = np.flatnonzero(((sig & 3) != 1) & (sig >= 4))
    rng = np.random.default_rng(7)
    checked = 0
    for idx in rng.permutation(hits)[:40]:
        ref_sig, g = cs.sample_gradient(d, int(idx))
        assert ref_sig == sig[idx]
        y, x = divmod(int(idx) % 4096, 64)
        sl = int(idx) // 4096
        h = 1e-7
        th0 = math.radians(50.0)
        fp = cs.trace(d, 0.5, th0 + h, 2.5, x, y, sl)[3]
        fm = cs.trace(d, 0.5, th0 - h, 2.5, x, y, sl)[3]
        fd_t = (fp - fm) / (2 * h) * 0.8 * 2.2 / 2
        if abs(fd_t - g[1]) > 1e-4 * abs(g[1]) + 1e-12:
            continue
        assert np.allclose(ps[idx], g, rtol=1e-6, atol=1e-12), (int(idx), ps[idx], g)
        checked += 1
        if checked == 24:
            break
    assert checked >= 20


def test_gradient_check_at_scale(cuda):
    """128x128x4: the full gradient (every sample, no mask) of the FP64 and
    FP32 adjoints against the central FP64 FD at h = 1e-4, within 1e-3
    relative in every component; the polar-axis factor of the step law keeps
    the pole-passing rays (L ~ 0) resolved, so nothing needs masking."""
    sc, target, params = _setup("fp64", 128, 128, 4)
    p = params.detach().numpy()
    fd = diff.fd_gradient(sc, p, target, precision="fp64", per_sample=True)
    r64 = diff.gradient_check(sc, p, target, precision="fp64", K=64, fd=fd)
    assert max(r64["rel_err_all"]) < 1e-3, r64
    assert max(r64["excluded_sample_frac"]) < 0.01, r64
    r32 = diff.gradient_check(sc, p, target, precision="mixed", K=64, fd=fd)
    assert max(r32["rel_err_all"]) < 1e-3, r32


def test_autotune_checkpoint_interval(cuda):
    """The K autotuner picks a measured-fastest K within the memory cap, and
    the reverse sweep's segment buffers do not grow with the rays."""
    sc = diff.scene_with(_scene(96, 96, 2), 0.5, math.radians(50.0), 0.8, 2.5)
    r = diff.autotune_K(sc, "mixed", Ks=(16, 64, 256), reps=1)
    assert r["K"] in (16, 64, 256)
    per = r["per_K"]
    assert per[str(r["K"])]["ms"] == min(v["ms"] for v in per.values() if v["fits"])
    capped = diff.autotune_K(sc, "mixed", Ks=(16, 64, 256), reps=1,
                             mem_cap=min(v["workspace_bytes"] for v in per.values()))
    assert per[str(capped["K"])]["workspace_bytes"] == min(v["workspace_bytes"] for v in per.values())


@pytest.mark.parametrize("K", [16, 64, 256])
def test_fp64_adjoint_matches_fd(cuda, K):
    import torch
    sc, target, params = _setup("fp64")
    img = diff.render_diff(params, sc, "fp64", K)
    loss = ((img.double() - target.double()) ** 2).sum()
    loss.backward()
    g = params.grad.numpy()
    fd = diff.fd_gradient(sc, params.detach().numpy(), target, h=1e-4, precision="fp64")
    rel = np.abs(g - fd) / np.maximum(np.abs(fd), 1e-12)
    # 1e-3 relative per component (the differentiable-render acceptance bar)
    assert (rel < 1e-3).all(), (K, g, fd, rel)


def test_checkpoint_interval_does_not_change_gradient(cuda):
    import torch
    sc, target, _ = _setup("fp64")
    grads = []
    for K in (16, 64, 256):
        params = torch.tensor([0.5, math.radians(50.0), 0.8, 2.5], dtype=torch.float64, requires_grad=True)
        loss = ((diff.render_diff(params, sc, "fp64", K).double() - target.double()) ** 2).sum()
        loss.backward()
        grads.append(params.grad.numpy())
    # the segment recomputation is a separate call site whose multiply-add
    # contraction may round differently from the forward loop: 1e-9 relative
    assert np.allclose(grads[0], grads[1], rtol=1e-9, atol=0) and np.allclose(grads[0], grads[2], rtol=1e-9, atol=0)


def test_fp32_adjoint_close_to_fd(cuda):
    import torch
    sc, target, params = _setup("mixed")
    loss = ((diff.render_diff(params, sc, "mixed", 16).double() - target.double()) ** 2).sum()
    loss.backward()
    g = params.grad.numpy()
    fd = diff.fd_gradient(sc, params.detach().numpy(), target, h=1e-4, precision="fp64")
    rel = np.abs(g - fd) / np.maximum(np.abs(fd), 1e-12)
    assert (rel < 2e-2).all(), (g, fd, rel)
