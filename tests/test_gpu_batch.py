"""Batched uneven scenes (one persistent launch, CUDA graph) against the
single-scene renderer: every ray runs the same arithmetic, so each scene of
the batch matches its own render bit for bit."""
import numpy as np
import pytest

import nullpath_gb300 as npx
from nullpath_gb300 import batch

pytestmark = pytest.mark.gpu


def _small_scenes(n=10):
    # the uneven workload's draws at an eighth of the resolution
    out = []
    for sc in batch.uneven_scenes(n, seed=1):
        r = max(8, sc.width // 8)
        out.append(sc.replace(width=r, height=r))
    return out


def test_batch_matches_single_scene_renders(cuda):
    import torch
    scenes = _small_scenes()
    b = batch.Batch(scenes)
    st = b.run(graph=False, stats=True)
    assert st.rays == sum(s.width * s.height * s.spp for s in scenes)
    for i, sc in enumerate(scenes):
        rgb, rc = b.image(i)
        ref_rgb, ref_rc = npx.render(sc, "mixed")
        torch.cuda.synchronize()
        assert torch.equal(rgb, ref_rgb), i
        assert torch.equal(rc, ref_rc), i
    b.close()


def test_batch_near_critical_closed_form(cuda):
    """Critical-curve sampled scenes at a = 0.9 and 0.998 (RK4 mixed path):
    the batch solves every near-critical ray in closed form, and each scene
    matches its single-scene render bit for bit; a scene that integrates its
    near-critical rays (NP_CRITICAL_INTEGRATE) keeps them on the FP64 warps."""
    import torch
    scenes = [npx.benchmark_scene(width=96, height=64, spp=4, spin=a).replace(jitter=npx.NP_JITTER_CRITICAL)
              for a in (0.9, 0.998)]
    scenes.append(scenes[0].replace(critical_solver=npx.NP_CRITICAL_INTEGRATE, seed=3))
    b = batch.Batch(scenes)
    st = b.run(graph=False, stats=True)
    singles = [npx.render(sc, "mixed", stats=True) for sc in scenes]
    assert st.deferred_rays == sum(s[2].deferred_rays for s in singles) > 0
    assert st.closed_form_rays == singles[0][2].closed_form_rays + singles[1][2].closed_form_rays > 0
    assert singles[2][2].closed_form_rays == 0
    for i in range(len(scenes)):
        rgb, rc = b.image(i)
        torch.cuda.synchronize()
        assert torch.equal(rgb, singles[i][0]) and torch.equal(rc, singles[i][1]), i
    b.close()


def test_graph_replay_and_tuning_are_deterministic(cuda):
    """Replays of one launch setting are bit-identical.  Chunk size and
    island batch never change a ray's arithmetic; the launch shapes are
    separate compilations under different register caps, where the code
    generator may fuse a multiply-add differently, so across shapes the
    images agree to float rounding."""
    import torch
    scenes = _small_scenes(8)
    b = batch.Batch(scenes)
    b.run(graph=False)
    ref = [b.image(i) for i in range(len(scenes))]
    for shape, chunk, ib in ((0, 64, 8), (0, 16, 4), (0, 256, 16), (1, 16, 4), (2, 256, 16), (3, 32, 12)):
        batch.set_tuning(shape, chunk, ib)
        first = None
        for _ in range(2):
            st = b.run(graph=True, stats=True)
            assert (st.chunk, st.island_batch) == (chunk, ib)
            imgs = [tuple(t.clone() for t in b.image(i)) for i in range(len(scenes))]
            if first is None:
                first = imgs
            for i in range(len(scenes)):
                rgb, rc = imgs[i]
                assert torch.equal(rgb, first[i][0]) and torch.equal(rc, first[i][1]), (shape, i)
                if shape == 0:
                    assert torch.equal(rgb, ref[i][0]) and torch.equal(rc, ref[i][1]), (shape, chunk, i)
                else:
                    bad = (rgb - ref[i][0]).abs() > 1e-3 * (1.0 + ref[i][0].abs())
                    assert bad.any(dim=0).float().mean().item() < 1e-3, (shape, i)
    batch.set_tuning()
    lat = b.latency_ms()
    assert (lat > 0).all() and lat.max() <= st.total_ms + 1e-3
    assert st.scene_ms_p50 <= st.scene_ms_p99 <= st.scene_ms_max
    b.close()


def test_autotuner_installs_a_valid_setting(cuda):
    b = batch.Batch(_small_scenes(6))
    t = batch.autotune(b)
    assert t["trials"] >= 10 and t["best_ms"] > 0
    assert t["block"] in (64, 128, 256) and t["chunk"] in (16, 32, 64, 128, 256)
    st = b.run(graph=True, stats=True)
    assert (st.block, st.chunk, st.island_batch) == (t["block"], t["chunk"], t["island_batch"])
    batch.set_tuning()
    b.close()


def test_batch_rejects_bad_scene(cuda):
    scenes = _small_scenes(3)
    scenes[1] = scenes[1].replace(spin=1.2)
    with pytest.raises(npx.NullPathError):
        batch.Batch(scenes)
    # the embedded 7(8) tracer is not batched: refused, not silently run as RK4
    scenes = _small_scenes(3)
    scenes[2] = npx.accurate_scene(scenes[2])
    with pytest.raises(npx.NullPathError):
        batch.Batch(scenes)
