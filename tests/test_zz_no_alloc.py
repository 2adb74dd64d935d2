"""The allocation-free render entry point.

Some callers cannot allocate device memory: hosts that own the whole GPU
through their own allocator, or that forbid allocation inside their frame
loop.  np_render_device_noalloc serves them from a fixed scratch array
compiled into the library.  This test calls it through the C ABI twice in a
row and checks each result against the allocating entry point
np_render_device on the same scene, with the tolerance the other parity
tests use; it also checks that a pass above NP_NOALLOC_MAX_RAYS is refused
and that a call takes no device memory.  The file name sorts last so that a
run stopping at the first failure has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

import nullpath_gb300 as npx
from nullpath_gb300._abi import NP_ERR_INVALID, NP_PREC_FP64, NP_PREC_MIXED

pytestmark = pytest.mark.gpu

NOALLOC_MAX_RAYS = 262144   # NP_NOALLOC_MAX_RAYS in include/np_render.h


def _noalloc(lib, sc, prec, rgb, rc, accumulate=0):
    import torch
    return lib.np_render_device_noalloc(C.byref(sc), prec, C.c_void_p(rgb.data_ptr()),
                                        C.c_void_p(rc.data_ptr()) if rc is not None else None,
                                        accumulate, C.c_void_p(torch.cuda.current_stream().cuda_stream))


@pytest.mark.parametrize("prec", [NP_PREC_MIXED, NP_PREC_FP64])
def test_noalloc_matches_allocating_entry_point(cuda, prec):
    import torch
    lib = npx.load()
    sc = npx.benchmark_scene(width=96, height=54, spp=4)
    ref_rgb, ref_rc = npx.render(sc, prec)
    torch.cuda.synchronize()
    for call in range(2):       # two calls in a row share the scratch array
        rgb = torch.full((3, sc.height, sc.width), -1.0, device="cuda")
        rc = torch.full((sc.height, sc.width), -1.0, device="cuda")
        assert _noalloc(lib, sc, prec, rgb, rc) == 0, lib.np_last_error()
        torch.cuda.synchronize()
        # same tolerance as the other parity tests (rtol 1e-6, atol 1e-7)
        assert torch.allclose(rgb, ref_rgb, rtol=1e-6, atol=1e-7), call
        assert torch.allclose(rc, ref_rc, rtol=1e-6, atol=1e-7), call


def test_noalloc_rejects_oversize_and_takes_no_memory(cuda):
    """A pass above the maximum is refused; a pass of exactly the maximum
    (256 x 256 x 4 rays) matches the allocating entry point and takes no
    device memory (free memory measured before the first call at that size,
    with the library already loaded, within 2 MiB for other users of the
    device)."""
    import torch
    lib = npx.load()
    big = npx.benchmark_scene(width=512, height=512, spp=2)     # 524,288 rays
    assert big.width * big.height * big.spp > NOALLOC_MAX_RAYS
    rgb = torch.zeros((3, 512, 512), device="cuda")
    rc = torch.zeros((512, 512), device="cuda")
    assert _noalloc(lib, big, NP_PREC_MIXED, rgb, rc) == NP_ERR_INVALID
    assert b"NP_NOALLOC_MAX_RAYS" in lib.np_last_error()
    sc = npx.benchmark_scene(width=256, height=256, spp=4)        # exactly the maximum
    assert sc.width * sc.height * sc.spp == NOALLOC_MAX_RAYS
    ref_rgb, ref_rc = npx.render(sc, NP_PREC_MIXED)
    out = torch.zeros((3, 256, 256), device="cuda")
    out_rc = torch.zeros((256, 256), device="cuda")
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        assert _noalloc(lib, sc, NP_PREC_MIXED, out, out_rc) == 0
        torch.cuda.synchronize()
    # read before any torch work: the comparisons below allocate temporaries,
    # which torch's caching allocator may take as new 2 MiB segments
    free1 = torch.cuda.mem_get_info()[0]
    assert torch.allclose(out, ref_rgb, rtol=1e-6, atol=1e-7)
    assert torch.allclose(out_rc, ref_rc, rtol=1e-6, atol=1e-7)
    assert abs(free1 - free0) <= 2 << 20


def test_noalloc_split_pass_matches_one_pass(cuda):
    """A pass split over two calls (samples 0-1, then 2-3 with sample_offset
    2 and accumulate = 1, rcross on the first call only) equals one
    four-sample np_render_device pass.  The wanghash jitter places a sample
    by its index alone (stratified jitter lays its strata out by the call's
    spp, so a split changes its pattern)."""
    import torch
    from nullpath_gb300._abi import NP_JITTER_WANGHASH
    lib = npx.load()
    sc = npx.benchmark_scene(width=64, height=36, spp=4).replace(jitter=NP_JITTER_WANGHASH)
    ref_rgb, ref_rc = npx.render(sc, NP_PREC_MIXED)
    rgb = torch.zeros((3, 36, 64), device="cuda")
    rc = torch.zeros((36, 64), device="cuda")
    assert _noalloc(lib, sc.replace(spp=2), NP_PREC_MIXED, rgb, rc) == 0
    assert _noalloc(lib, sc.replace(spp=2, sample_offset=2), NP_PREC_MIXED, rgb, None, accumulate=1) == 0
    torch.cuda.synchronize()
    assert torch.allclose(rgb, ref_rgb, rtol=1e-6, atol=1e-7)
    assert torch.equal(rc, ref_rc)
