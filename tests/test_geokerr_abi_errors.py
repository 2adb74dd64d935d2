"""Error paths of the GEOKERR C ABI (include/geokerr_c_api.h) that are
decided on the host before any device work: bad sizes, spins with |a| >= 1,
NULL buffers.  They return the reference's codes (geokerr_stream.cu:163-180:
-1 bad argument; geokerr_eval_lambda.f90:96-100: info = 1 for S <= 0) or
NP_ERR_INVALID, and never abort."""
import ctypes as C

import numpy as np

from nullpath_gb300 import geokerr as gk
from nullpath_gb300._abi import NP_ERR_INVALID


def test_f90_entry_rejects_empty_grid(built):
    lib = gk._lib()
    buf = [np.zeros(1) for _ in range(5)]
    tpmi, tpri, info = C.c_int(7), C.c_int(7), C.c_int(-9)
    lib.geokerr_eval_lambda(0.1, 0.8, 0.01, 0.5, 2.0, 4.0, 0.0, 0.0, 0.01, 0, *[gk._vp(b) for b in buf],
                            C.byref(tpmi), C.byref(tpri), C.byref(info))
    assert info.value == 1


def test_stream_wrappers_return_minus_one(built):
    lib = gk._lib()
    buf = [np.zeros(4) for _ in range(5)]
    ptrs = [gk._vp(b) for b in buf]
    for fn in (lib.geokerr_stream_cuda, lib.geokerr_complete_stream_cuda):
        assert fn(0.1, 0.01, 0.8, 0.5, 2.0, 4.0, 0.0, 0.01, 0, *ptrs) == -1        # S <= 0
        assert fn(0.1, 0.01, 0.8, 1.0, 2.0, 4.0, 0.0, 0.01, 4, *ptrs) == -1        # |a| >= 1
        assert fn(0.1, 0.01, 0.8, 0.5, 2.0, 4.0, 0.0, 0.01, 4, None, *ptrs[1:]) == -1   # NULL output


def test_batched_entries_reject_bad_sizes_and_spins(built):
    lib = gk._lib()
    nul = [None] * 8
    assert lib.np_geokerr_points_device(-1, 0.5, *[None] * 7, 1, 8, 0.5, *nul, None) == NP_ERR_INVALID
    assert lib.np_geokerr_points_device(4, 0.5, *[None] * 7, 1, 0, 0.5, *nul, None) == NP_ERR_INVALID
    assert lib.np_geokerr_points_device(4, 1.0, *[None] * 7, 1, 8, 0.5, *nul, None) == NP_ERR_INVALID
    assert lib.np_geokerr_points_device(0, 0.5, *[None] * 7, 1, 8, 0.5, *nul, None) == 0
    assert lib.np_geokerr_eval_lambda_device(-1, 0.5, *[None] * 8, 16, *[None] * 8, None, None) == NP_ERR_INVALID
    assert lib.np_geokerr_eval_lambda_device(4, 0.5, *[None] * 8, 0, *[None] * 8, None, None) == NP_ERR_INVALID
    assert lib.np_geokerr_eval_lambda_device(4, -1.0, *[None] * 8, 16, *[None] * 8, None, None) == NP_ERR_INVALID
    assert lib.np_geokerr_final_state_host(-1, *[None] * 13) == NP_ERR_INVALID
    assert lib.np_geokerr_final_state_host(2, *[None] * 13) == NP_ERR_INVALID
    assert gk.load().np_last_error() == b"bad arguments"
    assert lib.np_geokerr_final_state_host(0, *[None] * 13) == 0


def test_void_wrappers_ignore_null_and_empty(built):
    lib = gk._lib()
    # no output, no crash, no device work
    lib.compute_mino_time_batch_cuda(*[None] * 14, 0)
    lib.compute_mino_time_batch_cuda(*[None] * 14, 3)
    lib.geokerr_cuda_batch(*[None] * 10, 0, 10, 1.0)
    lib.geokerr_improved_batch(*[None] * 10, 3, 10, 1.0)
    lib.geokerr_single_case_(*[None] * 13)
