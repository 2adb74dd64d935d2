"""GB300-native Kerr null-geodesic tracer (sm_103a CUDA behind a C ABI).

Public Python surface (a thin layer over include/np_render.h):
    Scene, reference_defaults(), benchmark_scene()   scene description
    accurate_scene(scene)                            the same scene on the mixed 7(8) path (FP32 under
                                                     error control, Henon crossings)
    research_scene(scene)                            the same scene in research mode (FP64 7(8))
    render(scene, precision)                         device render (torch tensors)
    render_host(scene, precision)                    host buffers in, host buffers out
    trace_rays(scene, px, py, precision)             per-ray crossing report
    trace_invariants(scene, px, py)                  per-ray drift of H and Carter's Q (FP64)
"""
from ._abi import (Scene, RenderStats, isco_radius, reference_defaults, benchmark_scene, research_scene,
                   accurate_scene, NP_PREC_FP64, NP_PREC_MIXED, NP_UNITS_RS, NP_UNITS_M,
                   NP_JITTER_WANGHASH, NP_JITTER_STRATIFIED, NP_JITTER_CRITICAL, NP_CAMERA_STATIC, NP_CAMERA_ZAMO,
                   NP_INTEG_RK4, NP_INTEG_ADAPTIVE, NP_INTEG_RKF78, NP_CROSS_LINEAR, NP_CROSS_HERMITE,
                   NP_CROSS_ROOT,
                   NP_BG_GRADIENT, NP_BG_POINT, NP_ISLAND_HORIZON, NP_ISLAND_TURNING,
                   NP_ISLAND_CRITICAL, NP_ISLANDS_ALL, NP_ISLANDS_DEFAULT, NP_ISLAND_ARITH_DF,
                   NP_ISLAND_ARITH_FP64, NP_CRITICAL_CLOSED_FORM, NP_CRITICAL_INTEGRATE)
from ._lib import load, lib_path, NullPathError
from .render import render, render_host, trace_rays, trace_invariants, precision_code

__all__ = [
    "Scene", "RenderStats", "isco_radius", "reference_defaults", "benchmark_scene", "research_scene",
    "accurate_scene", "render", "render_host", "trace_rays", "trace_invariants", "precision_code", "load", "lib_path", "NullPathError",
    "NP_PREC_FP64", "NP_PREC_MIXED",
]
