"""Generates the golden fixtures in this folder.

Reference-mode cases (ref_*.npz) are rendered by oracle/_ref/libnpref.so,
i.e. by the reference's own physics headers (include/bh_kerr.h,
include/bh_common.h of danielchristiancazares/NullPath) compiled on this
host, with render.cu's per-pixel loop restated around them.  Benchmark-scene
cases (bench_*.npz) exercise extensions the reference does not have
(lengths in M, stratified jitter, r^-q disk, Hermite crossings); they are
rendered by the oracle restatement itself and serve as regression fixtures.

Run from the repository root after `make -C oracle`:
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from nullpath_gb300._abi import (reference_defaults, benchmark_scene, NP_INTEG_ADAPTIVE,  # noqa: E402
                                 NP_BG_POINT, NP_CAMERA_ZAMO)


def ref_cases():
    base = reference_defaults()
    return {
        "ref_a09_th80": base.replace(width=64, height=36, spp=2, spin=0.9, theta_deg=80.0, fov_y_deg=55.0),
        "ref_a0_th90": base.replace(width=48, height=27, spp=1, spin=0.0),
        "ref_a05_adaptive": base.replace(width=24, height=14, spp=1, spin=0.5, theta_deg=70.0,
                                         fov_y_deg=40.0, integrator=NP_INTEG_ADAPTIVE),
        "ref_a09_point_zamo": base.replace(width=40, height=24, spp=1, spin=0.9, theta_deg=85.0,
                                           fov_y_deg=30.0, background=NP_BG_POINT, camera=NP_CAMERA_ZAMO,
                                           disk_max_orders=2, sample_offset=3),
    }


def bench_cases():
    return {
        "bench_a09_64x36": benchmark_scene(width=64, height=36, spp=4),
        "bench_a0998_32x32": benchmark_scene(width=32, height=32, spp=4, spin=0.998, seed=5),
    }


def scene_dict(sc):
    return {k: getattr(sc, k) for k, _ in type(sc)._fields_}


def main():
    if oracle.load_ref() is None:
        raise SystemExit("oracle/_ref/libnpref.so is not built (needs the reference checkout)")
    for name, sc in ref_cases().items():
        rgb, rc = oracle.render_ref(sc)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), rgb=rgb, rcross=rc,
                            scene=np.array([repr(scene_dict(sc))]), source=np.array(["reference headers"]))
        print(name, rgb.shape, int((rc > 0).sum()), "disk px")
    for name, sc in bench_cases().items():
        rgb, rc = oracle.render(sc)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), rgb=rgb, rcross=rc,
                            scene=np.array([repr(scene_dict(sc))]), source=np.array(["oracle"]))
        print(name, rgb.shape, int((rc > 0).sum()), "disk px")


if __name__ == "__main__":
    main()
