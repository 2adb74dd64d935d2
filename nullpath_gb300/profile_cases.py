"""Small, fixed workloads of each GPU kernel of the library, for profiler
captures (ncu -k <kernel> -s <skip> -c 1): every case launches its kernel
`reps` times on cuda:0 after one warm-up launch and exits.

    python -m nullpath_gb300.profile_cases <case> [--reps N]

Cases (kernel names in parentheses):
    fp64_rk4        FP64 reference-form RK4 render, 160x90x1 benchmark frame
                    (render_fp64_kernel<0>)
    fp64_research   research mode, FP64 Fehlberg 7(8) with root-found
                    crossings and the invariant gate, 160x90x1 (render_fp64_kernel<1>)
    mixed_rk4       mixed path, reference step law, every island, 640x360x4
                    (render_mixed_kernel<4, 0>)
    mixed_rkf78     mixed 7(8) path, default islands, 640x360x4
                    (render_mixed_kernel<4, 1>)
    adjoint         differentiable render 128x128x2, FP32, K = 64
                    (adj_forward_kernel<float>, adj_backward_kernel<float>)
    batch           16 uneven scenes in one persistent launch (batch_mixed_kernel)
    critical        near-critical rays in closed form: 512x512x16 at a = 0.998
                    with critical-curve sampling, mixed 7(8) path, default
                    islands (critical_cf_kernel; render_mixed_kernel<4, 1>)
    geokerr         GEOKERR camera grid 128x128, 32 points per geodesic, closed
                    form (cf_setup_kernel, cf_points_kernel, cf_fallback_kernel)
    geokerr_taylor  the same grid on the Taylor solver (geokerr_points_kernel)
    carlson         2^20 Carlson R_F / R_D / R_J cases (carlson_batch_kernel)
"""
import argparse
import math

import numpy as np


def _fp64_rk4(reps):
    import nullpath_gb300 as npx
    sc = npx.benchmark_scene(width=160, height=90, spp=1)
    for _ in range(reps + 1):
        npx.render(sc, "fp64")


def _fp64_research(reps):
    import nullpath_gb300 as npx
    sc = npx.research_scene(npx.benchmark_scene(width=160, height=90, spp=1))
    for _ in range(reps + 1):
        npx.render(sc, "fp64")


def _mixed(reps, path):
    import nullpath_gb300 as npx
    base = npx.benchmark_scene(width=640, height=360, spp=4)
    sc = npx.accurate_scene(base) if path == "rkf78" else base.replace(islands=npx.NP_ISLANDS_ALL)
    for _ in range(reps + 1):
        npx.render(sc, "mixed")


def _critical(reps):
    import nullpath_gb300 as npx
    base = npx.benchmark_scene(width=512, height=512, spp=16, spin=0.998).replace(jitter=npx.NP_JITTER_CRITICAL)
    sc = npx.accurate_scene(base)
    for _ in range(reps + 1):
        npx.render(sc, "mixed")


def _adjoint(reps):
    import torch
    import nullpath_gb300 as npx
    from nullpath_gb300 import diff
    sc = diff.scene_with(npx.benchmark_scene(width=128, height=128, spp=2, spin=0.5, seed=2), 0.5,
                         math.radians(50.0), 0.8, 2.5)
    ones = torch.ones((3, 128, 128), dtype=torch.float32, device="cuda")
    for _ in range(reps + 1):
        adj = diff.Adjoint()
        adj.forward(sc, "mixed", 64)
        adj.backward(ones)
        adj.close()


def _batch(reps):
    from nullpath_gb300 import batch
    b = batch.Batch(batch.uneven_scenes(16, seed=1))
    for _ in range(reps + 1):
        b.run(graph=False)
    b.close()


def _geokerr(reps, method="closed_form"):
    from nullpath_gb300 import geokerr as gk
    a, mu0, u0 = 0.9, 0.5, 1e-6
    uplus = 1.0 / (1.0 + math.sqrt(1.0 - a * a))
    g = {k: v.cpu().numpy() for k, v in gk.camera_grid(a, mu0, 128, 128).items()}
    n = g["l"].size
    for _ in range(reps + 1):
        gk.points(a, np.full(n, u0), np.full(n, uplus), np.full(n, mu0), g["l"], g["q2"], g["su"], g["sm"],
                  tpr=1, nup=32, offset=0.5, method=method)


def _carlson(reps):
    from nullpath_gb300 import carlson
    n = 1 << 20
    rng = np.random.default_rng(3)
    x, y, z, p = (rng.uniform(0.1, 10.0, n) for _ in range(4))
    kinds = [("RF", "RD", "RJ")[k] for k in rng.integers(0, 3, n)]
    for _ in range(reps + 1):
        carlson.evaluate(kinds, x, y, z, p)


CASES = {"fp64_rk4": _fp64_rk4, "fp64_research": _fp64_research, "critical": _critical,
         "mixed_rk4": lambda r: _mixed(r, "rk4"), "mixed_rkf78": lambda r: _mixed(r, "rkf78"),
         "adjoint": _adjoint, "batch": _batch, "geokerr": _geokerr,
         "geokerr_taylor": lambda r: _geokerr(r, "taylor"), "carlson": _carlson}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=sorted(CASES))
    ap.add_argument("--reps", type=int, default=2)
    args = ap.parse_args()
    import torch
    torch.cuda.set_device(0)
    CASES[args.case](args.reps)
    torch.cuda.synchronize()
    print("done", args.case)


if __name__ == "__main__":
    main()
