"""The complex-step oracle of the differentiable render (oracle/adjoint_cs.py)
against central differences of its own map on samples whose map is smooth at
the difference step, and its colour against the FP64 render oracle."""
import math

import numpy as np

import nullpath_gb300 as npx
from nullpath_gb300 import diff
from oracle import adjoint_cs as cs


def _scene():
    sc = npx.benchmark_scene(width=32, height=32, spp=1, spin=0.5, seed=2)
    return cs.scene_dict(diff.scene_with(sc, 0.5, math.radians(50.0), 0.8, 2.5))


def test_complex_step_matches_central_difference():
    d = _scene()
    th0 = math.radians(50.0)
    for idx in (520, 660, 336, 588):
        sig, g = cs.sample_gradient(d, idx)
        assert sig >= 4 and sig % 4 == 0
        x, y = idx % 32, idx // 32
        h = 1e-6
        f = lambda a, th, q: cs.trace(d, a, th, q, x, y, 0)[3]
        w = 0.8 * 2.2
        fa = (f(0.5 + h, th0, 2.5) - f(0.5 - h, th0, 2.5)) / (2 * h) * w
        ft = (f(0.5, th0 + h, 2.5) - f(0.5, th0 - h, 2.5)) / (2 * h) * w
        fq = (f(0.5, th0, 2.5 + h) - f(0.5, th0, 2.5 - h)) / (2 * h) * w
        assert np.allclose([fa, ft, fq], [g[0], g[1], g[3]], rtol=1e-6, atol=1e-12), (idx, g, fa, ft, fq)
        # d/dgain is the colour sum itself
        assert abs(g[2] - 2.2 * f(0.5, th0, 2.5)) < 1e-15


def test_sky_and_captured_samples_have_no_gradient():
    d = _scene()
    seen = set()
    for idx in range(0, 1024, 7):
        sig, g = cs.sample_gradient(d, idx)
        if sig < 4 or sig % 4 == 1:
            assert g == [0.0, 0.0, 0.0, 0.0]
            seen.add(sig % 4)
    assert seen, "no sky or captured sample in the probe set"
