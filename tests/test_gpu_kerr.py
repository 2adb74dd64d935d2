"""The physics-header API (include/np_kerr.h) compiled for sm_103a against the
same header code on the host: camera rays and 300 FP64 RK4 steps agree to
1e-9 relative (the device contracts multiply-adds)."""
import numpy as np
import pytest

from nullpath_gb300 import kerr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("zamo", [False, True])
def test_device_matches_host(cuda, zamo):
    rng = np.random.default_rng(11)
    n = 256
    d = rng.normal(size=(n, 3))
    d[:, 0] = -np.abs(d[:, 0]) - 1.0
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    cam = np.zeros((n, 6))
    cam[:, 0] = rng.uniform(20.0, 60.0, n)
    cam[:, 1] = rng.uniform(0.3, 2.8, n)
    cam[:, 2] = rng.uniform(0.0, 6.0, n)
    cam[:, 3:] = d
    h_st, h_al = kerr.integrate(1.0, 0.7, cam, 300, h_scale=0.01, zamo=zamo, device=False)
    d_st, d_al = kerr.integrate(1.0, 0.7, cam, 300, h_scale=0.01, zamo=zamo, device=True)
    init_h, _ = kerr.integrate(1.0, 0.7, cam, 0, zamo=zamo, device=False)
    init_d, _ = kerr.integrate(1.0, 0.7, cam, 0, zamo=zamo, device=True)
    assert np.allclose(init_d, init_h, rtol=1e-13, atol=1e-13)
    same = h_al == d_al
    assert same.mean() > 0.98
    ok = same & (h_al == 1)
    assert np.allclose(d_st[ok], h_st[ok], rtol=1e-9, atol=1e-9)
