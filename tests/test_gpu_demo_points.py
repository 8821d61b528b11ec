"""gpu_step_points, the loader's demo entry point (src/gpu/gpu_api.h:75): one
kick-drift-kick leapfrog step under a softened pull toward the origin, checked
against a float64 NumPy model of the same step."""
import ctypes as C

import numpy as np
import pytest

import simstack_gb300 as sg

pytestmark = pytest.mark.gpu


def leapfrog(p, v, dt, eps2=0.01):
    def acc(q):
        r2 = (q * q).sum(0) + eps2
        return -q / r2 ** 1.5
    u = v + 0.5 * dt * acc(p)
    p = p + dt * u
    return p, u + 0.5 * dt * acc(p)


def test_step_points_matches_leapfrog(module):
    rng = np.random.default_rng(5)
    n = 10_000
    host = np.concatenate([rng.uniform(-2, 2, (3, n)), rng.uniform(-0.5, 0.5, (3, n))]).astype(np.float32)
    dev = module.alloc(host.nbytes)
    L = sg.lib()
    assert L.gpu_copy_to_device(dev, host.ctypes.data, host.nbytes) == 0
    ptr = [dev + i * n * 4 for i in range(6)]
    dt = 0.01
    for _ in range(3):
        assert L.gpu_step_points(*ptr, n, C.c_float(dt)) == 0
    out = np.empty_like(host)
    assert L.gpu_copy_to_host(out.ctypes.data, dev, out.nbytes) == 0
    p, v = host[:3].astype(np.float64), host[3:].astype(np.float64)
    for _ in range(3):
        p, v = leapfrog(p, v, dt)
    np.testing.assert_allclose(out[:3], p, rtol=2e-5, atol=2e-5)
    np.testing.assert_allclose(out[3:], v, rtol=2e-4, atol=2e-4)
    assert L.gpu_step_points(*ptr, 0, C.c_float(dt)) == 0   # empty set: nothing to do
