"""Seeded synthetic inputs are deterministic and have the stated shapes."""
from __future__ import annotations

import numpy as np

from msbg_gb300 import workloads as W


def test_sphere_cloud_deterministic():
    a = W.sphere_cloud(128, 4, 100, seed=W.workload_seed(1, 3))
    b = W.sphere_cloud(128, 4, 100, seed=W.workload_seed(1, 3))
    c = W.sphere_cloud(128, 4, 100, seed=W.workload_seed(1, 4))
    assert a.dtype == np.float32 and a.shape == (400, 3)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert a.min() >= 0 and a.max() < 128


def test_sphere_radius_and_jitter():
    pts = W.sphere_cloud(512, 1, 20000, seed=123, centre_range=(0.5, 0.5), radius_range=(0.05, 0.05))
    r = np.linalg.norm(pts - 256.0, axis=1)
    assert abs(r.mean() - 25.6) < 0.05
    assert 0.1 < r.std() < 0.25  # sigma 0.1 per axis -> ~0.1 radial (float32 rounding on top)


def test_ellipsoid_cloud_shape():
    pts = W.ellipsoid_cloud(4096, 3, 1000, seed=W.workload_seed(2))
    assert pts.shape == (3000, 3) and pts.dtype == np.float32
    assert pts.min() > 0.05 * 4096 and pts.max() < 0.95 * 4096


def test_named_workloads():
    assert W.SURFACE_512["n_objects"] * W.SURFACE_512["pts_per_object"] == 2_048_000
    assert W.SURFACE_4096["n_objects"] * W.SURFACE_4096["pts_per_object"] == 32_768_000
