"""Seeded synthetic inputs for the MSBG surface-reconstruction and Poisson workloads.

The reference demo builds its point cloud by instancing a PLY mesh
(src/msbg_demo.cpp:246-356).  The workloads here replace that with seeded
synthetic clouds of the stated shapes:

* ``sphere_cloud``   - spheres, points uniform on each surface plus Gaussian
  jitter (the 512^3 / bs16 FP32 surface workload uses 64 spheres x 32,000 pts).
* ``ellipsoid_cloud`` - randomly rotated ellipsoids, points at uniformly random
  directions scaled by the three semi-axes plus jitter (the 4096^3 / bs32
  three-level FP16 workload uses 1,024 clusters x 32,000 pts).

Every generator is deterministic: ``seed = 20261203 + 1000*workload + index``
feeds numpy's PCG64, and the float32 result is what both the GPU path and the
CPU oracle consume.
"""
from __future__ import annotations

import numpy as np

SEED_BASE = 20261203


def workload_seed(workload: int, index: int = 0) -> int:
    return SEED_BASE + 1000 * workload + index


def _unit_dirs(rng: np.random.Generator, n: int) -> np.ndarray:
    g = rng.standard_normal((n, 3))
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    return g


def sphere_cloud(res: int, n_spheres: int, pts_per_sphere: int, *, seed: int,
                 centre_range=(0.1, 0.9), radius_range=(0.02, 0.06),
                 jitter_vox: float = 0.1) -> np.ndarray:
    """Points (float32, shape [n,3], voxel units) on ``n_spheres`` sphere surfaces."""
    rng = np.random.Generator(np.random.PCG64(seed))
    c = rng.uniform(*centre_range, size=(n_spheres, 3)) * res
    r = rng.uniform(*radius_range, size=n_spheres) * res
    out = np.empty((n_spheres * pts_per_sphere, 3), dtype=np.float32)
    for s in range(n_spheres):
        d = _unit_dirs(rng, pts_per_sphere)
        p = c[s] + r[s] * d + rng.normal(0.0, jitter_vox, size=(pts_per_sphere, 3))
        out[s * pts_per_sphere:(s + 1) * pts_per_sphere] = p
    np.clip(out, 0.0, np.float32(res) * np.float32(0.999), out=out)
    return out


def _rotation(rng: np.random.Generator) -> np.ndarray:
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    ])


def ellipsoid_cloud(res: int, n_clusters: int, pts_per_cluster: int, *, seed: int,
                    centre_range=(0.1, 0.9), axis_range=(0.005, 0.03),
                    jitter_vox: float = 0.1) -> np.ndarray:
    """Points (float32, [n,3], voxel units) on randomly rotated ellipsoid surfaces."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = np.empty((n_clusters * pts_per_cluster, 3), dtype=np.float32)
    for k in range(n_clusters):
        c = rng.uniform(*centre_range, size=3) * res
        ax = rng.uniform(*axis_range, size=3) * res
        rot = _rotation(rng)
        d = _unit_dirs(rng, pts_per_cluster) * ax
        p = c + d @ rot.T + rng.normal(0.0, jitter_vox, size=(pts_per_cluster, 3))
        out[k * pts_per_cluster:(k + 1) * pts_per_cluster] = p
    np.clip(out, 0.0, np.float32(res) * np.float32(0.999), out=out)
    return out


# Named workloads -----------------------------------------------------------------

SURFACE_512 = dict(name="surface-512^3-bs16-fp32", res=512, bsx=16, n_levels=3,
                   n_objects=64, pts_per_object=32000, kind="sphere", n_iter=20, dt=0.1,
                   storage="f32")
SURFACE_4096 = dict(name="surface-4096^3-bs32-3lvl-fp16", res=4096, bsx=32, n_levels=3,
                    n_objects=1024, pts_per_object=32000, kind="ellipsoid", n_iter=50,
                    dt=0.1, storage="f16", fine_band=8.0, mid_band=16.0)


# A crop of the 4096^3 workload (first 96 of its 1,024 clusters, same seed), a
# few GB on the device: the case kernels are profiled on.
SURFACE_4096_CROP = dict(SURFACE_4096, name="surface-4096^3-bs32-3lvl-fp16-crop96", n_objects=96)


def make_points(spec: dict, workload: int, index: int = 0) -> np.ndarray:
    seed = workload_seed(workload, index)
    if spec["kind"] == "sphere":
        return sphere_cloud(spec["res"], spec["n_objects"], spec["pts_per_object"], seed=seed)
    return ellipsoid_cloud(spec["res"], spec["n_objects"], spec["pts_per_object"], seed=seed)
