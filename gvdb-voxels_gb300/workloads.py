"""Seeded synthetic point sets with the shapes of the benchmark configurations.

The reference ships no point dataset for this path (its only sample,
shared_assets/points.dat, is not in the repository), so every workload is
generated from a seed:

  plain_small      100k points, FP32 xyz uniform in [0,256)^3, seed 0, weight 1
  sph_slab         4M points in x in [0,512], y in [0,256], z in [0,1024] jittered
                   by N(0, 0.3 voxel), velocity components N(0,1); advect() moves
                   them by dt * u (dt = 0.5 voxel)
  differentiable   1M points uniform in [8,504)^3, weights U(0,1), radii U(1,3)
  batched_clouds   64 clouds, sizes log-uniform in [10k, 2M] (seed 7), mixtures of
                   1-16 Gaussian blobs (sigma 4-64) in 1024^3, weights U(0.5,1.5)
"""
import numpy as np


def plain_small(n=100_000, seed=0, extent=256.0):
    rng = np.random.default_rng(seed)
    pos = (rng.random((n, 3), dtype=np.float64) * extent).astype(np.float32)
    pos = np.minimum(pos, np.float32(np.nextafter(np.float32(extent), np.float32(0))))
    w = np.ones(n, np.float32)
    return pos, w


def sph_slab(n=4_000_000, seed=0, box=(512.0, 256.0, 1024.0), jitter=0.3):
    rng = np.random.default_rng(seed)
    base = rng.random((n, 3), dtype=np.float64) * np.asarray(box)
    pos = (base + rng.normal(0.0, jitter, (n, 3))).astype(np.float32)
    vel = rng.normal(0.0, 1.0, (n, 3)).astype(np.float32)
    return pos, vel


def advect(pos, vel, dt=0.5):
    return (pos + np.float32(dt) * vel).astype(np.float32)


def differentiable(n=1_000_000, seed=0, lo=8.0, hi=504.0):
    rng = np.random.default_rng(seed)
    pos = (lo + rng.random((n, 3)) * (hi - lo)).astype(np.float32)
    w = rng.random(n).astype(np.float32)
    r = (1.0 + 2.0 * rng.random(n)).astype(np.float32)
    return pos, w, r


def batched_clouds(count=64, seed=7, nmin=10_000, nmax=2_000_000, extent=1024.0):
    rng = np.random.default_rng(seed)
    sizes = np.floor(np.exp(rng.uniform(np.log(nmin), np.log(nmax), count))).astype(np.int64)
    clouds = []
    for n in sizes:
        k = int(rng.integers(1, 17))
        centres = rng.uniform(128.0, 896.0, (k, 3))
        sig = rng.uniform(4.0, 64.0, k)
        comp = rng.integers(0, k, int(n))
        p = centres[comp] + rng.normal(0.0, 1.0, (int(n), 3)) * sig[comp, None]
        p = np.clip(p, 0.0, extent - 1e-3).astype(np.float32)
        w = rng.uniform(0.5, 1.5, int(n)).astype(np.float32)
        clouds.append((p, w))
    return clouds
