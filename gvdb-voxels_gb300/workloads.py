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
  depth_fusion     frames of a depth camera (640x480, f = 525, principal point at the
                   centre) on a circle around a scene of 8 spheres and 2 planes in
                   2048^3, ray-cast analytically, back-projected with N(0, 0.5 voxel)
                   noise; per point a confidence |cos| of the incidence angle
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


def depth_fusion(frames=30, seed=3, width=640, height=480, f=525.0, noise=0.5, extent=2048.0, scale=1.0):
    """Yields (points, confidence) per frame: the surface points a pinhole depth
    camera sees, ray-cast analytically against 8 spheres and 2 planes (scene
    drawn from `seed`), back-projected to index space with noise.  `scale`
    shrinks the scene, the camera path and the extent together."""
    rng = np.random.default_rng(seed)
    c0 = np.full(3, 0.5 * extent)
    sc = c0 + rng.uniform(-300.0, 300.0, (8, 3)) * scale
    sr = rng.uniform(60.0, 180.0, 8) * scale
    planes = [(np.array([0.0, 1.0, 0.0]), c0[1] - 350.0 * scale),   # floor: n.x = d
              (np.array([0.0, 0.0, 1.0]), c0[2] - 900.0 * scale)]   # back wall, beyond the camera path
    u, v = np.meshgrid(np.arange(width, dtype=np.float64), np.arange(height, dtype=np.float64))
    dc = np.stack([(u - 0.5 * width) / f, (v - 0.5 * height) / f, np.ones_like(u)], -1).reshape(-1, 3)
    dc /= np.linalg.norm(dc, axis=1, keepdims=True)
    for k in range(frames):
        ang = 2.0 * np.pi * k / frames
        cam = c0 + np.array([700.0 * np.cos(ang), 150.0, 700.0 * np.sin(ang)]) * scale
        fwd = c0 - cam
        fwd /= np.linalg.norm(fwd)
        right = np.cross(fwd, np.array([0.0, 1.0, 0.0]))
        right /= np.linalg.norm(right)
        up = np.cross(right, fwd)
        d = dc[:, :1] * right + dc[:, 1:2] * (-up) + dc[:, 2:3] * fwd
        t = np.full(len(d), np.inf)
        nrm = np.zeros_like(d)
        for c, r in zip(sc, sr):
            oc = cam - c
            b = d @ oc
            disc = b * b - (oc @ oc - r * r)
            ok = disc > 0
            th = np.where(ok, -b - np.sqrt(np.where(ok, disc, 0.0)), np.inf)
            th = np.where(th > 1e-6, th, np.inf)
            better = th < t
            t = np.where(better, th, t)
            with np.errstate(invalid="ignore"):
                hitp = cam + th[:, None] * d
            nrm = np.where(better[:, None], (hitp - c) / r, nrm)
        for n_, dd in planes:
            den = d @ n_
            with np.errstate(divide="ignore", invalid="ignore"):
                th = (dd - cam @ n_) / den
            th = np.where((np.abs(den) > 1e-9) & (th > 1e-6), th, np.inf)
            better = th < t
            t = np.where(better, th, t)
            nrm = np.where(better[:, None], n_[None, :], nrm)
        hit = np.isfinite(t)
        p = cam + t[hit, None] * d[hit] + rng.normal(0.0, noise, (int(hit.sum()), 3))
        conf = np.abs((nrm[hit] * d[hit]).sum(1))
        keep = np.all((p >= 0.0) & (p < extent), axis=1)
        yield p[keep].astype(np.float32), conf[keep].astype(np.float32)
