"""Writes the golden fixtures of tests/golden/ from the REFERENCE's own kernels.

Runs where the reference's kernels run: a GPU with oracle/_ref/ built (the
PTX of the reference's cuda_gvdb_module.cu, see oracle/ref_build.py) and the
harness oracle/ref_harness.cu that drives them.  Each fixture holds seeded
inputs and what the reference computed from them:
  topo_full_r{0,1,2}.npz   full RebuildTopology: node pools, child lists, atlas map
  topo_incremental.npz     4 frames of RebuildTopology (full, full, incremental...)
  topo_accumulate.npz      3 frames of AccumulateTopology
  scatter.npz              InsertPoints + ScatterDensity (expand), interior bricks
  gather_{density,levelset}.npz   InsertPointsSubcell + the gathers, interior bricks
  apron.npz                UpdateApron(0, 0.75) of a seeded float channel

  python tests/golden/make_golden.py      (writes next to this file)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

LOGDIM = (3, 3, 3, 3, 5)


def grid(rh, channels=((0, 3),)):
    r = rh.RefGrid(LOGDIM)
    for c, t in channels:
        r.add_channel(c, t)
    return r


def pools(r):
    out = {"root_level": np.int32(r.root_level()), "used_leaves": np.int64(r.used_leaves())}
    for lev in range(r.root_level() + 1):
        nd = r.nodes(lev)
        out["nodes%d" % lev] = np.frombuffer(nd.tobytes(), np.uint8).reshape(len(nd), 64)
        if lev > 0:
            out["clist%d" % lev] = r.childlist(lev)
    return out


def cloud(n, seed, extent, lo=2.0):
    rng = np.random.default_rng(seed)
    return (rng.random((n, 3)) * np.asarray(extent) + lo).astype(np.float32)


def main():
    import ref_harness as rh

    if not rh.available():
        raise SystemExit("the reference's kernels are not built (oracle/_ref/cuda_gvdb_module.ptx)")
    rh.build()
    rh.load()

    for radius in (0.0, 1.0, 2.0):
        pos = cloud(4000, 11, (90.0, 70.0, 110.0))
        r = grid(rh)
        r.set_points(pos)
        assert r.rebuild(radius) == 0
        r.update_atlas()
        np.savez_compressed(os.path.join(HERE, "topo_full_r%d.npz" % radius), pos=pos, radius=np.float32(radius),
                            **pools(r))

    base = cloud(3000, 12, (80.0, 60.0, 90.0), lo=20.0)
    vel = np.random.default_rng(13).normal(0, 1, base.shape).astype(np.float32)
    for name, mode, frames in (("topo_incremental", 0, 4), ("topo_accumulate", 2, 3)):
        r = grid(rh)
        out = {}
        for f in range(frames):
            p = np.maximum(base + np.float32(3.0 * f) * vel, 0.5).astype(np.float32)
            r.set_points(p)
            assert r.rebuild(1.0, mode=mode) == 0
            r.update_atlas()
            out["pos%d" % f] = p
            out["mode%d" % f] = np.int32(r.last_mode())
            for k, v in pools(r).items():
                out["f%d_%s" % (f, k)] = v
        np.savez_compressed(os.path.join(HERE, name + ".npz"), frames=np.int32(frames), topo_mode=np.int32(mode),
                            **out)

    # ScatterDensity on a jittered lattice (no two 7-voxel stencils overlap: no race in the reference)
    g = np.stack(np.meshgrid(np.arange(12), np.arange(10), np.arange(14), indexing="ij"), -1).reshape(-1, 3)
    pos = (3.0 * g + 2.0 + np.random.default_rng(14).random(g.shape) * 0.9).astype(np.float32)
    r = grid(rh)
    r.set_points(pos)
    r.rebuild(0.0)
    r.update_atlas()
    r.scatter(1.5)
    used = r.used_leaves()
    np.savez_compressed(os.path.join(HERE, "scatter.npz"), pos=pos, radius=np.float32(1.5),
                        bricks=r.read_bricks(0)[:used, 1:-1, 1:-1, 1:-1], **pools(r))

    pos = cloud(2500, 15, (60.0, 50.0, 70.0), lo=4.0)
    for levelset in (False, True):
        r = grid(rh)
        r.set_points(pos)
        r.rebuild(2.0)
        r.update_atlas()
        n_sc = r.gather(levelset, 4, 1.0, 2.0)
        used = r.used_leaves()
        np.savez_compressed(os.path.join(HERE, "gather_%s.npz" % ("levelset" if levelset else "density")), pos=pos,
                            radius=np.float32(1.0), radius_ins=np.float32(2.0), subcell=np.int32(4),
                            sc_len=np.int64(n_sc), bricks=r.read_bricks(0)[:used, 1:-1, 1:-1, 1:-1], **pools(r))

    pos = cloud(400, 16, (40.0, 30.0, 40.0), lo=4.0)
    r = grid(rh)
    r.set_points(pos)
    r.rebuild(1.0)
    r.update_atlas()
    P = 10
    sd = r.atlas_subdim()
    # eighths in [-8, 8): exact in float32 and small once compressed
    data = (np.random.default_rng(17).integers(-64, 64, (sd[2] * sd[1] * sd[0], P, P, P)) / 8.0).astype(np.float32)
    r.write_dense(0, rh.bricks_to_dense(data, sd, P))
    r.update_apron(0, 0.75)
    used = r.used_leaves()
    np.savez_compressed(os.path.join(HERE, "apron.npz"), pos=pos, data_in=data[:used], boundval=np.float32(0.75),
                        bricks=r.read_bricks(0)[:used], **pools(r))
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
