"""GPU tests of the batched multi-grid splat: one persistent launch over the
bricks of many grids (plain, captured in a CUDA graph and replayed, and
autotuned) gives every grid exactly what its own gvx_splat gives."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LOGDIM = (3, 3, 3, 3, 5)


def clouds(count, seed, nmin=2_000, nmax=60_000):
    """uneven Gaussian-mixture clouds (the batched workload's generator, smaller sizes)"""
    import workloads

    return workloads.batched_clouds(count=count, seed=seed, nmin=nmin, nmax=nmax)


def make_grids(gvx, cl, vel=False, radius=1.0):
    grids = []
    for p, w in cl:
        g = gvx.Grid(0)
        g.configure(LOGDIM)
        g.add_channel(0, gvx.T_FLOAT, 1)
        if vel:
            g.add_channel(1, gvx.T_FLOAT3, 1)
        v = np.random.default_rng(len(p)).normal(0, 1, p.shape).astype(np.float32) if vel else None
        g.commit_points_host(p, vel=v, weight=w)
        g.rebuild_topology(len(p), radius, mode=gvx.TOPO_FULL)
        g.update_atlas()
        g.insert_points(len(p))
        grids.append(g)
    return grids


def read_all(grids, chans):
    """the channels' active bricks (the slots past them are not written by a splat)"""
    return [[g.read_channel(c)[:g.info()["used_leaves"]].copy() for c in chans] for g in grids]


def same(a, b):
    return all(np.array_equal(x, y) for ra, rb in zip(a, b) for x, y in zip(ra, rb))


@pytest.mark.parametrize("mode,vel", [("trilinear", False), ("cubic", True)])
def test_batch_matches_per_grid_splats(gvx_mod, mode, vel):
    m = gvx_mod.SPLAT_TRILINEAR if mode == "trilinear" else gvx_mod.SPLAT_CUBIC
    radius = 1.0 if mode == "trilinear" else 2.0
    grids = make_grids(gvx_mod, clouds(7, 5), vel=vel, radius=radius)
    chans = (0, 1) if vel else (0,)
    cv = 1 if vel else -1
    # per grid
    for g, (p, _) in zip(grids, clouds(7, 5)):
        g.splat(m, len(p), radius, chan_density=0, chan_vel=cv)
    ref = read_all(grids, chans)
    for g in grids:
        g.fill_channel(0, [9.0])
    b = gvx_mod.Batch(0)
    b.set_grids(grids)
    b.splat(m, radius, chan_density=0, chan_vel=cv, graph=False)
    assert same(read_all(grids, chans), ref)
    for g in grids:
        g.fill_channel(0, [9.0])
    b.splat(m, radius, chan_density=0, chan_vel=cv, graph=True)
    assert same(read_all(grids, chans), ref)
    # replay of the captured graph
    for g in grids:
        g.fill_channel(0, [9.0])
    b.splat(m, radius, chan_density=0, chan_vel=cv, graph=True)
    assert same(read_all(grids, chans), ref)
    b.close()


def test_batch_recaptures_when_a_grid_changes(gvx_mod):
    cl = clouds(5, 9)
    grids = make_grids(gvx_mod, cl)
    b = gvx_mod.Batch(0)
    b.set_grids(grids)
    b.splat(gvx_mod.SPLAT_TRILINEAR, 1.0, graph=True)
    # grid 2 gets new points and a new topology: its buffers move
    p = (cl[2][0] + 37.0).astype(np.float32)
    grids[2].commit_points_host(p, weight=cl[2][1])
    grids[2].rebuild_topology(len(p), 1.0, mode=gvx_mod.TOPO_FULL)
    grids[2].update_atlas()
    grids[2].insert_points(len(p))
    b.splat(gvx_mod.SPLAT_TRILINEAR, 1.0, graph=True)
    got = read_all(grids, (0,))
    for g, (q, _) in zip(grids, [cl[0], cl[1], (p, None), cl[3], cl[4]]):
        g.splat(gvx_mod.SPLAT_TRILINEAR, len(q), 1.0)
    assert same(got, read_all(grids, (0,)))
    b.close()


def test_batch_autotune_keeps_results(gvx_mod):
    cl = clouds(6, 13)
    grids = make_grids(gvx_mod, cl)
    for g, (p, _) in zip(grids, cl):
        g.splat(gvx_mod.SPLAT_TRILINEAR, len(p), 1.0)
    ref = read_all(grids, (0,))
    b = gvx_mod.Batch(0)
    b.set_grids(grids)
    b.splat(gvx_mod.SPLAT_TRILINEAR, 1.0, graph=True, tune=True)
    t = b.tuning()
    assert t["slab_layers"] >= 1 and t["blocks_per_sm"] >= 1 and t["ms"] > 0
    assert same(read_all(grids, (0,)), ref)
    b.close()


@pytest.mark.parametrize("threads", [0, 4])
def test_batch_topology_matches_per_grid_builds(gvx_mod, threads):
    """gvx_batch_topology staged from one host thread (threads 0) or from 4 host threads, grids on
    their own streams: the same pools, child lists, atlas maps and point groupings (checked through
    a splat) as one-by-one builds"""
    cl = clouds(9, 11)
    ref = make_grids(gvx_mod, cl, radius=1.0)
    grids = []
    for p, w in cl:
        g = gvx_mod.Grid(0)
        g.configure(LOGDIM)
        g.add_channel(0, gvx_mod.T_FLOAT, 1)
        g.commit_points_host(p, weight=w)
        grids.append(g)
    b = gvx_mod.Batch(0)
    b.set_grids(grids)
    b.topology(1.0, threads=threads)
    for g in grids:
        g.sync()
    for g, r, (p, _) in zip(grids, ref, cl):
        gi, ri = g.info(), r.info()
        assert gi["root_level"] == ri["root_level"] and gi["used_leaves"] == ri["used_leaves"]
        assert np.array_equal(g.read_atlas_map(), r.read_atlas_map())
        for lev in range(ri["root_level"] + 1):
            assert np.array_equal(g.read_nodes(lev), r.read_nodes(lev))
            if lev > 0:
                assert np.array_equal(g.read_childlist(lev), r.read_childlist(lev))
        g.splat(gvx_mod.SPLAT_TRILINEAR, len(p), 1.0, chan_density=0)
        r.splat(gvx_mod.SPLAT_TRILINEAR, len(p), 1.0, chan_density=0)
    assert same(read_all(grids, (0,)), read_all(ref, (0,)))
    b.close()
    for g in grids + ref:
        g.close()
