"""GPU parity of the incremental topology builds (RebuildTopology from its
third call on, and AccumulateTopology on an existing tree) against the oracle:
pools, child lists, flags, used-leaf counts and the rebuild mode must be
bit-exact after every frame, and a splat on the resulting tree must match."""
import numpy as np
import pytest

from parity_util import DENSITY_TOL, compare_topology, rel_error

pytestmark = pytest.mark.gpu

LOGDIM = (3, 3, 3, 3, 5)
UNDEF64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def new_pair(gvx, orc, logdim=LOGDIM, channels=((0, 3),)):
    g = gvx.Grid(0)
    g.configure(logdim)
    o = orc.Oracle(logdim)
    for c, t in channels:
        g.add_channel(c, t, 1)
        o.add_channel(c, t)
    return g, o


def step(gvx, orc, g, o, pos, radius, mode, min_depth=1, orig=(0.0, 0.0, 0.0)):
    g.commit_points_host(pos)
    g.rebuild_topology(len(pos), radius, orig=orig, mode=mode, min_depth=min_depth)
    g.finish_topology()
    g.update_atlas()
    assert o.rebuild_topology(pos, radius, orig=orig, mode=mode, min_depth=min_depth) == orc.OK
    o.update_atlas()
    compare_topology(g, o)
    assert g.info()["last_rebuild"] == o.last_mode()
    assert np.array_equal(g.read_atlas_map(), o.atlas_map())
    compare_bounds(g, o)


def compare_bounds(g, o):
    """FinishTopology's ComputeBounds (VG.cpp:1792-1816) against the oracle's
    restatement: mObjMin/Max, mVoxRes and the sticky mVoxResMax, exactly"""
    vmin, vmax, vres, vres_max = o.compute_bounds()
    inf = g.info()
    assert np.array_equal(np.float32(inf["obj_min"]), vmin)
    assert np.array_equal(np.float32(inf["obj_max"]), vmax)
    assert np.array_equal(np.float32(inf["vox_res"]), vres)
    assert np.array_equal(np.float32(inf["vox_res_max"]), vres_max)


def moving_slab(n, seed, frames, dt, box=(150.0, 90.0, 180.0)):
    rng = np.random.default_rng(seed)
    p0 = rng.random((n, 3)) * np.asarray(box) + 20.0
    v = rng.normal(0.0, 1.0, (n, 3))
    for f in range(frames):
        yield np.maximum(p0 + dt * f * v, 0.5).astype(np.float32)


@pytest.mark.parametrize("radius", [0.0, 1.0, 2.0])
def test_auto_frames_match_oracle(gvx_mod, orc, radius):
    g, o = new_pair(gvx_mod, orc)
    modes = []
    for pos in moving_slab(40_000, 3, 7, 1.5):
        step(gvx_mod, orc, g, o, pos, radius, gvx_mod.TOPO_AUTO)
        modes.append(o.last_mode())
    assert modes[:2] == [1, 1] and 2 in modes[2:]  # full, full (mCurrDepth quirk), then incremental


def test_accumulate_frames_match_oracle(gvx_mod, orc):
    g, o = new_pair(gvx_mod, orc)
    rng = np.random.default_rng(8)
    for f in range(5):
        centre = np.array([60.0 + 40.0 * f, 80.0, 100.0 + 25.0 * f])
        pos = (centre + rng.normal(0.0, 12.0, (15_000, 3))).astype(np.float32)
        pos = np.maximum(pos, 0.5).astype(np.float32)
        step(gvx_mod, orc, g, o, pos, 1.0, gvx_mod.TOPO_ACCUMULATE)
    assert o.last_mode() == 2
    assert (g.read_nodes(0)["flags"] == 1).all()  # accumulation keeps every leaf


def test_accumulate_below_root_level(gvx_mod, orc):
    # a wide first cloud puts the root at level 3; a small one then accumulates with depth 2
    g, o = new_pair(gvx_mod, orc)
    rng = np.random.default_rng(9)
    wide = (rng.random((20_000, 3)) * np.array([900.0, 300.0, 600.0]) + 1.0).astype(np.float32)
    step(gvx_mod, orc, g, o, wide, 1.0, gvx_mod.TOPO_ACCUMULATE)
    assert o.root_level() == 3
    small = (rng.random((3_000, 3)) * 40.0 + np.array([70.0, 70.0, 70.0])).astype(np.float32)
    step(gvx_mod, orc, g, o, small, 1.0, gvx_mod.TOPO_ACCUMULATE, min_depth=1)
    assert o.last_mode() == 2


def test_incremental_semantics_small(gvx_mod, orc):
    base = np.array([[10.5, 10.5, 10.5], [300.5, 200.5, 100.5], [60.5, 40.5, 20.5]], np.float32)
    g, o = new_pair(gvx_mod, orc)
    step(gvx_mod, orc, g, o, base, 0.0, gvx_mod.TOPO_AUTO)
    step(gvx_mod, orc, g, o, base, 0.0, gvx_mod.TOPO_AUTO)
    # a subset: no new node, so the markers are not applied and all 3 leaves stay
    step(gvx_mod, orc, g, o, base[:2], 0.0, gvx_mod.TOPO_AUTO)
    assert g.info()["last_rebuild"] == 0 and g.info()["used_leaves"] == 3
    # a point in a new leaf: the unmarked leaf is delinked
    moved = np.vstack([base[:2], [[120.5, 40.5, 20.5]]]).astype(np.float32)
    step(gvx_mod, orc, g, o, moved, 0.0, gvx_mod.TOPO_AUTO)
    n0 = g.read_nodes(0)
    i = [p.tolist() for p in n0["pos"]].index([56, 40, 16])
    assert n0["flags"][i] == 0 and n0["parent"][i] == UNDEF64
    # the point comes back: its leaf is allocated anew, the dead one stays in the pool
    step(gvx_mod, orc, g, o, base, 0.0, gvx_mod.TOPO_AUTO)
    assert g.info()["node_count"][0] == 5


def test_splat_on_incremental_tree(gvx_mod, orc):
    g, o = new_pair(gvx_mod, orc)
    frames = list(moving_slab(30_000, 5, 5, 2.0))
    for pos in frames:
        step(gvx_mod, orc, g, o, pos, 1.0, gvx_mod.TOPO_AUTO)
    pos = frames[-1]
    assert o.last_mode() in (0, 2)
    g.insert_points(len(pos))
    g.splat(gvx_mod.SPLAT_TRILINEAR, len(pos), 1.0, chan_density=0)
    o.splat(orc.SPLAT_TRILINEAR, pos, 1.0)
    got, ref = g.read_channel(0), o.read_channel(0)
    used = o.used_leaves()
    assert rel_error(got[:used], ref[:used]) <= DENSITY_TOL
    interior = got[:used, 1:-1, 1:-1, 1:-1].astype(np.float64)
    assert abs(float(interior.sum()) - len(pos)) <= 1e-5 * len(pos)


def test_full_request_after_incremental(gvx_mod, orc):
    g, o = new_pair(gvx_mod, orc)
    frames = list(moving_slab(20_000, 6, 4, 2.0))
    for pos in frames:
        step(gvx_mod, orc, g, o, pos, 1.0, gvx_mod.TOPO_AUTO)
    step(gvx_mod, orc, g, o, frames[0], 1.0, gvx_mod.TOPO_FULL)
    assert o.last_mode() == 1


def test_bounds_seeded_by_inactive_pool_node_zero(gvx_mod, orc):
    """ComputeBounds seeds min and max with level-0 pool node 0's position even
    when an incremental build has delinked that leaf (VG.cpp:1795-1797), and
    mVoxResMax keeps the widest box seen since Configure."""
    g, o = new_pair(gvx_mod, orc)
    a = np.array([[10.5, 10.5, 10.5], [300.5, 200.5, 100.5]], np.float32)
    step(gvx_mod, orc, g, o, a, 0.0, gvx_mod.TOPO_AUTO)
    step(gvx_mod, orc, g, o, a, 0.0, gvx_mod.TOPO_AUTO)
    wide = g.info()["vox_res_max"]
    b = np.array([[300.5, 200.5, 100.5], [120.5, 40.5, 20.5]], np.float32)
    step(gvx_mod, orc, g, o, b, 0.0, gvx_mod.TOPO_AUTO)
    n0 = g.read_nodes(0)
    assert n0["pos"][0].tolist() == [8, 8, 8] and n0["flags"][0] == 0
    inf = g.info()
    assert inf["obj_min"] == [8.0, 8.0, 8.0]  # from the delinked node 0, not from an active leaf
    assert inf["obj_max"] == [304.0, 208.0, 104.0]
    # a narrower cloud later: mVoxRes shrinks, mVoxResMax does not
    g2, o2 = new_pair(gvx_mod, orc)
    step(gvx_mod, orc, g2, o2, a, 0.0, gvx_mod.TOPO_FULL)
    narrow = np.array([[11.5, 11.5, 11.5], [20.5, 11.5, 11.5]], np.float32)
    step(gvx_mod, orc, g2, o2, narrow, 0.0, gvx_mod.TOPO_FULL)
    inf2 = g2.info()
    assert inf2["vox_res"] == [16.0, 8.0, 8.0] and inf2["vox_res_max"] == wide
    # FinishTopology(true, false) leaves the bounds as they were
    g2.commit_points_host(a)
    g2.rebuild_topology(len(a), 0.0, mode=gvx_mod.TOPO_FULL)
    g2.finish_topology(compute_bounds=False)
    assert g2.info()["obj_min"] == inf2["obj_min"] and g2.info()["obj_max"] == inf2["obj_max"]
