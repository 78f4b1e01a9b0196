"""GPU tests of gvx_batch_frame: whole frames of a batch of grids -- full
RebuildTopology, UpdateAtlas, InsertPoints and the batched splat -- unplanned
on the first frame, then planned builds without host waits, then one captured
CUDA graph replayed; every frame gives every grid the pools, child lists,
atlas map and splatted bricks of its own one-by-one calls, bit for bit, and a
cloud that leaves its plan is built again without it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LOGDIM = (3, 3, 3, 3, 5)


def clouds(count, seed, nmin=2_000, nmax=60_000):
    import workloads

    return workloads.batched_clouds(count=count, seed=seed, nmin=nmin, nmax=nmax)


def reference(gvx, p, w, topo_radius, mode, radius):
    """one grid built and splatted by the one-by-one calls"""
    g = gvx.Grid(0)
    g.configure(LOGDIM)
    g.add_channel(0, gvx.T_FLOAT, 1)
    g.commit_points_host(p, weight=w)
    g.rebuild_topology(len(p), topo_radius, mode=gvx.TOPO_FULL)
    g.update_atlas()
    g.insert_points(len(p))
    g.splat(mode, len(p), radius, chan_density=0)
    out = snapshot(g)
    g.close()
    return out


def snapshot(g):
    inf = g.info()
    used = inf["used_leaves"]
    amap = g.read_atlas_map()
    assert (amap[used:] == -1).all()
    return {"root": inf["root_level"], "used": used,
            "nodes": [g.read_nodes(l) for l in range(inf["root_level"] + 1)],
            "clist": [g.read_childlist(l) for l in range(1, inf["root_level"] + 1)],
            "amap": amap[:used].copy(), "den": g.read_channel(0)[:used].copy()}


def assert_same(a, b):
    assert a["root"] == b["root"] and a["used"] == b["used"]
    for x, y in zip(a["nodes"], b["nodes"]):
        assert np.array_equal(x, y)
    for x, y in zip(a["clist"], b["clist"]):
        assert np.array_equal(x, y)
    assert np.array_equal(a["amap"], b["amap"])
    assert np.array_equal(a["den"], b["den"])


def frame_grids(gvx, torch, cl):
    grids, keep = [], []
    for p, w in cl:
        g = gvx.Grid(0)  # its own stream
        g.configure(LOGDIM)
        g.add_channel(0, gvx.T_FLOAT, 1)
        pd, wd = torch.from_numpy(p).cuda(), torch.from_numpy(w).cuda()
        keep.append((pd, wd))
        g.set_points(len(p), pd)
        g.set_point_attribs(weight=wd)
        grids.append(g)
    return grids, keep


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("mode", ["trilinear", "cubic"])
def test_frames_match_per_grid_calls(gvx_mod, graph, mode):
    torch = pytest.importorskip("torch")
    m = gvx_mod.SPLAT_TRILINEAR if mode == "trilinear" else gvx_mod.SPLAT_CUBIC
    radius = 1.0 if mode == "trilinear" else 2.0
    cl = clouds(9, 11)
    refs = [reference(gvx_mod, p, w, 1.0, m, radius) for p, w in cl]
    grids, keep = frame_grids(gvx_mod, torch, cl)
    b = gvx_mod.Batch(0)
    b.set_grids(grids)
    paths = []
    for f in range(4):
        for g in grids:
            g.fill_channel(0, [9.0])
        b.frame(1.0, m, radius, graph=graph)
        paths.append(b.frame_path())
        for g, r in zip(grids, refs):
            assert_same(snapshot(g), r)
    assert paths == ([(0, 0), (1, 0), (2, 0), (2, 0)] if graph else [(0, 0), (1, 0), (1, 0), (1, 0)])
    # the grids stay usable by the one-by-one calls after planned frames
    for g, (p, _), r in zip(grids, cl, refs):
        g.fill_channel(0, [9.0])
        g.splat(m, len(p), radius, chan_density=0)
        assert np.array_equal(g.read_channel(0)[:r["used"]], r["den"])
    b.close()
    for g in grids:
        g.close()


def test_cloud_leaving_its_plan_is_built_again(gvx_mod):
    """points changed in place (same buffers, same count): a cloud moved out of its plan's root
    or key space, then a cloud refilled uniformly inside its own box (more bricks than its pools'
    capacities when the filled cloud needs more than count + 25% + 64 leaves); the grids whose plan
    failed are built again without it, the others replay under theirs, and every grid matches its
    one-by-one build"""
    torch = pytest.importorskip("torch")
    cl = clouds(6, 3)
    grids, keep = frame_grids(gvx_mod, torch, cl)
    b = gvx_mod.Batch(0)
    b.set_grids(grids)
    tri = gvx_mod.SPLAT_TRILINEAR
    for _ in range(3):
        b.frame(1.0, tri, 1.0)
    assert b.frame_path() == (2, 0)
    pts = [p.copy() for p, _ in cl]

    def check():
        for g, p, (_, w) in zip(grids, pts, cl):
            assert_same(snapshot(g), reference(gvx_mod, p, w, 1.0, tri, 1.0))

    # moved by 4096 voxels along x: a root of level <= 3 moves, a level-4 root's key space (the
    # cloud's extent of at most 128 leaves, widened and rounded up to a power of two) is left
    pts[1] = pts[1] + np.array([4096.0, 0.0, 0.0], np.float32)
    keep[1][0].copy_(torch.from_numpy(pts[1]))
    torch.cuda.synchronize()
    b.frame(1.0, tri, 1.0)
    assert b.frame_path() == (2, 1)
    check()
    # planned anew: the next frames run planned, then from a new graph
    b.frame(1.0, tri, 1.0)
    assert b.frame_path() == (1, 0)
    b.frame(1.0, tri, 1.0)
    assert b.frame_path() == (2, 0)
    check()
    # the largest cloud refilled uniformly inside its box
    k = int(np.argmax([len(p) for p in pts]))
    used0, root0 = grids[k].info()["used_leaves"], grids[k].info()["root_level"]
    lo, hi = pts[k].min(axis=0), pts[k].max(axis=0)
    rng = np.random.default_rng(5)
    pts[k] = (lo + rng.random(pts[k].shape) * (hi - lo)).astype(np.float32)
    keep[k][0].copy_(torch.from_numpy(pts[k]))
    torch.cuda.synchronize()
    b.frame(1.0, tri, 1.0)
    r = reference(gvx_mod, pts[k], cl[k][1], 1.0, tri, 1.0)
    assert b.frame_path() == (2, 1 if r["used"] > used0 + used0 // 4 + 64 or r["root"] != root0 else 0)
    check()
    b.close()
    for g in grids:
        g.close()


@pytest.mark.parametrize("vel", [False, True])
def test_replayed_frames_follow_moving_points(gvx_mod, vel):
    """points jittered in place every frame (the plans hold, the graph replays): every frame's
    pools, atlas map and bricks are those of one-by-one builds of that frame's points -- a replay
    recomputes everything from the points it reads"""
    torch = pytest.importorskip("torch")
    cl = clouds(5, 17)
    rng = np.random.default_rng(3)
    mode = gvx_mod.SPLAT_CUBIC if vel else gvx_mod.SPLAT_TRILINEAR
    radius = 2.0 if vel else 1.0
    cv = 1 if vel else -1
    grids, keep, vels = [], [], []
    for p, w in cl:
        g = gvx_mod.Grid(0)
        g.configure(LOGDIM)
        g.add_channel(0, gvx_mod.T_FLOAT, 1)
        if vel:
            g.add_channel(1, gvx_mod.T_FLOAT3, 1)
        v = rng.normal(0, 1, p.shape).astype(np.float32)
        pd, wd, vd = torch.from_numpy(p).cuda(), torch.from_numpy(w).cuda(), torch.from_numpy(v).cuda()
        keep.append((pd, wd, vd))
        vels.append(v)
        g.set_points(len(p), pd, vel=vd if vel else None)
        g.set_point_attribs(weight=wd)
        grids.append(g)
    b = gvx_mod.Batch(0)
    b.set_grids(grids)
    pts = [p.copy() for p, _ in cl]
    paths = []
    for f in range(5):
        for k in range(len(pts)):
            pts[k] = (pts[k] + rng.normal(0, 0.4, pts[k].shape)).astype(np.float32)
            keep[k][0].copy_(torch.from_numpy(pts[k]))
        torch.cuda.synchronize()
        b.frame(1.0, mode, radius, chan_vel=cv)
        paths.append(b.frame_path())
        for g, p, (_, w), v in zip(grids, pts, cl, vels):
            r = gvx_mod.Grid(0)
            r.configure(LOGDIM)
            r.add_channel(0, gvx_mod.T_FLOAT, 1)
            if vel:
                r.add_channel(1, gvx_mod.T_FLOAT3, 1)
            r.commit_points_host(p, vel=v if vel else None, weight=w)
            r.rebuild_topology(len(p), 1.0, mode=gvx_mod.TOPO_FULL)
            r.update_atlas()
            r.insert_points(len(p))
            r.splat(mode, len(p), radius, chan_density=0, chan_vel=cv)
            assert_same(snapshot(g), snapshot(r))
            if vel:
                u = g.info()["used_leaves"]
                assert np.array_equal(g.read_channel(1)[:u], r.read_channel(1)[:u])
            r.close()
    # unplanned, planned, then replays (a plan outgrown by the jitter would rebuild its grid and
    # the frame after it would run planned again)
    assert paths[0] == (0, 0) and paths[1][0] == 1 and sum(p[0] == 2 for p in paths[2:]) >= 2
    b.close()
    for g in grids:
        g.close()


def test_bad_point_in_a_planned_frame(gvx_mod):
    """a NaN position written in place into a replayed frame's points: the frame reports
    GVX_ERR_INVALID_ARG (the device error word, as an unplanned build reports it), and once the
    point is fixed the next frame builds again from scratch and matches one-by-one builds"""
    torch = pytest.importorskip("torch")
    cl = clouds(3, 21)
    grids, keep = frame_grids(gvx_mod, torch, cl)
    b = gvx_mod.Batch(0)
    b.set_grids(grids)
    tri = gvx_mod.SPLAT_TRILINEAR
    for _ in range(3):
        b.frame(1.0, tri, 1.0)
    assert b.frame_path() == (2, 0)
    saved = keep[1][0][7].clone()
    keep[1][0][7, 0] = float("nan")
    torch.cuda.synchronize()
    with pytest.raises(gvx_mod.GvxError) as e:
        b.frame(1.0, tri, 1.0)
    assert e.value.status == 1 and "grid 1" in str(e.value)  # GVX_ERR_INVALID_ARG
    keep[1][0][7] = saved
    torch.cuda.synchronize()
    b.frame(1.0, tri, 1.0)
    assert b.frame_path()[0] == 0
    for g, (p, w) in zip(grids, cl):
        assert_same(snapshot(g), reference(gvx_mod, p, w, 1.0, tri, 1.0))
    b.close()
    for g in grids:
        g.close()
