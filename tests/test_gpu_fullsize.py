"""GPU checks at the full sizes of the measured workloads, through properties
that hold at any size (the oracle finishes the small cases; these are too
large for it): determinism, exact linearity, mass conservation, containment
and monotone pools."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LOGDIM = (3, 3, 3, 3, 5)


def grid(gvx, channels):
    g = gvx.Grid(0)
    g.configure(LOGDIM)
    for c, t in channels:
        g.add_channel(c, t, 1)
    return g


def test_plain_small_trilinear_conserves_mass(gvx_mod):
    """100k points in 256^3: the trilinear weights of a point sum to its weight, and with topology
    radius 1 all eight voxels are interior voxels of active bricks"""
    import workloads

    pos, w = workloads.plain_small()
    g = grid(gvx_mod, ((0, gvx_mod.T_FLOAT),))
    g.commit_points_host(pos, weight=w)
    g.rebuild_topology(len(pos), 1.0, mode=gvx_mod.TOPO_FULL)
    g.update_atlas()
    g.insert_points(len(pos))
    g.splat(gvx_mod.SPLAT_TRILINEAR, len(pos), 1.0, chan_density=0)
    used = g.info()["used_leaves"]
    total = g.read_channel(0)[:used, 1:-1, 1:-1, 1:-1].astype(np.float64).sum()
    assert abs(total - float(w.sum())) <= 1e-6 * float(w.sum())


def test_sph_frame_determinism_linearity_containment(gvx_mod):
    """The 4M-point SPH frame: two runs give the same bytes; with one velocity u for every point the
    velocity channel is u times the density (the same weights, multiplied per term); every point's
    InsertPoints leaf holds it"""
    import torch
    import workloads

    pos, _ = workloads.sph_slab()
    n = len(pos)
    u = np.array([0.5, -2.0, 0.25], np.float32)  # powers of two: w*W*u is exact given w*W
    vel = np.broadcast_to(u, pos.shape).copy()
    g = grid(gvx_mod, ((0, gvx_mod.T_FLOAT), (1, gvx_mod.T_FLOAT3)))
    pd, vd = torch.from_numpy(pos).cuda(), torch.from_numpy(vel).cuda()
    g.set_points(n, pd, 0, 12, vd, 0, 12)
    g.rebuild_topology(n, 2.0, mode=gvx_mod.TOPO_FULL)
    g.update_atlas()
    pnode = g.insert_points(n, want_pnode=True)
    g.splat(gvx_mod.SPLAT_CUBIC, n, 2.0, chan_density=0, chan_vel=1)
    d1, v1 = g.read_channel(0), g.read_channel(1)
    g.splat(gvx_mod.SPLAT_CUBIC, n, 2.0, chan_density=0, chan_vel=1)
    assert np.array_equal(d1, g.read_channel(0)) and np.array_equal(v1, g.read_channel(1))
    for k in range(3):
        assert np.array_equal(v1[..., k], d1 * u[k]), k
    leaf = g.read_nodes(0)["pos"]
    inside = (pnode >= 0)
    assert inside.mean() > 0.999  # points with a negative jittered coordinate are dropped
    lp = leaf[pnode[inside]]
    assert np.array_equal(lp, (np.floor(pos[inside]).astype(np.int32) // 8) * 8)


def test_differentiable_splat_is_linear_in_weights(gvx_mod):
    """1M points, per-point weights and radii: doubling every weight doubles every voxel exactly"""
    import torch
    import workloads

    pos, w, r = workloads.differentiable()[:3]
    n = len(pos)
    g = grid(gvx_mod, ((0, gvx_mod.T_FLOAT),))
    pd = torch.from_numpy(pos).cuda()
    wd, rd = torch.from_numpy(w).cuda(), torch.from_numpy(r).cuda()
    g.set_points(n, pd)
    g.rebuild_topology(n, 1.5, mode=gvx_mod.TOPO_FULL)
    g.update_atlas()
    g.insert_points(n)
    g.set_point_attribs(weight=wd, radius=rd)
    g.splat(gvx_mod.SPLAT_CUBIC, n, 1.0, chan_density=0)
    a = g.read_channel(0)
    w2 = wd * 2
    g.set_point_attribs(weight=w2, radius=rd)
    g.splat(gvx_mod.SPLAT_CUBIC, n, 1.0, chan_density=0)
    assert np.array_equal(g.read_channel(0), 2 * a)


def test_fusion_frames_accumulate(gvx_mod):
    """30 depth frames: AccumulateTopology only appends leaves, and each frame's accumulating trilinear
    splat adds exactly that frame's mass"""
    import workloads

    g = grid(gvx_mod, ((0, gvx_mod.T_FLOAT),))
    prev_leaves = None
    mass = 0.0
    for pos, _ in workloads.depth_fusion(frames=30, seed=3):
        n = len(pos)
        g.commit_points_host(pos)
        g.rebuild_topology(n, 1.0, mode=gvx_mod.TOPO_ACCUMULATE)
        g.update_atlas()
        g.insert_points(n)
        g.splat(gvx_mod.SPLAT_TRILINEAR, n, 1.0, chan_density=0, accum=True)
        leaves = g.read_nodes(0)["pos"]
        if prev_leaves is not None:
            assert np.array_equal(leaves[:len(prev_leaves)], prev_leaves)
        prev_leaves = leaves
        mass += n
        used = g.info()["used_leaves"]
        total = g.read_channel(0)[:used, 1:-1, 1:-1, 1:-1].astype(np.float64).sum()
        assert abs(total - mass) <= 2e-6 * mass
