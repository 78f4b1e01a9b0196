"""CPU tests: the oracle against hand-worked answers derived from the reference
source (the reference itself ships no tests, fixtures or golden vectors)."""
import math

import numpy as np
import pytest

UNDEF64 = 0xFFFFFFFFFFFFFFFF


def two_points():
    return np.array([[10.5, 10.5, 10.5], [300.5, 200.5, 100.5]], np.float32)


def test_two_point_topology_r1(orc):
    o = orc.Oracle()
    o.add_channel(0, orc.T_FLOAT)
    assert o.rebuild_topology(two_points(), 1.0) == orc.OK
    # bbox (9..302, 9..202, 9..102) -> root at level 2 (range 512), VG.cpp:821-837
    assert o.root_level() == 2 and o.top_lev() == 2
    assert [o.num_nodes(l) for l in range(3)] == [3, 2, 1]
    n2, n1, n0 = o.nodes(2), o.nodes(1), o.nodes(0)
    assert n2["pos"].tolist() == [[0, 0, 0]]
    # level 1 in key order (x, y, z): PT.cuh:377-380 + sorted unique keys
    assert n1["pos"].tolist() == [[0, 0, 0], [256, 192, 64]]
    # leaves: the two containing leaves, then the extra leaf of the box
    # [int(p)-r, int(p)+2r] = y in [199, 202] (PT.cuh:481-482) appended after them
    assert n0["pos"].tolist() == [[8, 8, 8], [296, 200, 96], [296, 192, 96]]
    # parent references (pid << 16) | ((lev+1) << 8), ND.cuh:496
    assert n1["parent"].tolist() == [0x200, 0x200]
    assert n0["parent"].tolist() == [0x100, 0x10100, 0x10100]
    # child-list references Elem(1, lev, i), VG.cpp:1325 / AL.h:59
    assert n1["childlist"].tolist() == [0x101, 0x10101]
    assert n2["childlist"].tolist() == [0x201]
    root = o.childlist(2)
    assert {i: int(v) for i, v in enumerate(root) if v != UNDEF64} == {0: 0x100, 92: 0x10100}
    l1 = o.childlist(1).reshape(2, 512)
    assert {(n, i): int(l1[n, i]) for n in range(2) for i in range(512) if l1[n, i] != UNDEF64} == {
        (0, 73): 0x0, (1, 269): 0x10000, (1, 261): 0x20000}
    o.update_atlas()
    # atlas slot k -> (k mod 16, k/16 mod 16, k/256) * 10 + 1 (AL.cpp:705-715)
    assert o.nodes(0)["value"].tolist() == [[1, 1, 1], [11, 1, 1], [21, 1, 1]]
    amap = o.atlas_map()
    assert amap[:3].tolist() == [[8, 8, 8, 0], [296, 200, 96, 1], [296, 192, 96, 2]]
    assert (amap[3:] == -1).all()


def test_radius_below_one_has_no_extra_bricks(orc):
    o = orc.Oracle()
    assert o.rebuild_topology(two_points(), 0.5) == orc.OK
    assert o.num_nodes(0) == 2  # VG.cpp:1207: extra bricks only for radius >= 1


def test_negative_points_are_dropped(orc):
    o = orc.Oracle()
    pts = np.vstack([two_points(), [[-0.5, 5.0, 5.0]]]).astype(np.float32)
    assert o.rebuild_topology(pts, 0.0) == orc.OK
    # key lev 255 (PT.cuh:361-371): no leaf for the negative point
    assert o.nodes(0)["pos"].tolist() == [[8, 8, 8], [296, 200, 96]]


def test_single_point_is_degenerate(orc):
    # one point: every level below the root holds one node, so VDBInfo.top_lev
    # is level 0 and the reference descends from the wrong node (VG.cpp:3957-3968)
    o = orc.Oracle()
    st = o.rebuild_topology(np.array([[100.5, 37.25, 64.0]], np.float32), 0.0, allow_degenerate=True)
    assert st == orc.ERR_DEGENERATE


def test_trilinear_known_values(orc):
    o = orc.Oracle()
    o.add_channel(0, orc.T_FLOAT)
    pts = two_points()
    o.rebuild_topology(pts, 1.0)
    o.update_atlas()
    o.splat(orc.SPLAT_TRILINEAR, pts, 1.0, weight=np.array([1.0, 2.0], np.float32))
    d = o.read_channel(0)  # (slots, 10, 10, 10)
    # leaf 1 = (296,200,96): voxels 300..301, 200..201, 100..101 -> local 4..5, 0..1, 4..5 (+1 apron)
    blk = d[1]
    assert np.allclose(blk[5:7, 1:3, 5:7], 0.25)
    assert math.isclose(blk[1:9, 1:9, 1:9].sum(), 2.0)
    # leaf 0: 10.5 -> voxels 10,11 -> local 2,3
    assert np.allclose(d[0][3:5, 3:5, 3:5], 0.125)
    assert math.isclose(d[:, 1:9, 1:9, 1:9].sum(), 3.0)
    # the extra leaf (296,192,96) holds the y=200 voxels as +y apron copies (padded y = 9)
    assert np.array_equal(d[2][5:7, 9, 5:7], blk[5:7, 1, 5:7])


def test_cubic_known_values(orc):
    o = orc.Oracle()
    o.add_channel(0, orc.T_FLOAT)
    pts = np.array([[10.5, 10.5, 10.5], [300.0, 203.0, 100.0]], np.float32)
    o.rebuild_topology(pts, 2.0)
    o.update_atlas()
    o.splat(orc.SPLAT_CUBIC, pts, 2.0)
    leaves = o.nodes(0)["pos"].tolist()
    k = leaves.index([296, 200, 96])
    blk = o.read_channel(0)[k]
    c = (100 - 96 + 1, 203 - 200 + 1, 300 - 296 + 1)  # (z, y, x) padded
    inv_pi = 1.0 / math.pi
    assert math.isclose(blk[c], inv_pi, rel_tol=1e-12)                       # q = 0
    assert math.isclose(blk[c[0], c[1], c[2] + 1], 0.25 * inv_pi, rel_tol=1e-12)  # q = 1
    q = math.sqrt(2.0)
    assert math.isclose(blk[c[0], c[1] + 1, c[2] + 1], 0.25 * (2 - q) ** 3 * inv_pi, rel_tol=1e-12)
    assert blk[c[0], c[1], c[2] + 2] == 0.0                                  # q = 2


def test_ref_scatter_known_values(orc):
    o = orc.Oracle()
    o.add_channel(0, orc.T_FLOAT)
    pts = np.array([[10.5, 10.5, 10.5], [300.25, 200.5, 100.0]], np.float32)
    o.rebuild_topology(pts, 0.0)
    o.update_atlas()
    o.splat(orc.SPLAT_REF_SCATTER, pts, 1.0)
    blk = o.read_channel(0)[1]  # leaf (296,200,96): local p = (4.25, 0.5, 4.0), pi = (4, 0, 4)
    z, y, x = 4 + 1, 0 + 1, 4 + 1
    # distFunc (PT.cuh:516-523): (1 - d^2/r^2)^3, unclamped
    assert math.isclose(blk[z, y, x], (1 - 0.3125) ** 3, rel_tol=1e-12)
    assert math.isclose(blk[z, y, x - 1], (1 - 1.8125) ** 3, rel_tol=1e-12)
    assert math.isclose(blk[z, y - 1, x], (1 - 2.3125) ** 3, rel_tol=1e-12)  # the brick's own apron voxel


def test_gather_known_values(orc):
    o = orc.Oracle()
    o.add_channel(0, orc.T_FLOAT)
    pts = two_points()
    o.rebuild_topology(pts, 2.0)
    o.update_atlas()
    o.splat(orc.SPLAT_GATHER_DENSITY, pts, 1.0, subcell=4, radius_ins=2.0)
    leaves = o.nodes(0)["pos"].tolist()
    blk = o.read_channel(0)[leaves.index([296, 200, 96])]
    # GatherDensity (PT.cuh:721-726): max(0, R - |p - v|) at integer voxel positions
    assert math.isclose(blk[100 - 96 + 1, 1, 300 - 296 + 1], 1.0 - math.sqrt(0.75), rel_tol=1e-9)
    assert blk[100 - 96 + 1, 1, 299 - 296 + 1] == 0.0
    o.splat(orc.SPLAT_GATHER_LEVELSET, pts, 1.0, subcell=4, radius_ins=2.0)
    blk = o.read_channel(0)[leaves.index([296, 200, 96])]
    assert math.isclose(blk[100 - 96 + 1, 1, 300 - 296 + 1], math.sqrt(0.75) - 1.0, rel_tol=1e-9)


def test_gather_colour_and_entry_count(orc):
    o = orc.Oracle()
    o.add_channel(0, orc.T_FLOAT)
    o.add_channel(1, orc.T_UCHAR4)
    pts = np.array([[10.5, 10.5, 10.5], [100.5, 100.5, 100.5]], np.float32)
    clr = np.array([[200, 100, 50, 0], [10, 20, 30, 40]], np.uint8)
    o.rebuild_topology(pts, 0.0)
    o.update_atlas()
    # insertion radius 0: each point joins the one subcell [(int(p)/4)*4, (int(p+1)/4)*4] = [8, 8]
    n = o.gather(False, pts, 1.0, 0.0, subcell=4, chan=0, chan_clr=1, clr=clr)
    assert n == 2
    leaves = o.nodes(0)["pos"].tolist()
    c = o.read_channel(1)[leaves.index([8, 8, 8])]
    # (0,0,0,1) + clr/255 over one point, times 255, truncated and saturated (PT.cuh:724-732)
    assert c[1 + 2, 1 + 2, 1 + 2].tolist() == [200.0, 100.0, 50.0, 255.0]
    # a subcell with no point: 0/0 -> 0 for r,g,b and 1/0 -> 255 for alpha
    assert c[1 + 5, 1 + 5, 1 + 5].tolist() == [0.0, 0.0, 0.0, 255.0]


def test_apron_copies_neighbours_and_boundary(orc):
    o = orc.Oracle()
    o.add_channel(0, orc.T_FLOAT)
    pts = np.array([[10.5, 10.5, 10.5], [303.5, 200.5, 100.5], [304.5, 200.5, 100.5]], np.float32)
    o.rebuild_topology(pts, 0.0)
    o.update_atlas()
    o.splat(orc.SPLAT_TRILINEAR, pts, 1.0)
    o.update_apron(0, 7.0)
    leaves = o.nodes(0)["pos"].tolist()
    d = o.read_channel(0)
    a, b = d[leaves.index([296, 200, 96])], d[leaves.index([304, 200, 96])]
    # +x apron of brick a (padded x = 9) holds brick b's interior x = 0 (padded 1)
    assert np.array_equal(a[1:9, 1:9, 9], b[1:9, 1:9, 1])
    assert np.array_equal(b[1:9, 1:9, 0], a[1:9, 1:9, 8])
    # faces with no neighbouring brick take the boundary value
    assert (a[1:9, 1:9, 0] == 7.0).all() and (a[0, 1:9, 1:9] == 7.0).all()


def test_incremental_semantics(orc):
    base = np.array([[10.5, 10.5, 10.5], [300.5, 200.5, 100.5], [60.5, 40.5, 20.5]], np.float32)
    o = orc.Oracle()
    assert o.rebuild_topology(base, 0.0, mode=orc.TOPO_AUTO) == orc.OK
    assert o.last_mode() == 1
    # second call: mCurrDepth is still -1, so the reference rebuilds fully again (VG.cpp:1198-1203)
    assert o.rebuild_topology(base, 0.0, mode=orc.TOPO_AUTO) == orc.OK
    assert o.last_mode() == 1
    # third call with a subset: no new node -> markers are not applied (VG.cpp:1066)
    assert o.rebuild_topology(base[:2], 0.0, mode=orc.TOPO_AUTO) == orc.OK
    assert o.last_mode() == 0 and o.used_leaves() == 3
    # a new point in a new leaf: the leaf of point 3 loses its marker and is delinked
    moved = np.vstack([base[:2], [[120.5, 40.5, 20.5]]]).astype(np.float32)
    assert o.rebuild_topology(moved, 0.0, mode=orc.TOPO_AUTO) == orc.OK
    assert o.last_mode() == 2
    n0 = o.nodes(0)
    assert n0["pos"].tolist()[-1] == [120, 40, 16]
    flags = dict(zip(map(tuple, n0["pos"].tolist()), n0["flags"].tolist()))
    assert flags[(56, 40, 16)] == 0 and flags[(120, 40, 16)] == 1
    assert n0["parent"][[p.tolist() for p in n0["pos"]].index([56, 40, 16])] == UNDEF64
    assert o.used_leaves() == 3


def test_accumulate_keeps_leaves(orc):
    base = np.array([[10.5, 10.5, 10.5], [300.5, 200.5, 100.5], [60.5, 40.5, 20.5]], np.float32)
    o = orc.Oracle()
    o.rebuild_topology(base, 0.0, mode=orc.TOPO_ACCUMULATE)
    more = np.vstack([base[:2], [[120.5, 40.5, 20.5]]]).astype(np.float32)
    assert o.rebuild_topology(more, 0.0, mode=orc.TOPO_ACCUMULATE) == orc.OK
    assert o.last_mode() == 2 and o.used_leaves() == 4


def test_cpu_activate_space_leaf_set(orc):
    rng = np.random.default_rng(5)
    pts = (rng.random((3000, 3)) * 200.0 + 3.0).astype(np.float32)
    leaves, root = orc.activate_space_cpu(pts)
    o = orc.Oracle()
    o.rebuild_topology(pts, 0.0)
    a = {tuple(x) for x in leaves.tolist()}
    b = {tuple(x) for x in o.nodes(0)["pos"].tolist()}
    assert a == b
    assert root == o.root_level()


def _atlas_dense(bricks, sub):
    """brick-major (slots, P, P, P) -> the atlas as (Z, Y, X)"""
    P = bricks.shape[1]
    sx, sy, sz = sub
    return bricks.reshape(sz, sy, sx, P, P, P).transpose(0, 3, 1, 4, 2, 5).reshape(sz * P, sy * P, sx * P)


@pytest.mark.parametrize("skip", [True, False])
def test_compute_smooth_known_values(orc, skip):
    o = orc.Oracle()
    o.add_channel(0, orc.T_FLOAT)
    assert o.rebuild_topology(two_points(), 1.0) == orc.OK
    o.update_atlas()
    P = 10
    nslots = int(np.prod(o.atlas_subdim()))
    data = np.random.default_rng(3).integers(-64, 64, (nslots, P, P, P)) / 8.0
    o.write_channel(0, data)
    p1, p2 = 4.0, 0.25
    o.compute(orc.FUNC_SMOOTH, 0, 1, (p1, p2, 0.0), update_apron=False, skip_over_aprons=skip)
    # gvdbOpSmooth (OP.cuh:383-400): every brick interior voxel, whatever skipOverAprons
    d = data
    nb = (d[:, 1:-1, 1:-1, :-2] + d[:, 1:-1, 1:-1, 2:] + d[:, 1:-1, :-2, 1:-1] + d[:, 1:-1, 2:, 1:-1] +
          d[:, :-2, 1:-1, 1:-1] + d[:, 2:, 1:-1, 1:-1])
    want = data.copy()
    want[:, 1:-1, 1:-1, 1:-1] = (p1 * d[:, 1:-1, 1:-1, 1:-1] + nb) / (p1 + 6.0) + p2
    np.testing.assert_allclose(o.read_channel(0), want, rtol=0, atol=1e-12)


def test_compute_smooth_then_apron(orc):
    o = orc.Oracle()
    o.add_channel(0, orc.T_FLOAT)
    assert o.rebuild_topology(two_points(), 1.0) == orc.OK
    o.update_atlas()
    data = np.zeros((int(np.prod(o.atlas_subdim())), 10, 10, 10))
    data[0, 1:-1, 1:-1, 1:-1] = 1.0
    o.write_channel(0, data)
    o.compute(orc.FUNC_SMOOTH, 0, 2, (4.0, 0.0, 0.0), update_apron=True, skip_over_aprons=True, boundval=3.0)
    got = o.read_channel(0)
    # leaf 0 has no active neighbours: after each iteration its apron holds boundval 3
    assert got[0, 0, 5, 5] == 3.0 and got[0, 9, 9, 9] == 3.0
    # first iteration reads apron 0s: a corner interior voxel has 3 interior neighbours,
    # (4 + 3) / 10 = 0.7; the second reads the apron's 3s
    c1 = np.zeros((10, 10, 10))
    c1[1:-1, 1:-1, 1:-1] = 1.0
    it1 = c1.copy()
    it1[1:-1, 1:-1, 1:-1] = (4 * c1[1:-1, 1:-1, 1:-1] + c1[1:-1, 1:-1, :-2] + c1[1:-1, 1:-1, 2:] +
                             c1[1:-1, :-2, 1:-1] + c1[1:-1, 2:, 1:-1] + c1[:-2, 1:-1, 1:-1] + c1[2:, 1:-1, 1:-1]) / 10
    assert math.isclose(it1[1, 1, 1], 0.7)
    it1[0, :, :] = it1[-1, :, :] = it1[:, 0, :] = it1[:, -1, :] = it1[:, :, 0] = it1[:, :, -1] = 3.0
    it2 = it1.copy()
    it2[1:-1, 1:-1, 1:-1] = (4 * it1[1:-1, 1:-1, 1:-1] + it1[1:-1, 1:-1, :-2] + it1[1:-1, 1:-1, 2:] +
                             it1[1:-1, :-2, 1:-1] + it1[1:-1, 2:, 1:-1] + it1[:-2, 1:-1, 1:-1] + it1[2:, 1:-1, 1:-1]) / 10
    np.testing.assert_allclose(got[0, 1:-1, 1:-1, 1:-1], it2[1:-1, 1:-1, 1:-1], rtol=0, atol=1e-12)


@pytest.mark.parametrize("skip", [False, True])
def test_compute_fill_region(orc, skip):
    o = orc.Oracle()
    o.add_channel(0, orc.T_FLOAT)
    assert o.rebuild_topology(two_points(), 1.0) == orc.OK
    o.update_atlas()
    sub = o.atlas_subdim()
    assert sub == (16, 16, 1)
    o.compute(orc.FUNC_FILL_F, 0, 1, (2.5, 0.0, 0.0), update_apron=False, skip_over_aprons=skip)
    dense = _atlas_dense(o.read_channel(0), sub)
    # GVDB_VOXUNPACKED (OP.cuh:220-223): voxel blockIdx*8 + threadIdx + 1 over 8^3 blocks covering
    # getAtlasRes (160, 160, 10) or, skipping aprons, getAtlasPackres (128, 128, 8)
    hi = (129, 129, 9) if skip else (160, 160, 10)
    want = np.zeros_like(dense)
    want[1:hi[2], 1:hi[1], 1:hi[0]] = 2.5
    assert np.array_equal(dense, want)


def test_compute_fill_pattern_and_colours(orc):
    o = orc.Oracle()
    o.add_channel(0, orc.T_FLOAT)
    o.add_channel(1, orc.T_UCHAR4)
    o.add_channel(2, orc.T_UCHAR)
    assert o.rebuild_topology(two_points(), 1.0) == orc.OK
    o.update_atlas()
    sub = o.atlas_subdim()
    o.compute(orc.FUNC_FILL_F, 0, 1, (0.0, 0.0, -1.0), update_apron=False, skip_over_aprons=False)
    dense = _atlas_dense(o.read_channel(0), sub)
    s = lambda i: math.sin(i * 12 / (math.pi * 30.0))  # noqa: E731  (3.141592 in the reference)
    assert math.isclose(dense[3, 7, 11], s(11) + s(7) + s(3), abs_tol=1e-5)
    # CLR2INT (OP.cuh:20): 255 * (0.5, 1, 2, 1) truncated and ORed unmasked: the 510 of blue
    # spills into alpha's byte
    o.compute(orc.FUNC_FILL_C4, 1, 1, (0.5, 1.0, 2.0), update_apron=False, skip_over_aprons=False)
    c = o.read_channel(1)
    assert c[0, 1, 1, 1].tolist() == [127, 255, 254, 255]
    assert c[0, 0, 0, 0].tolist() == [0, 0, 0, 0]
    for p1, want in ((7.9, 7), (300.0, 255), (-3.0, 0)):
        o.compute(orc.FUNC_FILL_C, 2, 1, (p1, 0.0, 0.0), update_apron=False, skip_over_aprons=False)
        assert o.read_channel(2)[0, 1, 1, 1] == want


def test_fp16_gather_known_values(orc):
    """InsertPointsSubcell_FP16 + GatherLevelSet_FP16 (PT.cuh:154-216, 775-813): the point comes back
    as q / 65535 * range + min with q = trunc((w - min) / range * 65535), each a float32 step"""
    pos = np.array([[10.3, 11.7, 12.2], [13.9, 9.1, 10.6], [300.5, 200.5, 100.5]], np.float32)
    o = orc.Oracle()
    o.add_channel(0, orc.T_FLOAT)
    assert o.rebuild_topology(pos, 1.0) == orc.OK
    o.update_atlas()
    lo, hi = o.pos_bounds()
    # GetBoundingBox (VG.cpp:5452-5462): min - 1 and max + 2, clamped at 0
    f32 = np.float32
    assert lo.tolist() == [f32(10.3) - f32(1), f32(9.1) - f32(1), f32(10.6) - f32(1)]
    assert hi.tolist() == [f32(300.5) + f32(2), f32(200.5) + f32(2), f32(100.5) + f32(2)]
    n_sc = o.gather_fp16(pos, 1.0, 1.0, subcell=4, chan=0)
    assert n_sc > 0
    f = np.float32
    rng = (hi - lo).astype(f)
    q = np.floor(((pos - lo).astype(f) / rng).astype(f) * f(65535)).astype(np.uint16)
    back = ((q.astype(f) / f(65535)).astype(f) * rng).astype(f) + lo
    ch = o.read_channel(0)
    leaf = o.nodes(0)
    # the voxel (12, 10, 11) lies in leaf (8, 8, 8), slot 0: the two first points are listed in its subcell
    assert leaf["pos"][0].tolist() == [8, 8, 8]
    v = np.array([12, 10, 11], f)
    d = (back[:2] - v).astype(f)
    s2 = (d[:, 0] * d[:, 0]).astype(f)
    s2 = (s2 + (d[:, 1] * d[:, 1]).astype(f)).astype(f)
    s2 = (s2 + (d[:, 2] * d[:, 2]).astype(f)).astype(f)
    want = min(f(3.0), *(np.sqrt(s2).astype(f) - f(1.0)))
    assert ch[0, 1 + 3, 1 + 2, 1 + 4] == want  # local (4, 2, 3), padded, stored [z][y][x]
    # a voxel no listed point reaches keeps 3
    assert ch[0, 1 + 0, 1 + 7, 1 + 7] == 3.0


def test_scatter_colours(orc):
    """ScatterDensity with point colours (PT.cuh:555-571, 610-642)"""
    pos = np.array([[10.2, 10.2, 10.2], [10.7, 10.4, 10.9], [10.5, 10.5, 10.1], [20.5, 10.5, 10.5]], np.float32)
    clr = np.array([[10, 20, 30, 40], [20, 40, 61, 50], [0, 0, 0, 0], [7, 8, 9, 10]], np.uint8)
    o = orc.Oracle()
    o.add_channel(0, orc.T_FLOAT)
    o.add_channel(1, orc.T_UCHAR4)
    o.add_channel(3, orc.T_UCHAR4)
    assert o.rebuild_topology(pos, 0.0) == orc.OK
    o.update_atlas()
    o.scatter_density(pos, 1.5, clr=clr, avg_color=False)
    c3 = o.read_channel(3)
    # voxel (10, 10, 10) of leaf (8, 8, 8): the three first points race; the highest index wins
    assert c3[0, 1 + 2, 1 + 2, 1 + 2].tolist() == [0, 0, 0, 0]
    assert c3[1, 1 + 2, 1 + 2, 1 + 4].tolist() == [7, 8, 9, 10]
    o.clear_channel(0)
    o.scatter_density(pos, 1.5, clr=clr, avg_color=True)
    c1 = o.read_channel(1)
    # integer means (10+20+0)/3, (20+40+0)/3, (30+61+0)/3, alpha 255
    assert c1[0, 1 + 2, 1 + 2, 1 + 2].tolist() == [10, 20, 30, 255]
    # after an avgColor call the colour buffer exists: a plain call then writes no colour
    o.clear_channel(3)
    o.scatter_density(pos, 1.5, clr=clr, avg_color=False)
    assert not o.read_channel(3).any()


def test_convert_and_transform_known_values(orc):
    src = np.array([[0, 65535, 1000], [7, 8, 9]], np.uint16)
    out = orc.convert_and_transform(src, 2, wmin=(-1.0, 0.0, 2.0), wdelta=(0.5, 2.0 ** -16, 1.0),
                                    trans=(1.0, 0.25, -3.0), scal=(2.0, 4.0, 0.5))
    assert out.tolist() == [[-1.0, 65535 * 2.0 ** -14 + 0.25, 498.0], [6.0, 8 * 2.0 ** -14 + 0.25, 2.5]]
    f = np.array([[1.5, -2.0, 3.25]], np.float32)
    assert orc.convert_and_transform(f, 4, (0, 0, 0), (1, 1, 1)).tolist() == [[1.5, -2.0, 3.25]]


def test_cpu_tree_known_answer(orc):
    """ActivateSpace (VG.cpp:2805-2855) from an empty tree: the first point's leaf is the root,
    the second point Reparents to the level-2 node covering both (VG.cpp:2726-2763); the old
    root comes back as a child through the stop-node path"""
    t = orc.CpuTree()
    t.activate(two_points())
    assert t.root() == 0x200  # Elem(0, 2, 0)
    n0, n1, n2 = t.nodes(0), t.nodes(1), t.nodes(2)
    assert n0["pos"].tolist() == [[8, 8, 8], [296, 200, 96]]
    assert n1["pos"].tolist() == [[0, 0, 0], [256, 192, 64]]
    assert n2["pos"].tolist() == [[0, 0, 0]]
    assert (n0["flags"] == 1).all() and (n0["value"] == -1).all()
    assert n0["parent"].tolist() == [0x100, 0x10100] and n1["parent"].tolist() == [0x200, 0x200]
    assert n2["parent"].tolist() == [0xFFFFFFFF]
    assert n1["childlist"].tolist() == [0x101, 0x10101] and n2["childlist"].tolist() == [0x201]
    assert n0["childlist"].tolist() == [0xFFFFFFFF, 0xFFFFFFFF]
    l1 = t.childlist(1).reshape(2, 512)
    assert {(n, i): int(l1[n, i]) for n in range(2) for i in range(512) if l1[n, i] != UNDEF64} == {
        (0, 73): 0x0, (1, 269): 0x10000}
    root = t.childlist(2)
    assert {i: int(v) for i, v in enumerate(root) if v != UNDEF64} == {0: 0x100, 92: 0x10100}
    # a point in an existing leaf adds nothing
    t.activate(np.array([[9.9, 12.0, 15.5]], np.float32))
    assert len(t.nodes(0)) == 2


def test_compute_bounds_known_answers(orc):
    """ComputeBounds (VG.cpp:1792-1816) on the two-point tree: leaves at
    (8,8,8), (296,200,96), (296,192,96), range 8 -> min (8,8,8), max
    (304,208,104); mVoxResMax is sticky while mVoxRes follows the last tree."""
    o = orc.Oracle()
    o.add_channel(0, orc.T_FLOAT)
    assert o.rebuild_topology(two_points(), 1.0) == orc.OK
    vmin, vmax, vres, vres_max = o.compute_bounds()
    assert vmin.tolist() == [8, 8, 8] and vmax.tolist() == [304, 208, 104]
    assert vres.tolist() == [296, 200, 96] and vres_max.tolist() == [296, 200, 96]
    small = np.array([[10.5, 10.5, 10.5], [20.5, 10.5, 10.5]], np.float32)
    assert o.rebuild_topology(small, 0.0, mode=orc.TOPO_FULL) == orc.OK
    vmin, vmax, vres, vres_max = o.compute_bounds()
    assert vmin.tolist() == [8, 8, 8] and vmax.tolist() == [24, 16, 16]
    assert vres.tolist() == [16, 8, 8] and vres_max.tolist() == [296, 200, 96]
