"""GPU parity tests: libgvx (through the C ABI) against the oracle on the same
seeded inputs.  Topology, pools, child lists and the atlas map must be
bit-exact; FP32 densities must be within DENSITY_TOL of the FP64 oracle."""
import numpy as np
import pytest

from parity_util import DENSITY_TOL, compare_topology, rel_error, rel_error_significant

pytestmark = pytest.mark.gpu

LOGDIM = (3, 3, 3, 3, 5)


def make_pair(gvx, orc, pos, radius, weight=None, vel=None, radius_pp=None, channels=((0, 3),), logdim=LOGDIM,
              orig=(0, 0, 0)):
    g = gvx.Grid(0)
    g.configure(logdim)
    o = orc.Oracle(logdim)
    for c, t in channels:
        g.add_channel(c, t, 1)
        o.add_channel(c, t)
    g.commit_points_host(pos, vel=vel, weight=weight, radius=radius_pp)
    g.rebuild_topology(len(pos), radius, orig=orig, mode=gvx.TOPO_FULL)
    g.finish_topology()
    g.update_atlas()
    assert o.rebuild_topology(pos, radius, orig=orig) == orc.OK
    o.update_atlas()
    return g, o


@pytest.fixture(scope="module")
def c1():
    import workloads

    return workloads.plain_small()


@pytest.mark.parametrize("radius", [0.0, 1.0, 2.0, 3.0])
def test_topology_plain_small(gvx_mod, orc, c1, radius):
    pos, w = c1
    g, o = make_pair(gvx_mod, orc, pos, radius)
    compare_topology(g, o)
    assert np.array_equal(g.read_atlas_map(), o.atlas_map())
    assert g.info()["atlas_subdim"] == list(o.atlas_subdim())


@pytest.mark.parametrize("logdim", [(3, 3, 3, 3, 4), (2, 3, 3, 3, 3), (4, 4, 3, 3, 3), (3, 4, 5, 5, 5)])
def test_topology_other_configs(gvx_mod, orc, logdim):
    rng = np.random.default_rng(11)
    pos = (rng.random((30_000, 3)) * np.array([700.0, 300.0, 900.0])).astype(np.float32)
    g, o = make_pair(gvx_mod, orc, pos, 1.0, logdim=logdim)
    compare_topology(g, o)


def test_topology_with_origin_and_negative_points(gvx_mod, orc):
    rng = np.random.default_rng(4)
    pos = (rng.normal(60.0, 40.0, (20_000, 3))).astype(np.float32)  # some coordinates < 0 after orig
    orig = (5.0, -3.0, 2.5)
    g, o = make_pair(gvx_mod, orc, pos, 1.0, orig=orig)
    compare_topology(g, o)


def test_topology_is_deterministic(gvx_mod, orc, c1):
    pos, _ = c1
    g, _o = make_pair(gvx_mod, orc, pos, 1.0)
    a = [g.read_nodes(l) for l in range(3)]
    g.rebuild_topology(len(pos), 1.0, mode=gvx_mod.TOPO_FULL)
    g.update_atlas()
    b = [g.read_nodes(l) for l in range(3)]
    for x, y in zip(a, b):
        assert x.tobytes() == y.tobytes()


def test_trilinear_plain_small(gvx_mod, orc, c1):
    pos, w = c1
    g, o = make_pair(gvx_mod, orc, pos, 1.0, weight=w)
    g.splat(gvx_mod.SPLAT_TRILINEAR, len(pos), 1.0, chan_density=0)
    o.splat(orc.SPLAT_TRILINEAR, pos, 1.0, weight=w)
    got, ref = g.read_channel(0), o.read_channel(0)
    assert got.shape == ref.shape
    assert rel_error(got, ref) <= DENSITY_TOL
    interior = got[:, 1:-1, 1:-1, 1:-1].astype(np.float64)  # aprons hold copies of neighbours
    assert abs(float(interior.sum()) - float(w.sum())) <= 1e-5 * float(w.sum())


def test_cubic_with_velocity(gvx_mod, orc):
    rng = np.random.default_rng(2)
    pos = (rng.random((60_000, 3)) * np.array([128.0, 96.0, 160.0]) + 2.0).astype(np.float32)
    vel = rng.normal(0, 1, (60_000, 3)).astype(np.float32)
    g, o = make_pair(gvx_mod, orc, pos, 2.0, vel=vel, channels=((0, 3), (1, 4)))
    g.splat(gvx_mod.SPLAT_CUBIC, len(pos), 2.0, chan_density=0, chan_vel=1)
    o.splat(orc.SPLAT_CUBIC, pos, 2.0, vel=vel, chan_vel=1)
    d, dr = g.read_channel(0), o.read_channel(0)
    assert rel_error(d, dr) <= DENSITY_TOL
    v, vr = g.read_channel(1), o.read_channel(1)
    assert rel_error_significant(v[..., :3], vr[..., :3]) <= 1e-4
    assert np.abs(v[..., :3] - vr[..., :3]).max() <= 1e-5 * np.abs(vr).max()


def test_cubic_per_point_radius_and_weight(gvx_mod, orc):
    import workloads

    pos, w, r = workloads.differentiable(n=40_000, seed=3, lo=8.0, hi=120.0)
    g, o = make_pair(gvx_mod, orc, pos, 3.0, weight=w, radius_pp=r)
    g.splat(gvx_mod.SPLAT_CUBIC, len(pos), 0.0, chan_density=0)
    o.splat(orc.SPLAT_CUBIC, pos, 0.0, weight=w, radius_pp=r)
    assert rel_error(g.read_channel(0), o.read_channel(0)) <= DENSITY_TOL


def test_apron_after_trilinear(gvx_mod, orc, c1):
    pos, w = c1
    g, o = make_pair(gvx_mod, orc, pos, 1.0, weight=w)
    g.splat(gvx_mod.SPLAT_TRILINEAR, len(pos), 1.0, chan_density=0)
    o.splat(orc.SPLAT_TRILINEAR, pos, 1.0, weight=w)
    g.update_apron(0, 0.5)
    o.update_apron(0, 0.5)
    got, ref = g.read_channel(0), o.read_channel(0)
    assert rel_error(got, ref) <= DENSITY_TOL
    # the apron is a copy: bit-exact against the device's own interior values
    P = got.shape[1]
    amap = g.read_atlas_map()
    used = g.info()["used_leaves"]
    lut = {tuple(amap[s, :3]): s for s in range(used)}
    s = 0
    nb = lut.get((amap[s, 0] + 8, amap[s, 1], amap[s, 2]))
    if nb is not None:
        assert np.array_equal(got[s][1:P - 1, 1:P - 1, P - 1], got[nb][1:P - 1, 1:P - 1, 1])


def test_apron_float3_channel(gvx_mod, orc):
    rng = np.random.default_rng(9)
    pos = (rng.random((20_000, 3)) * 90.0 + 1.0).astype(np.float32)
    vel = rng.normal(0, 1, (20_000, 3)).astype(np.float32)
    g, o = make_pair(gvx_mod, orc, pos, 1.0, vel=vel, channels=((0, 3), (1, 4)))
    g.splat(gvx_mod.SPLAT_TRILINEAR, len(pos), 1.0, chan_density=0, chan_vel=1)
    o.splat(orc.SPLAT_TRILINEAR, pos, 1.0, vel=vel, chan_vel=1)
    g.update_apron(1, -1.0)
    o.update_apron(1, -1.0)
    v, vr = g.read_channel(1), o.read_channel(1)
    assert np.abs(v[..., :3] - vr[..., :3]).max() <= 1e-5 * np.abs(vr).max()


def test_ref_scatter(gvx_mod, orc, c1):
    pos, _ = c1
    g, o = make_pair(gvx_mod, orc, pos, 0.0)
    g.clear_channel(0)
    g.scatter_density(len(pos), 1.5, 1.0, expand=True)
    o.splat(orc.SPLAT_REF_SCATTER, pos, 1.5, expand=True)
    got, ref = g.read_channel(0).astype(np.float64), o.read_channel(0)
    # the unclamped (1 - d^2/r^2)^3 is negative off-centre, so voxel sums cancel;
    # the FP32 error is judged against the largest magnitude: max|a-b| <= 1e-6 max|b|
    assert np.abs(got - ref).max() <= 1e-6 * np.abs(ref).max()
    assert rel_error_significant(got, ref, frac=1e-2) <= DENSITY_TOL


def test_accumulate_adds(gvx_mod, orc, c1):
    pos, w = c1
    g, o = make_pair(gvx_mod, orc, pos, 1.0, weight=w)
    g.splat(gvx_mod.SPLAT_TRILINEAR, len(pos), 1.0, chan_density=0)
    g.splat(gvx_mod.SPLAT_TRILINEAR, len(pos), 1.0, chan_density=0, accum=True)
    o.splat(orc.SPLAT_TRILINEAR, pos, 1.0, weight=w)
    o.splat(orc.SPLAT_TRILINEAR, pos, 1.0, weight=w, accum=True)
    assert rel_error(g.read_channel(0), o.read_channel(0)) <= DENSITY_TOL


def test_dense_readback_layout(gvx_mod, orc, c1):
    pos, w = c1
    g, _ = make_pair(gvx_mod, orc, pos[:5000], 1.0, weight=w[:5000])
    g.splat(gvx_mod.SPLAT_TRILINEAR, 5000, 1.0, chan_density=0)
    bm = g.read_channel(0)
    dense = g.read_channel_dense(0)
    inf = g.info()
    sx, sy, _sz = inf["atlas_subdim"]
    P = bm.shape[1]
    for s in (0, 1, 17, 300):
        if s >= bm.shape[0]:
            continue
        bx, by, bz = s % sx, (s // sx) % sy, s // (sx * sy)
        assert np.array_equal(dense[bz * P:(bz + 1) * P, by * P:(by + 1) * P, bx * P:(bx + 1) * P], bm[s])


def test_borrowed_device_pointers(gvx_mod, orc):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(1)
    pos = (rng.random((10_000, 4)) * 70.0 + 1.0).astype(np.float32)  # stride 16 bytes, xyz + pad
    dev = torch.from_numpy(pos).cuda()
    g = gvx_mod.Grid(0)
    g.configure(LOGDIM)
    g.add_channel(0, gvx_mod.T_FLOAT, 1)
    g.set_points(len(pos), dev, 0, 16)
    g.rebuild_topology(len(pos), 1.0, mode=gvx_mod.TOPO_FULL)
    g.update_atlas()
    g.splat(gvx_mod.SPLAT_TRILINEAR, len(pos), 1.0, chan_density=0)
    o = orc.Oracle(LOGDIM)
    o.add_channel(0, orc.T_FLOAT)
    o.rebuild_topology(pos[:, :3], 1.0)
    o.update_atlas()
    o.splat(orc.SPLAT_TRILINEAR, pos[:, :3], 1.0)
    compare_topology(g, o)
    assert rel_error(g.read_channel(0), o.read_channel(0)) <= DENSITY_TOL
    torch.cuda.synchronize()


def test_errors_are_status_codes(gvx_mod):
    g = gvx_mod.Grid(0)
    with pytest.raises(gvx_mod.GvxError) as e:
        g.rebuild_topology(10, 1.0)
    assert e.value.status == 2  # NOT_CONFIGURED
    g.configure(LOGDIM)
    g.add_channel(0, gvx_mod.T_FLOAT, 1)
    pts = np.full((100, 3), 3.5, np.float32)  # extents inside one brick -> depth 0
    g.commit_points_host(pts)
    with pytest.raises(gvx_mod.GvxError) as e:
        g.rebuild_topology(100, 0.0)
    assert e.value.status == 7  # DEPTH
    with pytest.raises(gvx_mod.GvxError):
        g.add_channel(1, gvx_mod.T_FLOAT, 2)  # apron 2 is not supported by the apron update
    with pytest.raises(gvx_mod.GvxError):
        g.splat(gvx_mod.SPLAT_TRILINEAR, 100, 1.0)  # no topology


def _adjacent_pairs(amap, used, brick):
    lut = {tuple(amap[s, :3]): s for s in range(used)}
    for s in range(used):
        x, y, z = amap[s, :3]
        for d, (dx, dy, dz) in enumerate(((brick, 0, 0), (0, brick, 0), (0, 0, brick))):
            nb = lut.get((x + dx, y + dy, z + dz))
            if nb is not None:
                yield s, nb, d


def test_splat_writes_exact_apron_copies(gvx_mod, orc):
    rng = np.random.default_rng(21)
    pos = (rng.random((30_000, 3)) * np.array([80.0, 64.0, 100.0]) + 3.0).astype(np.float32)
    vel = rng.normal(0, 1, (30_000, 3)).astype(np.float32)
    g, o = make_pair(gvx_mod, orc, pos, 2.0, vel=vel, channels=((0, 3), (1, 4)))
    g.splat(gvx_mod.SPLAT_CUBIC, len(pos), 2.0, chan_density=0, chan_vel=1)
    o.splat(orc.SPLAT_CUBIC, pos, 2.0, vel=vel, chan_vel=1)
    d, v = g.read_channel(0), g.read_channel(1)
    # interior and apron against the oracle (the oracle adds every contribution to all copies)
    assert rel_error(d, o.read_channel(0)) <= DENSITY_TOL
    amap = g.read_atlas_map()
    used = g.info()["used_leaves"]
    P = d.shape[1]
    n = 0
    for s, nb, axis in _adjacent_pairs(amap, used, P - 2):
        # +axis apron of s (padded P-1) is the interior layer 1 of nb, and vice versa: bitwise
        if axis == 0:
            a1, b1, a2, b2 = d[s][:, :, P - 1], d[nb][:, :, 1], d[nb][:, :, 0], d[s][:, :, P - 2]
        elif axis == 1:
            a1, b1, a2, b2 = d[s][:, P - 1, :], d[nb][:, 1, :], d[nb][:, 0, :], d[s][:, P - 2, :]
        else:
            a1, b1, a2, b2 = d[s][P - 1], d[nb][1], d[nb][0], d[s][P - 2]
        assert a1.tobytes() == b1.tobytes() and a2.tobytes() == b2.tobytes()
        n += 1
    assert n > 100
    # a following UpdateApron(chan, 0) has nothing to do
    before = g.kernel_launches()
    g.update_apron(0, 0.0)
    g.update_apron(1, 0.0)
    assert g.kernel_launches() == before
    assert g.read_channel(0).tobytes() == d.tobytes() and g.read_channel(1).tobytes() == v.tobytes()


def test_splat_is_deterministic(gvx_mod, orc, c1):
    pos, w = c1
    g, _ = make_pair(gvx_mod, orc, pos, 2.0, weight=w)
    g.splat(gvx_mod.SPLAT_CUBIC, len(pos), 2.0, chan_density=0)
    a = g.read_channel(0).tobytes()
    g.splat(gvx_mod.SPLAT_CUBIC, len(pos), 2.0, chan_density=0)
    assert g.read_channel(0).tobytes() == a


def test_apron_kernel_matches_fused_copies(gvx_mod, orc, c1):
    pos, w = c1
    g, _ = make_pair(gvx_mod, orc, pos, 1.0, weight=w)
    g.splat(gvx_mod.SPLAT_TRILINEAR, len(pos), 1.0, chan_density=0)
    fused = g.read_channel(0)
    g.update_apron(0, 0.25)  # different boundary value: the apron kernel runs
    g.update_apron(0, 0.0)   # and back: must reproduce the splat's apron exactly
    assert g.read_channel(0).tobytes() == fused.tobytes()


def test_radix_sort_entry_point(gvx_mod):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(13)
    for n, bits in ((1, 8), (4095, 12), (200_003, 21), (65_536, 32)):
        keys = rng.integers(0, 1 << bits, n, dtype=np.uint64).astype(np.uint32)
        vals = np.arange(n, dtype=np.uint32)
        kd = torch.from_numpy(keys.view(np.int32)).cuda()
        vd = torch.from_numpy(vals.view(np.int32)).cuda()
        ko, vo = torch.empty_like(kd), torch.empty_like(vd)
        g = gvx_mod.Grid(0)
        gvx_mod.radix_sort(g, kd, vd, ko, vo, n, bits)
        g.sync()
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(ko.cpu().numpy().view(np.uint32), keys[order])
        assert np.array_equal(vo.cpu().numpy().view(np.uint32), vals[order])
        g.close()


def test_plain_small_32_cubed_bricks(gvx_mod, orc):
    """the secondary C1 row: the samples' literal Configure(3,3,3,3,5) -- 32^3 bricks (padded 34^3, slab
    tiles clamped to shared memory): topology, trilinear splat with its fused aprons, then UpdateApron.
    In 256^3 the first pass holds one level-1 node, the reference's top_lev quirk (VG.cpp:3957-3968)
    that the oracle reports as degenerate; this slab spans two level-1 nodes along x."""
    rng = np.random.default_rng(0)
    pos = (rng.random((60_000, 3)) * np.array([400.0, 90.0, 90.0]) + 1.0).astype(np.float32)
    w = np.ones(len(pos), np.float32)
    logdim = (5, 3, 3, 3, 3)
    g, o = make_pair(gvx_mod, orc, pos, 1.0, logdim=logdim)
    compare_topology(g, o)
    g.commit_points_host(pos, weight=w)
    g.insert_points(len(pos))
    g.splat(gvx_mod.SPLAT_TRILINEAR, len(pos), 1.0, chan_density=0)
    o.splat(orc.SPLAT_TRILINEAR, pos, 1.0, weight=w, chan_density=0)
    used = o.used_leaves()
    assert rel_error(g.read_channel(0)[:used], o.read_channel(0)[:used]) <= DENSITY_TOL
    g.update_apron(0, 0.5)
    o.update_apron(0, 0.5)
    assert rel_error(g.read_channel(0)[:used], o.read_channel(0)[:used]) <= DENSITY_TOL


@pytest.mark.parametrize("mode", ["trilinear", "cubic"])
def test_dense_cluster_against_oracle(gvx_mod, orc, mode):
    """many points per voxel (a Gaussian cluster of sigma 2.5 voxels next to a sparse background):
    long hit batches, many cells per batch and deep same-row ordering in every slab"""
    rng = np.random.default_rng(41)
    dense = rng.normal(0.0, 2.5, (40_000, 3)) + np.array([40.0, 36.0, 44.0])
    sparse = rng.random((5_000, 3)) * np.array([80.0, 72.0, 88.0]) + 2.0
    pos = np.concatenate([dense, sparse]).astype(np.float32)
    pos = pos[(pos > 1.0).all(axis=1)]
    vel = rng.normal(0, 1, pos.shape).astype(np.float32)
    w = (0.5 + rng.random(len(pos))).astype(np.float32)
    if mode == "trilinear":
        g, o = make_pair(gvx_mod, orc, pos, 1.0, weight=w)
        g.splat(gvx_mod.SPLAT_TRILINEAR, len(pos), 1.0, chan_density=0)
        o.splat(orc.SPLAT_TRILINEAR, pos, 1.0, weight=w)
        assert rel_error(g.read_channel(0), o.read_channel(0)) <= DENSITY_TOL
    else:
        g, o = make_pair(gvx_mod, orc, pos, 2.0, weight=w, vel=vel, channels=((0, 3), (1, 4)))
        g.splat(gvx_mod.SPLAT_CUBIC, len(pos), 2.0, chan_density=0, chan_vel=1)
        o.splat(orc.SPLAT_CUBIC, pos, 2.0, weight=w, vel=vel, chan_vel=1)
        assert rel_error(g.read_channel(0), o.read_channel(0)) <= DENSITY_TOL
        v, vr = g.read_channel(1), o.read_channel(1)
        assert np.abs(v[..., :3] - vr[..., :3]).max() <= 1e-5 * np.abs(vr).max()


@pytest.mark.parametrize("radius", [1.0, 1.5, 2.0])
def test_cubic_lattice_points_on_support_edges(gvx_mod, orc, radius):
    """points on integer and half-integer coordinates, brick faces included: voxels exactly at
    distance R (weight 0, excluded) and rows exactly at dy^2 + dz^2 = R^2"""
    g1 = np.arange(2.0, 60.0, 1.5)
    pos = np.stack(np.meshgrid(g1, g1[:24], g1[:30], indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
    g, o = make_pair(gvx_mod, orc, pos, radius)
    g.splat(gvx_mod.SPLAT_CUBIC, len(pos), radius, chan_density=0)
    o.splat(orc.SPLAT_CUBIC, pos, radius)
    assert rel_error(g.read_channel(0), o.read_channel(0)) <= DENSITY_TOL


def test_push_tiles_match_padded_slabs(gvx_mod, orc):
    """a dense cloud (over 8 points a brick) splats density with velocity through push tiles (apron
    rows written by the neighbours); an accumulating splat onto cleared channels takes the
    padded-slab tiles (every apron voxel computed from the points).  With the topology dilated by
    the splat radius no footprint leaves the tree, so both give every padded voxel, aprons
    included, bit for bit"""
    rng = np.random.default_rng(33)
    pos = (rng.random((80_000, 3)) * np.array([72.0, 56.0, 88.0]) + 2.0).astype(np.float32)
    vel = rng.normal(0, 1, pos.shape).astype(np.float32)
    w = (0.5 + rng.random(len(pos))).astype(np.float32)
    g, o = make_pair(gvx_mod, orc, pos, 2.0, weight=w, vel=vel, channels=((0, 3), (1, 4)))
    used = g.info()["used_leaves"]
    assert len(pos) >= 8 * used  # dense: the push tiles
    g.splat(gvx_mod.SPLAT_CUBIC, len(pos), 2.0, chan_density=0, chan_vel=1)
    d1, v1 = g.read_channel(0)[:used].copy(), g.read_channel(1)[:used].copy()
    g.clear_channel(0)
    g.clear_channel(1)
    g.splat(gvx_mod.SPLAT_CUBIC, len(pos), 2.0, chan_density=0, chan_vel=1, accum=True)
    d2, v2 = g.read_channel(0)[:used], g.read_channel(1)[:used]
    assert d1.tobytes() == d2.tobytes()
    assert v1[..., :3].tobytes() == v2[..., :3].tobytes()
    o.splat(orc.SPLAT_CUBIC, pos, 2.0, weight=w, vel=vel, chan_vel=1)
    assert rel_error(d1, o.read_channel(0)[:used]) <= DENSITY_TOL
