"""GPU tests that pin the oracle (and libgvx) to the REFERENCE's own kernels.

The reference's kernels (cuda_gvdb_module.cu, compiled to PTX from the
reference sources by oracle/ref_build.py) run through oracle/ref_harness.cu,
which restates the reference's host orchestration.  Topology and apron copies
must agree bit for bit; the FP32 fast-math scatter and gathers of the
reference within the stated tolerances."""
import numpy as np
import pytest

from parity_util import compare_topology

pytestmark = pytest.mark.gpu

rh = pytest.importorskip("ref_harness")
if not rh.available():
    pytest.skip("reference kernels not built (oracle/_ref/cuda_gvdb_module.ptx)", allow_module_level=True)

FIELDS = ("lev", "flags", "pos", "value", "parent", "childlist")


def same_pools(a, b, levels):
    for lev in range(levels):
        na, nb = a.nodes(lev), b.nodes(lev)
        assert len(na) == len(nb), "level %d: %d vs %d nodes" % (lev, len(na), len(nb))
        for f in FIELDS:
            assert np.array_equal(na[f], nb[f]), "level %d field %s" % (lev, f)
        if lev > 0:
            assert np.array_equal(a.childlist(lev), b.childlist(lev)), "level %d child lists" % lev
    assert a.used_leaves() == b.used_leaves()


def pair(orc, logdim=(3, 3, 3, 3, 5), channels=((0, 3),)):
    r = rh.RefGrid(logdim)
    o = orc.Oracle(logdim)
    for c, t in channels:
        r.add_channel(c, t)
        o.add_channel(c, t)
    return r, o


def slab(n, seed, box=(160.0, 96.0, 200.0), jitter=0.3):
    rng = np.random.default_rng(seed)
    p = rng.random((n, 3)) * np.asarray(box) + rng.normal(0, jitter, (n, 3)) + 1.0
    return p.astype(np.float32)


@pytest.mark.parametrize("radius", [0.0, 1.0, 2.0])
def test_full_topology_matches_reference_kernels(orc, gvx_mod, radius):
    import workloads

    pos, _ = workloads.plain_small(n=40_000, seed=0)
    r, o = pair(orc)
    r.set_points(pos)
    assert r.rebuild(radius) == 0
    r.update_atlas()
    assert o.rebuild_topology(pos, radius) == orc.OK
    o.update_atlas()
    assert r.root_level() == o.root_level()
    same_pools(r, o, o.root_level() + 1)
    # and libgvx against both
    g = gvx_mod.Grid(0)
    g.configure((3, 3, 3, 3, 5))
    g.add_channel(0, gvx_mod.T_FLOAT, 1)
    g.commit_points_host(pos)
    g.rebuild_topology(len(pos), radius, mode=gvx_mod.TOPO_FULL)
    g.update_atlas()
    compare_topology(g, o)


@pytest.mark.parametrize("logdim", [(3, 3, 3, 3, 4), (2, 3, 3, 3, 3), (4, 4, 3, 3, 3)])
def test_full_topology_other_configs(orc, logdim):
    pos = slab(20_000, 5, box=(600.0, 300.0, 700.0))
    r, o = pair(orc, logdim)
    r.set_points(pos)
    assert r.rebuild(1.0) == 0
    r.update_atlas()
    assert o.rebuild_topology(pos, 1.0) == orc.OK
    o.update_atlas()
    same_pools(r, o, o.root_level() + 1)


@pytest.mark.parametrize("accumulate", [False, True])
def test_incremental_frames_match_reference_kernels(orc, gvx_mod, accumulate):
    pos = slab(30_000, 3)
    vel = np.random.default_rng(4).normal(0, 1, pos.shape).astype(np.float32)
    r, o = pair(orc)
    g = gvx_mod.Grid(0)
    g.configure((3, 3, 3, 3, 5))
    g.add_channel(0, gvx_mod.T_FLOAT, 1)
    mode = 2 if accumulate else 0
    for frame in range(6):
        p = (pos + np.float32(2.0 * frame) * vel).astype(np.float32)
        p = np.maximum(p, 0.5).astype(np.float32)
        r.set_points(p)
        st_r = r.rebuild(1.0, mode=mode)
        st_o = o.rebuild_topology(p, 1.0, mode=mode)
        assert st_r == 0 and st_o == orc.OK
        assert r.last_mode() == o.last_mode()
        r.update_atlas()
        o.update_atlas()
        same_pools(r, o, o.root_level() + 1)
        g.commit_points_host(p)
        g.rebuild_topology(len(p), 1.0, mode=mode)
        g.update_atlas()
        assert g.info()["last_rebuild"] == o.last_mode()
        compare_topology(g, o)


@pytest.mark.parametrize("typ", [3, 4])
def test_apron_matches_reference_kernels(orc, typ):
    pos = slab(20_000, 7)
    r, o = pair(orc, channels=((0, typ),))
    r.set_points(pos)
    r.rebuild(1.0)
    r.update_atlas()
    o.rebuild_topology(pos, 1.0)
    o.update_atlas()
    P = 10
    rng = np.random.default_rng(1)
    bricks = o.read_channel(0)
    data = rng.normal(0, 1, bricks.shape).astype(np.float32)
    if typ == 4:
        data[..., 3] = 0.0
    o.write_channel(0, data.astype(np.float64))
    r.write_dense(0, rh.bricks_to_dense(data, r.atlas_subdim(), P))
    r.update_apron(0, 0.75)
    o.update_apron(0, 0.75)
    got = r.read_bricks(0)
    ref = o.read_channel(0).astype(np.float32)
    used = o.used_leaves()
    assert np.array_equal(got[:used], ref[:used])


def test_scatter_matches_reference_kernels(orc):
    # a jittered lattice of spacing 3: no two 7-voxel stencils overlap, so the
    # reference's non-atomic read-modify-write has no collision
    g = np.stack(np.meshgrid(np.arange(30), np.arange(20), np.arange(25), indexing="ij"), -1).reshape(-1, 3)
    rng = np.random.default_rng(2)
    pos = (3.0 * g + 2.0 + rng.random(g.shape) * 0.9).astype(np.float32)
    r, o = pair(orc)
    r.set_points(pos)
    r.rebuild(0.0)
    r.update_atlas()
    o.rebuild_topology(pos, 0.0)
    o.update_atlas()
    r.scatter(1.5)
    o.splat(orc.SPLAT_REF_SCATTER, pos, 1.5)
    got = r.read_bricks(0)[:o.used_leaves()].astype(np.float64)
    ref = o.read_channel(0)[:o.used_leaves()]
    # fast-math FP32 in the reference: |a-b| <= 1e-5 max|b|
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("levelset", [False, True])
def test_gathers_match_reference_kernels(orc, gvx_mod, levelset):
    pos = slab(15_000, 9, box=(100.0, 80.0, 120.0))
    r, o = pair(orc)
    r.set_points(pos)
    r.rebuild(2.0)
    r.update_atlas()
    o.rebuild_topology(pos, 2.0)
    o.update_atlas()
    r.gather(levelset, 4, 1.0, 2.0)
    o.splat(orc.SPLAT_GATHER_LEVELSET if levelset else orc.SPLAT_GATHER_DENSITY, pos, 1.0, subcell=4, radius_ins=2.0)
    used = o.used_leaves()
    got = r.read_bricks(0)[:used, 1:-1, 1:-1, 1:-1].astype(np.float64)
    ref = o.read_channel(0)[:used, 1:-1, 1:-1, 1:-1]
    # the reference takes sqrtf with --use_fast_math: absolute error <= 1e-5 of the radius scale
    assert np.abs(got - ref).max() <= 1e-5 * max(1.0, np.abs(ref).max())
    # libgvx against the reference kernels directly
    g = gvx_mod.Grid(0)
    g.configure((3, 3, 3, 3, 5))
    g.add_channel(0, gvx_mod.T_FLOAT, 1)
    g.commit_points_host(pos)
    g.rebuild_topology(len(pos), 2.0, mode=gvx_mod.TOPO_FULL)
    g.update_atlas()
    n = g.insert_points_subcell(4, len(pos), 2.0)
    if levelset:
        g.gather_levelset(4, len(pos), 1.0, n, chan=0)
    else:
        g.gather_density(4, len(pos), 1.0, n, chan=0)
    mine = g.read_channel(0)[:used, 1:-1, 1:-1, 1:-1].astype(np.float64)
    assert np.abs(mine - got).max() <= 1e-5 * max(1.0, np.abs(got).max())


@pytest.mark.parametrize("src_bits", [2, 4])
def test_convert_matches_reference_kernel(orc, src_bits):
    """ConvertAndTransform: gPointCloud's point decode, (wmin + q * wdelta) * scal + trans; the
    reference's build contracts both multiply-adds to FMAs, which the oracle restates"""
    rng = np.random.default_rng(61 + src_bits)
    n = 200_000
    if src_bits == 2:
        src = rng.integers(0, 65536, (n, 3)).astype(np.uint16)
    else:
        src = (rng.standard_normal((n, 3)) * 500).astype(np.float32)
    wmin, wmax = np.array([-12.5, 3.25, 0.7], np.float32), np.array([1020.3, 511.9, 250.1], np.float32)
    wdelta = ((wmax - wmin) / np.float32(65535.0)).astype(np.float32)
    args = (wmin, wdelta, (0.5, -1.0, 2.0), (0.9, 1.1, 1.0))
    a = rh.convert_and_transform(src, src_bits, *args)
    b = orc.convert_and_transform(src, src_bits, *args)
    assert np.array_equal(a, b), "%d of %d values differ" % (int((a != b).sum()), a.size)


def test_fp16_gather_matches_reference_kernels(orc, gvx_mod):
    """InsertPointsSubcell_FP16 + GatherLevelSet_FP16: the entry count bit for bit; the level set
    within one quantisation step, the reference dividing with fast-math (2 ulp) where the oracle
    and libgvx round correctly"""
    import torch

    pos = slab(30_000, 62)
    r, o = pair(orc)
    r.set_points(pos)
    assert r.rebuild(2.0) == 0
    r.update_atlas()
    assert o.rebuild_topology(pos, 2.0) == orc.OK
    o.update_atlas()
    rmin, rrange = r.pos_bounds()
    omin, omax = o.pos_bounds()
    assert np.array_equal(rmin, omin) and np.array_equal(rrange, (omax - omin).astype(np.float32))
    n_r = r.gather_fp16(4, 1.0, 1.0)
    n_o = o.gather_fp16(pos, 1.0, 1.0, subcell=4, chan=0)
    assert n_r == n_o
    used = o.used_leaves()
    a = r.read_bricks(0)[:used, 1:-1, 1:-1, 1:-1].astype(np.float64)
    b = o.read_channel(0)[:used, 1:-1, 1:-1, 1:-1]
    step = float(np.sqrt(3.0)) * float(rrange.max()) / 65535.0
    assert np.abs(a - b).max() <= step + 1e-5 * max(1.0, float(np.abs(b).max()))
    # libgvx against the reference's kernels the same way
    g = gvx_mod.Grid(0)
    g.configure((3, 3, 3, 3, 5))
    g.add_channel(0, gvx_mod.T_FLOAT, 1)
    pd = torch.from_numpy(pos).cuda()
    g.set_points(len(pos), pd)
    g.rebuild_topology(len(pos), 2.0, mode=gvx_mod.TOPO_FULL)
    g.update_atlas()
    n_g = g.insert_points_subcell_fp16(4, len(pos), 1.0)
    g.gather_levelset_fp16(4, len(pos), 1.0, n_g, chan=0)
    assert n_g == n_r
    c = g.read_channel(0)[:used, 1:-1, 1:-1, 1:-1].astype(np.float64)
    assert np.abs(c - a).max() <= step + 1e-5 * max(1.0, float(np.abs(a).max()))
    print("FP16 level set: %.4f of voxels bit-identical to the reference's kernels" % float((c == a).mean()))
