"""GPU parity of the FP16 subcell path (InsertPointsSubcell_FP16 +
GatherLevelSet_FP16, the gPointCloud sequence), the colour half of
ScatterDensity and ConvertAndTransform against the oracle.  All three are
integer or single-rounding float work restated step for step, so they are
compared bit for bit; only the FP64 smoothing after the gather is compared
within a tolerance."""
import numpy as np
import pytest

from parity_util import DENSITY_TOL, rel_error_significant

pytestmark = pytest.mark.gpu

LOGDIM = (3, 3, 3, 3, 5)
# float sums of 7 terms against FP64: |a - b| <= SMOOTH_TOL * max(1, max|b|)
SMOOTH_TOL = 2e-6


def cloud(n, seed, extent=(120.0, 90.0, 150.0), lo=2.0):
    rng = np.random.default_rng(seed)
    return (rng.random((n, 3)) * np.asarray(extent) + lo).astype(np.float32)


def grid_pair(gvx, orc, pos, radius, channels, clr=None, trans=(0.0, 0.0, 0.0)):
    import torch

    g = gvx.Grid(0)
    g.configure(LOGDIM)
    o = orc.Oracle(LOGDIM)
    for c, t in channels:
        g.add_channel(c, t, 1)
        o.add_channel(c, t)
    pd = torch.from_numpy(np.ascontiguousarray(pos, np.float32)).cuda()
    cd = None if clr is None else torch.from_numpy(np.ascontiguousarray(clr, np.uint8).view(np.int32)).cuda()
    g.set_points(len(pos), pd, clr=cd)
    g._keep_dev = (pd, cd)
    g.rebuild_topology(len(pos), radius, orig=trans, mode=gvx.TOPO_FULL)
    g.update_atlas()
    assert o.rebuild_topology(pos, radius, orig=trans) == orc.OK
    o.update_atlas()
    inf = g.info()
    lo, hi = o.pos_bounds()
    assert np.array_equal(np.asarray(inf["bbox_min"], np.float32), lo)
    assert np.array_equal(np.asarray(inf["bbox_max"], np.float32), hi)
    return g, o


@pytest.mark.parametrize("trans", [(0.0, 0.0, 0.0), (3.5, 0.0, 1.25)])
def test_fp16_levelset_bit_exact(gvx_mod, orc, trans):
    pos = cloud(20000, 41)
    r = 1.0
    g, o = grid_pair(gvx_mod, orc, pos, 2 * r, ((0, gvx_mod.T_FLOAT),), trans=trans)
    g.clear_channel(0)
    n_g = g.insert_points_subcell_fp16(4, len(pos), r, trans=trans)
    g.gather_levelset_fp16(4, len(pos), r, n_g, trans=trans, chan=0)
    n_o = o.gather_fp16(pos, r, r, subcell=4, chan=0, trans=trans)
    assert n_g == n_o > len(pos)
    used = o.used_leaves()
    a = g.read_channel(0)[:used, 1:-1, 1:-1, 1:-1]
    b = o.read_channel(0)[:used, 1:-1, 1:-1, 1:-1]
    assert np.array_equal(a, b.astype(np.float32)), float(np.abs(a - b).max())


def test_fp16_colours_bit_exact(gvx_mod, orc):
    pos = cloud(12000, 42, extent=(80.0, 60.0, 70.0))
    clr = np.random.default_rng(43).integers(0, 256, (len(pos), 4)).astype(np.uint8)
    g, o = grid_pair(gvx_mod, orc, pos, 2.0, ((0, gvx_mod.T_FLOAT), (1, gvx_mod.T_UCHAR4)), clr=clr)
    used = o.used_leaves()
    # colours into a uchar4 channel
    n_g = g.insert_points_subcell_fp16(4, len(pos), 1.0)
    g.gather_levelset_fp16(4, len(pos), 1.0, n_g, chan=0, chan_clr=1)
    n_o = o.gather_fp16(pos, 1.0, 1.0, subcell=4, chan=0, chan_clr=1, clr=clr)
    assert n_g == n_o
    assert np.array_equal(g.read_channel(0)[:used, 1:-1, 1:-1, 1:-1],
                          o.read_channel(0)[:used, 1:-1, 1:-1, 1:-1].astype(np.float32))
    assert np.array_equal(g.read_channel(1)[:used, 1:-1, 1:-1, 1:-1],
                          o.read_channel(1)[:used, 1:-1, 1:-1, 1:-1].astype(np.uint8))
    # gPointCloud passes the level-set channel as the colour channel too: the colour bits stay
    g.gather_levelset_fp16(4, len(pos), 1.0, n_g, chan=0, chan_clr=0)
    o.gather_fp16(pos, 1.0, 1.0, subcell=4, chan=0, chan_clr=0, clr=clr)
    a = g.read_channel(0)[:used, 1:-1, 1:-1, 1:-1].view(np.uint32)
    bf = o.read_channel(0)[:used, 1:-1, 1:-1, 1:-1].astype(np.float32)
    b = bf.view(np.uint32)
    # colour words that read as signalling NaNs come back quieted from the oracle's FP64 storage
    a_cmp = np.where(np.isnan(bf), a | np.uint32(0x00400000), a)
    assert np.array_equal(a_cmp, b)
    assert np.isnan(bf).mean() < 0.5


def test_fp16_needs_fp16_lists(gvx_mod, orc):
    pos = cloud(3000, 44)
    g, _ = grid_pair(gvx_mod, orc, pos, 2.0, ((0, gvx_mod.T_FLOAT),))
    n = g.insert_points_subcell(4, len(pos), 1.0)
    with pytest.raises(gvx_mod.GvxError):
        g.gather_levelset_fp16(4, len(pos), 1.0, n, chan=0)
    n = g.insert_points_subcell_fp16(4, len(pos), 1.0)
    with pytest.raises(gvx_mod.GvxError):
        g.gather_levelset(4, len(pos), 1.0, n, chan=0)


def test_point_cloud_pipeline(gvx_mod, orc):
    """gPointCloud's render_update: RebuildTopology(2r), UpdateAtlas, ClearChannel, the FP16 pair,
    UpdateApron(0, 3), Compute(FUNC_SMOOTH, 0, m_smooth, m_smoothp, true, true, 3)"""
    pos = cloud(40000, 45, extent=(200.0, 120.0, 160.0))
    r = 1.5
    g, o = grid_pair(gvx_mod, orc, pos, 2 * r, ((0, gvx_mod.T_FLOAT),))
    g.clear_channel(0)
    n = g.insert_points_subcell_fp16(4, len(pos), r)
    g.gather_levelset_fp16(4, len(pos), r, n, chan=0)
    g.update_apron(0, 3.0)
    g.compute(gvx_mod.FUNC_SMOOTH, 0, 3, (1.0, 0.0, 0.0), update_apron=True, skip_over_aprons=True, boundval=3.0)
    o.gather_fp16(pos, r, r, subcell=4, chan=0)
    o.update_apron(0, 3.0)
    o.compute(orc.FUNC_SMOOTH, 0, 3, (1.0, 0.0, 0.0), update_apron=True, skip_over_aprons=True, boundval=3.0)
    used = o.used_leaves()
    a = g.read_channel(0)[:used].astype(np.float64)
    b = o.read_channel(0)[:used]
    assert float(np.abs(a - b).max()) <= SMOOTH_TOL * max(1.0, float(np.abs(b).max()))


def test_scatter_colours_match_oracle(gvx_mod, orc):
    # clusters of 1-4 points per voxel on a lattice of spacing 3 (ScatterDensity's density is
    # compared where its 7-voxel stencils do not overlap between clusters)
    rng = np.random.default_rng(46)
    gx = np.stack(np.meshgrid(np.arange(16), np.arange(12), np.arange(14), indexing="ij"), -1).reshape(-1, 3)
    reps = rng.integers(1, 5, len(gx))
    base = np.repeat(3.0 * gx + 2.0, reps, axis=0)
    pos = (base + rng.random(base.shape) * 0.9).astype(np.float32)
    clr = rng.integers(0, 256, (len(pos), 4)).astype(np.uint8)
    ch = ((0, gvx_mod.T_FLOAT), (1, gvx_mod.T_UCHAR4), (2, gvx_mod.T_FLOAT), (3, gvx_mod.T_UCHAR4))
    g, o = grid_pair(gvx_mod, orc, pos, 0.0, ch, clr=clr)
    used = o.used_leaves()
    for c in (0, 1, 3):
        g.clear_channel(c)
    g.insert_points(len(pos))
    g.scatter_density(len(pos), 1.5, avg_color=False)
    o.scatter_density(pos, 1.5, clr=clr, avg_color=False)
    assert np.array_equal(g.read_channel(3)[:used], o.read_channel(3)[:used].astype(np.uint8))
    assert not g.read_channel(1).any()
    g.clear_channel(0)
    o.clear_channel(0)
    g.scatter_density(len(pos), 1.5, avg_color=True)
    o.scatter_density(pos, 1.5, clr=clr, avg_color=True)
    assert np.array_equal(g.read_channel(1)[:used], o.read_channel(1)[:used].astype(np.uint8))
    den_g, den_o = g.read_channel(0)[:used], o.read_channel(0)[:used]
    assert np.abs(den_g - den_o).max() <= 1e-6 * np.abs(den_o).max()
    assert rel_error_significant(den_g, den_o, frac=1e-2) <= DENSITY_TOL
    # after an avgColor call, a plain call writes no colour (the reference's colour buffer exists)
    g.clear_channel(3)
    o.clear_channel(3)
    g.scatter_density(len(pos), 1.5, avg_color=False)
    o.scatter_density(pos, 1.5, clr=clr, avg_color=False)
    assert not g.read_channel(3).any() and not o.read_channel(3).any()


@pytest.mark.parametrize("src_bits", [2, 4])
def test_convert_and_transform_bit_exact(gvx_mod, orc, src_bits):
    import torch

    rng = np.random.default_rng(47 + src_bits)
    n = 300_001
    if src_bits == 2:
        src = rng.integers(0, 65536, (n, 3)).astype(np.uint16)
        sd = torch.from_numpy(src.view(np.int16)).cuda()
    else:
        src = (rng.standard_normal((n, 3)) * 1000).astype(np.float32)
        sd = torch.from_numpy(src).cuda()
    wmin, wmax = np.array([-3.7, 12.25, 0.1], np.float32), np.array([811.3, 95.5, 400.9], np.float32)
    wdelta = ((wmax - wmin) / np.float32(65535.0)).astype(np.float32)
    trans, scal = (1.5, -2.25, 0.0), (0.75, 1.0, 3.0)
    g = gvx_mod.Grid(0)
    dst = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    g.convert_and_transform(sd, src_bits, dst, n, wmin, wdelta, trans, scal)
    torch.cuda.synchronize()
    want = orc.convert_and_transform(src, src_bits, wmin, wdelta, trans, scal)
    assert np.array_equal(dst.cpu().numpy(), want)
