"""GPU parity of InsertPointsSubcell + GatherDensity / GatherLevelSet against
the oracle: the entry count (pSCPntsLength) must be identical, the gathered
values within the FP32 tolerance below, colours within one step of 1/255."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LOGDIM = (3, 3, 3, 3, 5)
# FP32 sqrt against the FP64 oracle: |a - b| <= GATHER_TOL * max(1, max|b|)
GATHER_TOL = 1e-5


def build(gvx, orc, pos, topo_radius, channels=((0, 3),), logdim=LOGDIM, clr=None):
    import torch

    g = gvx.Grid(0)
    g.configure(logdim)
    o = orc.Oracle(logdim)
    for c, t in channels:
        g.add_channel(c, t, 1)
        o.add_channel(c, t)
    pd = torch.from_numpy(np.ascontiguousarray(pos, np.float32)).cuda()
    cd = None if clr is None else torch.from_numpy(np.ascontiguousarray(clr, np.uint8).view(np.int32)).cuda()
    g.set_points(len(pos), pd, clr=cd)
    g._keep_dev = (pd, cd)
    g.rebuild_topology(len(pos), topo_radius, mode=gvx.TOPO_FULL)
    g.update_atlas()
    assert o.rebuild_topology(pos, topo_radius) == orc.OK
    o.update_atlas()
    return g, o


def close(got, ref):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.abs(got - ref).max()) <= GATHER_TOL * max(1.0, float(np.abs(ref).max()))


@pytest.fixture(scope="module")
def c1():
    import workloads

    return workloads.plain_small()


@pytest.mark.parametrize("levelset", [False, True])
def test_gather_plain_small(gvx_mod, orc, c1, levelset):
    pos, _ = c1
    g, o = build(gvx_mod, orc, pos, 1.0)
    n_g = g.insert_points_subcell(4, len(pos), 2.0)
    if levelset:
        g.gather_levelset(4, len(pos), 1.0, n_g, chan=0)
    else:
        g.gather_density(4, len(pos), 1.0, n_g, chan=0)
    n_o = o.gather(levelset, pos, 1.0, 2.0, subcell=4, chan=0)
    assert n_g == n_o and n_g > len(pos)
    used = o.used_leaves()
    assert close(g.read_channel(0)[:used], o.read_channel(0)[:used])


@pytest.mark.parametrize("subcell", [1, 2, 8])
def test_gather_subcell_sizes(gvx_mod, orc, subcell):
    rng = np.random.default_rng(21)
    pos = (rng.random((20_000, 3)) * np.array([90.0, 70.0, 110.0]) + 3.0).astype(np.float32)
    g, o = build(gvx_mod, orc, pos, 2.0)
    n_g = g.insert_points_subcell(subcell, len(pos), 1.5)
    g.gather_levelset(subcell, len(pos), 0.75, n_g, chan=0)
    n_o = o.gather(True, pos, 0.75, 1.5, subcell=subcell, chan=0)
    assert n_g == n_o
    used = o.used_leaves()
    assert close(g.read_channel(0)[:used], o.read_channel(0)[:used])


def test_gather_accumulates(gvx_mod, orc):
    rng = np.random.default_rng(22)
    pos = (rng.random((30_000, 3)) * 120.0 + 4.0).astype(np.float32)
    g, o = build(gvx_mod, orc, pos, 2.0)
    half = len(pos) // 2
    # density from the first half, then accumulate the second half on top
    n_g = g.insert_points_subcell(4, half, 2.0)
    g.gather_density(4, half, 1.2, n_g, chan=0)
    o.gather(False, pos[:half], 1.2, 2.0, subcell=4, chan=0)
    import torch

    pd2 = torch.from_numpy(pos[half:].copy()).cuda()
    g.set_points(len(pos) - half, pd2)
    n_g2 = g.insert_points_subcell(4, len(pos) - half, 2.0)
    g.gather_density(4, len(pos) - half, 1.2, n_g2, chan=0, accum=True)
    n_o2 = o.gather(False, pos[half:], 1.2, 2.0, subcell=4, chan=0, accum=True)
    assert n_g2 == n_o2
    used = o.used_leaves()
    assert close(g.read_channel(0)[:used], o.read_channel(0)[:used])


def test_gather_colour_average(gvx_mod, orc):
    rng = np.random.default_rng(23)
    pos = (rng.random((15_000, 3)) * 80.0 + 5.0).astype(np.float32)
    clr = rng.integers(0, 256, (len(pos), 4), dtype=np.uint8)
    clr[:, 3] = rng.integers(0, 100, len(pos))  # keeps the averaged alpha mostly inside [0, 1]
    g, o = build(gvx_mod, orc, pos, 1.0, channels=((0, 3), (1, 2)), clr=clr)
    n_g = g.insert_points_subcell(4, len(pos), 2.0)
    g.gather_density(4, len(pos), 1.0, n_g, chan=0, chan_clr=1)
    n_o = o.gather(False, pos, 1.0, 2.0, subcell=4, chan=0, chan_clr=1, clr=clr)
    assert n_g == n_o
    used = o.used_leaves()
    assert close(g.read_channel(0)[:used], o.read_channel(0)[:used])
    got = g.read_channel(1)[:used].astype(np.int64)
    ref = o.read_channel(1)[:used].astype(np.int64)
    assert got.shape == ref.shape
    inner = (slice(None), slice(1, -1), slice(1, -1), slice(1, -1))
    assert np.abs(got[inner] - ref[inner]).max() <= 1  # FP32 sums vs FP64, truncated to uchar


def test_gather_on_incremental_tree(gvx_mod, orc):
    rng = np.random.default_rng(24)
    p0 = rng.random((20_000, 3)) * np.array([100.0, 80.0, 120.0]) + 20.0
    v = rng.normal(0, 1, p0.shape)
    g = gvx_mod.Grid(0)
    g.configure(LOGDIM)
    g.add_channel(0, gvx_mod.T_FLOAT, 1)
    o = orc.Oracle(LOGDIM)
    o.add_channel(0, 3)
    for f in range(4):
        pos = np.maximum(p0 + 3.0 * f * v, 0.5).astype(np.float32)
        g.commit_points_host(pos)
        g.rebuild_topology(len(pos), 2.0, mode=gvx_mod.TOPO_AUTO)
        g.update_atlas()
        assert o.rebuild_topology(pos, 2.0, mode=orc.TOPO_AUTO) == orc.OK
        o.update_atlas()
    assert o.last_mode() == 2 and (o.nodes(0)["flags"] == 0).any()
    n_g = g.insert_points_subcell(4, len(pos), 2.0)
    g.gather_levelset(4, len(pos), 1.0, n_g, chan=0)
    n_o = o.gather(True, pos, 1.0, 2.0, subcell=4, chan=0)
    assert n_g == n_o
    used = o.used_leaves()
    assert close(g.read_channel(0)[:used], o.read_channel(0)[:used])


def test_gather_density_with_no_entries_writes_nothing(gvx_mod, orc):
    rng = np.random.default_rng(25)
    pos = (rng.random((5_000, 3)) * 60.0 + 5.0).astype(np.float32)
    g, o = build(gvx_mod, orc, pos, 1.0)
    g.fill_channel(0, [0.5])
    g.insert_points_subcell(4, len(pos), 2.0)
    g.gather_density(4, len(pos), 1.0, 0, chan=0)  # pSCPntsLength 0: the reference returns at once
    assert (g.read_channel(0) == 0.5).all()


def test_gather_needs_matching_lists(gvx_mod, orc):
    rng = np.random.default_rng(26)
    pos = (rng.random((5_000, 3)) * 60.0 + 5.0).astype(np.float32)
    g, _ = build(gvx_mod, orc, pos, 1.0)
    n = g.insert_points_subcell(4, len(pos), 2.0)
    with pytest.raises(gvx_mod.GvxError) as e:
        g.gather_density(2, len(pos), 1.0, n, chan=0)
    assert e.value.status == 8  # GVX_ERR_STATE
    g.rebuild_topology(len(pos), 1.0, mode=gvx_mod.TOPO_FULL)
    g.update_atlas()
    with pytest.raises(gvx_mod.GvxError):
        g.gather_levelset(4, len(pos), 1.0, n, chan=0)
