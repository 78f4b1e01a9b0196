"""GPU tests of the host-side topology (ActivateSpace / RebuildTopologyCPU +
FinishTopology): the pools libgvx commits equal, node for node and child list
for child list, the oracle's restatement of the reference's host tree; the
committed tree serves UpdateAtlas and InsertPoints; activation on top of a
GPU-built tree (gFluidSurface's CPU path) only appends."""
import numpy as np
import pytest

from parity_util import assert_nodes_equal

pytestmark = pytest.mark.gpu

LOGDIM = (3, 3, 3, 3, 5)
UNDEFL = 0xFFFFFFFF
UNDEF64 = 0xFFFFFFFFFFFFFFFF
ALL = ("lev", "flags", "pos", "value", "parent", "childlist")


def grid(gvx):
    g = gvx.Grid(0)
    g.configure(LOGDIM)
    g.add_channel(0, gvx.T_FLOAT, 1)
    return g


def same_as_cpu_tree(g, t):
    inf = g.info()
    assert inf["root_level"] == (t.root() >> 8) & 0xFF
    for lev in range(inf["root_level"] + 1):
        assert_nodes_equal(g.read_nodes(lev), t.nodes(lev), lev, ALL)
        if lev:
            assert np.array_equal(g.read_childlist(lev), t.childlist(lev)), lev


@pytest.mark.parametrize("orig", [(0.0, 0.0, 0.0), (7.25, 0.5, 30.0)])
def test_rebuild_topology_cpu_matches_oracle(gvx_mod, orc, orig):
    rng = np.random.default_rng(81)
    pos = (rng.random((30_000, 3)) * np.array([400.0, 300.0, 700.0]) + 1.0).astype(np.float32)
    g = grid(gvx_mod)
    g.commit_points_host(pos)
    g.rebuild_topology_cpu(pos, orig)
    g.finish_topology()
    t = orc.CpuTree(LOGDIM)
    t.activate(pos, orig)
    same_as_cpu_tree(g, t)
    # UpdateAtlas gives the leaves their bricks in pool order; InsertPoints finds every point's leaf
    g.update_atlas()
    nd = g.read_nodes(0)
    assert (nd["value"][:, 0] >= 0).all()
    pnode = g.insert_points(len(pos), trans=orig, want_pnode=True)
    w = np.floor((pos + np.asarray(orig, np.float32)).astype(np.float32)).astype(np.int32)
    assert (pnode >= 0).all() and np.array_equal(nd["pos"][pnode], (w // 8) * 8)


def test_activate_space_return_values(gvx_mod, orc):
    g = grid(gvx_mod)
    pts = np.array([[10.5, 10.5, 10.5], [300.5, 200.5, 100.5]], np.float32)
    # the first point's leaf is the new root: it "exists" once created (ActivateSpace returns it)
    first = g.activate_space(pts[0])
    assert first == 0  # Elem(0, 0, 0)
    assert g.activate_space(pts[1]) == UNDEFL  # a new leaf
    assert g.activate_space([9.9, 12.0, 15.5]) == 0  # inside leaf 0
    assert g.activate_space([297.0, 201.0, 99.0]) == 0x10000  # leaf 1
    g.finish_topology()
    t = orc.CpuTree(LOGDIM)
    t.activate(pts)
    same_as_cpu_tree(g, t)
    # Clear empties the tree; the same calls rebuild it
    g.clear()
    g.rebuild_topology_cpu(pts)
    g.finish_topology()
    same_as_cpu_tree(g, t)


def test_activation_extends_a_gpu_tree(gvx_mod, orc):
    """gFluidSurface's CPU path: ActivateSpace of every other point on the tree the GPU built"""
    rng = np.random.default_rng(82)
    a = (rng.random((20_000, 3)) * np.array([200.0, 150.0, 300.0]) + 2.0).astype(np.float32)
    b = (rng.random((20_000, 3)) * np.array([500.0, 300.0, 700.0]) + 2.0).astype(np.float32)
    g = grid(gvx_mod)
    g.commit_points_host(a)
    g.rebuild_topology(len(a), 1.0, mode=gvx_mod.TOPO_FULL)
    g.update_atlas()
    before = [g.read_nodes(l) for l in range(g.info()["root_level"] + 1)]
    for p in b[::2]:
        g.activate_space(p)
    g.finish_topology()
    inf = g.info()
    # the old pools are a prefix of the new ones (nodes are only appended; the old root keeps index 0
    # while it stays the root, a new root sits at index 0 of the level above)
    for lev, old in enumerate(before):
        new = g.read_nodes(lev)
        assert len(new) >= len(old)
        assert np.array_equal(new["pos"][:len(old)], old["pos"]), lev
    # every activated point has its leaf, and the tree is consistent: each child's parent owns it
    leaves = set(map(tuple, g.read_nodes(0)["pos"].tolist()))
    for p in b[::2]:
        assert tuple(((np.floor(p).astype(np.int64)) // 8 * 8).tolist()) in leaves
    pools = [g.read_nodes(lev) for lev in range(inf["root_level"] + 1)]
    for lev in range(1, inf["root_level"] + 1):
        cl = g.read_childlist(lev).reshape(len(pools[lev]), -1)
        owner, slot = np.nonzero(cl != np.uint64(UNDEF64))
        kids = cl[owner, slot]
        assert ((kids >> np.uint64(8)) & np.uint64(0xFF) == lev - 1).all()
        parents = pools[lev - 1]["parent"][(kids >> np.uint64(16)).astype(np.int64)]
        assert np.array_equal(parents, (np.uint64(lev) << np.uint64(8)) | (owner.astype(np.uint64) << np.uint64(16)))
    g.update_atlas()
    assert g.info()["used_leaves"] == len(g.read_nodes(0))
