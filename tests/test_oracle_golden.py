"""CPU tests: the oracle against golden fixtures written by the REFERENCE's own
kernels (tests/golden/*.npz, made by tests/golden/make_golden.py on a GPU from
the PTX of the reference's cuda_gvdb_module.cu and the harness that drives it).
Topology bit for bit; the reference's fast-math FP32 splat values within
|a - b| <= 1e-5 * max(1, max|b|) of the FP64 oracle."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIELDS = ("lev", "flags", "pos", "value", "parent", "childlist")
LOGDIM = (3, 3, 3, 3, 5)


def load(name):
    p = os.path.join(GOLDEN, name)
    if not os.path.exists(p):
        pytest.skip("golden fixture %s not generated" % name)
    return dict(np.load(p))


def same_pools(o, g, orc, prefix=""):
    assert o.root_level() == int(g[prefix + "root_level"])
    for lev in range(o.root_level() + 1):
        ref = np.frombuffer(g[prefix + "nodes%d" % lev].tobytes(), orc.NODE_DTYPE)
        got = o.nodes(lev)
        assert len(got) == len(ref), "level %d: %d nodes vs %d" % (lev, len(got), len(ref))
        for f in FIELDS:
            assert np.array_equal(got[f], ref[f]), "level %d field %s" % (lev, f)
        if lev > 0:
            assert np.array_equal(o.childlist(lev), g[prefix + "clist%d" % lev]), "level %d child lists" % lev
    assert o.used_leaves() == int(g[prefix + "used_leaves"])


def close(got, ref):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    return float(np.abs(got - ref).max()) <= 1e-5 * max(1.0, float(np.abs(ref).max()))


@pytest.mark.parametrize("radius", [0, 1, 2])
def test_full_topology_golden(orc, radius):
    g = load("topo_full_r%d.npz" % radius)
    o = orc.Oracle(LOGDIM)
    o.add_channel(0, orc.T_FLOAT)
    assert o.rebuild_topology(g["pos"], float(g["radius"])) == orc.OK
    o.update_atlas()
    same_pools(o, g, orc)


@pytest.mark.parametrize("name", ["topo_incremental", "topo_accumulate"])
def test_frame_sequences_golden(orc, name):
    g = load(name + ".npz")
    o = orc.Oracle(LOGDIM)
    o.add_channel(0, orc.T_FLOAT)
    for f in range(int(g["frames"])):
        assert o.rebuild_topology(g["pos%d" % f], 1.0, mode=int(g["topo_mode"])) == orc.OK
        o.update_atlas()
        assert o.last_mode() == int(g["mode%d" % f]), "frame %d" % f
        same_pools(o, g, orc, prefix="f%d_" % f)


def test_scatter_golden(orc):
    g = load("scatter.npz")
    o = orc.Oracle(LOGDIM)
    o.add_channel(0, orc.T_FLOAT)
    o.rebuild_topology(g["pos"], 0.0)
    o.update_atlas()
    same_pools(o, g, orc)
    o.splat(orc.SPLAT_REF_SCATTER, g["pos"], float(g["radius"]))
    assert close(o.read_channel(0)[: o.used_leaves(), 1:-1, 1:-1, 1:-1], g["bricks"])


@pytest.mark.parametrize("kind", ["density", "levelset"])
def test_gathers_golden(orc, kind):
    g = load("gather_%s.npz" % kind)
    o = orc.Oracle(LOGDIM)
    o.add_channel(0, orc.T_FLOAT)
    o.rebuild_topology(g["pos"], 2.0)
    o.update_atlas()
    same_pools(o, g, orc)
    n = o.gather(kind == "levelset", g["pos"], float(g["radius"]), float(g["radius_ins"]), subcell=int(g["subcell"]))
    assert n == int(g["sc_len"])
    assert close(o.read_channel(0)[: o.used_leaves(), 1:-1, 1:-1, 1:-1], g["bricks"])


def test_apron_golden(orc):
    g = load("apron.npz")
    o = orc.Oracle(LOGDIM)
    o.add_channel(0, orc.T_FLOAT)
    o.rebuild_topology(g["pos"], 1.0)
    o.update_atlas()
    same_pools(o, g, orc)
    data = o.read_channel(0)
    data[: len(g["data_in"])] = g["data_in"]
    o.write_channel(0, data)
    o.update_apron(0, float(g["boundval"]))
    # apron copies are exact: every voxel of the used bricks bit for bit (as float32)
    assert np.array_equal(o.read_channel(0)[: o.used_leaves()].astype(np.float32), g["bricks"])
