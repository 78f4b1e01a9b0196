"""GPU test of the host-side tree queries of the nvdb::VolumeGVDB drop-in
(getNodeAtPoint, isActive, getValue, getChildNode over the pools and child
lists read back on demand), driven by a C++ program written like an
application of the reference (tests/cpp/volume_gvdb_queries.cpp).

The expected answers are computed here from the level-0 pool alone: the leaf
at a position is the node whose box holds it, an integer position is active
iff some leaf holds it, and the value there is the brick voxel of that leaf's
atlas slot in the brick-major channel readback (a different path from the
dense atlas that getValue indexes)."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "gvdb-voxels_gb300")
SRC = os.path.join(ROOT, "tests", "cpp", "volume_gvdb_queries.cpp")
NODE = np.dtype([("lev", "u1"), ("flags", "u1"), ("prio", "u1"), ("pad", "u1"), ("pos", "<i4", 3),
                 ("value", "<i4", 3), ("vrange", "<f4", 3), ("parent", "<u8"), ("childlist", "<u8"),
                 ("mask", "<u8")])
ID_UNDEFL = 0xFFFFFFFF


@pytest.fixture(scope="module")
def program(gvx_mod, tmp_path_factory):
    out = str(tmp_path_factory.mktemp("cppq") / "volume_gvdb_queries")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", out, "-L", PKG,
           "-lgvx_volume", "-lgvx", "-Wl,-rpath," + PKG]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def run(program, tmp_path, pos, qs, radius):
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(inp, "wb") as f:
        np.array([len(pos), len(qs)], np.int32).tofile(f)
        np.array([radius], np.float32).tofile(f)
        np.ascontiguousarray(pos, np.float32).tofile(f)
        np.ascontiguousarray(qs, np.float32).tofile(f)
    r = subprocess.run([program, inp, outp], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    buf = open(outp, "rb").read()
    off = 4  # levels
    cnt = int(np.frombuffer(buf, np.uint64, 1, off)[0])
    off += 8
    nodes = np.frombuffer(buf, NODE, cnt, off)
    off += 64 * cnt
    off += 12  # atlas res
    root = int(np.frombuffer(buf, np.uint64, 1, off)[0])
    off += 8
    rec = np.frombuffer(buf, np.dtype([("leaf", "<u8"), ("active", "<i4"), ("value", "<f4")]), len(qs), off)
    off += 16 * len(qs)
    slots = int(np.frombuffer(buf, np.int32, 1, off)[0])
    off += 4
    amap = np.frombuffer(buf, np.int32, 4 * slots, off).reshape(slots, 4)
    off += 16 * slots
    chan = np.frombuffer(buf, np.float32, slots * 1000, off).reshape(slots, 10, 10, 10)
    return nodes, root, rec, amap, chan


def test_tree_queries_match_the_pools(program, tmp_path):
    rng = np.random.default_rng(5)
    pos = (rng.random((20_000, 3)) * np.array([150.0, 90.0, 200.0]) + 4.0).astype(np.float32)
    # queries: the points themselves (inside leaves), random positions around the volume (some
    # outside every leaf, some outside the root), and brick corners
    qs = np.concatenate([pos[:1500],
                         (rng.random((1500, 3)) * np.array([300.0, 300.0, 400.0]) - 20.0).astype(np.float32),
                         (np.floor(pos[1500:1700] / 8) * 8).astype(np.float32)])
    nodes, root, rec, amap, chan = run(program, tmp_path, pos, qs, 1.0)
    assert root != 0xFFFFFFFFFFFFFFFF and (root & 0xFF) == 0 and ((root >> 16) == 0)

    key = {tuple(p): i for i, p in enumerate(nodes["pos"].tolist()) if nodes["flags"][i]}
    slot_of = {int(leaf): s for s, leaf in enumerate(amap[:, 3])}
    # the leaf whose box holds each query (leaf boxes are [pos, pos + 8) on every axis)
    corner = (np.floor(qs.astype(np.float64) / 8.0) * 8).astype(np.int64)
    expect_leaf = np.array([key.get(tuple(c), -1) if (q >= 0).all() else -1
                            for c, q in zip(corner.tolist(), qs)], np.int64)
    got_leaf = np.where(rec["leaf"] == ID_UNDEFL, -1, (rec["leaf"] >> 16).astype(np.int64))
    assert np.array_equal(got_leaf, expect_leaf)
    assert ((rec["leaf"][got_leaf >= 0] & 0xFFFF) == 0).all()  # Elem(0, 0, ndx)
    assert (got_leaf[:1500] >= 0).all() and (got_leaf[-200:] >= 0).all()
    assert (got_leaf[1500:3000] < 0).any()

    # isActive takes the position truncated toward zero, as Vector3DI(Vector3DF) does
    ti = np.trunc(qs).astype(np.int64)
    tc = (ti // 8) * 8
    expect_active = np.array([bool((t >= 0).all()) and tuple(c) in key for t, c in zip(ti, tc.tolist())], np.int32)
    assert np.array_equal(rec["active"], expect_active)

    # getValue: the voxel of the leaf's brick at the truncated offset, read from the brick-major channel
    for i in np.nonzero(got_leaf >= 0)[0]:
        lf = int(got_leaf[i])
        d = np.trunc(qs[i].astype(np.float64) - nodes["pos"][lf]).astype(int)
        s = slot_of[lf]
        assert rec["value"][i] == chan[s, d[2] + 1, d[1] + 1, d[0] + 1], i
    assert np.all(rec["value"][got_leaf < 0] == 0.0)
    assert np.abs(rec["value"][:1500]).max() > 0.0
