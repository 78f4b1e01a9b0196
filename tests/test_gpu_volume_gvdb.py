"""GPU test of the nvdb::VolumeGVDB drop-in class (include/gvx_volume_gvdb.h):
a C++ program written like an application of the reference drives it
(tests/cpp/volume_gvdb_points.cpp); its node pools must equal the oracle's
bit for bit, every point's leaf (AUX_PNODE) must hold the point, and the
brick values must match the oracle within the density tolerance."""
import os
import subprocess

import numpy as np
import pytest

from parity_util import DENSITY_TOL, rel_error, rel_error_significant

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "gvdb-voxels_gb300")
SRC = os.path.join(ROOT, "tests", "cpp", "volume_gvdb_points.cpp")
NODE = np.dtype([("lev", "u1"), ("flags", "u1"), ("prio", "u1"), ("pad", "u1"), ("pos", "<i4", 3),
                 ("value", "<i4", 3), ("vrange", "<f4", 3), ("parent", "<u8"), ("childlist", "<u8"),
                 ("mask", "<u8")])


@pytest.fixture(scope="module")
def program(gvx_mod, tmp_path_factory):
    out = str(tmp_path_factory.mktemp("cpp") / "volume_gvdb_points")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", out, "-L", PKG,
           "-lgvx_volume", "-lgvx", "-Wl,-rpath," + PKG]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def run(program, tmp_path, pos, mode, radius):
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(inp, "wb") as f:
        np.array([len(pos), mode], np.int32).tofile(f)
        np.array([radius], np.float32).tofile(f)
        np.ascontiguousarray(pos, np.float32).tofile(f)
    r = subprocess.run([program, inp, outp], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    buf = open(outp, "rb").read()
    off = 0
    levels = int(np.frombuffer(buf, np.int32, 1, off)[0])
    off += 4
    nodes = []
    for _ in range(levels):
        cnt = int(np.frombuffer(buf, np.uint64, 1, off)[0])
        off += 8
        nodes.append(np.frombuffer(buf, NODE, cnt, off))
        off += 64 * cnt
    used = int(np.frombuffer(buf, np.uint64, 1, off)[0])
    off += 8
    pnode = np.frombuffer(buf, np.int32, len(pos), off)
    off += 4 * len(pos)
    # AtlasRetrieveBrickXYZ writes z fastest, [x][y][z]: to [z][y][x] like the channel readback
    bricks = np.frombuffer(buf, np.float32, used * 512, off).reshape(used, 8, 8, 8).transpose(0, 3, 2, 1)
    return nodes, used, pnode, bricks


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_volume_gvdb_class_matches_oracle(program, orc, tmp_path, mode):
    rng = np.random.default_rng(31 + mode)
    if mode in (0, 2):
        # a jittered lattice of spacing 3: ScatterDensity's 7-voxel stencils do not overlap
        gx = np.stack(np.meshgrid(np.arange(24), np.arange(16), np.arange(20), indexing="ij"), -1).reshape(-1, 3)
        pos = (3.0 * gx + 2.0 + rng.random(gx.shape) * 0.9).astype(np.float32)
        radius = 1.5
    elif mode == 1:
        pos = (rng.random((30_000, 3)) * np.array([100.0, 70.0, 130.0]) + 3.0).astype(np.float32)
        radius = 2.0
    else:
        pos = (rng.random((30_000, 3)) * np.array([100.0, 70.0, 130.0]) + 3.0).astype(np.float32)
        radius = 1.0
    nodes, used, pnode, bricks = run(program, tmp_path, pos, mode, radius)
    o = orc.Oracle((3, 3, 3, 3, 5))
    o.add_channel(0, orc.T_FLOAT)
    assert o.rebuild_topology(pos, 2 * radius if mode == 3 else radius) == orc.OK
    o.update_atlas()
    for lev in range(o.root_level() + 1):
        ref = o.nodes(lev)
        assert len(nodes[lev]) == len(ref)
        for f in ("lev", "flags", "pos", "value", "parent", "childlist"):
            assert np.array_equal(nodes[lev][f], ref[f]), (lev, f)
    assert used == o.used_leaves()
    # every point's leaf holds it
    leaf_pos = nodes[0]["pos"][pnode]
    assert (pnode >= 0).all() and np.array_equal(leaf_pos, (np.floor(pos).astype(np.int32) // 8) * 8)
    if mode == 3:
        o.gather_fp16(pos, radius, radius, subcell=4, chan=0)
        o.update_apron(0, 3.0)
        o.compute(orc.FUNC_SMOOTH, 0, 2, (1.0, 0.0, 0.0), update_apron=True, skip_over_aprons=True, boundval=3.0)
    elif mode in (0, 2):
        o.splat(orc.SPLAT_REF_SCATTER, pos, radius)
        o.update_apron(0, 0.0)
        if mode == 2:
            o.compute(orc.FUNC_SMOOTH, 0, 2, (4.0, 0.0, 0.0), update_apron=True, skip_over_aprons=True)
    else:
        o.splat(orc.SPLAT_CUBIC, pos, radius)
    ref = o.read_channel(0)[:used, 1:-1, 1:-1, 1:-1]
    # bricks come out in pool order of the active leaves = atlas slot order
    if mode == 3:
        # the FP16 gather is bit-exact; the two smoothing passes are float sums against FP64
        assert np.abs(bricks - ref).max() <= 2e-6 * max(1.0, np.abs(ref).max())
    elif mode == 2:
        # smoothing averages the scatter's FP32 error down; judged as the scatter is
        assert np.abs(bricks - ref).max() <= 1e-6 * np.abs(ref).max()
        assert rel_error_significant(bricks, ref, frac=1e-2) <= DENSITY_TOL
    elif mode == 0:
        # ScatterDensity's (1 - d^2/r^2)^3 loses FP32 relative accuracy where d ~ r: judged
        # against the largest magnitude, and relatively on the significant voxels
        assert np.abs(bricks - ref).max() <= 1e-6 * np.abs(ref).max()
        assert rel_error_significant(bricks, ref, frac=1e-2) <= DENSITY_TOL
    else:
        assert rel_error(bricks, ref) <= DENSITY_TOL
