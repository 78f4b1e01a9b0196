"""GPU tests of SaveVBX / LoadVBX: the file libgvx writes, read back by an
independent reader in the reference LoadVBX's field order (tests/vbx_format.py),
holds the grid's pools, child lists and dense atlases byte for byte; loading
it into a fresh grid restores pools and channels exactly, and the loaded grid
splats the same points to the same bytes."""
import numpy as np
import pytest

from vbx_format import read_vbx

pytestmark = pytest.mark.gpu

LOGDIM = (3, 3, 3, 3, 5)


def made_grid(gvx, n=60_000, seed=71):
    import torch

    rng = np.random.default_rng(seed)
    pos = (rng.random((n, 3)) * np.array([150.0, 90.0, 120.0]) + 3.0).astype(np.float32)
    vel = rng.normal(0.0, 1.0, (n, 3)).astype(np.float32)
    clr = rng.integers(0, 256, (n, 4)).astype(np.uint8)
    g = gvx.Grid(0)
    g.configure(LOGDIM)
    g.add_channel(0, gvx.T_FLOAT, 1)
    g.add_channel(1, gvx.T_FLOAT3, 1)
    g.add_channel(2, gvx.T_UCHAR4, 1)
    pd, vd = torch.from_numpy(pos).cuda(), torch.from_numpy(vel).cuda()
    cd = torch.from_numpy(clr.view(np.int32)).cuda()
    g.set_points(n, pd, 0, 12, vd, 0, 12, clr=cd)
    g._keep_dev = (pd, vd, cd)
    g.rebuild_topology(n, 2.0, mode=gvx.TOPO_FULL)
    g.finish_topology()
    g.update_atlas()
    g.insert_points(n)
    g.splat(gvx.SPLAT_CUBIC, n, 2.0, chan_density=0, chan_vel=1)
    g.fill_channel(2, [10, 20, 30, 40])
    return g, (pd, vd, cd)


def test_vbx_file_matches_reference_layout(gvx_mod, tmp_path):
    g, _ = made_grid(gvx_mod)
    path = str(tmp_path / "grid.vbx")
    g.save_vbx(path)
    f = read_vbx(path)
    inf = g.info()
    assert (f["major"], f["minor"], f["num_grids"]) == (1, 11, 1)
    assert f["transform"] == [(0.0, 0.0, 0.0), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0)]
    assert f["trailing_bytes"] == 0
    gr = f["grids"][0]
    assert (gr["dtype"], gr["components"], gr["compression"]) == (ord("f"), 1, 0)
    assert (gr["topology_type"], gr["layout"], gr["apron"], gr["channels"]) == (2, 0, 1, 3)
    assert gr["brick_dims"] == (8, 8, 8) and gr["leaf_count"] == inf["node_count"][0]
    assert gr["atlas_bricks"] == tuple(inf["atlas_subdim"]) and gr["atlas_res"] == tuple(inf["atlas_res"])
    assert gr["levels"] == 5 and gr["root"] == inf["root_level"] << 8
    for lev, lt in enumerate(gr["level_table"]):
        assert lt["log2dim"] == LOGDIM[lev] and lt["res"] == 1 << LOGDIM[lev] and lt["width0"] == 64
        assert lt["count0"] == inf["node_count"][lev]
        assert np.array_equal(gr["nodes"][lev].view(np.uint8), g.read_nodes(lev).view(np.uint8))
        if lev == 0:
            assert lt["count1"] == 0 and lt["width1"] == 0
        else:
            assert lt["width1"] == 8 * (1 << (3 * LOGDIM[lev])) and lt["count1"] == lt["count0"]
            assert np.array_equal(gr["childlists"][lev], g.read_childlist(lev))
    for c, (typ, a) in enumerate(gr["atlas"]):
        dense = g.read_channel_dense(c)
        if typ == gvx_mod.T_FLOAT3:
            dense = dense[..., :3]
        assert np.array_equal(a, dense)
    assert gr["atlas_bytes"] == gr["atlas"][0][1].nbytes


def test_vbx_round_trip(gvx_mod, tmp_path):
    g, (pd, vd, cd) = made_grid(gvx_mod)
    path = str(tmp_path / "grid.vbx")
    g.save_vbx(path)
    h = gvx_mod.Grid(0)
    h.load_vbx(path)
    a, b = g.info(), h.info()
    for k in ("levels", "root_level", "node_count", "used_leaves", "atlas_subdim", "atlas_res", "apron", "channels",
              "root_pos"):
        assert a[k] == b[k], k
    for lev in range(a["root_level"] + 1):
        assert np.array_equal(g.read_nodes(lev).view(np.uint8), h.read_nodes(lev).view(np.uint8)), lev
        if lev:
            assert np.array_equal(g.read_childlist(lev), h.read_childlist(lev)), lev
    for c in range(3):
        x, y = g.read_channel(c), h.read_channel(c)
        if c == 1:  # FLOAT3 keeps xyz on file
            x, y = x[..., :3], y[..., :3]
        assert np.array_equal(x, y), c
    # the loaded tree serves the path: the same points splat to the same bytes
    n = pd.shape[0]
    h.set_points(n, pd, 0, 12, vd, 0, 12, clr=cd)
    h.insert_points(n)
    h.splat(gvx_mod.SPLAT_CUBIC, n, 2.0, chan_density=0, chan_vel=1)
    assert np.array_equal(g.read_channel(0), h.read_channel(0))
    assert np.array_equal(g.read_channel(1), h.read_channel(1))
    # after a load the next RebuildTopology is a full one (Clear sets mRebuildTopo)
    h.rebuild_topology(n, 2.0, mode=gvx_mod.TOPO_AUTO)
    assert h.info()["last_rebuild"] == 1
    h.update_atlas()
    for lev in range(a["root_level"] + 1):
        assert np.array_equal(g.read_nodes(lev).view(np.uint8), h.read_nodes(lev).view(np.uint8)), lev


def test_vbx_errors(gvx_mod, tmp_path):
    h = gvx_mod.Grid(0)
    with pytest.raises(gvx_mod.GvxError) as e:
        h.load_vbx(str(tmp_path / "missing.vbx"))
    assert e.value.status == 9
    bad = tmp_path / "short.vbx"
    bad.write_bytes(b"\x01\x0b" + b"\x00" * 40)
    with pytest.raises(gvx_mod.GvxError):
        h.load_vbx(str(bad))
    g = gvx_mod.Grid(0)
    g.configure(LOGDIM)
    g.add_channel(0, gvx_mod.T_FLOAT, 1)
    with pytest.raises(gvx_mod.GvxError):
        g.save_vbx(str(tmp_path / "empty.vbx"))  # no topology yet


def test_vbx_through_the_drop_in_class(gvx_mod, tmp_path):
    """SaveVBX / LoadVBX of nvdb::VolumeGVDB (tests/cpp/volume_gvdb_vbx.cpp)"""
    import os
    import subprocess

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    pkg = os.path.join(root, "gvdb-voxels_gb300")
    exe = str(tmp_path / "volume_gvdb_vbx")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(root, "include"),
           os.path.join(root, "tests", "cpp", "volume_gvdb_vbx.cpp"), "-o", exe, "-L", pkg, "-lgvx_volume", "-lgvx",
           "-Wl,-rpath," + pkg]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    pos = (np.random.default_rng(72).random((20_000, 3)) * np.array([90.0, 70.0, 110.0]) + 2.0).astype(np.float32)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([len(pos)], np.int32).tofile(f)
        pos.tofile(f)
    r = subprocess.run([exe, str(inp), str(tmp_path / "grid.vbx")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr + r.stdout
    assert "bricks identical" in r.stdout and not r.stdout.startswith("0 ")


def test_vbx_counts_beyond_the_file_are_rejected(gvx_mod, tmp_path):
    """a header whose tables would need more bytes than the file holds fails before allocating"""
    import struct

    hdr = struct.pack("<BB", 1, 11) + struct.pack("<12f", 0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 0, 0)
    hdr += struct.pack("<i", 1) + struct.pack("<Q", 2 + 48 + 4 + 8)
    hdr += b"\0" * 256 + struct.pack("<BBB", ord("f"), 1, 0) + struct.pack("<3f", 1, 1, 1)
    hdr += struct.pack("<i3iiiQBiB3i3i", 1, 8, 8, 8, 1, 1, 0, 2, 0, 0, 16, 16, 1, 160, 160, 10)
    hdr += struct.pack("<iQ", 5, 0x200)
    for lev, ld in enumerate((3, 3, 3, 3, 5)):
        r = 1 << ld
        hdr += struct.pack("<ii3iiiii", ld, r, r, r, r, 1 << 30, 64, (1 << 30) if lev else 0, 8 * r ** 3 if lev else 0)
    path = tmp_path / "huge.vbx"
    path.write_bytes(hdr + b"\0" * 1024)
    h = gvx_mod.Grid(0)
    with pytest.raises(gvx_mod.GvxError) as e:
        h.load_vbx(str(path))
    assert e.value.status == 9
