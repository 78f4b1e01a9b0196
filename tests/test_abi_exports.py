"""CPU tests: libgvx.so loads and exports every entry point include/gvx.h declares.
No compute call is made here (there may be no GPU)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for f in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ \*]*?\b(gvx_[a-z0-9_]+)\s*\(", txt, re.M)
    return sorted(set(names))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("gvx_create", "gvx_configure", "gvx_add_channel", "gvx_set_points", "gvx_rebuild_topology",
                 "gvx_update_atlas", "gvx_insert_points", "gvx_scatter_density", "gvx_insert_points_subcell",
                 "gvx_gather_density", "gvx_gather_levelset", "gvx_splat", "gvx_update_apron"):
        assert must in names


def test_library_exports_every_declared_symbol(gvx_mod):
    lib = gvx_mod.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, "libgvx.so lacks %s" % missing
    assert b"sm_103a" in lib.gvx_version()
    assert isinstance(lib.gvx_last_error(), bytes)


def test_library_has_no_oracle_dependency(gvx_mod):
    # the product library never links the oracle
    lib = ctypes.CDLL(gvx_mod.LIB_PATH)
    assert not hasattr(lib, "orc_create")


def test_volume_class_compiles_and_links(gvx_mod, tmp_path):
    """the nvdb::VolumeGVDB drop-in (include/gvx_volume_gvdb.h, libgvx_volume.so) links a
    program written against it (run on the GPU by test_gpu_volume_gvdb.py)"""
    import subprocess

    pkg = os.path.join(ROOT, "gvdb-voxels_gb300")
    assert os.path.exists(os.path.join(pkg, "libgvx_volume.so"))
    out = str(tmp_path / "volume_gvdb_points")
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "volume_gvdb_points.cpp"), "-o", out, "-L", pkg, "-lgvx_volume",
           "-lgvx", "-Wl,-rpath," + pkg]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
