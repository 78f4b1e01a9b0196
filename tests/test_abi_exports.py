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
