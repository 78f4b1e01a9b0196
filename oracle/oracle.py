"""ctypes binding of the CPU oracle (gvx_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA library.  Only tests/,
__graft_entry__.smoke() and the CPU-baseline / reference arm of bench.py use
it; the product (libgvx.so and gvdb-voxels_gb300/) never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "gvx_oracle.c")

OK, ERR_ARG, ERR_DEPTH, ERR_DEGENERATE, ERR_STATE, ERR_NOMEM = 0, 1, 2, 3, 4, 5
TOPO_AUTO, TOPO_FULL, TOPO_ACCUMULATE = 0, 1, 2
FUNC_FILL_F, FUNC_FILL_C, FUNC_FILL_C4, FUNC_SMOOTH = 110, 111, 112, 113
SPLAT_TRILINEAR, SPLAT_CUBIC, SPLAT_REF_SCATTER, SPLAT_GATHER_DENSITY, SPLAT_GATHER_LEVELSET = 0, 1, 2, 3, 4
T_UCHAR, T_UCHAR4, T_FLOAT, T_FLOAT3, T_FLOAT4 = 0, 2, 3, 4, 5

NODE_DTYPE = np.dtype([("lev", "u1"), ("flags", "u1"), ("prio", "u1"), ("pad", "u1"),
                       ("pos", "<i4", (3,)), ("value", "<i4", (3,)), ("vrange", "<f4", (3,)),
                       ("parent", "<u8"), ("childlist", "<u8"), ("mask", "<u8")])


def build():
    """gcc the restatement into oracle/liboracle.so (no FMA contraction: the float
    steps it restates round one by one, on x86 and Arm alike)"""
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-D_POSIX_C_SOURCE=200809L", "-ffp-contract=off", "-o",
           LIB_PATH + ".tmp", SRC, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n%s" % r.stderr)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(SRC):
        build()
    lib = ctypes.CDLL(LIB_PATH)
    vp, i, f, d, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_int64
    sig = {
        "orc_create": ([i, vp, i, i, i, i], vp), "orc_destroy": ([vp], None),
        "orc_add_channel": ([vp, i, i], i), "orc_clear_channel": ([vp, i], i),
        "orc_rebuild_topology": ([vp, i, vp, i, f, vp, i, i], i), "orc_update_atlas": ([vp], i),
        "orc_root_level": ([vp], i), "orc_top_lev": ([vp], i), "orc_num_nodes": ([vp, i], i),
        "orc_num_used_leaves": ([vp], i), "orc_last_mode": ([vp], i),
        "orc_get_nodes": ([vp, i, vp, i], i), "orc_get_childlist": ([vp, i, vp, i64], i),
        "orc_atlas_subdim": ([vp, vp], i), "orc_get_atlas_map": ([vp, vp, i], i),
        "orc_splat": ([vp, i, i, vp, i, vp, vp, vp, i, f, vp, i, i, i, i, i, f], i),
        "orc_gather": ([vp, i, i, vp, i, vp, f, f, vp, i, i, i, i, vp], i),
        "orc_gather_fp16": ([vp, i, vp, i, vp, f, f, vp, i, i, i, vp], i), "orc_pos_bounds": ([vp, vp], None),
        "orc_compute_bounds": ([vp, vp], i), "orc_atlas_layout_only": ([vp], i),
        "orc_splat_sample": ([vp, i, i, vp, i, vp, vp, vp, i, f, vp, vp, i, i, vp, vp], i),
        "orc_scatter_density": ([vp, i, vp, i, vp, f, vp, i, i], i),
        "orc_convert_and_transform": ([i, vp, i, vp, vp, vp, vp, vp], i),
        "orc_update_apron_faces": ([vp, i], i),
        "orc_cpu_tree_new": ([i, vp], vp), "orc_cpu_tree_free": ([vp], None),
        "orc_cpu_tree_activate": ([vp, i, vp, i, vp], i), "orc_cpu_tree_count": ([vp, i], i),
        "orc_cpu_tree_root": ([vp], i64), "orc_cpu_tree_nodes": ([vp, i, vp, i], i),
        "orc_cpu_tree_childlist": ([vp, i, vp, i64], i),
        "orc_compute": ([vp, i, i, i, vp, i, i, d], i),
        "orc_update_apron": ([vp, i, d], i), "orc_channel_size": ([vp, i], i64),
        "orc_read_channel": ([vp, i, vp, i64], i), "orc_write_channel": ([vp, i, vp, i64], i),
        "orc_activate_space_cpu": ([i, vp, i, vp, i, vp, vp, i, vp], i),
        "orc_now_seconds": ([], d),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def _p(a):
    return None if a is None else a.ctypes.data


class OracleError(RuntimeError):
    def __init__(self, status, what):
        super().__init__("oracle status %d in %s" % (status, what))
        self.status = status


class Oracle:
    """One oracle grid: FP64 restatement of a VolumeGVDB."""

    def __init__(self, logdim=(3, 3, 3, 3, 5), apron=1, axiscnt=(16, 16, 1)):
        self.lib = load()
        ld = np.ascontiguousarray(logdim, np.int32)
        self.h = self.lib.orc_create(len(logdim), _p(ld), apron, *axiscnt)
        if not self.h:
            raise OracleError(ERR_ARG, "orc_create")
        self.logdim = tuple(logdim)
        self.apron = apron
        self.ncomp = {}

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, st, what, allow_degenerate=False):
        if st != OK and not (allow_degenerate and st == ERR_DEGENERATE):
            raise OracleError(st, what)
        return st

    def add_channel(self, chan, typ):
        self._ck(self.lib.orc_add_channel(self.h, chan, typ), "add_channel")
        self.ncomp[chan] = 4 if typ in (T_FLOAT3, T_FLOAT4, T_UCHAR4) else 1

    def clear_channel(self, chan):
        self._ck(self.lib.orc_clear_channel(self.h, chan), "clear_channel")

    def rebuild_topology(self, pos, radius, orig=(0, 0, 0), mode=TOPO_FULL, min_depth=1, allow_degenerate=False):
        pos = np.ascontiguousarray(pos, np.float32)
        o = np.ascontiguousarray(orig, np.float32)
        return self._ck(self.lib.orc_rebuild_topology(self.h, pos.shape[0], _p(pos), 3, float(radius), _p(o),
                                                      mode, min_depth), "rebuild_topology", allow_degenerate)

    def atlas_layout_only(self):
        """slot assignment without channel storage (for sampled checks of large grids)"""
        self._ck(self.lib.orc_atlas_layout_only(self.h), "atlas_layout_only")

    def update_atlas(self):
        self._ck(self.lib.orc_update_atlas(self.h), "update_atlas")

    def root_level(self):
        return self.lib.orc_root_level(self.h)

    def top_lev(self):
        return self.lib.orc_top_lev(self.h)

    def num_nodes(self, level):
        return self.lib.orc_num_nodes(self.h, level)

    def used_leaves(self):
        return self.lib.orc_num_used_leaves(self.h)

    def last_mode(self):
        return self.lib.orc_last_mode(self.h)

    def nodes(self, level):
        n = self.num_nodes(level)
        out = np.zeros(n, NODE_DTYPE)
        self._ck(self.lib.orc_get_nodes(self.h, level, _p(out), n), "get_nodes")
        return out

    def childlist(self, level):
        r = 1 << self.logdim[level]
        n = self.num_nodes(level) * r * r * r
        out = np.zeros(n, np.uint64)
        self._ck(self.lib.orc_get_childlist(self.h, level, _p(out), n), "get_childlist")
        return out

    def atlas_subdim(self):
        out = np.zeros(3, np.int32)
        self.lib.orc_atlas_subdim(self.h, _p(out))
        return tuple(int(x) for x in out)

    def atlas_map(self):
        sd = self.atlas_subdim()
        n = sd[0] * sd[1] * sd[2]
        out = np.zeros((n, 4), np.int32)
        self._ck(self.lib.orc_get_atlas_map(self.h, _p(out), n), "get_atlas_map")
        return out

    def splat(self, mode, pos, radius=1.0, weight=None, radius_pp=None, vel=None, trans=(0, 0, 0),
              chan_density=0, chan_vel=-1, accum=False, expand=True, subcell=4, radius_ins=0.0,
              allow_degenerate=False):
        pos = np.ascontiguousarray(pos, np.float32)
        w = None if weight is None else np.ascontiguousarray(weight, np.float32)
        r = None if radius_pp is None else np.ascontiguousarray(radius_pp, np.float32)
        v = None if vel is None else np.ascontiguousarray(vel, np.float32)
        t = np.ascontiguousarray(trans, np.float32)
        st = self.lib.orc_splat(self.h, mode, pos.shape[0], _p(pos), 3, _p(w), _p(r), _p(v), 3, float(radius),
                                _p(t), chan_density, chan_vel, int(accum), int(expand), subcell, float(radius_ins))
        return self._ck(st, "splat", allow_degenerate)

    def splat_sample(self, mode, pos, leaves, radius=1.0, weight=None, radius_pp=None, vel=None, trans=(0, 0, 0),
                     zero_unowned=True, dens=None, velout=None):
        """TRILINEAR / CUBIC splat values (FP64) of the padded bricks of the
        level-0 pool nodes `leaves`, without atlas channels.  Adds into `dens`
        (k, P, P, P) and `velout` (k, P, P, P, 3) when given (accumulation),
        else into zeros; returns (dens, velout or None)."""
        pos = np.ascontiguousarray(pos, np.float32)
        lv = np.ascontiguousarray(leaves, np.int32)
        w = None if weight is None else np.ascontiguousarray(weight, np.float32)
        r = None if radius_pp is None else np.ascontiguousarray(radius_pp, np.float32)
        v = None if vel is None else np.ascontiguousarray(vel, np.float32)
        t = np.ascontiguousarray(trans, np.float32)
        P = (1 << self.logdim[0]) + 2 * self.apron
        if dens is None:
            dens = np.zeros((len(lv), P, P, P), np.float64)
        if velout is None and v is not None:
            velout = np.zeros((len(lv), P, P, P, 3), np.float64)
        assert dens.flags.c_contiguous and dens.dtype == np.float64
        st = self.lib.orc_splat_sample(self.h, mode, pos.shape[0], _p(pos), 3, _p(w), _p(r), _p(v), 3,
                                       float(radius), _p(t), _p(lv), len(lv), int(zero_unowned), _p(dens),
                                       _p(velout))
        self._ck(st, "splat_sample")
        return dens, velout

    def gather(self, levelset, pos, radius, radius_ins, subcell=4, chan=0, chan_clr=-1, clr=None,
               trans=(0, 0, 0), accum=False, allow_degenerate=False):
        """InsertPointsSubcell + GatherDensity / GatherLevelSet; returns the
        number of (point, subcell) entries"""
        pos = np.ascontiguousarray(pos, np.float32)
        c = None if clr is None else np.ascontiguousarray(clr, np.uint8).reshape(-1, 4)
        t = np.ascontiguousarray(trans, np.float32)
        n = ctypes.c_int64(0)
        st = self.lib.orc_gather(self.h, int(levelset), pos.shape[0], _p(pos), 3, _p(c), float(radius),
                                 float(radius_ins), _p(t), subcell, chan, chan_clr, int(accum), ctypes.byref(n))
        self._ck(st, "gather", allow_degenerate)
        return n.value

    def scatter_density(self, pos, radius, clr=None, trans=(0, 0, 0), expand=True, avg_color=False,
                        allow_degenerate=False):
        """ScatterDensity (VG.cpp:5624-5660): REF_SCATTER into channel 0 and, with point
        colours, channel 1 (avg_color) or channel 3"""
        pos = np.ascontiguousarray(pos, np.float32)
        c = None if clr is None else np.ascontiguousarray(clr, np.uint8).reshape(-1, 4)
        t = np.ascontiguousarray(trans, np.float32)
        st = self.lib.orc_scatter_density(self.h, pos.shape[0], _p(pos), 3, _p(c), float(radius), _p(t),
                                          int(expand), int(avg_color))
        return self._ck(st, "scatter_density", allow_degenerate)

    def gather_fp16(self, pos, radius, radius_ins, subcell=4, chan=0, chan_clr=-1, clr=None, trans=(0, 0, 0),
                    allow_degenerate=False):
        """InsertPointsSubcell_FP16 + GatherLevelSet_FP16; returns the entry count"""
        pos = np.ascontiguousarray(pos, np.float32)
        c = None if clr is None else np.ascontiguousarray(clr, np.uint8).reshape(-1, 4)
        t = np.ascontiguousarray(trans, np.float32)
        n = ctypes.c_int64(0)
        st = self.lib.orc_gather_fp16(self.h, pos.shape[0], _p(pos), 3, _p(c), float(radius), float(radius_ins),
                                      _p(t), subcell, chan, chan_clr, ctypes.byref(n))
        self._ck(st, "gather_fp16", allow_degenerate)
        return n.value

    def pos_bounds(self):
        """(mPosMin, mPosMax) of the last GetBoundingBox"""
        out = np.zeros(6, np.float32)
        self.lib.orc_pos_bounds(self.h, _p(out))
        return out[:3], out[3:]

    def compute_bounds(self):
        """ComputeBounds (VG.cpp:1792-1816): (mVoxMin, mVoxMax, mVoxRes, mVoxResMax)"""
        out = np.zeros(12, np.float32)
        self._ck(self.lib.orc_compute_bounds(self.h, _p(out)), "compute_bounds")
        return out[:3], out[3:6], out[6:9], out[9:]

    def compute(self, effect, chan, iterations, params, update_apron, skip_over_aprons, boundval=0.0):
        """Compute (VG.cpp:4534-4558): FUNC_FILL_F/C/C4 (110-112), FUNC_SMOOTH (113)"""
        p = np.ascontiguousarray(params, np.float32)
        self._ck(self.lib.orc_compute(self.h, effect, chan, iterations, _p(p), int(update_apron),
                                      int(skip_over_aprons), float(boundval)), "compute")

    def update_apron(self, chan, boundval=0.0):
        self._ck(self.lib.orc_update_apron(self.h, chan, float(boundval)), "update_apron")

    def update_apron_faces(self, chan):
        self._ck(self.lib.orc_update_apron_faces(self.h, chan), "update_apron_faces")

    def write_channel(self, chan, data):
        data = np.ascontiguousarray(data, np.float64).ravel()
        self._ck(self.lib.orc_write_channel(self.h, chan, _p(data), data.size), "write_channel")

    def read_channel(self, chan):
        n = self.lib.orc_channel_size(self.h, chan)
        out = np.zeros(n, np.float64)
        self._ck(self.lib.orc_read_channel(self.h, chan, _p(out), n), "read_channel")
        P = (1 << self.logdim[0]) + 2 * self.apron
        nc = self.ncomp[chan]
        return out.reshape((-1, P, P, P) + ((nc,) if nc > 1 else ()))


class CpuTree:
    """The reference's host tree (ActivateSpace / RebuildTopologyCPU), kept across calls"""

    def __init__(self, logdim=(3, 3, 3, 3, 5)):
        self.lib = load()
        ld = np.ascontiguousarray(logdim, np.int32)
        self.h = self.lib.orc_cpu_tree_new(len(logdim), _p(ld))
        self.logdim = tuple(logdim)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_cpu_tree_free(self.h)
            self.h = None

    def activate(self, pos, orig=(0, 0, 0)):
        pos = np.ascontiguousarray(pos, np.float32)
        o = np.ascontiguousarray(orig, np.float32)
        st = self.lib.orc_cpu_tree_activate(self.h, pos.shape[0], _p(pos), 3, _p(o))
        if st != OK:
            raise OracleError(st, "cpu_tree_activate")

    def root(self):
        return self.lib.orc_cpu_tree_root(self.h)

    def nodes(self, lev):
        n = self.lib.orc_cpu_tree_count(self.h, lev)
        out = np.zeros(n, NODE_DTYPE)
        if n:
            self.lib.orc_cpu_tree_nodes(self.h, lev, _p(out), n)
        return out

    def childlist(self, lev):
        r = 1 << self.logdim[lev]
        n = self.lib.orc_cpu_tree_count(self.h, lev) * r * r * r
        out = np.zeros(n, np.uint64)
        if n:
            self.lib.orc_cpu_tree_childlist(self.h, lev, _p(out), n)
        return out


def convert_and_transform(src, src_bits, wmin, wdelta, trans=(0, 0, 0), scal=(1, 1, 1)):
    """ConvertAndTransform on host arrays: (n, 3) uint16 (src_bits 2) or float32 (4) -> (n, 3) float32"""
    lib = load()
    a = np.ascontiguousarray(src, np.uint16 if src_bits == 2 else np.float32)
    out = np.zeros((a.shape[0], 3), np.float32)
    vecs = [np.ascontiguousarray(v, np.float32) for v in (wmin, wdelta, trans, scal)]
    st = lib.orc_convert_and_transform(a.shape[0], _p(a), src_bits, _p(out), *[_p(v) for v in vecs])
    if st != OK:
        raise OracleError(st, "convert_and_transform")
    return out


def activate_space_cpu(pos, logdim=(3, 3, 3, 3, 5), orig=(0, 0, 0)):
    """host CPU topology (ActivateSpace per point): leaf positions and root level"""
    lib = load()
    pos = np.ascontiguousarray(pos, np.float32)
    ld = np.ascontiguousarray(logdim, np.int32)
    o = np.ascontiguousarray(orig, np.float32)
    cap = pos.shape[0] + 1
    out = np.zeros((cap, 3), np.int32)
    root = ctypes.c_int(-1)
    n = lib.orc_activate_space_cpu(len(logdim), _p(ld), pos.shape[0], _p(pos), 3, _p(o), _p(out), cap,
                                   ctypes.byref(root))
    if n < 0:
        raise OracleError(ERR_ARG, "activate_space_cpu")
    return out[:n], root.value
