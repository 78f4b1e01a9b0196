"""ctypes binding of the reference-kernel harness (oracle/ref_harness.cu).

TEST INFRASTRUCTURE ONLY.  Builds oracle/_ref/libref_harness.so from
ref_harness.cu (nvcc) and loads the reference's kernels from
oracle/_ref/cuda_gvdb_module.ptx (built by ref_build.py from the reference's
own sources).  Used by tests/ to pin the oracle against the reference.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "_ref")
SRC = os.path.join(HERE, "ref_harness.cu")
LIB = os.path.join(REF, "libref_harness.so")
PTX = os.path.join(REF, "cuda_gvdb_module.ptx")

NODE_DTYPE = np.dtype([("lev", "u1"), ("flags", "u1"), ("prio", "u1"), ("pad", "u1"),
                       ("pos", "<i4", (3,)), ("value", "<i4", (3,)), ("vrange", "<f4", (3,)),
                       ("parent", "<u8"), ("childlist", "<u8"), ("mask", "<u8")])


def available():
    return os.path.exists(PTX)


def build():
    if not available():
        return None
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-gencode",
           "arch=compute_103a,code=sm_103a", SRC, "-o", LIB + ".tmp", "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("harness build failed:\n%s" % r.stderr[-3000:])
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        build()
    lib = ctypes.CDLL(LIB)
    vp, i, f, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_int64
    sig = {"rh_error": ([], ctypes.c_char_p), "rh_load": ([ctypes.c_char_p], i),
           "rh_create": ([i, vp, i, i, i, i], vp), "rh_destroy": ([vp], None),
           "rh_add_channel": ([vp, i, i], i), "rh_set_points": ([vp, i, vp], i),
           "rh_rebuild": ([vp, f, vp, i, i], i), "rh_update_atlas": ([vp], i),
           "rh_clear_channel": ([vp, i], i), "rh_write_channel_dense": ([vp, i, vp], i),
           "rh_read_channel_dense": ([vp, i, vp], i), "rh_channel_bytes": ([vp, i], i64),
           "rh_scatter": ([vp, f, vp, i], i), "rh_gather": ([vp, i, i, f, f, vp, i, i], i),
           "rh_sc_len": ([vp], i), "rh_update_apron": ([vp, i, f], i), "rh_root_level": ([vp], i),
           "rh_num_nodes": ([vp, i], i), "rh_used_leaves": ([vp], i), "rh_last_mode": ([vp], i),
           "rh_atlas_subdim": ([vp, vp], i), "rh_get_nodes": ([vp, i, vp, i], i),
           "rh_get_childlist": ([vp, i, vp, i64], i),
           "rh_gather_fp16": ([vp, i, f, f, vp, i], i), "rh_pos_bounds": ([vp, vp], i),
           "rh_convert": ([i, vp, i, vp, vp, vp, vp, vp], i)}
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if lib.rh_load(PTX.encode()) != 0:
        raise RuntimeError("reference kernels did not load: %s" % lib.rh_error().decode())
    _lib = lib
    return lib


def _p(a):
    return None if a is None else a.ctypes.data


class RefGrid:
    """A VolumeGVDB driven through the reference's own kernels."""

    def __init__(self, logdim=(3, 3, 3, 3, 5), apron=1, axiscnt=(16, 16, 1)):
        self.lib = load()
        ld = np.ascontiguousarray(logdim, np.int32)
        self.h = self.lib.rh_create(len(logdim), _p(ld), apron, *axiscnt)
        if not self.h:
            raise RuntimeError("rh_create failed")
        self.logdim = tuple(logdim)
        self.apron = apron
        self.types = {}

    def close(self):
        if self.h:
            self.lib.rh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, st, what):
        if st != 0:
            raise RuntimeError("%s: status %d %s" % (what, st, self.lib.rh_error().decode()))
        return st

    def add_channel(self, chan, typ):
        self._ck(self.lib.rh_add_channel(self.h, chan, typ), "add_channel")
        self.types[chan] = typ

    def set_points(self, pos):
        pos = np.ascontiguousarray(pos, np.float32)
        self._ck(self.lib.rh_set_points(self.h, pos.shape[0], _p(pos)), "set_points")

    def rebuild(self, radius, orig=(0, 0, 0), mode=1, min_depth=1):
        o = np.ascontiguousarray(orig, np.float32)
        return self.lib.rh_rebuild(self.h, float(radius), _p(o), mode, min_depth)

    def update_atlas(self):
        self._ck(self.lib.rh_update_atlas(self.h), "update_atlas")

    def clear_channel(self, chan):
        self._ck(self.lib.rh_clear_channel(self.h, chan), "clear_channel")

    def _shape(self, chan):
        sd = self.atlas_subdim()
        P = (1 << self.logdim[0]) + 2 * self.apron
        nc = 4 if self.types[chan] == 4 else 1
        return (sd[2] * P, sd[1] * P, sd[0] * P) + ((nc,) if nc > 1 else ())

    def read_dense(self, chan):
        out = np.zeros(self._shape(chan), np.float32)
        self._ck(self.lib.rh_read_channel_dense(self.h, chan, _p(out)), "read_channel")
        return out

    def write_dense(self, chan, data):
        data = np.ascontiguousarray(data, np.float32).reshape(self._shape(chan))
        self._ck(self.lib.rh_write_channel_dense(self.h, chan, _p(data)), "write_channel")

    def read_bricks(self, chan):
        """the channel in brick-major order (slots, P, P, P[, c]) for comparison with libgvx/oracle"""
        return dense_to_bricks(self.read_dense(chan), self.atlas_subdim(), (1 << self.logdim[0]) + 2 * self.apron)

    def scatter(self, radius, trans=(0, 0, 0), expand=True):
        t = np.ascontiguousarray(trans, np.float32)
        self._ck(self.lib.rh_scatter(self.h, float(radius), _p(t), int(expand)), "scatter")

    def gather(self, levelset, subcell, radius, radius_ins, trans=(0, 0, 0), chan=0, accum=False):
        t = np.ascontiguousarray(trans, np.float32)
        self._ck(self.lib.rh_gather(self.h, int(levelset), subcell, float(radius), float(radius_ins), _p(t), chan,
                                    int(accum)), "gather")
        return self.lib.rh_sc_len(self.h)

    def gather_fp16(self, subcell, radius, radius_ins, trans=(0, 0, 0), chan=0):
        """InsertPointsSubcell_FP16 + GatherLevelSet_FP16 through the reference's kernels"""
        t = np.ascontiguousarray(trans, np.float32)
        self._ck(self.lib.rh_gather_fp16(self.h, subcell, float(radius), float(radius_ins), _p(t), chan),
                 "gather_fp16")
        return self.lib.rh_sc_len(self.h)

    def pos_bounds(self):
        """(mPosMin, mPosRange) of the last GetBoundingBox"""
        out = np.zeros(6, np.float32)
        self.lib.rh_pos_bounds(self.h, _p(out))
        return out[:3], out[3:]

    def update_apron(self, chan, boundval=0.0):
        self._ck(self.lib.rh_update_apron(self.h, chan, float(boundval)), "update_apron")

    def root_level(self):
        return self.lib.rh_root_level(self.h)

    def num_nodes(self, lev):
        return self.lib.rh_num_nodes(self.h, lev)

    def used_leaves(self):
        return self.lib.rh_used_leaves(self.h)

    def last_mode(self):
        return self.lib.rh_last_mode(self.h)

    def atlas_subdim(self):
        out = np.zeros(3, np.int32)
        self.lib.rh_atlas_subdim(self.h, _p(out))
        return tuple(int(x) for x in out)

    def nodes(self, lev):
        n = self.num_nodes(lev)
        out = np.zeros(n, NODE_DTYPE)
        self._ck(self.lib.rh_get_nodes(self.h, lev, _p(out), n), "get_nodes")
        return out

    def childlist(self, lev):
        r = 1 << self.logdim[lev]
        n = self.num_nodes(lev) * r * r * r
        out = np.zeros(n, np.uint64)
        self._ck(self.lib.rh_get_childlist(self.h, lev, _p(out), n), "get_childlist")
        return out


def convert_and_transform(src, src_bits, wmin, wdelta, trans=(0, 0, 0), scal=(1, 1, 1)):
    """ConvertAndTransform through the reference's gvdbConvAndTransform kernel"""
    lib = load()
    a = np.ascontiguousarray(src, np.uint16 if src_bits == 2 else np.float32)
    out = np.zeros((a.shape[0], 3), np.float32)
    vecs = [np.ascontiguousarray(v, np.float32) for v in (wmin, wdelta, trans, scal)]
    if lib.rh_convert(a.shape[0], _p(a), src_bits, _p(out), *[_p(v) for v in vecs]) != 0:
        raise RuntimeError("rh_convert: %s" % lib.rh_error().decode())
    return out


def dense_to_bricks(dense, subdim, P):
    sx, sy, sz = subdim
    extra = dense.shape[3:]
    d = dense.reshape((sz, P, sy, P, sx, P) + extra)
    order = (0, 2, 4, 1, 3, 5) + tuple(range(6, 6 + len(extra)))
    return d.transpose(order).reshape((sx * sy * sz, P, P, P) + extra)


def bricks_to_dense(bricks, subdim, P):
    sx, sy, sz = subdim
    extra = bricks.shape[4:]
    b = bricks.reshape((sz, sy, sx, P, P, P) + extra)
    order = (0, 3, 1, 4, 2, 5) + tuple(range(6, 6 + len(extra)))
    return b.transpose(order).reshape((sz * P, sy * P, sx * P) + extra)
