"""ctypes binding of libgvx.so (include/gvx.h) for tests, benchmarks and Python callers.

The binding is a thin mirror of the C ABI: every method calls exactly one
gvx_* entry point and raises GvxError with the library's message when the
status is not GVX_OK.  There is no fallback: if libgvx.so is missing or has no
CUDA device to run on, the calls fail.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgvx.so")

OK = 0
ERR_NAMES = {1: "INVALID_ARG", 2: "NOT_CONFIGURED", 3: "CAPACITY", 4: "DEVICE", 5: "TIMEOUT",
             6: "UNSUPPORTED", 7: "DEPTH", 8: "STATE", 9: "IO"}
ERR_TIMEOUT = 5

T_UCHAR, T_UCHAR4, T_FLOAT, T_FLOAT3, T_FLOAT4 = 0, 2, 3, 4, 5
TOPO_AUTO, TOPO_FULL, TOPO_ACCUMULATE = 0, 1, 2
SPLAT_TRILINEAR, SPLAT_CUBIC = 0, 1
FUNC_FILL_F, FUNC_FILL_C, FUNC_FILL_C4, FUNC_SMOOTH = 110, 111, 112, 113

NODE_DTYPE = np.dtype([("lev", "u1"), ("flags", "u1"), ("prio", "u1"), ("pad", "u1"),
                       ("pos", "<i4", (3,)), ("value", "<i4", (3,)), ("vrange", "<f4", (3,)),
                       ("parent", "<u8"), ("childlist", "<u8"), ("mask", "<u8")])
assert NODE_DTYPE.itemsize == 64

_ELEM = {T_FLOAT: (np.float32, 1), T_FLOAT3: (np.float32, 4), T_FLOAT4: (np.float32, 4),
         T_UCHAR: (np.uint8, 1), T_UCHAR4: (np.uint8, 4)}


class GvxError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("gvx status %d (%s): %s" % (status, ERR_NAMES.get(status, "?"), msg))
        self.status = status


class Info(ctypes.Structure):
    _fields_ = [("levels", ctypes.c_int), ("logdim", ctypes.c_int * 10), ("brick_res", ctypes.c_int),
                ("apron", ctypes.c_int), ("root_level", ctypes.c_int), ("top_lev", ctypes.c_int),
                ("node_count", ctypes.c_int64 * 10), ("used_leaves", ctypes.c_int64),
                ("atlas_subdim", ctypes.c_int * 3), ("atlas_res", ctypes.c_int * 3), ("channels", ctypes.c_int),
                ("last_rebuild", ctypes.c_int), ("root_pos", ctypes.c_int * 3), ("bbox_min", ctypes.c_float * 3),
                ("bbox_max", ctypes.c_float * 3), ("obj_min", ctypes.c_float * 3), ("obj_max", ctypes.c_float * 3),
                ("vox_res", ctypes.c_float * 3), ("vox_res_max", ctypes.c_float * 3),
                ("planned_builds", ctypes.c_int64)]


_lib = None


def load(path=None):
    """Load libgvx.so (raises if it was not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("libgvx.so not built at %s (run __graft_entry__.build())" % p)
    lib = ctypes.CDLL(p)
    vp, i, f, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_int64
    fp = ctypes.POINTER(ctypes.c_float)
    ip = ctypes.POINTER(ctypes.c_int)
    sig = {
        "gvx_last_error": ([], ctypes.c_char_p), "gvx_version": ([], ctypes.c_char_p),
        "gvx_create": ([i, ctypes.POINTER(vp)], i), "gvx_destroy": ([vp], i),
        "gvx_set_stream": ([vp, vp], i), "gvx_sync": ([vp], i),
        "gvx_configure": ([vp, i, ip, ip], i), "gvx_set_channel_default": ([vp, i, i, i], i),
        "gvx_add_channel": ([vp, i, i, i], i), "gvx_clear_channel": ([vp, i], i),
        "gvx_fill_channel": ([vp, i, fp], i),
        "gvx_set_points": ([vp, i, vp, i, i, vp, i, i, vp, i, i], i),
        "gvx_set_point_attribs": ([vp, vp, vp], i),
        "gvx_commit_points_host": ([vp, i, vp, i, vp, i, vp, vp], i),
        "gvx_rebuild_topology": ([vp, i, f, fp, i, i], i), "gvx_request_full_rebuild": ([vp, i], i),
        "gvx_finish_topology": ([vp], i), "gvx_finish_topology_ex": ([vp, i, i], i), "gvx_update_atlas": ([vp], i),
        "gvx_insert_points": ([vp, i, fp, vp], i),
        "gvx_scatter_density": ([vp, i, f, f, fp, i, i], i),
        "gvx_insert_points_subcell": ([vp, i, i, f, fp, ip], i),
        "gvx_gather_density": ([vp, i, i, f, fp, i, i, i, i], i),
        "gvx_gather_levelset": ([vp, i, i, f, fp, i, i, i, i], i),
        "gvx_splat": ([vp, i, i, f, fp, i, i, i], i),
        "gvx_splat_backward": ([vp, i, i, f, fp, vp, vp, vp, vp], i),
        "gvx_splat_backward_ex": ([vp, i, i, f, fp, vp, vp, vp, vp, i], i),
        "gvx_update_apron": ([vp, i, f], i), "gvx_update_apron_all": ([vp], i),
        "gvx_compute": ([vp, i, i, i, fp, i, i, f], i),
        "gvx_insert_points_subcell_fp16": ([vp, i, i, f, fp, ctypes.POINTER(i)], i),
        "gvx_gather_levelset_fp16": ([vp, i, i, f, fp, i, i, i], i),
        "gvx_convert_and_transform": ([vp, vp, i, vp, i, i, fp, fp, fp, fp], i),
        "gvx_channel_type": ([vp, i, ip], i),
        "gvx_update_apron_faces": ([vp, i], i), "gvx_update_neighbors": ([vp], i),
        "gvx_clear": ([vp], i), "gvx_activate_space": ([vp, fp, ctypes.POINTER(ctypes.c_uint64)], i),
        "gvx_rebuild_topology_cpu": ([vp, i, fp, vp], i),
        "gvx_save_vbx": ([vp, ctypes.c_char_p], i), "gvx_load_vbx": ([vp, ctypes.c_char_p, i, i], i),
        "gvx_memcpy": ([i, vp, vp, ctypes.c_size_t, i], i),
        "gvx_get_info": ([vp, ctypes.POINTER(Info)], i),
        "gvx_read_nodes": ([vp, i, vp, i64], i), "gvx_read_childlist": ([vp, i, vp, i64], i),
        "gvx_read_atlas_map": ([vp, vp, i64], i), "gvx_channel_bytes": ([vp, i, ctypes.POINTER(i64)], i),
        "gvx_read_channel": ([vp, i, vp, i64], i), "gvx_read_channel_dense": ([vp, i, vp, i64], i),
        "gvx_channel_device_ptr": ([vp, i, ctypes.POINTER(vp), ctypes.POINTER(i64)], i),
        "gvx_retrieve_brick": ([vp, i, ip, vp, i64], i),
        "gvx_kernel_launches": ([vp, ctypes.POINTER(i64)], i),
        "gvx_radix_sort": ([vp, vp, vp, vp, vp, ctypes.c_uint32, i], i),
        "gvx_radix_sort_noalloc": ([vp, vp, vp, vp, ctypes.c_uint32, i, vp], i),
        "gvx_radix_sort_noalloc_status": ([vp], i),
        "gvx_test_sort_noalloc_withheld_tile": ([vp, vp, vp, vp, ctypes.c_uint32, vp], i),
        "gvx_batch_create": ([i, ctypes.POINTER(vp)], i), "gvx_batch_destroy": ([vp], i),
        "gvx_batch_set_stream": ([vp, vp], i), "gvx_batch_set_grids": ([vp, ctypes.POINTER(vp), i], i),
        "gvx_batch_splat": ([vp, i, f, i, i, i, i], i),
        "gvx_batch_get_tuning": ([vp, ip, ip, fp], i),
        "gvx_batch_topology": ([vp, f, i, i], i),
        "gvx_batch_frame": ([vp, f, i, f, i, i, i], i),
        "gvx_batch_frame_path": ([vp, ip, ip], i),
        "gvx_test_sort_withheld_tile": ([vp, vp, vp, vp, vp, ctypes.c_uint32], i),
        "gvx_batch_kernel_launches": ([vp, ctypes.POINTER(i64)], i),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _lib = lib
    return lib


def _f3(v):
    v = (0.0, 0.0, 0.0) if v is None else v
    return (ctypes.c_float * 3)(*[float(x) for x in v])


def _ptr(a):
    """device pointer of a torch tensor / int, or host pointer of a numpy array"""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    raise TypeError(type(a))


class Grid:
    """One gvx_grid handle (one VolumeGVDB)."""

    def __init__(self, device=0, lib=None):
        self.lib = lib or load()
        h = ctypes.c_void_p()
        self._check(self.lib.gvx_create(device, ctypes.byref(h)))
        self.h = h
        self.device = device
        self._types = {}
        self._keep = (None, None)

    def _check(self, st):
        if st != OK:
            raise GvxError(st, self.lib.gvx_last_error().decode(errors="replace"))

    def close(self):
        if getattr(self, "h", None):
            self.lib.gvx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- setup
    def configure(self, logdim=(3, 3, 3, 3, 5)):
        ld = (ctypes.c_int * len(logdim))(*logdim)
        self._check(self.lib.gvx_configure(self.h, len(logdim), ld, None))
        self.logdim = tuple(logdim)

    def set_channel_default(self, cx, cy, cz):
        self._check(self.lib.gvx_set_channel_default(self.h, cx, cy, cz))

    def add_channel(self, chan, typ, apron=1):
        self._check(self.lib.gvx_add_channel(self.h, chan, typ, apron))
        self._types[chan] = typ

    def clear_channel(self, chan):
        self._check(self.lib.gvx_clear_channel(self.h, chan))

    def fill_channel(self, chan, value):
        v = (ctypes.c_float * 4)(*(list(value) + [0.0] * (4 - len(value))))
        self._check(self.lib.gvx_fill_channel(self.h, chan, v))

    def set_stream(self, stream_ptr):
        self._check(self.lib.gvx_set_stream(self.h, ctypes.c_void_p(stream_ptr)))

    def sync(self):
        self._check(self.lib.gvx_sync(self.h))

    # --- points
    def set_points(self, n, pos, pos_offset=0, pos_stride=12, vel=None, vel_offset=0, vel_stride=12, clr=None,
                   clr_offset=0, clr_stride=4):
        self._check(self.lib.gvx_set_points(self.h, n, _ptr(pos), pos_offset, pos_stride, _ptr(vel), vel_offset,
                                            vel_stride, _ptr(clr), clr_offset, clr_stride))

    def set_point_attribs(self, weight=None, radius=None):
        self._check(self.lib.gvx_set_point_attribs(self.h, _ptr(weight), _ptr(radius)))

    def commit_points_host(self, pos, vel=None, weight=None, radius=None):
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        arrs = [pos]
        vel = None if vel is None else np.ascontiguousarray(vel, dtype=np.float32)
        weight = None if weight is None else np.ascontiguousarray(weight, dtype=np.float32)
        radius = None if radius is None else np.ascontiguousarray(radius, dtype=np.float32)
        arrs += [a for a in (vel, weight, radius) if a is not None]
        # the copies run asynchronously into one of two device buffer sets: hold the arrays of
        # the last two commits
        self._keep = (arrs, self._keep[0])
        n = pos.shape[0]
        self._check(self.lib.gvx_commit_points_host(self.h, n, _ptr(pos), pos.strides[0], _ptr(vel),
                                                    vel.strides[0] if vel is not None else 0, _ptr(weight),
                                                    _ptr(radius)))
        return n

    # --- topology
    def rebuild_topology(self, n, radius, orig=None, mode=TOPO_FULL, min_depth=1):
        self._check(self.lib.gvx_rebuild_topology(self.h, n, float(radius), _f3(orig), mode, min_depth))

    def request_full_rebuild(self, on=True):
        self._check(self.lib.gvx_request_full_rebuild(self.h, int(on)))

    def finish_topology(self, commit_pool=True, compute_bounds=True):
        self._check(self.lib.gvx_finish_topology_ex(self.h, int(commit_pool), int(compute_bounds)))

    def update_atlas(self):
        self._check(self.lib.gvx_update_atlas(self.h))

    # --- splats
    def insert_points(self, n, trans=None, want_pnode=False):
        out = np.empty(n, np.int32) if want_pnode else None
        self._check(self.lib.gvx_insert_points(self.h, n, _f3(trans), _ptr(out)))
        return out

    def scatter_density(self, n, radius, amp=1.0, trans=None, expand=True, avg_color=False):
        self._check(self.lib.gvx_scatter_density(self.h, n, float(radius), float(amp), _f3(trans), int(expand),
                                                 int(avg_color)))

    def splat(self, mode, n, radius, trans=None, chan_density=0, chan_vel=-1, accum=False):
        self._check(self.lib.gvx_splat(self.h, mode, n, float(radius), _f3(trans), chan_density, chan_vel,
                                       int(accum)))

    def splat_backward(self, mode, n, radius, dl_drho, grad_pos, grad_w, grad_r=None, trans=None, recompute=False):
        """device buffers (torch tensors or raw pointers): dL/drho in the density
        channel layout in, dL/dp (n x 3), dL/dw (n) and dL/dR (n) out; recompute:
        the sorted-key permutation is recomputed from the positions, not reused"""
        self._check(self.lib.gvx_splat_backward_ex(self.h, mode, n, float(radius), _f3(trans), _ptr(dl_drho),
                                                   _ptr(grad_pos), _ptr(grad_w), _ptr(grad_r),
                                                   BWD_RECOMPUTE if recompute else 0))

    def insert_points_subcell(self, subcell, n, radius, trans=None):
        ln = ctypes.c_int(0)
        self._check(self.lib.gvx_insert_points_subcell(self.h, subcell, n, float(radius), _f3(trans),
                                                       ctypes.byref(ln)))
        return ln.value

    def gather_density(self, subcell, n, radius, sc_len, trans=None, chan=0, chan_clr=-1, accum=False):
        self._check(self.lib.gvx_gather_density(self.h, subcell, n, float(radius), _f3(trans), sc_len, chan,
                                                chan_clr, int(accum)))

    def gather_levelset(self, subcell, n, radius, sc_len, trans=None, chan=0, chan_clr=-1, accum=False):
        self._check(self.lib.gvx_gather_levelset(self.h, subcell, n, float(radius), _f3(trans), sc_len, chan,
                                                 chan_clr, int(accum)))

    def insert_points_subcell_fp16(self, subcell, n, radius, trans=None):
        out = ctypes.c_int(0)
        self._check(self.lib.gvx_insert_points_subcell_fp16(self.h, subcell, n, float(radius), _f3(trans),
                                                            ctypes.byref(out)))
        return out.value

    def gather_levelset_fp16(self, subcell, n, radius, sc_len, trans=None, chan=0, chan_clr=-1):
        self._check(self.lib.gvx_gather_levelset_fp16(self.h, subcell, n, float(radius), _f3(trans), sc_len, chan,
                                                      chan_clr))

    def convert_and_transform(self, src, src_bits, dst, n, wmin, wdelta, trans=(0, 0, 0), scal=(1, 1, 1)):
        """ConvertAndTransform: device uint16x3 (src_bits 2) or float3 (4) points -> device float3"""
        self._check(self.lib.gvx_convert_and_transform(self.h, _ptr(src), src_bits, _ptr(dst), 4, n, _f3(wmin),
                                                       _f3(wdelta), _f3(trans), _f3(scal)))

    def update_apron_faces(self, chan):
        self._check(self.lib.gvx_update_apron_faces(self.h, chan))

    def update_neighbors(self):
        self._check(self.lib.gvx_update_neighbors(self.h))

    def clear(self):
        self._check(self.lib.gvx_clear(self.h))

    def activate_space(self, pos):
        """ActivateSpace: the leaf's id when it existed, else ID_UNDEFL (0xFFFFFFFF)"""
        out = ctypes.c_uint64(0)
        self._check(self.lib.gvx_activate_space(self.h, _f3(pos), ctypes.byref(out)))
        return out.value

    def rebuild_topology_cpu(self, pos, orig=None):
        """RebuildTopologyCPU over host float3 points"""
        p = np.ascontiguousarray(pos, np.float32)
        self._check(self.lib.gvx_rebuild_topology_cpu(self.h, p.shape[0], _f3(orig), _ptr(p)))

    def _channel_type(self, chan):
        t = ctypes.c_int(-1)
        self._check(self.lib.gvx_channel_type(self.h, chan, ctypes.byref(t)))
        return t.value

    def save_vbx(self, path):
        self._check(self.lib.gvx_save_vbx(self.h, os.fsencode(path)))

    def load_vbx(self, path, force_major=0, force_minor=0):
        """LoadVBX: configures the grid and its channels from the file"""
        self._check(self.lib.gvx_load_vbx(self.h, os.fsencode(path), force_major, force_minor))
        self._types = {c: t for c in range(32) for t in [self._channel_type(c)] if t >= 0}

    def update_apron(self, chan=None, boundval=0.0):
        if chan is None:
            self._check(self.lib.gvx_update_apron_all(self.h))
        else:
            self._check(self.lib.gvx_update_apron(self.h, chan, float(boundval)))

    def compute(self, effect, chan, iterations, params, update_apron, skip_over_aprons, boundval=0.0):
        """Compute(effect, channel, num_iterations, parameters, bUpdateApron, skipOverAprons, boundval)"""
        p = (ctypes.c_float * 3)(*[float(x) for x in params])
        self._check(self.lib.gvx_compute(self.h, effect, chan, iterations, p, int(update_apron),
                                         int(skip_over_aprons), float(boundval)))

    # --- queries
    def info(self):
        inf = Info()
        self._check(self.lib.gvx_get_info(self.h, ctypes.byref(inf)))
        d = {k: getattr(inf, k) for k, _ in Info._fields_}
        for k, v in list(d.items()):
            if not isinstance(v, (int, float)):
                d[k] = list(v)
        return d

    def read_nodes(self, level):
        n = self.info()["node_count"][level]
        out = np.zeros(n, NODE_DTYPE)
        self._check(self.lib.gvx_read_nodes(self.h, level, _ptr(out), n))
        return out

    def read_childlist(self, level):
        inf = self.info()
        r = 1 << inf["logdim"][level]
        n = inf["node_count"][level] * r * r * r
        out = np.zeros(n, np.uint64)
        self._check(self.lib.gvx_read_childlist(self.h, level, _ptr(out), n))
        return out

    def read_atlas_map(self):
        sd = self.info()["atlas_subdim"]
        n = sd[0] * sd[1] * sd[2]
        out = np.zeros((n, 4), np.int32)
        self._check(self.lib.gvx_read_atlas_map(self.h, _ptr(out), n))
        return out

    def channel_bytes(self, chan):
        b = ctypes.c_int64(0)
        self._check(self.lib.gvx_channel_bytes(self.h, chan, ctypes.byref(b)))
        return b.value

    def read_channel(self, chan):
        """brick-major native layout: (slots, P, P, P[, ncomp]) with x fastest"""
        inf = self.info()
        P = inf["brick_res"] + 2 * inf["apron"]
        dt, nc = _ELEM[self._types[chan]]
        nbytes = self.channel_bytes(chan)
        out = np.zeros(nbytes // np.dtype(dt).itemsize, dt)
        self._check(self.lib.gvx_read_channel(self.h, chan, _ptr(out), nbytes))
        shp = (-1, P, P, P) + ((nc,) if nc > 1 else ())
        return out.reshape(shp)

    def read_slots(self, chan, slots):
        """the bricks of the given atlas slots, (len(slots), P, P, P[, ncomp]),
        copied slot by slot (a sample of a channel too large to read whole)"""
        inf = self.info()
        P = inf["brick_res"] + 2 * inf["apron"]
        dt, nc = _ELEM[self._types[chan]]
        ptr, nbytes = self.channel_device_ptr(chan)
        per = P * P * P * nc * np.dtype(dt).itemsize
        out = np.zeros((len(slots), P, P, P) + ((nc,) if nc > 1 else ()), dt)
        for k, s in enumerate(np.asarray(slots, np.int64)):
            if s < 0 or (s + 1) * per > nbytes:
                raise ValueError("slot %d outside channel %d" % (s, chan))
            self._check(self.lib.gvx_memcpy(self.device, _ptr(out[k]), ctypes.c_void_p(ptr + int(s) * per), per, 1))
        return out

    def read_channel_dense(self, chan):
        """the reference's 3D-array layout: (Z, Y, X[, ncomp])"""
        inf = self.info()
        dt, nc = _ELEM[self._types[chan]]
        nbytes = self.channel_bytes(chan)
        out = np.zeros(nbytes // np.dtype(dt).itemsize, dt)
        self._check(self.lib.gvx_read_channel_dense(self.h, chan, _ptr(out), nbytes))
        X, Y, Z = inf["atlas_res"]
        shp = (Z, Y, X) + ((nc,) if nc > 1 else ())
        return out.reshape(shp)

    def write_channel(self, chan, data):
        """host data in the brick-major native layout (as read_channel returns) into the channel"""
        dt, _ = _ELEM[self._types[chan]]
        a = np.ascontiguousarray(data, dt)
        ptr, nbytes = self.channel_device_ptr(chan)
        if a.nbytes != nbytes:
            raise ValueError("channel %d holds %d bytes, got %d" % (chan, nbytes, a.nbytes))
        self._check(self.lib.gvx_memcpy(self.device, ptr, _ptr(a), nbytes, 0))

    def channel_device_ptr(self, chan):
        p = ctypes.c_void_p()
        b = ctypes.c_int64()
        self._check(self.lib.gvx_channel_device_ptr(self.h, chan, ctypes.byref(p), ctypes.byref(b)))
        return p.value, b.value

    def kernel_launches(self):
        c = ctypes.c_int64()
        self._check(self.lib.gvx_kernel_launches(self.h, ctypes.byref(c)))
        return c.value


def radix_sort(grid, keys_in, vals_in, keys_out, vals_out, n, bits):
    """gvx_radix_sort on device buffers (torch tensors or raw pointers)"""
    grid._check(grid.lib.gvx_radix_sort(grid.h, _ptr(keys_in), _ptr(vals_in), _ptr(keys_out), _ptr(vals_out),
                                        int(n), int(bits)))


BATCH_GRAPH, BATCH_TUNE = 1, 2
BWD_RECOMPUTE = 1


class Batch:
    """One gvx_batch handle: the splats of many grids in one persistent launch."""

    def __init__(self, device=0, lib=None):
        self.lib = lib or load()
        h = ctypes.c_void_p()
        st = self.lib.gvx_batch_create(device, ctypes.byref(h))
        if st:
            raise GvxError(st, self.lib.gvx_last_error().decode())
        self.h = h
        self._grids = []

    def _check(self, st):
        if st:
            raise GvxError(st, self.lib.gvx_last_error().decode())

    def close(self):
        if self.h:
            self.lib.gvx_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr):
        self._check(self.lib.gvx_batch_set_stream(self.h, ctypes.c_void_p(stream_ptr)))

    def set_grids(self, grids):
        self._grids = list(grids)
        arr = (ctypes.c_void_p * len(grids))(*[g.h.value for g in grids])
        self._check(self.lib.gvx_batch_set_grids(self.h, arr, len(grids)))

    def splat(self, mode, radius, chan_density=0, chan_vel=-1, accum=False, graph=True, tune=False):
        flags = (BATCH_GRAPH if graph else 0) | (BATCH_TUNE if tune else 0)
        self._check(self.lib.gvx_batch_splat(self.h, mode, float(radius), chan_density, chan_vel, int(accum), flags))

    def topology(self, radius, mode=None, threads=0):
        """gvx_batch_topology: RebuildTopology + UpdateAtlas + InsertPoints of every grid, staged
        from this thread (threads 0) or as per-grid calls from a pool of host threads"""
        self._check(self.lib.gvx_batch_topology(self.h, float(radius), TOPO_FULL if mode is None else mode,
                                                int(threads)))

    def frame(self, topo_radius, mode, radius, chan_density=0, chan_vel=-1, graph=True, tune=False):
        """gvx_batch_frame: full RebuildTopology + UpdateAtlas + InsertPoints of every grid, then the
        batched splat; planned builds (and, with graph, one captured CUDA graph) once plans exist"""
        flags = (BATCH_GRAPH if graph else 0) | (BATCH_TUNE if tune else 0)
        self._check(self.lib.gvx_batch_frame(self.h, float(topo_radius), mode, float(radius), chan_density, chan_vel,
                                              flags))

    def frame_path(self):
        """(path, rebuilt) of the last frame: path 0 unplanned, 1 planned, 2 graph replay; rebuilt =
        grids built again without their plan"""
        p, r = ctypes.c_int(0), ctypes.c_int(0)
        self._check(self.lib.gvx_batch_frame_path(self.h, ctypes.byref(p), ctypes.byref(r)))
        return p.value, r.value

    def tuning(self):
        la, bp, ms = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_float(0)
        self._check(self.lib.gvx_batch_get_tuning(self.h, ctypes.byref(la), ctypes.byref(bp), ctypes.byref(ms)))
        return {"slab_layers": la.value, "blocks_per_sm": bp.value, "ms": ms.value}

    def kernel_launches(self):
        c = ctypes.c_int64()
        self._check(self.lib.gvx_batch_kernel_launches(self.h, ctypes.byref(c)))
        return c.value
