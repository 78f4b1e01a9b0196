"""A reader of VBX files written independently of libgvx, in the field order of
the reference's LoadVBX (gvdb_volume_gvdb.cpp:507-686): the tests check the
files libgvx writes against it."""
import struct

import numpy as np

NODE = np.dtype([("lev", "u1"), ("flags", "u1"), ("prio", "u1"), ("pad", "u1"), ("pos", "<i4", (3,)),
                 ("value", "<i4", (3,)), ("vrange", "<f4", (3,)), ("parent", "<u8"), ("childlist", "<u8"),
                 ("mask", "<u8")])
VOXEL = {0: (np.uint8, 1), 2: (np.uint8, 4), 3: (np.float32, 1), 4: (np.float32, 3), 5: (np.float32, 4)}


class Reader:
    def __init__(self, data):
        self.d, self.o = data, 0

    def take(self, fmt):
        v = struct.unpack_from("<" + fmt, self.d, self.o)
        self.o += struct.calcsize("<" + fmt)
        return v if len(v) > 1 else v[0]

    def raw(self, n):
        b = self.d[self.o:self.o + n]
        self.o += n
        return b


def read_vbx(path):
    r = Reader(open(path, "rb").read())
    f = {"major": r.take("B"), "minor": r.take("B")}
    if (f["major"] == 1 and f["minor"] >= 11) or f["major"] > 1:
        f["transform"] = [r.take("3f") for _ in range(4)]
    f["num_grids"] = r.take("i")
    if f["major"] >= 2:
        f["masks"] = r.take("B")
    f["grid_offsets"] = [r.take("Q") for _ in range(f["num_grids"])]
    grids = []
    for _ in range(f["num_grids"]):
        assert r.o == f["grid_offsets"][len(grids)]
        g = {"name": r.raw(256), "dtype": r.take("B"), "components": r.take("B"), "compression": r.take("B"),
             "voxel_size": r.take("3f"), "leaf_count": r.take("i"), "brick_dims": r.take("3i"),
             "apron": r.take("i"), "channels": r.take("i"), "atlas_bytes": r.take("Q"),
             "topology_type": r.take("B"), "reuse": r.take("i"), "layout": r.take("B"),
             "atlas_bricks": r.take("3i"), "atlas_res": r.take("3i"), "levels": r.take("i"), "root": r.take("Q")}
        g["level_table"] = []
        for _ in range(g["levels"]):
            g["level_table"].append({"log2dim": r.take("i"), "res": r.take("i"), "range": r.take("3i"),
                                     "count0": r.take("i"), "width0": r.take("i"), "count1": r.take("i"),
                                     "width1": r.take("i")})
        g["nodes"] = []
        for lt in g["level_table"]:
            rows = np.frombuffer(r.raw(lt["count0"] * lt["width0"]), np.uint8).reshape(lt["count0"], lt["width0"])
            g["nodes"].append(np.frombuffer(rows[:, :64].tobytes(), NODE))
        g["childlists"] = []
        for lt in g["level_table"]:
            g["childlists"].append(np.frombuffer(r.raw(lt["count1"] * lt["width1"]), "<u8"))
        X, Y, Z = g["atlas_res"]
        g["atlas"] = []
        for _ in range(g["channels"]):
            typ, stride = r.take("i"), r.take("i")
            dt, nc = VOXEL[typ]
            assert stride == np.dtype(dt).itemsize * nc
            a = np.frombuffer(r.raw(X * Y * Z * stride), dt).reshape((Z, Y, X) + ((nc,) if nc > 1 else ()))
            g["atlas"].append((typ, a))
        grids.append(g)
    f["grids"] = grids
    f["trailing_bytes"] = len(r.d) - r.o
    return f
