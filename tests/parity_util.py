"""Comparison helpers shared by the parity tests."""
import numpy as np

NODE_FIELDS = ("lev", "flags", "pos", "value", "parent", "childlist")

# FP32 densities vs the FP64 oracle: |a-b| / (|b| + FLOOR * max|b|) <= TOL
DENSITY_TOL = 1e-5
DENSITY_FLOOR = 1e-6


def assert_nodes_equal(a, b, level, fields=NODE_FIELDS):
    assert len(a) == len(b), "level %d: %d nodes vs %d in the oracle" % (level, len(a), len(b))
    for f in fields:
        if not np.array_equal(a[f], b[f]):
            bad = np.nonzero(np.any((a[f] != b[f]).reshape(len(a), -1), axis=1))[0]
            i = int(bad[0])
            raise AssertionError("level %d field %s differs at %d nodes; first %d: %r vs %r"
                                 % (level, f, len(bad), i, a[i][f], b[i][f]))


def rel_error(got, ref, floor=DENSITY_FLOOR):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    scale = max(float(np.abs(ref).max()), 1e-30)
    return float((np.abs(got - ref) / (np.abs(ref) + floor * scale)).max())


def rel_error_significant(got, ref, frac=1e-3):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    scale = max(float(np.abs(ref).max()), 1e-30)
    m = np.abs(ref) >= frac * scale
    if not m.any():
        return 0.0
    return float((np.abs(got[m] - ref[m]) / np.abs(ref[m])).max())


def compare_topology(g, o, check_childlists=True):
    inf = g.info()
    assert inf["root_level"] == o.root_level()
    for lev in range(o.root_level() + 1):
        assert inf["node_count"][lev] == o.num_nodes(lev), "level %d count" % lev
        assert_nodes_equal(g.read_nodes(lev), o.nodes(lev), lev)
        if check_childlists and lev > 0:
            a, b = g.read_childlist(lev), o.childlist(lev)
            assert np.array_equal(a, b), "level %d child lists differ at %d slots" % (lev, int((a != b).sum()))
    assert inf["used_leaves"] == o.used_leaves()


def leaf_slots(nodes, subdim, P):
    """atlas slot of every level-0 node from its mValue (the atlas voxel of its
    interior corner): slot = (bz * sy + by) * sx + bx, -1 without a slot"""
    v = np.asarray(nodes["value"], np.int64)
    b = v // P
    slot = (b[:, 2] * subdim[1] + b[:, 1]) * subdim[0] + b[:, 0]
    return np.where(v[:, 0] < 0, -1, slot)
