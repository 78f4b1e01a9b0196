"""GPU test of the double-buffered host commit (CommitData of host points): the
points of frame k+1 are committed from pinned host memory while frame k's
splat still runs, before frame k's results are read back.  Each frame must
come out bit for bit as on a fresh grid that ran the same frame alone, and the
serial order (commit, frame, read) must give the same results too.  One frame
commits strided records, so the staged copy and its packing kernel run on the
side stream as well."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LOGDIM = (3, 3, 3, 3, 5)
RADIUS = 2.0


def frames(count, n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        centres = rng.random((6, 3)) * 300.0 + 40.0
        pos = centres[rng.integers(0, 6, n)] + rng.normal(0.0, 9.0 + 2.0 * k, (n, 3))
        vel = rng.normal(0.0, 1.0, (n, 3))
        w = rng.random(n) + 0.5
        out.append((np.abs(pos).astype(np.float32), vel.astype(np.float32), w.astype(np.float32)))
    return out


def new_grid(gvx):
    g = gvx.Grid(0)
    g.configure(LOGDIM)
    g.add_channel(0, gvx.T_FLOAT, 1)
    g.add_channel(1, gvx.T_FLOAT3, 1)
    return g


def run_frame(g, gvx, n):
    g.rebuild_topology(n, RADIUS, mode=gvx.TOPO_FULL)
    g.finish_topology()
    g.update_atlas()
    g.insert_points(n)
    g.splat(gvx.SPLAT_CUBIC, n, RADIUS, chan_density=0, chan_vel=1)
    g.update_apron(0, 0.0)
    g.update_apron(1, 0.0)


def results(g):
    # the atlas only grows: a grid that ran a larger frame before holds more (unused) slots
    inf = g.info()
    used = inf["used_leaves"]
    return ([g.read_nodes(lev) for lev in range(inf["root_level"] + 1)], g.read_atlas_map()[:used],
            g.read_channel(0)[:used], g.read_channel(1)[:used])


def assert_same(a, b, k):
    for lev, (x, y) in enumerate(zip(a[0], b[0])):
        assert np.array_equal(x, y), "frame %d level %d nodes" % (k, lev)
    assert np.array_equal(a[1], b[1]), "frame %d atlas map" % k
    for c in (2, 3):
        assert np.array_equal(a[c].view(np.uint32), b[c].view(np.uint32)), "frame %d channel %d" % (k, c - 2)


def commit_pinned(g, host, k):
    pos, vel, w = host[k]
    lib = g.lib
    n = pos.shape[0]
    stride = pos.stride(0) * 4
    st = lib.gvx_commit_points_host(g.h, n, pos.data_ptr(), stride, vel.data_ptr(), 12, w.data_ptr(), None)
    g._check(st)


def pinned_frames(fr, n, strided_frame):
    import torch

    host = []
    for k, (pos, vel, w) in enumerate(fr):
        if k == strided_frame:  # float4 records, the fourth float ignored
            p = torch.zeros((n, 4), dtype=torch.float32, pin_memory=True)
            p[:, :3].copy_(torch.from_numpy(pos))
            p[:, 3] = -1.0
        else:
            p = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
            p.copy_(torch.from_numpy(pos))
        v = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
        v.copy_(torch.from_numpy(vel))
        ww = torch.empty(n, dtype=torch.float32, pin_memory=True)
        ww.copy_(torch.from_numpy(w))
        host.append((p, v, ww))
    return host


def fresh_results(gvx_mod, fr, n):
    expect = []
    for pos, vel, w in fr:
        f = new_grid(gvx_mod)
        f.commit_points_host(pos, vel=vel, weight=w)
        run_frame(f, gvx_mod, n)
        expect.append(results(f))
        f.close()
    return expect


def test_pipelined_commits_match_fresh_frames(gvx_mod):
    n = 300_000
    fr = frames(4, n, seed=11)
    strided_frame = 2
    host = pinned_frames(fr, n, strided_frame)
    expect = fresh_results(gvx_mod, fr, n)

    # pipelined: frame k+1 committed after frame k's work is queued, before its readback
    g = new_grid(gvx_mod)
    commit_pinned(g, host, 0)
    for k in range(len(fr)):
        run_frame(g, gvx_mod, n)
        if k + 1 < len(fr):
            commit_pinned(g, host, k + 1)
        assert_same(results(g), expect[k], k)
    g.close()

    # serial order on one grid, twice through the frames (both buffer sets reused)
    g = new_grid(gvx_mod)
    for rep in range(2):
        for k in range(len(fr)):
            commit_pinned(g, host, k)
            run_frame(g, gvx_mod, n)
            assert_same(results(g), expect[k], k)
    g.close()


def test_pipelined_commits_on_a_caller_stream(gvx_mod):
    """the same pipelined order with the grid on a caller's stream (gvx_set_stream): the
    buffer-set events are recorded on that stream"""
    import torch

    n = 200_000
    fr = frames(3, n, seed=12)
    host = pinned_frames(fr, n, -1)
    expect = fresh_results(gvx_mod, fr, n)
    s = torch.cuda.Stream()
    g = new_grid(gvx_mod)
    g.set_stream(s.cuda_stream)
    for rep in range(2):
        commit_pinned(g, host, 0)
        for k in range(len(fr)):
            run_frame(g, gvx_mod, n)
            if k + 1 < len(fr):
                commit_pinned(g, host, k + 1)
            assert_same(results(g), expect[k], k)
    g.close()
