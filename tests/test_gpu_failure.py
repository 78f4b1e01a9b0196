"""GPU test of failure detection without a GPU fault: a device spin-wait that
runs out.  One radix-sort pass is launched with its first tile withheld, so the
decoupled look-back of the next tile waits for a flag that nothing sets; the
wait gives up after its limit (about two seconds), the call returns a timeout
status, and the grid and the CUDA context go on working."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_sort_lookback_wait_times_out_and_the_grid_goes_on(gvx_mod):
    torch = pytest.importorskip("torch")
    g = gvx_mod.Grid(0)
    n = 20_000  # five tiles of 4096 keys
    rng = np.random.default_rng(3)
    keys_np = rng.integers(0, 1 << 20, n, dtype=np.int64).astype(np.uint32)
    keys = torch.from_numpy(keys_np.view(np.int32)).cuda()
    vals = torch.arange(n, dtype=torch.int32, device="cuda")
    ko, vo = torch.empty_like(keys), torch.empty_like(vals)
    t0 = time.perf_counter()
    st = g.lib.gvx_test_sort_withheld_tile(g.h, keys.data_ptr(), vals.data_ptr(), ko.data_ptr(), vo.data_ptr(), n)
    waited = time.perf_counter() - t0
    assert st == gvx_mod.ERR_TIMEOUT, st
    assert b"timed out" in g.lib.gvx_last_error()
    assert 0.5 < waited < 60.0
    # the same grid sorts correctly afterwards, and so does a new one
    for grid in (g, gvx_mod.Grid(0)):
        gvx_mod.radix_sort(grid, keys, vals, ko, vo, n, 20)
        grid.sync()
        order = np.argsort(keys_np, kind="stable")
        assert np.array_equal(ko.cpu().numpy().view(np.uint32), keys_np[order])
        assert np.array_equal(vo.cpu().numpy(), order.astype(np.int32))
        grid.close()


def test_injected_faults_are_status_codes_and_the_grid_goes_on(gvx_mod):
    """faults made on the host, each reported as a status with its text, none fatal: a NaN position,
    a per-point radius beyond the 26 neighbouring bricks, a stride that is not a multiple of 4 bytes,
    and a device allocation far beyond the GPU's memory; the same grid then builds and splats"""
    import ctypes

    lib = gvx_mod.load()
    g = gvx_mod.Grid(0)
    g.configure((3, 3, 3, 3, 5))
    g.add_channel(0, gvx_mod.T_FLOAT, 1)
    rng = np.random.default_rng(4)
    pts = (rng.random((5000, 3)) * 60.0 + 2.0).astype(np.float32)

    bad = pts.copy()
    bad[1234, 1] = np.nan
    g.commit_points_host(bad)
    with pytest.raises(gvx_mod.GvxError) as e:
        g.rebuild_topology(len(bad), 1.0, mode=gvx_mod.TOPO_FULL)
    assert e.value.status == 1 and "NaN" in str(e.value)

    g.commit_points_host(pts, radius=np.full(len(pts), 9.0, np.float32))  # brick 8: at most 7
    g.rebuild_topology(len(pts), 2.0, mode=gvx_mod.TOPO_FULL)
    g.update_atlas()
    g.splat(gvx_mod.SPLAT_CUBIC, len(pts), 0.0, chan_density=0)
    with pytest.raises(gvx_mod.GvxError) as e:
        g.sync()
    assert e.value.status == 6 and "radius" in str(e.value)
    g.sync()  # reported once

    st = lib.gvx_commit_points_host(g.h, len(pts), pts.ctypes.data, 14, None, 12, None, None)
    assert st == 1 and b"stride" in lib.gvx_last_error()

    ptr = ctypes.c_void_p()
    st = lib.gvx_device_alloc(0, ctypes.c_size_t(1 << 52), ctypes.byref(ptr))
    assert st == 4 and not ptr.value

    # nothing of the above sticks: the same grid builds and splats, and the next sync reports success
    g.commit_points_host(pts)
    g.rebuild_topology(len(pts), 1.0, mode=gvx_mod.TOPO_FULL)
    g.update_atlas()
    g.splat(gvx_mod.SPLAT_TRILINEAR, len(pts), 1.0, chan_density=0)
    g.sync()
    ch = g.read_channel(0)[: g.info()["used_leaves"]]
    assert abs(float(ch[:, 1:-1, 1:-1, 1:-1].astype(np.float64).sum()) - len(pts)) < 1e-2
    g.close()
