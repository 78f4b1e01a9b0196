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
