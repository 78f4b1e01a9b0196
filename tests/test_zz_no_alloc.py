"""GPU test of gvx_radix_sort_noalloc, the sort entry point for callers that
cannot allocate device memory (their host hands the library a fixed memory
budget, or owns every device allocation itself).

It must give exactly what gvx_radix_sort (which allocates its scratch on
first use) gives, on consecutive calls that reuse its static scratch array.
This file is collected last so that a run stopping at its first failure has
already run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_KEYS = 1 << 18  # GVX_NOALLOC_SORT_MAX_KEYS in include/gvx.h


def _sort_both(gvx_mod, torch, grid, keys, vals, bits):
    n = len(keys)
    kd = torch.from_numpy(keys.view(np.int32)).cuda()
    vd = torch.from_numpy(vals.view(np.int32)).cuda()
    ko_ref, vo_ref = torch.empty_like(kd), torch.empty_like(vd)
    ko, vo = torch.full_like(kd, -1), torch.full_like(vd, -1)
    gvx_mod.radix_sort(grid, kd, vd, ko_ref, vo_ref, n, bits)
    grid.sync()
    st = grid.lib.gvx_radix_sort_noalloc(kd.data_ptr(), vd.data_ptr(), ko.data_ptr(), vo.data_ptr(), n, bits,
                                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, grid.lib.gvx_last_error().decode()
    torch.cuda.synchronize()
    return (ko.cpu().numpy().view(np.uint32), vo.cpu().numpy().view(np.uint32),
            ko_ref.cpu().numpy().view(np.uint32), vo_ref.cpu().numpy().view(np.uint32))


def test_noalloc_sort_matches_allocating_sort_twice(gvx_mod):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(17)
    grid = gvx_mod.Grid(0)
    # two calls in a row: the second starts from the first one's leftover scratch
    for n, bits in ((200_000, 21), (MAX_KEYS, 27)):
        keys = rng.integers(0, 1 << bits, n, dtype=np.uint64).astype(np.uint32)
        vals = rng.permutation(n).astype(np.uint32)
        ko, vo, kr, vr = _sort_both(gvx_mod, torch, grid, keys, vals, bits)
        assert np.array_equal(ko, kr) and np.array_equal(vo, vr)
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(ko, keys[order]) and np.array_equal(vo, vals[order])
    grid.close()


def test_noalloc_sort_in_place(gvx_mod):
    """Sorting in place: with an odd pass count (bits 17..24 -> 3 passes) the
    first pass writes the output, which here is the input itself."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(23)
    grid = gvx_mod.Grid(0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for n, bits in ((150_000, 21), (MAX_KEYS, 16), (70_001, 5)):
        keys = rng.integers(0, 1 << bits, n, dtype=np.uint64).astype(np.uint32)
        vals = rng.permutation(n).astype(np.uint32)
        kd = torch.from_numpy(keys.view(np.int32)).cuda()
        vd = torch.from_numpy(vals.view(np.int32)).cuda()
        st = grid.lib.gvx_radix_sort_noalloc(kd.data_ptr(), vd.data_ptr(), kd.data_ptr(), vd.data_ptr(), n, bits,
                                             stream)
        assert st == 0, grid.lib.gvx_last_error().decode()
        assert grid.lib.gvx_radix_sort_noalloc_status(stream) == 0
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(kd.cpu().numpy().view(np.uint32), keys[order])
        assert np.array_equal(vd.cpu().numpy().view(np.uint32), vals[order])
    # the two outputs must not overlap
    kd = torch.zeros(1000, dtype=torch.int32, device="cuda")
    st = grid.lib.gvx_radix_sort_noalloc(kd.data_ptr(), kd.data_ptr(), kd.data_ptr(), kd.data_ptr() + 400, 1000,
                                         10, stream)
    assert st == 1  # GVX_ERR_INVALID_ARG
    grid.close()


def test_noalloc_sort_reports_a_timed_out_wait(gvx_mod):
    """A look-back wait that runs out (first tile withheld by the test hook,
    no GPU fault) is reported by gvx_radix_sort_noalloc_status, once; the next
    sort on the same static scratch is correct."""
    torch = pytest.importorskip("torch")
    lib = gvx_mod.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    n = 40_000
    rng = np.random.default_rng(5)
    keys = rng.integers(0, 1 << 8, n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    kd = torch.from_numpy(keys.view(np.int32)).cuda()
    vd = torch.from_numpy(vals.view(np.int32)).cuda()
    ko, vo = torch.empty_like(kd), torch.empty_like(vd)
    assert lib.gvx_radix_sort_noalloc_status(stream) == 0
    st = lib.gvx_test_sort_noalloc_withheld_tile(kd.data_ptr(), vd.data_ptr(), ko.data_ptr(), vo.data_ptr(), n,
                                                 stream)
    assert st == 0, lib.gvx_last_error().decode()
    assert lib.gvx_radix_sort_noalloc_status(stream) == 5  # GVX_ERR_TIMEOUT
    assert b"look-back" in lib.gvx_last_error()
    assert lib.gvx_radix_sort_noalloc_status(stream) == 0  # read once, then clear
    st = lib.gvx_radix_sort_noalloc(kd.data_ptr(), vd.data_ptr(), ko.data_ptr(), vo.data_ptr(), n, 8, stream)
    assert st == 0
    assert lib.gvx_radix_sort_noalloc_status(stream) == 0
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(ko.cpu().numpy().view(np.uint32), keys[order])
    assert np.array_equal(vo.cpu().numpy().view(np.uint32), vals[order])


def test_noalloc_sort_rejects_sizes_beyond_its_scratch(gvx_mod):
    torch = pytest.importorskip("torch")
    lib = gvx_mod.load()
    n = MAX_KEYS + 1
    kd = torch.zeros(n, dtype=torch.int32, device="cuda")
    out = torch.zeros(n, dtype=torch.int32, device="cuda")
    st = lib.gvx_radix_sort_noalloc(kd.data_ptr(), kd.data_ptr(), out.data_ptr(), out.data_ptr(), n, 20, None)
    assert st == 3  # GVX_ERR_CAPACITY
    assert b"static scratch limit" in lib.gvx_last_error()
