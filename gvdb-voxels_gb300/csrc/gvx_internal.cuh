// gvx_internal.cuh -- shared declarations of the libgvx CUDA sources.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "gvx.h"

#define GVX_MAXLEV 10
#define GVX_MAXCH 32

#define ID_UNDEFL_U64 0xFFFFFFFFull          // ID_UNDEFL (gvdb_types.h:55) stored in 64 bits
#define ID_UNDEF64_U64 0xFFFFFFFFFFFFFFFFull // ID_UNDEF64 (gvdb_types.h:56)
#define GVX_NOHIT 1.0e10f                    // NOHIT (gvdb_types.h:53)

// device error word bits
#define GVX_DERR_TIMEOUT 1u      // a bounded spin-wait gave up
#define GVX_DERR_CAPACITY 2u     // a kernel found more items than its buffer holds
#define GVX_DERR_DEGENERATE 4u   // a node lies outside the root / a level-0 key domain
#define GVX_DERR_BADPOINT 8u     // NaN position
#define GVX_DERR_RADIUS 16u      // a per-point splat radius reaches past the 26 neighbouring bricks

// 64-byte node record, layout of VDBNode (cuda_gvdb_nodes.cuh:24-35) / Node (gvdb_node.h:27-40)
struct __align__(16) GvxNode {
    uint8_t lev, flags, prio, pad;
    int32_t pos[3];
    int32_t value[3];
    float vrange[3];
    uint64_t parent;
    uint64_t childlist;
    uint64_t mask;
};
static_assert(sizeof(GvxNode) == 64, "node layout");

// Compact level-0 key space of one topology build: leaf coordinates relative to
// `lo` (aligned to the level depth-1 node size), `bits[a]` bits per axis, packed
// x-major: key = (x << (by+bz)) | (y << bz) | z, so key order is the reference's
// (x, y, z) node order.  Level-l coordinates are the level-0 ones >> shift_l.
struct KeySpace {
    int lo[3];       // absolute leaf coordinates of compact (0,0,0)
    int bits[3];     // per-axis bits at level 0
    int total_bits;  // bx + by + bz
};

__host__ __device__ inline uint32_t ks_pack(const KeySpace& ks, int cx, int cy, int cz, int shift)
{
    int by = ks.bits[1] > shift ? ks.bits[1] - shift : 0;
    int bz = ks.bits[2] > shift ? ks.bits[2] - shift : 0;
    return ((uint32_t)cx << (by + bz)) | ((uint32_t)cy << bz) | (uint32_t)cz;
}
__host__ __device__ inline void ks_unpack(const KeySpace& ks, uint32_t key, int shift, int* c)
{
    int by = ks.bits[1] > shift ? ks.bits[1] - shift : 0;
    int bz = ks.bits[2] > shift ? ks.bits[2] - shift : 0;
    c[2] = (int)(key & ((1u << bz) - 1u));
    c[1] = (int)((key >> bz) & ((1u << by) - 1u));
    c[0] = (int)(key >> (by + bz));
}
__host__ __device__ inline int ks_bits_at(const KeySpace& ks, int shift)
{
    int t = 0;
    for (int a = 0; a < 3; a++) t += ks.bits[a] > shift ? ks.bits[a] - shift : 0;
    return t;
}
__host__ __device__ inline int ks_extent(const KeySpace& ks, int a, int shift)
{
    return 1 << (ks.bits[a] > shift ? ks.bits[a] - shift : 0);
}

// A set of keys held as a bitmap with per-word exclusive prefix popcounts
// (rank in O(1)).
// Work units 0 .. total-1 handed to the warps of a persistent launch from a
// counter (zeroed before the launch): kUnitClaim consecutive units per atomic,
// the warp's next claim requested before it works through the current one, so
// that its latency is hidden.  For launches of many units of even cost (the
// subcell gathers: 1.77 -> 1.64 ms on 1.68M subcells); where costly units
// cluster, whole claims held by one warp leave others idle at the end.  The
// counter may run past `total` by a few claims per warp: totals stay below 2^31.
constexpr uint32_t kUnitClaim = 4;
struct WarpUnits {
    uint32_t cur = 0, lim = 0, pre = 0;
    __device__ explicit WarpUnits(uint32_t* counter, int lane)
    {
        if (lane == 0) pre = atomicAdd(counter, kUnitClaim);
    }
    // the warp's next unit (warp-uniform), false when the work is done
    __device__ bool next(uint32_t* counter, uint32_t total, int lane, uint32_t& u)
    {
        if (cur == lim) {
            cur = __shfl_sync(0xFFFFFFFFu, pre, 0);
            lim = cur + kUnitClaim;
            if (cur >= total) return false;
            if (lane == 0) pre = atomicAdd(counter, kUnitClaim);
        }
        if (cur >= total) return false;
        u = cur++;
        return true;
    }
};

// A count a kernel takes either from the host (p null) or from device memory
// (p[i0] + p[i1], i1 < 0 for none), clamped to `cap` (the capacity of the
// buffers it sizes): launches enqueued before the count is known on the host
// (the planned builds of batched grids) stay inside their buffers whatever
// the count turns out to be.
struct DevCount {
    const uint32_t* p;
    int i0, i1;
    uint32_t host, cap;
    __device__ uint32_t get() const
    {
        if (!p) return host;
        const uint32_t v = p[i0] + (i1 >= 0 ? p[i1] : 0u);
        return v < cap ? v : cap;
    }
};
inline DevCount dc_host(uint32_t n) { return DevCount{nullptr, 0, -1, n, n}; }
inline DevCount dc_dev(const uint32_t* p, int i0, int i1, uint32_t cap) { return DevCount{p, i0, i1, 0u, cap}; }

struct BitRank {
    uint32_t* bits;
    uint32_t* prefix;
    uint32_t words;
};
__device__ inline bool br_test(const BitRank& b, uint32_t key)
{
    return (b.bits[key >> 5] >> (key & 31)) & 1u;
}
__device__ inline uint32_t br_rank(const BitRank& b, uint32_t key)
{
    uint32_t w = b.bits[key >> 5] & ((1u << (key & 31)) - 1u);
    return b.prefix[key >> 5] + __popc(w);
}

// host-side growable device buffer
struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    template <class T> T* as() const { return (T*)p; }
};

// error reporting helpers (gvx_api.cu)
void gvx_set_error(const char* fmt, ...);
gvx_status gvx_cuda_fail(cudaError_t e, const char* what);
#define GVX_CK(call)                                                   \
    do {                                                               \
        cudaError_t _e = (call);                                       \
        if (_e != cudaSuccess) return gvx_cuda_fail(_e, #call);        \
    } while (0)

#define GVX_CK_STATUS(call)             \
    do {                                \
        gvx_status _s = (call);         \
        if (_s != GVX_OK) return _s;    \
    } while (0)

cudaError_t gvx_ensure(DevBuf& b, size_t bytes);
void gvx_free(DevBuf& b);
// Device allocations and frees made by gvx_ensure / gvx_free in this process (a
// captured CUDA graph holds buffer addresses: it is replayed only while no
// buffer has moved since its capture).
uint64_t gvx_alloc_epoch();
// While alive, gvx_ensure on this thread fails (cudaErrorNotPermitted) instead of
// allocating: work queued inside a stream capture must find its buffers sized.
struct GvxNoAllocScope {
    GvxNoAllocScope();
    ~GvxNoAllocScope();
    bool prev;
};

// ---- onesweep radix sort (gvx_sort.cu) -----------------------------------
struct SortScratch {
    DevBuf hist;      // passes * 256 counts
    DevBuf base;      // passes * 256 exclusive bases
    DevBuf lookback;  // tiles * 256 status words
    DevBuf counter;   // tile counters, one per pass
};
// one sort pass with its first tile withheld: the bounded look-back times out (a test hook)
gvx_status gvx_sort_pass_withheld_tile(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout,
                                       uint32_t n, SortScratch& s, cudaStream_t st, uint32_t* d_err,
                                       int64_t* launches);
// Sorts (keys, vals) by the low `bits` bits of the keys, stable.  The keys
// must already be in keys[0]/vals[0]; the result ends in buffer index *result
// (0 or 1).  If the histogram of the pass digits was accumulated by the
// producer of the keys (hist_ready), it is used as is.
gvx_status gvx_sort_pairs(uint32_t* keys[2], uint32_t* vals[2], uint32_t n, int bits, SortScratch& s,
                          bool hist_ready, cudaStream_t st, uint32_t* d_err, int* result, int64_t* launches);
int gvx_sort_passes(int bits);
// zero the global histogram before a fused key producer accumulates into it
gvx_status gvx_sort_prepare_hist(SortScratch& s, int bits, cudaStream_t st);
uint32_t* gvx_sort_hist_ptr(SortScratch& s);

// device helper used by key producers: accumulate digit histograms of a key
// into the shared histogram `sh` (passes * 256 uint32)
__device__ inline void gvx_sort_count_key(uint32_t* sh, uint32_t key, int passes)
{
    for (int p = 0; p < passes; p++) atomicAdd(&sh[p * 256 + ((key >> (8 * p)) & 255u)], 1u);
}

// ---- generic exclusive scan of popcounts of a bitmap (gvx_topology.cu) -----
gvx_status gvx_bitmap_prefix(const uint32_t* bits, uint32_t* prefix, uint32_t words, uint32_t* total,
                             DevBuf& tmp, cudaStream_t st, int64_t* launches);
// exclusive scan of n uint32 values (in -> out, may not alias), total -> *total if non-null
gvx_status gvx_scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* total, DevBuf& tmp,
                        cudaStream_t st, int64_t* launches);
