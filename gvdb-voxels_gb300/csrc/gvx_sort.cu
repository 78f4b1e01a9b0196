// gvx_sort.cu -- hand-written onesweep LSD radix sort of 32-bit brick keys.
//
// Replaces the reference's thrust::sort of 64-bit keys (gvdb_cutils.cu:11-16,
// called from VolumeGVDB::RadixSortByByte, gvdb_volume_gvdb.cpp:904-928).
// Only the significant bits of the compact brick key are sorted (8 bits per
// pass), the digit histograms of all passes come from one upfront count (fused
// into the key producer when it can), and every pass is a single kernel: tile
// ranking with warp match_any, decoupled look-back across tiles for the digit
// offsets, then a scatter staged through shared memory so that global writes
// of one digit bucket are contiguous.  Stable: equal keys keep input order.
//
// Every look-back wait is bounded: after ~2 s of polling the kernel records
// GVX_DERR_TIMEOUT in the device error word and carries on, so a lost
// predecessor can never hang the GPU.
#include "gvx_internal.cuh"

namespace {
constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;  // 4096 keys per tile
constexpr int kWarps = kThreads / 32;
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kFlagMask = 3u << 30;
constexpr uint32_t kCountMask = (1u << 30) - 1u;
constexpr long long kSpinCycles = 4000000000LL;
}  // namespace

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v)
{
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__global__ void k_sort_hist(const uint32_t* __restrict__ keys, uint32_t n, int passes, uint32_t* hist)
{
    __shared__ uint32_t sh[4 * 256];
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) sh[i] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        gvx_sort_count_key(sh, keys[i], passes);
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x)
        if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// exclusive scan of every pass histogram: one block of 256 threads per pass
__global__ void k_sort_bases(const uint32_t* __restrict__ hist, uint32_t* __restrict__ base)
{
    __shared__ uint32_t s[256];
    const int p = blockIdx.x, t = threadIdx.x;
    const uint32_t v = hist[p * 256 + t];
    s[t] = v;
    __syncthreads();
    for (int off = 1; off < 256; off <<= 1) {
        uint32_t x = t >= off ? s[t - off] : 0u;
        __syncthreads();
        s[t] += x;
        __syncthreads();
    }
    base[p * 256 + t] = s[t] - v;
}

// 4 resident tiles per SM (registers capped at 64): unbounded, the compiler's register use left room
// for one tile per SM and a 32M-key sort took 1.7 ms instead of 1.0 ms
__global__ void __launch_bounds__(kThreads, 4) k_onesweep(const uint32_t* __restrict__ kin,
                                                       const uint32_t* __restrict__ vin,
                                                       uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                       uint32_t n, int shift, const uint32_t* __restrict__ base,
                                                       uint32_t* lookback, uint32_t* counter, uint32_t* err)
{
    __shared__ uint32_t s_whist[kWarps][256];
    __shared__ uint32_t s_tstart[256];
    __shared__ uint32_t s_gstart[256];
    __shared__ uint32_t s_keys[kTile];
    __shared__ uint32_t s_vals[kTile];
    __shared__ uint32_t s_wsum[kWarps];
    __shared__ uint32_t s_tile;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(counter, 1u);
    for (int i = tid; i < kWarps * 256; i += kThreads) (&s_whist[0][0])[i] = 0u;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t tbase = tile * (uint32_t)kTile;
    const uint32_t wbase = tbase + (uint32_t)warp * 32u * kItems;

    uint32_t k[kItems], v[kItems];
    uint32_t r[kItems];
#pragma unroll
    for (int j = 0; j < kItems; j++) {
        const uint32_t idx = wbase + (uint32_t)j * 32u + lane;
        if (idx < n) {
            k[j] = kin[idx];
            v[j] = vin[idx];
        } else {
            k[j] = 0xFFFFFFFFu;
            v[j] = 0u;
        }
    }
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int j = 0; j < kItems; j++) {
        const uint32_t idx = wbase + (uint32_t)j * 32u + lane;
        const bool valid = idx < n;
        const uint32_t d = (k[j] >> shift) & 255u;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, valid ? d : 256u);
        const int leader = __ffs(peers) - 1;
        uint32_t prev = 0u;
        if (lane == leader && valid) {
            prev = s_whist[warp][d];
            s_whist[warp][d] = prev + __popc(peers);
        }
        prev = __shfl_sync(0xFFFFFFFFu, prev, leader);
        r[j] = prev + __popc(peers & lt);
        __syncwarp();
    }
    __syncthreads();

    // thread `tid` owns digit `tid`: per-warp offsets, tile count, look-back
    uint32_t cnt = 0u;
#pragma unroll
    for (int w = 0; w < kWarps; w++) {
        const uint32_t c = s_whist[w][tid];
        s_whist[w][tid] = cnt;
        cnt += c;
    }
    uint32_t* my = lookback + (size_t)tile * 256u + tid;
    uint32_t excl = 0u;
    if (tile == 0) {
        st_relaxed(my, kFlagPrefix | cnt);
    } else {
        st_relaxed(my, kFlagAgg | cnt);
        int t = (int)tile - 1;
        const long long t0 = clock64();
        while (t >= 0) {
            const uint32_t w = ld_relaxed(lookback + (size_t)t * 256u + tid);
            const uint32_t f = w & kFlagMask;
            if (f == 0u) {
                if (clock64() - t0 > kSpinCycles) {
                    atomicOr(err, GVX_DERR_TIMEOUT);
                    break;
                }
                continue;
            }
            excl += w & kCountMask;
            if (f == kFlagPrefix) break;
            t--;
        }
        st_relaxed(my, kFlagPrefix | ((excl + cnt) & kCountMask));
    }
    s_gstart[tid] = base[tid] + excl;

    // exclusive scan of the tile counts over the 256 digits
    uint32_t x = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_wsum[warp] = x;
    __syncthreads();
    uint32_t wpre = 0u;
    for (int w = 0; w < warp; w++) wpre += s_wsum[w];
    s_tstart[tid] = wpre + x - cnt;
    __syncthreads();

    // stage the tile in digit order
#pragma unroll
    for (int j = 0; j < kItems; j++) {
        const uint32_t idx = wbase + (uint32_t)j * 32u + lane;
        if (idx < n) {
            const uint32_t d = (k[j] >> shift) & 255u;
            const uint32_t pos = s_tstart[d] + s_whist[warp][d] + r[j];
            s_keys[pos] = k[j];
            s_vals[pos] = v[j];
        }
    }
    __syncthreads();
    const uint32_t cnt_tile = min((uint32_t)kTile, n - tbase);
    for (uint32_t i = tid; i < cnt_tile; i += kThreads) {
        const uint32_t key = s_keys[i];
        const uint32_t d = (key >> shift) & 255u;
        const uint32_t g = s_gstart[d] + (i - s_tstart[d]);
        kout[g] = key;
        vout[g] = s_vals[i];
    }
}

int gvx_sort_passes(int bits) { return bits <= 0 ? 0 : (bits + 7) / 8; }

uint32_t* gvx_sort_hist_ptr(SortScratch& s) { return s.hist.as<uint32_t>(); }

gvx_status gvx_sort_prepare_hist(SortScratch& s, int bits, cudaStream_t st)
{
    (void)bits;
    GVX_CK(gvx_ensure(s.hist, 4 * 256 * sizeof(uint32_t)));
    GVX_CK(cudaMemsetAsync(s.hist.p, 0, 4 * 256 * sizeof(uint32_t), st));
    return GVX_OK;
}

gvx_status gvx_sort_pairs(uint32_t* keys[2], uint32_t* vals[2], uint32_t n, int bits, SortScratch& s,
                          bool hist_ready, cudaStream_t st, uint32_t* d_err, int* result, int64_t* launches)
{
    *result = 0;
    const int passes = gvx_sort_passes(bits);
    if (n <= 1 || passes == 0) return GVX_OK;
    if (passes > 4) {
        gvx_set_error("sort: %d key bits exceed 32", bits);
        return GVX_ERR_INVALID_ARG;
    }
    if (n > kCountMask) {
        gvx_set_error("sort: %u keys exceed the 2^30 limit", n);
        return GVX_ERR_CAPACITY;
    }
    const uint32_t tiles = (n + kTile - 1) / kTile;
    GVX_CK(gvx_ensure(s.hist, 4 * 256 * sizeof(uint32_t)));
    GVX_CK(gvx_ensure(s.base, 4 * 256 * sizeof(uint32_t)));
    GVX_CK(gvx_ensure(s.lookback, (size_t)passes * tiles * 256 * sizeof(uint32_t)));
    GVX_CK(gvx_ensure(s.counter, 4 * sizeof(uint32_t)));
    if (!hist_ready) {
        GVX_CK(cudaMemsetAsync(s.hist.p, 0, 4 * 256 * sizeof(uint32_t), st));
        const uint32_t blocks = tiles < 1024 ? tiles : 1024;
        k_sort_hist<<<blocks, 256, 0, st>>>(keys[0], n, passes, s.hist.as<uint32_t>());
        (*launches)++;
    }
    k_sort_bases<<<passes, 256, 0, st>>>(s.hist.as<uint32_t>(), s.base.as<uint32_t>());
    (*launches)++;
    GVX_CK(cudaMemsetAsync(s.lookback.p, 0, (size_t)passes * tiles * 256 * sizeof(uint32_t), st));
    GVX_CK(cudaMemsetAsync(s.counter.p, 0, 4 * sizeof(uint32_t), st));
    int cur = 0;
    for (int p = 0; p < passes; p++) {
        k_onesweep<<<tiles, kThreads, 0, st>>>(keys[cur], vals[cur], keys[cur ^ 1], vals[cur ^ 1], n, 8 * p,
                                              s.base.as<uint32_t>() + p * 256,
                                              s.lookback.as<uint32_t>() + (size_t)p * tiles * 256,
                                              s.counter.as<uint32_t>() + p, d_err);
        (*launches)++;
        cur ^= 1;
    }
    GVX_CK(cudaGetLastError());
    *result = cur;
    return GVX_OK;
}

// One pass of the sort with its first tile withheld (a test of the bounded
// look-back): the tile counter starts at 1 and tiles - 1 blocks run, so every
// block takes a tile in range, and the tile after the withheld one waits for a
// flag that nothing sets.  Its wait gives up after kSpinCycles and records
// GVX_DERR_TIMEOUT; it then publishes the prefix it has (a lower bound of the
// true one, so every scatter index stays below n) and the later tiles finish.
gvx_status gvx_sort_pass_withheld_tile(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout,
                                       uint32_t n, SortScratch& s, cudaStream_t st, uint32_t* d_err,
                                       int64_t* launches)
{
    const uint32_t tiles = (n + kTile - 1) / kTile;
    if (tiles < 2) {
        gvx_set_error("sort test: %u keys make one tile; at least two are needed", n);
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(gvx_ensure(s.hist, 4 * 256 * sizeof(uint32_t)));
    GVX_CK(gvx_ensure(s.base, 4 * 256 * sizeof(uint32_t)));
    GVX_CK(gvx_ensure(s.lookback, (size_t)tiles * 256 * sizeof(uint32_t)));
    GVX_CK(gvx_ensure(s.counter, 4 * sizeof(uint32_t)));
    GVX_CK(cudaMemsetAsync(s.hist.p, 0, 4 * 256 * sizeof(uint32_t), st));
    k_sort_hist<<<tiles < 1024 ? tiles : 1024, 256, 0, st>>>(kin, n, 1, s.hist.as<uint32_t>());
    k_sort_bases<<<1, 256, 0, st>>>(s.hist.as<uint32_t>(), s.base.as<uint32_t>());
    GVX_CK(cudaMemsetAsync(s.lookback.p, 0, (size_t)tiles * 256 * sizeof(uint32_t), st));
    static const uint32_t one = 1u;
    GVX_CK(cudaMemcpyAsync(s.counter.p, &one, sizeof(one), cudaMemcpyHostToDevice, st));
    k_onesweep<<<tiles - 1, kThreads, 0, st>>>(kin, vin, kout, vout, n, 0, s.base.as<uint32_t>(),
                                               s.lookback.as<uint32_t>(), s.counter.as<uint32_t>(), d_err);
    *launches += 3;
    GVX_CK(cudaGetLastError());
    return GVX_OK;
}
