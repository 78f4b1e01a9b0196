// gvx_topology.cu -- dynamic brick topology from points, on the device.
//
// Reference path (paths relative to the reference project):
//   VolumeGVDB::RebuildTopology          gvdb_volume_gvdb.cpp:1181-1218
//   GetBoundingBox / DetermineDepth      gvdb_volume_gvdb.cpp:5404-5467, 821-837
//   ActivateBricksGPU                    gvdb_volume_gvdb.cpp:1229-1413
//   ActivateExtraBricksGPU               gvdb_volume_gvdb.cpp:931-1016
//   gvdbCalcBrickId / CalcExtraBrickId   cuda_gvdb_particles.cuh:352-382, 467-512
//   gvdbLinkBricks                       cuda_gvdb_nodes.cuh:470-505
//   UpdateAtlas                          gvdb_volume_gvdb.cpp:2630-2704
//
// The reference computes one 64-bit key per point per level, sorts all of
// them, copies the unique keys to the host, allocates nodes in a host loop,
// links them with a root descent per node and repeats the cycle for the
// dilated ("extra") bricks.  Here the node set of every level is derived on the
// device from ONE sort of 32-bit compact level-0 keys:
//   D0 = leaves holding points, X0 = leaves of the dilation boxes not in D0,
//   level l nodes = parents of (D0 u X0), split the same way,
// each set held as a bitmap with per-word prefix popcounts, so pool order
// (sorted direct nodes, then sorted extra nodes: the order of the reference's
// two passes), parent indices and child-list slots are all O(1) rank lookups.
// The host reads back 24 bytes (bounding box) and the per-level counts.
#include <limits.h>
#include <math.h>
#include <string.h>

#include <atomic>

#include "gvx_grid.cuh"

namespace {

__device__ __forceinline__ uint32_t f2ord(float f)
{
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
inline float ord2f(uint32_t u)
{
    const uint32_t b = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
    float f;
    memcpy(&f, &b, 4);
    return f;
}

__device__ __forceinline__ void load_pos(const char* base, int off, int stride, uint32_t i, float* w)
{
    const float* p = (const float*)(base + (size_t)i * (size_t)stride + off);
    w[0] = p[0];
    w[1] = p[1];
    w[2] = p[2];
}

inline int ceil_log2(int64_t v)
{
    int b = 0;
    while ((int64_t(1) << b) < v) b++;
    return b;
}

}  // namespace

// ---------------------------------------------------------------------------
// bounding box of pos + orig over ALL points (GetBoundingBox includes points
// that the key kernel later drops)
__global__ void k_bbox(const char* pos, int off, int stride, uint32_t n, float ox, float oy, float oz,
                       uint32_t* out, uint32_t* err)
{
    uint32_t mn[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, mx[3] = {0u, 0u, 0u};
    bool nan = false;
    const uint32_t nt = gridDim.x * blockDim.x, t = blockIdx.x * blockDim.x + threadIdx.x;
    const char* base = pos + off;
    if (stride == 12 && ((uintptr_t)base & 15u) == 0 && nt % 3u == 0) {
        // packed float3, 16-byte aligned: four points in three float4 loads.  Float4 j holds
        // floats 4j .. 4j+3, whose axes are (j + k) mod 3; the thread count is a multiple of 3,
        // so j mod 3 = t mod 3 on every iteration and component k keeps one axis throughout.
        const float4* v = (const float4*)base;
        const uint64_t nflt = 3ull * n, nv = nflt / 4;
        const uint32_t ph = t % 3u;
        const float oc[3] = {ph == 0 ? ox : (ph == 1 ? oy : oz), ph == 0 ? oy : (ph == 1 ? oz : ox),
                             ph == 0 ? oz : (ph == 1 ? ox : oy)};
        uint32_t cmn[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, cmx[4] = {0u, 0u, 0u, 0u};
        for (uint64_t j = t; j < nv; j += nt) {
            const float4 q = v[j];
            const float w[4] = {q.x + oc[0], q.y + oc[1], q.z + oc[2], q.w + oc[0]};
#pragma unroll
            for (int k = 0; k < 4; k++) {
                if (w[k] != w[k]) nan = true;
                const uint32_t o = f2ord(w[k]);
                cmn[k] = min(cmn[k], o);
                cmx[k] = max(cmx[k], o);
            }
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const uint32_t a = (ph + (uint32_t)k) % 3u;
            mn[a] = min(mn[a], cmn[k]);
            mx[a] = max(mx[a], cmx[k]);
        }
        if (t == 0) {  // the floats after the last whole float4
            const float o3[3] = {ox, oy, oz};
            for (uint64_t f = nv * 4; f < nflt; f++) {
                const uint32_t a = (uint32_t)(f % 3u);
                const float w = ((const float*)base)[f] + o3[a];
                if (w != w) nan = true;
                mn[a] = min(mn[a], f2ord(w));
                mx[a] = max(mx[a], f2ord(w));
            }
        }
    } else {
        for (uint32_t i = t; i < n; i += nt) {
            float w[3];
            load_pos(pos, off, stride, i, w);
            w[0] += ox;
            w[1] += oy;
            w[2] += oz;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                if (w[a] != w[a]) nan = true;
                const uint32_t o = f2ord(w[a]);
                mn[a] = min(mn[a], o);
                mx[a] = max(mx[a], o);
            }
        }
    }
    // warp, then block, then one atomic per block and bound (6 addresses take every atomic)
#pragma unroll
    for (int a = 0; a < 3; a++) {
        for (int s = 16; s > 0; s >>= 1) {
            mn[a] = min(mn[a], __shfl_xor_sync(0xFFFFFFFFu, mn[a], s));
            mx[a] = max(mx[a], __shfl_xor_sync(0xFFFFFFFFu, mx[a], s));
        }
    }
    __shared__ uint32_t s_b[32][6];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if (lane == 0)
        for (int a = 0; a < 3; a++) {
            s_b[wid][a] = mn[a];
            s_b[wid][3 + a] = mx[a];
        }
    __syncthreads();
    if (threadIdx.x < 6) {
        uint32_t v = s_b[0][threadIdx.x];
        for (int w = 1; w < nw; w++) v = threadIdx.x < 3 ? min(v, s_b[w][threadIdx.x]) : max(v, s_b[w][threadIdx.x]);
        if (threadIdx.x < 3)
            atomicMin(&out[threadIdx.x], v);
        else
            atomicMax(&out[threadIdx.x], v);
    }
    if (nan) atomicOr(err, GVX_DERR_BADPOINT);
}

// compact level-0 key of every point (invalid points -> invalid_key, sorted
// last), identity values, and the digit histograms of the sort.  kshift 3: the
// key is (leaf key << 3) | octant, octant = 4 hx + 2 hy + hz the half of the
// brick (2^lb voxels) that the point's voxel lies in on every axis, so the
// stable sort leaves every leaf's points in (octant, index) order; invalid_key
// is the shifted one then
__global__ void k_keys(const char* pos, int off, int stride, uint32_t n, float ox, float oy, float oz,
                       KeySpace ks, float inv_b, int kshift, int lb, int passes, uint32_t invalid_key,
                       uint32_t* keys, uint32_t* vals, uint32_t* hist, uint32_t* err)
{
    __shared__ uint32_t sh[4 * 256];
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) sh[i] = 0u;
    __syncthreads();
    bool degen = false;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float w[3];
        load_pos(pos, off, stride, i, w);
        w[0] += ox;
        w[1] += oy;
        w[2] += oz;
        uint32_t key = invalid_key;
        if (w[0] >= 0.f && w[1] >= 0.f && w[2] >= 0.f) {
            int c[3];
            bool in = true;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                c[a] = (int)(w[a] * inv_b) - ks.lo[a];  // floor(w / b), exact for a power-of-two b
                if (c[a] < 0 || c[a] >= (1 << ks.bits[a])) in = false;
            }
            if (in) {
                key = ks_pack(ks, c[0], c[1], c[2], 0) << kshift;
                if (kshift) {
                    // voxel x >= the brick's corner + half  <=>  bit lb-1 of x (x >= 0, bricks aligned)
                    int oct = 7;
                    if (lb > 0)
                        oct = ((((int)w[0]) >> (lb - 1)) & 1) << 2 | ((((int)w[1]) >> (lb - 1)) & 1) << 1 |
                              ((((int)w[2]) >> (lb - 1)) & 1);
                    key |= (uint32_t)oct;
                }
            } else {
                degen = true;
            }
        }
        keys[i] = key;
        vals[i] = i;
        gvx_sort_count_key(sh, key, passes);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x)
        if (sh[i]) atomicAdd(&hist[i], sh[i]);
    if (degen) atomicOr(err, GVX_DERR_DEGENERATE);
}

// first point of every run of equal valid leaf keys (sorted keys >> kshift) sets the key's bit
__global__ void k_mark_runs(const uint32_t* __restrict__ skeys, uint32_t n, int kshift, uint32_t invalid_key,
                            uint32_t* bits)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = skeys[i] >> kshift;
    if (k >= invalid_key) return;
    if (i == 0 || (skeys[i - 1] >> kshift) != k) atomicOr(&bits[k >> 5], 1u << (k & 31));
}

// dilation mask of every direct leaf: OR over its points of the leaves touched
// by the box [int(p)-r, int(p)+2r] (cuda_gvdb_particles.cuh:481-482), encoded
// as 27 bits (dz+1)*9 + (dy+1)*3 + (dx+1)
// (hi_mul = 2 for the full rebuild's box, 1 for the incremental box [int(p)-r, int(p)+r], PT.cuh:433-434)
__global__ void k_point_masks(const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ svals, uint32_t n,
                              int kshift, uint32_t invalid_key, BitRank d0, const char* pos, int off, int stride,
                              float ox, float oy, float oz, float radius, float hi_mul, int brick, uint32_t* masks)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < n;
    uint32_t key = live ? skeys[i] >> kshift : invalid_key;
    const bool valid = key < invalid_key;
    uint32_t m = 0u;
    int leaf = -1;
    if (valid) {
        leaf = (int)br_rank(d0, key);
        float w[3];
        load_pos(pos, off, stride, svals[i], w);
        w[0] += ox;
        w[1] += oy;
        w[2] += oz;
        int lo[3], hi[3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int ip = (int)w[a];
            const int bmin = (int)((float)ip - radius);
            const int bmax = (int)((float)ip + hi_mul * radius);
            const int cl = ip / brick;
            lo[a] = bmin / brick - cl;  // C truncation, as bmin/rres*rres
            hi[a] = bmax / brick - cl;
            lo[a] = max(lo[a], -1);
            hi[a] = min(hi[a], 1);
        }
        for (int dz = lo[2]; dz <= hi[2]; dz++)
            for (int dy = lo[1]; dy <= hi[1]; dy++)
                for (int dx = lo[0]; dx <= hi[0]; dx++) m |= 1u << ((dz + 1) * 9 + (dy + 1) * 3 + (dx + 1));
    }
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, valid ? (uint32_t)leaf : 0xFFFFFFFFu);
    const uint32_t agg = __reduce_or_sync(peers, m);
    const int lane = threadIdx.x & 31;
    if (valid && lane == __ffs(peers) - 1) atomicOr(&masks[leaf], agg);
}

// leaves of the dilation boxes that hold no point -> X0 bitmap; lim: per axis, the first key-space
// coordinate past the root (a key space rounded up to powers of two may reach past it)
__global__ void k_dilate(const uint32_t* __restrict__ dlist, const uint32_t* __restrict__ count, KeySpace ks,
                         int3 lim, const uint32_t* __restrict__ masks, BitRank d0, uint32_t* x0bits, uint32_t* err)
{
    // grid-stride over the leaves (their count is on the device; the grid is sized for the points)
    const uint32_t cnt = *count, stride = gridDim.x * blockDim.x;
    bool degen = false;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += stride) {
        const uint32_t m = masks[j] & ~(1u << 13);
        if (!m) continue;
        int c[3];
        ks_unpack(ks, dlist[j], 0, c);
        for (int b = 0; b < 27; b++) {
            if (!((m >> b) & 1u)) continue;
            const int nx = c[0] + (b % 3) - 1, ny = c[1] + (b / 3) % 3 - 1, nz = c[2] + b / 9 - 1;
            if (nx < 0 || ny < 0 || nz < 0 || nx >= lim.x || ny >= lim.y || nz >= lim.z) {
                degen = true;  // the reference descends outside the root here
                continue;
            }
            const uint32_t nk = ks_pack(ks, nx, ny, nz, 0);
            if (!br_test(d0, nk)) atomicOr(&x0bits[nk >> 5], 1u << (nk & 31));
        }
    }
    if (degen) atomicOr(err, GVX_DERR_DEGENERATE);
}

struct UpperDesc {
    int nlev;                  // levels 1..nlev are described (nlev = depth-1)
    uint32_t words[GVX_MAXLEV];
    uint32_t off[GVX_MAXLEV];  // per level: D bits, X bits, D prefix, X prefix (words each)
    int tshift[GVX_MAXLEV];
};

// parents of direct leaves -> D_l bitmaps
__global__ void k_upper_direct(const uint32_t* __restrict__ dlist, const uint32_t* __restrict__ count, KeySpace ks,
                               UpperDesc ud, uint32_t* upper)
{
    // grid-stride over the leaves in whole warps (the match_any below takes every lane)
    const uint32_t cnt = *count, stride = gridDim.x * blockDim.x;
    for (uint32_t j0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); j0 < cnt; j0 += stride) {
        const uint32_t j = j0 + (threadIdx.x & 31u);
        const bool valid = j < cnt;
        int c[3] = {0, 0, 0};
        if (valid) ks_unpack(ks, dlist[j], 0, c);
        for (int l = 1; l <= ud.nlev; l++) {
            const int t = ud.tshift[l];
            const uint32_t k = valid ? ks_pack(ks, c[0] >> t, c[1] >> t, c[2] >> t, t) : 0xFFFFFFFFu;
            const uint32_t peers = __match_any_sync(0xFFFFFFFFu, k);
            if (valid && (threadIdx.x & 31) == __ffs(peers) - 1)
                atomicOr(&upper[ud.off[l] + (k >> 5)], 1u << (k & 31));
        }
    }
}

// parents of extra leaves -> A_l bitmaps (X_l = A_l & ~D_l later)
__global__ void k_upper_extra(const uint32_t* __restrict__ x0bits, uint32_t words, KeySpace ks, UpperDesc ud,
                              uint32_t* upper)
{
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= words) return;
    uint32_t bits = x0bits[w];
    uint32_t last[GVX_MAXLEV];
    for (int l = 0; l < GVX_MAXLEV; l++) last[l] = 0xFFFFFFFFu;
    while (bits) {
        const int b = __ffs(bits) - 1;
        bits &= bits - 1u;
        int c[3];
        ks_unpack(ks, w * 32u + (uint32_t)b, 0, c);
        for (int l = 1; l <= ud.nlev; l++) {
            const int t = ud.tshift[l];
            const uint32_t k = ks_pack(ks, c[0] >> t, c[1] >> t, c[2] >> t, t);
            if (k == last[l]) continue;
            last[l] = k;
            atomicOr(&upper[ud.off[l] + ud.words[l] + (k >> 5)], 1u << (k & 31));
        }
    }
}

// small bitmaps: one block per (level, D|X); X = A & ~D first; exclusive
// prefix popcounts, total -> counts[2 + 2*(l-1) + which]
__global__ void k_prefix_upper(UpperDesc ud, uint32_t* upper, uint32_t* counts)
{
    const int l = 1 + blockIdx.x / 2, which = blockIdx.x & 1;
    if (l > ud.nlev) return;
    const uint32_t words = ud.words[l];
    uint32_t* D = upper + ud.off[l];
    uint32_t* B = upper + ud.off[l] + (which ? words : 0u);
    uint32_t* pre = upper + ud.off[l] + 2u * words + (which ? words : 0u);
    __shared__ uint32_t s_w[32];
    __shared__ uint32_t s_carry;
    if (threadIdx.x == 0) s_carry = 0u;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (uint32_t base = 0; base < words; base += blockDim.x) {
        const uint32_t w = base + threadIdx.x;
        uint32_t v = 0u;
        if (w < words) {
            uint32_t bits = B[w];
            if (which) {
                bits &= ~D[w];
                B[w] = bits;
            }
            v = __popc(bits);
        }
        uint32_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_w[warp] = x;
        __syncthreads();
        uint32_t wp = 0u;
        for (int i = 0; i < warp; i++) wp += s_w[i];
        uint32_t tot = 0u;
        for (int i = 0; i < nw; i++) tot += s_w[i];
        if (w < words) pre[w] = s_carry + wp + x - v;
        __syncthreads();
        if (threadIdx.x == 0) s_carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) counts[2 + 2 * (l - 1) + which] = s_carry;
}

// ---------------------------------------------------------------------------
// generic exclusive prefix of popcounts over a bitmap (reduce, scan, apply)
namespace {
constexpr int kPfxThreads = 256;
constexpr int kPfxPerThread = 16;
constexpr uint32_t kPfxChunk = kPfxThreads * kPfxPerThread;
}  // namespace

// POPC: the scanned values are the popcounts of bitmap words, else the words themselves
template <bool POPC>
__device__ __forceinline__ uint32_t pfx_value(uint32_t v)
{
    return POPC ? (uint32_t)__popc(v) : v;
}

// per block of kPfxChunk words: the sum (all loads issued before any add: the block's chunk is
// one round trip, not kPfxPerThread)
template <bool POPC>
__global__ void __launch_bounds__(kPfxThreads) k_pfx_reduce(const uint32_t* __restrict__ bits, uint32_t words,
                                                            uint32_t* block_sums)
{
    const uint32_t base = blockIdx.x * kPfxChunk + threadIdx.x;
    uint32_t v[kPfxPerThread];
#pragma unroll
    for (int k = 0; k < kPfxPerThread; k++) {
        const uint32_t w = base + (uint32_t)k * kPfxThreads;
        v[k] = w < words ? bits[w] : 0u;
    }
    uint32_t s = 0u;
#pragma unroll
    for (int k = 0; k < kPfxPerThread; k++) s += pfx_value<POPC>(v[k]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
    __shared__ uint32_t ws[kPfxThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0u;
        for (int i = 0; i < kPfxThreads / 32; i++) t += ws[i];
        block_sums[blockIdx.x] = t;
    }
}

// the block's chunk in and out through shared memory (coalesced global loads and stores; index i
// of the chunk at i + i/32, so that a thread's kPfxPerThread consecutive values and the warps'
// strided rows are both free of bank conflicts), each thread scanning kPfxPerThread consecutive
// values after the block offset from the earlier blocks' sums
template <bool POPC>
__global__ void __launch_bounds__(kPfxThreads) k_pfx_apply(const uint32_t* __restrict__ bits, uint32_t words,
                                                           const uint32_t* __restrict__ block_sums, uint32_t* prefix,
                                                           uint32_t* total)
{
    __shared__ uint32_t s_v[kPfxChunk + kPfxChunk / 32];
    __shared__ uint32_t s_w[kPfxThreads / 32];
    __shared__ uint32_t s_off;
    const uint32_t cbase = blockIdx.x * kPfxChunk;
#pragma unroll
    for (int k = 0; k < kPfxPerThread; k++) {
        const uint32_t i = (uint32_t)k * kPfxThreads + threadIdx.x, w = cbase + i;
        s_v[i + (i >> 5)] = w < words ? pfx_value<POPC>(bits[w]) : 0u;
    }
    {
        uint32_t o = 0u;
        for (uint32_t i = threadIdx.x; i < blockIdx.x; i += kPfxThreads) o += block_sums[i];
        for (int k = 16; k > 0; k >>= 1) o += __shfl_xor_sync(0xFFFFFFFFu, o, k);
        if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = o;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0u;
            for (int k = 0; k < kPfxThreads / 32; k++) t += s_w[k];
            s_off = t;
            if (total && blockIdx.x + 1 == gridDim.x) *total = t + block_sums[blockIdx.x];
        }
        __syncthreads();
    }
    const uint32_t block_off = s_off;
    uint32_t cnt[kPfxPerThread];
    uint32_t s = 0u;
#pragma unroll
    for (int k = 0; k < kPfxPerThread; k++) {
        const uint32_t i = threadIdx.x * kPfxPerThread + k;
        cnt[k] = s_v[i + (i >> 5)];
        s += cnt[k];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = s;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    __syncthreads();  // s_w is reused
    if (lane == 31) s_w[warp] = x;
    __syncthreads();
    uint32_t run = block_off + x - s;
    for (int k = 0; k < warp; k++) run += s_w[k];
#pragma unroll
    for (int k = 0; k < kPfxPerThread; k++) {
        const uint32_t i = threadIdx.x * kPfxPerThread + k;
        s_v[i + (i >> 5)] = run;
        run += cnt[k];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kPfxPerThread; k++) {
        const uint32_t i = (uint32_t)k * kPfxThreads + threadIdx.x, w = cbase + i;
        if (w < words) prefix[w] = s_v[i + (i >> 5)];
    }
}

template <bool POPC>
static gvx_status pfx_run(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* total, DevBuf& tmp, cudaStream_t st,
                          int64_t* launches)
{
    const uint32_t nb = std::max<uint32_t>(1u, (n + kPfxChunk - 1) / kPfxChunk);
    GVX_CK(gvx_ensure(tmp, (size_t)(nb + 1) * sizeof(uint32_t)));
    k_pfx_reduce<POPC><<<nb, kPfxThreads, 0, st>>>(in, n, tmp.as<uint32_t>());
    k_pfx_apply<POPC><<<nb, kPfxThreads, 0, st>>>(in, n, tmp.as<uint32_t>(), out, total);
    *launches += 2;
    GVX_CK(cudaGetLastError());
    return GVX_OK;
}

gvx_status gvx_bitmap_prefix(const uint32_t* bits, uint32_t* prefix, uint32_t words, uint32_t* total, DevBuf& tmp,
                             cudaStream_t st, int64_t* launches)
{
    return pfx_run<true>(bits, prefix, words, total, tmp, st, launches);
}

gvx_status gvx_scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* total, DevBuf& tmp, cudaStream_t st,
                        int64_t* launches)
{
    return pfx_run<false>(in, out, n, total, tmp, st, launches);
}

// set bits -> sorted key list (select)
__global__ void k_select(const uint32_t* __restrict__ bits, const uint32_t* __restrict__ prefix, uint32_t words,
                         uint32_t* out, uint32_t cap)
{
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= words) return;
    uint32_t b = bits[w];
    uint32_t o = prefix[w];
    while (b && o < cap) {  // cap: the list's capacity
        const int k = __ffs(b) - 1;
        b &= b - 1u;
        out[o++] = w * 32u + (uint32_t)k;
    }
}

struct NodeLevelArgs {
    int lev, depth;
    uint32_t ucount, xcount;
    const uint32_t* dlist;
    const uint32_t* xlist;
    KeySpace ks;
    int tshift, tshift_parent, logdim_parent, res_parent;
    int lo[3];         // absolute level-l node coordinates of compact (0,0,0)
    int root_rel[3];   // root position in level-l node units (when the parent is the root)
    int range;
    BitRank pd, px;    // parent level bitmaps (unused when the parent is the root)
    uint32_t pucount;
    GvxNode* nodes;
    uint64_t* pclist;
    uint32_t* leaf_key;  // level 0 only
    // planned builds: the counts from device memory (dc[ci_u], dc[ci_x], dc[ci_pu]; ci_pu < 0: none),
    // this level's node capacity and the parent level's (0: no parent check)
    const uint32_t* dc;
    int ci_u, ci_x, ci_pu;
    uint32_t cap, pcap;
};

// one node per thread: Node record, parent reference, and the parent's child-list slot
// (SetupNode VG.cpp:2512-2524, gvdbLinkBricks cuda_gvdb_nodes.cuh:470-505)
__global__ void k_write_nodes(NodeLevelArgs a)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t ucount = a.ucount, xcount = a.xcount, pucount = a.pucount;
    if (a.dc) {
        ucount = min(a.dc[a.ci_u], a.cap);
        xcount = min(a.dc[a.ci_x], a.cap - ucount);
        pucount = a.ci_pu >= 0 ? a.dc[a.ci_pu] : 0u;
    }
    if (i >= ucount + xcount) return;
    const uint32_t key = i < ucount ? a.dlist[i] : a.xlist[i - ucount];
    int c[3];
    ks_unpack(a.ks, key, a.tshift, c);
    GvxNode nd;
    nd.lev = (uint8_t)a.lev;
    nd.flags = 1;
    nd.prio = 0;
    nd.pad = 0;
    for (int k = 0; k < 3; k++) {
        nd.pos[k] = (a.lo[k] + c[k]) * a.range;
        nd.value[k] = -1;
        nd.vrange[k] = 0.f;
    }
    nd.mask = 0ull;
    nd.childlist = a.lev > 0 ? (1ull | ((uint64_t)a.lev << 8) | ((uint64_t)i << 16)) : ID_UNDEFL_U64;
    uint32_t pidx;
    int rel[3];
    const int res = a.res_parent;
    bool linked = true;
    if (a.lev + 1 == a.depth) {
        pidx = 0u;
        for (int k = 0; k < 3; k++) {
            rel[k] = a.lo[k] + c[k] - a.root_rel[k];
            // (a key space rounded up to powers of two may reach past the root: a planned build's
            // points there make it void -- the frame's root differs -- and are not linked)
            linked = linked && rel[k] >= 0 && rel[k] < res;
        }
    } else {
        const int sh = a.logdim_parent;
        const uint32_t pk = ks_pack(a.ks, c[0] >> sh, c[1] >> sh, c[2] >> sh, a.tshift_parent);
        pidx = br_test(a.pd, pk) ? br_rank(a.pd, pk) : pucount + br_rank(a.px, pk);
        for (int k = 0; k < 3; k++) rel[k] = c[k] & (res - 1);
    }
    nd.parent = ((uint64_t)pidx << 16) | ((uint64_t)(a.lev + 1) << 8);
    const int bit = (rel[2] * res + rel[1]) * res + rel[0];
    // (a parent beyond its pool's capacity: no link -- the planned build is void)
    if (linked && (!a.pcap || pidx < a.pcap))
        a.pclist[(size_t)pidx * res * res * res + bit] = ((uint64_t)i << 16) | ((uint64_t)a.lev << 8);
    a.nodes[i] = nd;
    if (a.leaf_key) a.leaf_key[i] = key;
}

__global__ void k_write_root(GvxNode* root, int lev, int px, int py, int pz)
{
    GvxNode nd;
    nd.lev = (uint8_t)lev;
    nd.flags = 1;
    nd.prio = 0;
    nd.pad = 0;
    nd.pos[0] = px;
    nd.pos[1] = py;
    nd.pos[2] = pz;
    for (int k = 0; k < 3; k++) {
        nd.value[k] = -1;
        nd.vrange[k] = 0.f;
    }
    nd.parent = ID_UNDEFL_U64;
    nd.childlist = 1ull | ((uint64_t)lev << 8);
    nd.mask = 0ull;
    *root = nd;
}

// run of equal leaf keys in sorted order -> [start, end) of its leaf.  With octants in the keys
// (kshift 3) also the first sorted index of every octant of the leaf's points (leaf_oct[8 l + o] =
// start + the points of octants < o), written at the starts of the octant runs and at the leaf's end
__global__ void k_group_runs(const uint32_t* __restrict__ skeys, uint32_t n, int kshift, uint32_t invalid_key,
                             LeafLookup L, int2* leaf_range, int* leaf_oct)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t sk = skeys[i], k = sk >> kshift;
    if (k >= invalid_key) return;
    const uint32_t prev = i == 0 ? 0xFFFFFFFFu : skeys[i - 1];
    const bool first = i == 0 || (prev >> kshift) != k;
    const bool last = i + 1 == n || (skeys[i + 1] >> kshift) != k;
    const bool ostart = kshift && (first || prev != sk);
    if (!first && !last && !ostart) return;
    int c[3];
    ks_unpack(L.ks, k, 0, c);
    const int leaf = ll_find(L, c[0], c[1], c[2]);
    if (leaf < 0) return;
    if (first) leaf_range[leaf].x = (int)i;
    if (last) leaf_range[leaf].y = (int)(i + 1);
    if (kshift) {
        int* lo = leaf_oct + (size_t)leaf * 8;
        const int o = (int)(sk & 7u);
        if (ostart)
            for (int q = first ? 0 : (int)(prev & 7u) + 1; q <= o; q++) lo[q] = (int)i;
        if (last)
            for (int q = o + 1; q < 8; q++) lo[q] = (int)(i + 1);
    }
}

// Points of every leaf in octant order: a stable partition of the leaf's range
// of sorted point indices by the half of the brick that each point's voxel
// (floor of the translated position, as the keys take it) lies in on every
// axis, octant = 4 hx + 2 hy + hz, and the first index of every octant.  The
// sorted order becomes (leaf key, octant, point index); the splat reads only
// the octants of a neighbouring brick whose points can reach its slab.  For
// key spaces too wide for the octant in the sort key (more than 2^28 leaf
// cells; otherwise the sort itself orders the octants).  A segment of G lanes
// per leaf, launched with G = 32 (segments of 8 lanes were slower on leaves
// of very different sizes: the longest leaf of a warp sets its trip count);
// the segment's lanes 0-7 keep the octants' counters.  With A.spos the sorted
// point attributes of the leaves' points are written in the same pass (as
// k_permute writes them); entries outside the leaf ranges are not, and no
// reader takes them (a point is splatted only when its own leaf exists).
template <int G>
__global__ void k_octant_partition(const int2* __restrict__ leaf_range, DevCount nlc,
                                   const GvxNode* __restrict__ nodes0, const char* pos, int off, int stride, float ox,
                                   float oy, float oz, int half, const uint32_t* __restrict__ vin,
                                   uint32_t* __restrict__ vout, int* __restrict__ leaf_oct, GvxSortedAttr A)
{
    static_assert(G == 8 || G == 16 || G == 32, "segments of 8, 16 or 32 lanes");
    const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int sl = lane & (G - 1), sb = lane - sl;  // lane in the segment, the segment's first lane
    const uint32_t smask = G == 32 ? 0xFFFFFFFFu : (((1u << G) - 1u) << sb);
    const uint32_t nl = nlc.get();
    if ((gt & ~31u) / G >= nl) return;  // whole warps: the warp's first leaf is past the last
    const uint32_t leaf = gt / G;
    const bool live = leaf < nl;
    int2 r = make_int2(0, 0);
    int bx = 0, by = 0, bz = 0;
    if (live) {
        r = leaf_range[leaf];
        bx = nodes0[leaf].pos[0] + half;
        by = nodes0[leaf].pos[1] + half;
        bz = nodes0[leaf].pos[2] + half;
    }
    // translated position and octant of sorted entry i (octant -1 past the leaf's range)
    auto fetch = [&](int i, uint32_t& v, float* w) {
        if (i >= r.y) return -1;
        v = vin[i];
        load_pos(pos, off, stride, v, w);
        w[0] += ox;
        w[1] += oy;
        w[2] += oz;
        const int x = (int)floorf(w[0]), y = (int)floorf(w[1]), z = (int)floorf(w[2]);
        return (x >= bx ? 4 : 0) | (y >= by ? 2 : 0) | (z >= bz ? 1 : 0);
    };
    const int nch = __reduce_max_sync(0xFFFFFFFFu, (r.y - r.x + G - 1) / G);  // chunks of the warp's longest leaf
    int cnt = 0;  // segment lane o < 8: points of octant o
    uint32_t v0 = 0u;  // the segment's first G points, kept for the placement pass
    float w0[3] = {0.f, 0.f, 0.f};
    int o0 = -1;
    for (int c = 0; c < nch; c++) {
        uint32_t v = 0u;
        float w[3];
        const int o = fetch(r.x + c * G + sl, v, w);
        if (c == 0) {
            v0 = v;
            o0 = o;
            w0[0] = w[0];
            w0[1] = w[1];
            w0[2] = w[2];
        }
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, o == k) & smask;
            if (sl == k) cnt += __popc(m);
        }
    }
    int incl = cnt;
#pragma unroll
    for (int s = 1; s < 8; s <<= 1) {
        const int t = __shfl_up_sync(0xFFFFFFFFu, incl, s, G);
        if (sl >= s) incl += t;
    }
    int run = r.x + incl - cnt;  // segment lane o < 8: next index of octant o
    if (live && sl < 8) leaf_oct[(size_t)leaf * 8 + sl] = run;
    for (int c = 0; c < nch; c++) {
        uint32_t v = v0;
        float w[3] = {w0[0], w0[1], w0[2]};
        int o = o0;
        if (c > 0) o = fetch(r.x + c * G + sl, v, w);
        const uint32_t same = __match_any_sync(0xFFFFFFFFu, o < 0 ? 0xFFFFFFFFu : (uint32_t)(o | (sb << 3)));
        const int dst = __shfl_sync(0xFFFFFFFFu, run, sb + (o < 0 ? 0 : o)) + __popc(same & ((1u << lane) - 1u));
        if (o >= 0) vout[dst] = v;
        if (A.spos) {
            float rr = 0.0f;
            if (o >= 0) {
                A.spos[dst] = make_float4(w[0], w[1], w[2], A.weight ? A.weight[v] : 1.0f);
                if (A.radius) rr = A.radius[v];
                if (A.svel) {
                    float4 q = make_float4(0.f, 0.f, 0.f, rr);
                    if (A.vel) {
                        const float* u = (const float*)(A.vel + (size_t)v * A.vel_stride + A.vel_off);
                        q.x = u[0];
                        q.y = u[1];
                        q.z = u[2];
                    }
                    A.svel[dst] = q;
                }
                rr = rr != rr ? 3.0e38f : fmaxf(rr, 0.0f);
            }
            if (A.rmax) {
                const unsigned int mm = __reduce_max_sync(0xFFFFFFFFu, __float_as_uint(rr));
                // most warps find the maximum already there: read before the atomic
                if (lane == 0 && mm && mm > *(volatile unsigned int*)A.rmax) atomicMax(A.rmax, mm);
            }
        }
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, o == k) & smask;
            if (sl == k) run += __popc(m);
        }
    }
}

// 27-neighbourhood of every leaf (leaf pool indices, -1 where no leaf; all -1
// for an inactive leaf, whose key is kNoKey)
constexpr uint32_t kNoKey = 0xFFFFFFFFu;
__global__ void k_neighbors(const uint32_t* __restrict__ leaf_key, DevCount nl, LeafLookup L, int* nbr)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nleaves = nl.get();
    if (t >= nleaves * 27u) return;
    const uint32_t leaf = t / 27u, d = t % 27u;
    const uint32_t key = leaf_key[leaf];
    if (key == kNoKey) {
        nbr[t] = -1;
        return;
    }
    int c[3];
    ks_unpack(L.ks, key, 0, c);
    nbr[t] = ll_find(L, c[0] + (int)(d % 3u) - 1, c[1] + (int)((d / 3u) % 3u) - 1, c[2] + (int)(d / 9u) - 1);
}

// active leaves (mFlags) -> bitmap over pool indices
__global__ void k_flag_bits(const GvxNode* __restrict__ nodes, DevCount nc, uint32_t* bits)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = nc.get();
    const bool f = i < n && nodes[i].flags;
    const uint32_t b = __ballot_sync(0xFFFFFFFFu, f);
    if ((threadIdx.x & 31) == 0 && i < ((n + 31u) & ~31u)) bits[i >> 5] = b;
}

// UpdateAtlas: active leaf k (pool order) -> atlas slot k, mValue, atlas map
// (VG.cpp:2650-2690, AL.cpp:692-715)
__global__ void k_atlas_assign(GvxNode* nodes, DevCount nc, const uint32_t* __restrict__ fbits,
                               const uint32_t* __restrict__ fprefix, int sx, int sy, int P, int apron,
                               int* leaf_slot, int* slot_leaf, int4* amap)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc.get()) return;
    if (!((fbits[i >> 5] >> (i & 31)) & 1u)) {
        leaf_slot[i] = -1;
        return;
    }
    const uint32_t s = fprefix[i >> 5] + __popc(fbits[i >> 5] & ((1u << (i & 31)) - 1u));
    const int a2 = sx * sy;
    const int z = (int)s / a2, rem = (int)s - z * a2;
    const int y = rem / sx, x = rem - y * sx;
    GvxNode* nd = nodes + i;
    nd->value[0] = x * P + apron;
    nd->value[1] = y * P + apron;
    nd->value[2] = z * P + apron;
    leaf_slot[i] = (int)s;
    slot_leaf[s] = (int)i;
    amap[s] = make_int4(nd->pos[0], nd->pos[1], nd->pos[2], (int)i);
}

// GetBoundingBox's accumulators before k_bbox: min = all ones, max = 0 (order-preserving bits)
__global__ void k_bbox_reset(uint32_t* out)
{
    if (threadIdx.x < 6) out[threadIdx.x] = threadIdx.x < 3 ? 0xFFFFFFFFu : 0u;
}

__global__ void k_bounds_init(int* out)
{
    if (threadIdx.x < 3) out[threadIdx.x] = 0x7FFFFFFF;
    else if (threadIdx.x < 6) out[threadIdx.x] = (int)0x80000000;
}

// ComputeBounds (VG.cpp:1792-1816): bbox of active leaves
__global__ void k_leaf_bounds(const GvxNode* __restrict__ nodes, uint32_t n, int range, int* out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;  // whole warps: the grid is a multiple of 32
    int mn[3] = {INT_MAX, INT_MAX, INT_MAX}, mx[3] = {INT_MIN, INT_MIN, INT_MIN};
    if (i < n && nodes[i].flags) {
        for (int a = 0; a < 3; a++) {
            mn[a] = nodes[i].pos[a];
            mx[a] = nodes[i].pos[a] + range;
        }
    }
    // warp, then block, then one atomic per block and bound
#pragma unroll
    for (int a = 0; a < 3; a++) {
        for (int s = 16; s > 0; s >>= 1) {
            mn[a] = min(mn[a], __shfl_xor_sync(0xFFFFFFFFu, mn[a], s));
            mx[a] = max(mx[a], __shfl_xor_sync(0xFFFFFFFFu, mx[a], s));
        }
    }
    __shared__ int s_b[32][6];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if (lane == 0)
        for (int a = 0; a < 3; a++) {
            s_b[wid][a] = mn[a];
            s_b[wid][3 + a] = mx[a];
        }
    __syncthreads();
    if (threadIdx.x < 6) {
        int v = s_b[0][threadIdx.x];
        for (int w = 1; w < nw; w++) v = threadIdx.x < 3 ? min(v, s_b[w][threadIdx.x]) : max(v, s_b[w][threadIdx.x]);
        if (threadIdx.x < 3) {
            if (v != INT_MAX) atomicMin(&out[threadIdx.x], v);
        } else if (v != INT_MIN) {
            atomicMax(&out[threadIdx.x], v);
        }
    }
}

// ---------------------------------------------------------------------------
// incremental rebuild: ActivateIncreBricksGPU (VG.cpp:1020-1156),
// gvdbCalcIncreBrickId / gvdbCalcIncreExtraBrickId (PT.cuh:384-465),
// gvdbLinkBricks (ND.cuh:470-505), gvdbDelinkLeafBricks / gvdbDelinkBricks
// (ND.cuh:401-467).
//
// In the reference a node is reachable by a root descent exactly when its
// parent reference is set: delinking clears the slot in the parent's child
// list and writes ID_UNDEF64 into the node, and only reachable nodes gain
// children.  The descents therefore become bitmap tests over one compact key
// space: L_l = linked level-l nodes, T_l = nodes the points' boxes touch,
// N_l = T_l & ~L_l = the nodes the reference allocates, in key order.

enum { kSetLinked = 0, kSetActive = 1 };

__device__ __forceinline__ bool node_key(const GvxNode& nd, const KeySpace& ks, int t, int range, uint32_t* key)
{
    int c[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        c[a] = nd.pos[a] / range - (ks.lo[a] >> t);
        if (c[a] < 0 || c[a] >= ks_extent(ks, a, t)) return false;
    }
    *key = ks_pack(ks, c[0], c[1], c[2], t);
    return true;
}

__device__ __forceinline__ bool in_node_set(const GvxNode& nd, int set)
{
    return set == kSetActive ? nd.flags != 0 : nd.parent != ID_UNDEF64_U64;
}

// bitmap of a level's linked (or active) nodes; linked nodes outside the key
// space cannot be touched and are left out, an active leaf outside it is an error
__global__ void k_node_bits(const GvxNode* __restrict__ nodes, uint32_t n, KeySpace ks, int t, int range, int set,
                            uint32_t* bits, uint32_t* err)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const GvxNode nd = nodes[i];
    if (!in_node_set(nd, set)) return;
    uint32_t key;
    if (node_key(nd, ks, t, range, &key))
        atomicOr(&bits[key >> 5], 1u << (key & 31));
    else if (set == kSetActive)
        atomicOr(err, GVX_DERR_DEGENERATE);
}

// rank in the set's bitmap -> pool index; with `leaf_key`, also the compact key
// of every leaf (kNoKey where the leaf is not in the set)
__global__ void k_node_remap(const GvxNode* __restrict__ nodes, uint32_t n, KeySpace ks, int t, int range, int set,
                             BitRank br, int* remap, uint32_t* leaf_key)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const GvxNode nd = nodes[i];
    uint32_t key = kNoKey;
    if (in_node_set(nd, set) && node_key(nd, ks, t, range, &key))
        remap[br_rank(br, key)] = (int)i;
    else
        key = kNoKey;
    if (leaf_key) leaf_key[i] = key;
}

// N = (D | A) & ~L: touched (by a point, or by a point's box) and not linked
__global__ void k_new_bits(const uint32_t* __restrict__ D, const uint32_t* __restrict__ A,
                           const uint32_t* __restrict__ L, uint32_t* N, uint32_t words)
{
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w < words) N[w] = (D[w] | A[w]) & ~L[w];
}

// markers of the existing leaves (VG.cpp:1028-1043, 1078-1085): a linked leaf
// inside some point's box gets 1, every other leaf keeps its flag
// (AccumulateTopology) or gets 0
__global__ void k_apply_markers(GvxNode* nodes, uint32_t n, KeySpace ks, int range, const uint32_t* __restrict__ d0,
                                const uint32_t* __restrict__ x0, int accum)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const GvxNode nd = nodes[i];
    uint8_t m = accum ? nd.flags : 0;
    uint32_t key;
    if (nd.parent != ID_UNDEF64_U64 && node_key(nd, ks, 0, range, &key) &&
        (((d0[key >> 5] | x0[key >> 5]) >> (key & 31)) & 1u))
        m = 1;
    nodes[i].flags = m;
}

struct IncNodeArgs {
    int lev;
    uint32_t count;        // new nodes of this level
    uint32_t base;         // pool index of the first one (the old pool size)
    const uint32_t* keys;  // their compact keys, sorted
    KeySpace ks;
    int tshift, range;
    int lo[3];             // absolute level-l coordinates of compact (0,0,0)
    GvxNode* nodes;
    int parent_root;       // the parent level is the root's
    int root_rel[3];       // root position in level-l node units
    BitRank pl;            // linked parents, with their pool indices in premap
    const int* premap;
    BitRank pn;            // new parents (bits null when the parent level gets none)
    uint32_t pbase;        // pool index of the first new parent
    int logdim_parent, res_parent, tshift_parent;
    uint64_t* pclist;
    uint32_t* err;
};

// one new node per thread: SetupNode (VG.cpp:2512-2524) and its link
// (gvdbLinkBricks); the parent is a linked node or a new one of this build
__global__ void k_inc_write_nodes(IncNodeArgs a)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.count) return;
    const uint32_t i = a.base + j;
    int c[3];
    ks_unpack(a.ks, a.keys[j], a.tshift, c);
    GvxNode nd;
    nd.lev = (uint8_t)a.lev;
    nd.flags = 1;
    nd.prio = 0;
    nd.pad = 0;
    for (int k = 0; k < 3; k++) {
        nd.pos[k] = (a.lo[k] + c[k]) * a.range;
        nd.value[k] = -1;
        nd.vrange[k] = 0.f;
    }
    nd.mask = 0ull;
    nd.childlist = a.lev > 0 ? (1ull | ((uint64_t)a.lev << 8) | ((uint64_t)i << 16)) : ID_UNDEFL_U64;
    const int res = a.res_parent;
    uint32_t pidx = 0u;
    int rel[3];
    bool ok = true;
    if (a.parent_root) {
        for (int k = 0; k < 3; k++) {
            rel[k] = a.lo[k] + c[k] - a.root_rel[k];
            if (rel[k] < 0 || rel[k] >= res) ok = false;
        }
    } else {
        const int sh = a.logdim_parent;
        const uint32_t pk = ks_pack(a.ks, c[0] >> sh, c[1] >> sh, c[2] >> sh, a.tshift_parent);
        if (br_test(a.pl, pk))
            pidx = (uint32_t)a.premap[br_rank(a.pl, pk)];
        else if (a.pn.bits && br_test(a.pn, pk))
            pidx = a.pbase + br_rank(a.pn, pk);
        else
            ok = false;
        for (int k = 0; k < 3; k++) rel[k] = c[k] & (res - 1);
    }
    if (ok) {
        nd.parent = ((uint64_t)pidx << 16) | ((uint64_t)(a.lev + 1) << 8);
        const int bit = (rel[2] * res + rel[1]) * res + rel[0];
        a.pclist[(size_t)pidx * res * res * res + bit] = ((uint64_t)i << 16) | ((uint64_t)a.lev << 8);
    } else {
        nd.parent = ID_UNDEFL_U64;  // no parent to link to: the reference's descent fails here
        atomicOr(a.err, GVX_DERR_DEGENERATE);
    }
    a.nodes[i] = nd;
}

// clear node i's slot in its parent's child list and its parent reference
__device__ void unlink_node(GvxNode* nodes, uint32_t i, const GvxNode& nd, const GvxNode* __restrict__ pnodes,
                            uint32_t pcount, uint64_t* pclist, int res_p, int range, uint32_t* err)
{
    const uint64_t pid = nd.parent >> 16;
    if (pid >= pcount) {
        atomicOr(err, GVX_DERR_DEGENERATE);
        return;
    }
    const GvxNode& pn = pnodes[pid];
    int b[3];
    for (int a = 0; a < 3; a++) {
        const int d = nd.pos[a] - pn.pos[a];
        b[a] = d / range;
        if (d < 0 || b[a] >= res_p) {
            atomicOr(err, GVX_DERR_DEGENERATE);
            return;
        }
    }
    const uint64_t cl = pn.childlist >> 16;  // == pid: lists are allocated in lockstep with the nodes
    if (cl >= pcount) {
        atomicOr(err, GVX_DERR_DEGENERATE);
        return;
    }
    const size_t vc = (size_t)res_p * res_p * res_p;
    pclist[(size_t)cl * vc + (b[2] * res_p + b[1]) * res_p + b[0]] = ID_UNDEF64_U64;
    nodes[i].parent = ID_UNDEF64_U64;
}

// gvdbDelinkLeafBricks (ND.cuh:401-428): unmarked leaves leave the tree
__global__ void k_delink_leaves(GvxNode* nodes, uint32_t n, const GvxNode* __restrict__ pnodes, uint32_t pcount,
                                uint64_t* pclist, int res_p, int range, uint32_t* err)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const GvxNode nd = nodes[i];
    if (nd.flags || nd.parent == ID_UNDEF64_U64) return;
    unlink_node(nodes, i, nd, pnodes, pcount, pclist, res_p, range, err);
}

// gvdbDelinkBricks (ND.cuh:430-467) for one level, one warp per node: a linked
// node with any child stays active, a childless one leaves the tree
__global__ void k_delink_upper(GvxNode* nodes, uint32_t n, const uint64_t* __restrict__ clist, uint32_t vc,
                               const GvxNode* __restrict__ pnodes, uint32_t pcount, uint64_t* pclist, int res_p,
                               int range, uint32_t* err)
{
    const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= n) return;  // warp-uniform
    const GvxNode nd = nodes[i];
    if (nd.parent == ID_UNDEF64_U64) {
        if (lane == 0) nodes[i].flags = 0;
        return;
    }
    const uint64_t* cl = clist + (size_t)i * vc;
    bool any = false;
    for (uint32_t s0 = 0; s0 < vc; s0 += 32u) {
        const uint32_t s = s0 + (uint32_t)lane;
        if (__any_sync(0xFFFFFFFFu, s < vc && cl[s] != ID_UNDEF64_U64)) {
            any = true;
            break;
        }
    }
    if (lane != 0) return;
    if (any) {
        nodes[i].flags = 1;
        return;
    }
    nodes[i].flags = 0;
    unlink_node(nodes, i, nd, pnodes, pcount, pclist, res_p, range, err);
}

// ---------------------------------------------------------------------------
// host orchestration

static inline unsigned blocks_for(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

// decodes a device error word that was read back (and clears it on the device:
// each error is reported once)
static gvx_status report_device_error(gvx_grid* g, uint32_t e, const char* stage)
{
    if (e) GVX_CK(cudaMemsetAsync(g->d_err.p, 0, sizeof(uint32_t), g->stream));
    if (e & GVX_DERR_TIMEOUT) {
        gvx_set_error("%s: a device spin-wait timed out", stage);
        return GVX_ERR_TIMEOUT;
    }
    if (e & GVX_DERR_CAPACITY) {
        gvx_set_error("%s: device buffer capacity exceeded", stage);
        return GVX_ERR_CAPACITY;
    }
    if (e & GVX_DERR_BADPOINT) {
        gvx_set_error("%s: NaN point position", stage);
        return GVX_ERR_INVALID_ARG;
    }
    if (e & GVX_DERR_RADIUS) {
        gvx_set_error("%s: a per-point radius exceeds brick-1 (footprint beyond the 26 neighbouring bricks)", stage);
        return GVX_ERR_UNSUPPORTED;
    }
    return GVX_OK;
}

gvx_status gvx_check_device_error(gvx_grid* g, const char* stage)
{
    uint32_t e = 0;
    GVX_CK(cudaMemcpyAsync(&e, g->d_err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, g->stream));
    GVX_CK(cudaStreamSynchronize(g->stream));
    return report_device_error(g, e, stage);
}

// `bytes` (at most 256) of device memory and the device error word in one round
// trip through pinned staging, then the error word reported as above
// (queued: the copies into the staging; then, once the stream has passed them,
// readback_finish takes the bytes and reports the error word)
static gvx_status readback_start(gvx_grid* g, const void* src, size_t bytes, const char* stage)
{
    if (bytes > 256) {
        gvx_set_error("%s: readback of %zu bytes", stage, bytes);
        return GVX_ERR_INVALID_ARG;
    }
    if (!g->h_pin) GVX_CK(cudaMallocHost(&g->h_pin, 512));
    GVX_CK(cudaMemcpyAsync(g->h_pin, src, bytes, cudaMemcpyDeviceToHost, g->stream));
    GVX_CK(cudaMemcpyAsync((char*)g->h_pin + 256, g->d_err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, g->stream));
    return GVX_OK;
}

static gvx_status readback_finish(gvx_grid* g, void* dst, size_t bytes, const char* stage)
{
    GVX_CK(cudaStreamSynchronize(g->stream));
    memcpy(dst, g->h_pin, bytes);
    uint32_t e = 0;
    memcpy(&e, (const char*)g->h_pin + 256, sizeof(e));
    return report_device_error(g, e, stage);
}

static gvx_status readback_checked(gvx_grid* g, void* dst, const void* src, size_t bytes, const char* stage)
{
    gvx_status rc = readback_start(g, src, bytes, stage);
    return rc ? rc : readback_finish(g, dst, bytes, stage);
}

static gvx_status ensure_grid_scratch(gvx_grid* g)
{
    GVX_CK(gvx_ensure(g->d_err, 64));
    GVX_CK(gvx_ensure(g->d_bbox, 64));
    GVX_CK(gvx_ensure(g->d_counts, 64 * sizeof(uint32_t)));
    return GVX_OK;
}

// sort the points by compact key in key space `ks` (positions + t), fill
// leaf_range for the leaves of `L` (whose key space must be ks)
static gvx_status sort_points(gvx_grid* g, int n, const float t[3], const KeySpace& ks, bool fuse_hist)
{
    GVX_CK(gvx_ensure(g->keys[0], (size_t)n * 4));
    GVX_CK(gvx_ensure(g->keys[1], (size_t)n * 4));
    GVX_CK(gvx_ensure(g->vals[0], (size_t)n * 4));
    GVX_CK(gvx_ensure(g->vals[1], (size_t)n * 4));
    // the octant below the leaf key when the key space leaves room for it (28 bits of leaves)
    const int kshift = ks.total_bits <= 28 ? 3 : 0;
    int lb = 0;
    while ((1 << lb) < g->brick) lb++;
    const uint32_t invalid_key = 1u << (ks.total_bits + kshift);
    const int bits = ks.total_bits + kshift + 1;
    const int passes = gvx_sort_passes(bits);
    gvx_status rc = gvx_sort_prepare_hist(g->sort, bits, g->stream);
    if (rc) return rc;
    const unsigned kb = std::min(blocks_for(n, 256), 152u * 8u);
    k_keys<<<kb, 256, 0, g->stream>>>(g->pts.pos, g->pts.pos_off, g->pts.pos_stride, (uint32_t)n, t[0], t[1], t[2],
                                      ks, 1.0f / (float)g->brick, kshift, lb, passes, invalid_key,
                                      g->keys[0].as<uint32_t>(), g->vals[0].as<uint32_t>(),
                                      gvx_sort_hist_ptr(g->sort), g->d_err.as<uint32_t>());
    g->launches++;
    uint32_t* kk[2] = {g->keys[0].as<uint32_t>(), g->keys[1].as<uint32_t>()};
    uint32_t* vv[2] = {g->vals[0].as<uint32_t>(), g->vals[1].as<uint32_t>()};
    int res = 0;
    rc = gvx_sort_pairs(kk, vv, (uint32_t)n, bits, g->sort, fuse_hist, g->stream, g->d_err.as<uint32_t>(), &res,
                        &g->launches);
    if (rc) return rc;
    g->sorted_buf = res;
    g->key_shift = kshift;
    g->n_sorted = (uint32_t)n;
    for (int a = 0; a < 3; a++) g->sort_trans[a] = t[a];
    g->perm_valid = false;
    g->oct_valid = false;
    return GVX_OK;
}

static gvx_status fill_leaf_ranges(gvx_grid* g, uint32_t nleaves)
{
    GVX_CK(gvx_ensure(g->leaf_range, (size_t)(nleaves + 1) * sizeof(int2)));
    GVX_CK(gvx_ensure(g->leaf_oct, (size_t)(nleaves + 1) * 8 * sizeof(int)));
    GVX_CK(cudaMemsetAsync(g->leaf_range.p, 0, (size_t)(nleaves + 1) * sizeof(int2), g->stream));
    GVX_CK(cudaMemsetAsync(g->leaf_oct.p, 0, (size_t)(nleaves + 1) * 8 * sizeof(int), g->stream));
    if (g->n_sorted) {
        k_group_runs<<<blocks_for(g->n_sorted, 256), 256, 0, g->stream>>>(
            g->keys[g->sorted_buf].as<uint32_t>(), g->n_sorted, g->key_shift, 1u << g->lookup.ks.total_bits,
            g->lookup, g->leaf_range.as<int2>(), g->leaf_oct.as<int>());
        g->launches++;
    }
    g->oct_leaves = nleaves;
    g->oct_valid = false;
    GVX_CK(cudaGetLastError());
    return GVX_OK;
}

// the sorted point attributes (as k_permute writes them), one thread per sorted entry
__global__ void k_attr_permute(const uint32_t* __restrict__ svals, uint32_t n, const char* pos, int off, int stride,
                               float ox, float oy, float oz, GvxSortedAttr A)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < n;
    const uint32_t v = live ? svals[i] : 0u;
    float rr = 0.0f;
    if (live) {
        float w[3];
        load_pos(pos, off, stride, v, w);
        A.spos[i] = make_float4(w[0] + ox, w[1] + oy, w[2] + oz, A.weight ? A.weight[v] : 1.0f);
        if (A.radius) rr = A.radius[v];
        if (A.svel) {
            float4 q = make_float4(0.f, 0.f, 0.f, rr);
            if (A.vel) {
                const float* u = (const float*)(A.vel + (size_t)v * A.vel_stride + A.vel_off);
                q.x = u[0];
                q.y = u[1];
                q.z = u[2];
            }
            A.svel[i] = q;
        }
        rr = rr != rr ? 3.0e38f : fmaxf(rr, 0.0f);
    }
    if (A.rmax) {
        const unsigned int mm = __reduce_max_sync(0xFFFFFFFFu, __float_as_uint(rr));
        if ((threadIdx.x & 31) == 0 && mm && mm > *(volatile unsigned int*)A.rmax) atomicMax(A.rmax, mm);
    }
}

// Octant order inside every leaf, once per grouping, for the splats.  With the
// octants in the sort keys the sorted order is already (leaf key, octant,
// index) and fill_leaf_ranges has the octant starts: only the sorted attributes
// are written, one thread per entry.  Otherwise k_octant_partition partitions
// into the other value buffer (a copy of the sorted values, so entries outside
// the leaf ranges keep theirs), then copies back.
gvx_status gvx_topo_octants(gvx_grid* g, const GvxSortedAttr* attr)
{
    if (g->oct_valid) return GVX_OK;
    GvxSortedAttr none;
    memset(&none, 0, sizeof(none));
    const uint32_t nleaves = g->oct_leaves;
    if (g->key_shift) {
        if (g->n_sorted && attr && attr->spos) {
            k_attr_permute<<<blocks_for(g->n_sorted, 256), 256, 0, g->stream>>>(
                g->vals[g->sorted_buf].as<uint32_t>(), g->n_sorted, g->pts.pos, g->pts.pos_off, g->pts.pos_stride,
                g->sort_trans[0], g->sort_trans[1], g->sort_trans[2], *attr);
            g->launches++;
            GVX_CK(cudaGetLastError());
        }
    } else if (g->n_sorted && nleaves) {
        uint32_t* vin = g->vals[g->sorted_buf].as<uint32_t>();
        uint32_t* vtmp = g->vals[1 - g->sorted_buf].as<uint32_t>();
        const size_t vb = (size_t)g->n_sorted * sizeof(uint32_t);
        GVX_CK(cudaMemcpyAsync(vtmp, vin, vb, cudaMemcpyDeviceToDevice, g->stream));
        const DevCount nlc = g->oct_count.p ? g->oct_count : dc_host(nleaves);
        k_octant_partition<32><<<blocks_for((uint64_t)nleaves * 32u, 256), 256, 0, g->stream>>>(
            g->leaf_range.as<int2>(), nlc, g->nodes[0].as<GvxNode>(), g->pts.pos, g->pts.pos_off, g->pts.pos_stride,
            g->sort_trans[0], g->sort_trans[1], g->sort_trans[2], g->brick / 2, vin, vtmp, g->leaf_oct.as<int>(),
            attr ? *attr : none);
        g->launches++;
        GVX_CK(cudaMemcpyAsync(vin, vtmp, vb, cudaMemcpyDeviceToDevice, g->stream));
        GVX_CK(cudaGetLastError());
    }
    g->oct_valid = true;
    g->perm_valid = false;  // the sorted attributes follow the new order (the caller sets it when attr wrote them)
    return GVX_OK;
}

// k_dilate's per-axis limit: the key space's end or the root's (rootpos in voxels, the root's
// side in leaves), whichever comes first
static int3 dilate_limit(const KeySpace& ks, const int rootpos[3], int brick, int root_leaves)
{
    int l[3];
    for (int a = 0; a < 3; a++)
        l[a] = (int)std::min<int64_t>(int64_t(1) << ks.bits[a], (int64_t)rootpos[a] / brick + root_leaves - ks.lo[a]);
    return make_int3(l[0], l[1], l[2]);
}

static gvx_status grow_nodes(gvx_grid* g, int lev, int64_t cnt)
{
    GVX_CK(gvx_ensure(g->nodes[lev], (size_t)std::max<int64_t>(cnt, 1) * sizeof(GvxNode)));
    if (lev > 0) {
        const size_t vc = (size_t)g->res[lev] * g->res[lev] * g->res[lev];
        GVX_CK(gvx_ensure(g->clist[lev], (size_t)std::max<int64_t>(cnt, 1) * vc * sizeof(uint64_t)));
    }
    return GVX_OK;
}

// FULL rebuild: ActivateBricksGPU + ActivateExtraBricksGPU semantics
// A full build between its counts readback being queued and being read: what
// topo_full_complete needs of topo_full_launch.
struct FullBuild {
    int n;
    float radius;
    float o[3];
    int depth;
    int rootpos[3];
    KeySpace ks;
    uint32_t words0;
    UpperDesc ud;
    float mn[3], mx[3];  // the points' bounding box (GetBoundingBox before its margins)
};

// A staged RebuildTopology between its stages (gvx_topo_stage1..3), and the last full build of the
// grid (staged or not: what a plan is made from)
struct gvx_topo_staged {
    int n;
    float radius;
    int mode, min_depth;
    bool pending;
    FullBuild fb;
    bool last_full;     // the last full build (fb) finished, and the tree is still that one
    uint64_t last_gen;  // topo_gen after it
};

static gvx_status topo_full_launch_ks(gvx_grid* g, int n, float radius, const float o[3], int depth,
                                      const int rootpos[3], const KeySpace& ks, FullBuild& fb, bool queue_readback);

// the compact level-0 key space of a full build over the points' bounding box
// (+ dilation margin), inside the root
// (widen > 0: every axis's range grows by 1/widen of its length + 1 leaf on each side, inside
// the root -- the key space of a plan; hi_out: the last leaf coordinate of the range per axis)
static gvx_status full_key_space(gvx_grid* g, float radius, int depth, const int rootpos[3], const float mn[3],
                                 const float mx[3], KeySpace& ks, int widen = 0, int* hi_out = nullptr)
{
    const int b = g->brick;
    const int root_span = g->range[depth] / b;  // leaves per root side
    const int align = 1 << g->tshift[depth - 1];
    int64_t total_bits = 0;
    for (int a = 0; a < 3; a++) {
        const int rl = rootpos[a] / b;
        const float lo_v = mn[a] > 0.f ? mn[a] : 0.f;
        int lo = (int)floorf((lo_v - radius - 2.0f) / (float)b);
        int hi = mx[a] < 0.f ? rl : (int)floorf((mx[a] + 2.0f * radius + 2.0f) / (float)b);
        if (widen > 0 && hi >= lo) {
            const int m = (hi - lo + 1) / widen + 1;
            lo -= m;
            hi += m;
        }
        lo = std::max(lo, rl);
        hi = std::min(hi, rl + root_span - 1);
        if (hi < lo) hi = lo;
        lo = rl + ((lo - rl) / align) * align;
        ks.lo[a] = lo;
        ks.bits[a] = ceil_log2((int64_t)hi - lo + 1);
        if (hi_out) hi_out[a] = hi;
        total_bits += ks.bits[a];
    }
    if (total_bits > 30) {
        gvx_set_error("RebuildTopology: point extents span 2^%lld leaf cells; the compact key space holds 2^30",
                      (long long)total_bits);
        return GVX_ERR_UNSUPPORTED;
    }
    ks.total_bits = (int)total_bits;
    return GVX_OK;
}

// Everything of a full build (VG.cpp:1229-1413) up to the node counts, which are
// queued for the host; topo_full_complete reads them and writes the pools.
static gvx_status topo_full_launch(gvx_grid* g, int n, float radius, const float o[3], int depth,
                                   const int rootpos[3], const float mn[3], const float mx[3], FullBuild& fb)
{
    const int b = g->brick;
    if (radius >= 1.0f && radius > 0.5f * (float)(b - 1)) {
        gvx_set_error("RebuildTopology: radius %g exceeds (brick-1)/2 = %g (dilation beyond the 26 neighbours)",
                      radius, 0.5 * (b - 1));
        return GVX_ERR_UNSUPPORTED;
    }
    KeySpace ks;
    gvx_status rc = full_key_space(g, radius, depth, rootpos, mn, mx, ks);
    if (rc) return rc;
    for (int a = 0; a < 3; a++) {
        fb.mn[a] = mn[a];
        fb.mx[a] = mx[a];
    }
    return topo_full_launch_ks(g, n, radius, o, depth, rootpos, ks, fb, true);
}

// a full build in key space `ks` up to its node counts (d_counts), which are queued for the
// host when queue_readback
static gvx_status topo_full_launch_ks(gvx_grid* g, int n, float radius, const float o[3], int depth,
                                      const int rootpos[3], const KeySpace& ks, FullBuild& fb, bool queue_readback)
{
    cudaStream_t st = g->stream;
    const int b = g->brick;
    const bool extra = radius >= 1.0f;
    const uint32_t words0 = std::max<uint32_t>(1u, (uint32_t)((1ull << ks.total_bits) / 32ull));
    const uint32_t invalid_key = 1u << ks.total_bits;

    // ---- scratch
    GVX_CK(gvx_ensure(g->d0_bits, (size_t)words0 * 4));
    GVX_CK(gvx_ensure(g->d0_prefix, (size_t)words0 * 4));
    GVX_CK(gvx_ensure(g->x0_bits, (size_t)words0 * 4));
    GVX_CK(gvx_ensure(g->x0_prefix, (size_t)words0 * 4));
    GVX_CK(gvx_ensure(g->masks, (size_t)std::max(n, 1) * 4));
    GVX_CK(gvx_ensure(g->leaf_key, (size_t)std::max(n, 1) * 4));
    GVX_CK(cudaMemsetAsync(g->d0_bits.p, 0, (size_t)words0 * 4, st));
    GVX_CK(cudaMemsetAsync(g->x0_bits.p, 0, (size_t)words0 * 4, st));
    GVX_CK(cudaMemsetAsync(g->d_counts.p, 0, 64 * sizeof(uint32_t), st));

    UpperDesc ud;
    memset(&ud, 0, sizeof(ud));
    ud.nlev = depth - 1;
    uint32_t upper_words = 0;
    for (int l = 1; l <= ud.nlev; l++) {
        ud.tshift[l] = g->tshift[l];
        const int bl = ks_bits_at(ks, g->tshift[l]);
        ud.words[l] = std::max<uint32_t>(1u, (uint32_t)((1ull << bl) / 32ull));
        ud.off[l] = upper_words;
        upper_words += 4u * ud.words[l];
    }
    GVX_CK(gvx_ensure(g->upper, (size_t)std::max<uint32_t>(upper_words, 1u) * 4));
    if (upper_words) GVX_CK(cudaMemsetAsync(g->upper.p, 0, (size_t)upper_words * 4, st));

    // ---- one sort of the compact level-0 keys
    gvx_status rc = sort_points(g, n, o, ks, true);
    if (rc) return rc;
    const uint32_t* skeys = g->keys[g->sorted_buf].as<uint32_t>();
    const uint32_t* svals = g->vals[g->sorted_buf].as<uint32_t>();
    uint32_t* counts = g->d_counts.as<uint32_t>();

    // ---- D0: leaves holding points
    k_mark_runs<<<blocks_for(n, 256), 256, 0, st>>>(skeys, (uint32_t)n, g->key_shift, invalid_key,
                                                    g->d0_bits.as<uint32_t>());
    g->launches++;
    rc = gvx_bitmap_prefix(g->d0_bits.as<uint32_t>(), g->d0_prefix.as<uint32_t>(), words0, counts + 0, g->tmp_scan,
                           st, &g->launches);
    if (rc) return rc;
    BitRank d0{g->d0_bits.as<uint32_t>(), g->d0_prefix.as<uint32_t>(), words0};
    k_select<<<blocks_for(words0, 256), 256, 0, st>>>(d0.bits, d0.prefix, words0, g->leaf_key.as<uint32_t>(), 0xFFFFFFFFu);
    g->launches++;

    // ---- X0: dilation leaves (radius >= 1, VG.cpp:1207-1208)
    BitRank x0{g->x0_bits.as<uint32_t>(), g->x0_prefix.as<uint32_t>(), words0};
    if (extra) {
        GVX_CK(cudaMemsetAsync(g->masks.p, 0, (size_t)n * 4, st));
        k_point_masks<<<blocks_for(n, 256), 256, 0, st>>>(skeys, svals, (uint32_t)n, g->key_shift, invalid_key, d0, g->pts.pos,
                                                          g->pts.pos_off, g->pts.pos_stride, o[0], o[1], o[2],
                                                          radius, 2.0f, b, g->masks.as<uint32_t>());
        k_dilate<<<std::min(blocks_for(n, 256), 152u * 8u), 256, 0, st>>>(
            g->leaf_key.as<uint32_t>(), counts + 0, ks, dilate_limit(ks, rootpos, b, g->range[depth] / b),
            g->masks.as<uint32_t>(), d0, x0.bits, g->d_err.as<uint32_t>());
        g->launches += 2;
    }
    rc = gvx_bitmap_prefix(x0.bits, x0.prefix, words0, counts + 1, g->tmp_scan, st, &g->launches);
    if (rc) return rc;

    // ---- upper levels: parents of D0 (direct) and of X0 (extra)
    if (ud.nlev > 0) {
        k_upper_direct<<<std::min(blocks_for(n, 256), 152u * 8u), 256, 0, st>>>(g->leaf_key.as<uint32_t>(), counts + 0, ks, ud,
                                                           g->upper.as<uint32_t>());
        k_upper_extra<<<blocks_for(words0, 256), 256, 0, st>>>(x0.bits, words0, ks, ud, g->upper.as<uint32_t>());
        k_prefix_upper<<<2 * ud.nlev, 256, 0, st>>>(ud, g->upper.as<uint32_t>(), counts);
        g->launches += 3;
    }
    GVX_CK(cudaGetLastError());

    // ---- counts to the host (the one mid-build synchronisation)
    fb.n = n;
    fb.radius = radius;
    fb.depth = depth;
    for (int a = 0; a < 3; a++) {
        fb.o[a] = o[a];
        fb.rootpos[a] = rootpos[a];
    }
    fb.ks = ks;
    fb.words0 = words0;
    fb.ud = ud;
    return queue_readback ? readback_start(g, counts, 64 * sizeof(uint32_t), "RebuildTopology") : GVX_OK;
}

static gvx_status topo_full_complete(gvx_grid* g, const FullBuild& fb)
{
    cudaStream_t st = g->stream;
    const int n = fb.n, depth = fb.depth;
    const float* o = fb.o;
    const int* rootpos = fb.rootpos;
    const KeySpace ks = fb.ks;
    const uint32_t words0 = fb.words0;
    const UpperDesc& ud = fb.ud;
    const uint32_t* counts = g->d_counts.as<uint32_t>();
    (void)counts;
    const BitRank d0{g->d0_bits.as<uint32_t>(), g->d0_prefix.as<uint32_t>(), words0};
    const BitRank x0{g->x0_bits.as<uint32_t>(), g->x0_prefix.as<uint32_t>(), words0};
    uint32_t hc[64];
    gvx_status rc = readback_finish(g, hc, sizeof(hc), "RebuildTopology");
    if (rc) return rc;
    const uint32_t U0 = hc[0], X0 = hc[1];
    uint32_t Ul[GVX_MAXLEV] = {}, Xl[GVX_MAXLEV] = {};
    Ul[0] = U0;
    Xl[0] = X0;
    for (int l = 1; l < depth; l++) {
        Ul[l] = hc[2 + 2 * (l - 1)];
        Xl[l] = hc[3 + 2 * (l - 1)];
    }

    // ---- pools and lists
    for (int l = 0; l < GVX_MAXLEV; l++) g->count[l] = 0;
    for (int l = 0; l < depth; l++) {
        rc = grow_nodes(g, l, (int64_t)Ul[l] + Xl[l]);
        if (rc) return rc;
        g->count[l] = (int64_t)Ul[l] + Xl[l];
    }
    rc = grow_nodes(g, depth, 1);
    if (rc) return rc;
    g->count[depth] = 1;
    for (int l = 1; l <= depth; l++) {
        const size_t vc = (size_t)g->res[l] * g->res[l] * g->res[l];
        GVX_CK(cudaMemsetAsync(g->clist[l].p, 0xFF, (size_t)g->count[l] * vc * sizeof(uint64_t), st));
    }
    size_t list_words = (size_t)X0 + 1;
    for (int l = 1; l < depth; l++) list_words += (size_t)Ul[l] + Xl[l];
    GVX_CK(gvx_ensure(g->lists, list_words * 4));
    uint32_t* x0list = g->lists.as<uint32_t>();
    k_select<<<blocks_for(words0, 256), 256, 0, st>>>(x0.bits, x0.prefix, words0, x0list, 0xFFFFFFFFu);
    g->launches++;
    uint32_t* lp = x0list + X0 + 1;
    const uint32_t* dl[GVX_MAXLEV] = {};
    const uint32_t* xl[GVX_MAXLEV] = {};
    dl[0] = g->leaf_key.as<uint32_t>();  // D0 list (overwritten in place by k_write_nodes with the same keys)
    xl[0] = x0list;
    for (int l = 1; l < depth; l++) {
        uint32_t* base = g->upper.as<uint32_t>() + ud.off[l];
        const uint32_t w = ud.words[l];
        k_select<<<blocks_for(w, 256), 256, 0, st>>>(base, base + 2 * w, w, lp, 0xFFFFFFFFu);
        dl[l] = lp;
        lp += Ul[l];
        k_select<<<blocks_for(w, 256), 256, 0, st>>>(base + w, base + 3 * w, w, lp, 0xFFFFFFFFu);
        xl[l] = lp;
        lp += Xl[l];
        g->launches += 2;
    }
    // leaf keys in pool order: D0 (already there) then X0
    GVX_CK(gvx_ensure(g->leaf_key, (size_t)std::max<uint64_t>((uint64_t)U0 + X0, (uint64_t)n) * 4 + 4));
    // (ensure may have reallocated: D0 list must be rebuilt in that case)
    k_select<<<blocks_for(words0, 256), 256, 0, st>>>(d0.bits, d0.prefix, words0, g->leaf_key.as<uint32_t>(), 0xFFFFFFFFu);
    dl[0] = g->leaf_key.as<uint32_t>();
    if (X0)
        GVX_CK(cudaMemcpyAsync(g->leaf_key.as<uint32_t>() + U0, x0list, (size_t)X0 * 4, cudaMemcpyDeviceToDevice, st));
    g->launches++;

    // ---- nodes, parents and child lists, top-down
    k_write_root<<<1, 1, 0, st>>>(g->nodes[depth].as<GvxNode>(), depth, rootpos[0], rootpos[1], rootpos[2]);
    g->launches++;
    for (int l = depth - 1; l >= 0; l--) {
        NodeLevelArgs a;
        memset(&a, 0, sizeof(a));
        a.lev = l;
        a.depth = depth;
        a.ucount = Ul[l];
        a.xcount = Xl[l];
        a.dlist = dl[l];
        a.xlist = xl[l];
        a.ks = ks;
        a.tshift = g->tshift[l];
        a.tshift_parent = g->tshift[l + 1];
        a.logdim_parent = g->logdim[l + 1];
        a.res_parent = g->res[l + 1];
        for (int k = 0; k < 3; k++) {
            a.lo[k] = ks.lo[k] >> g->tshift[l];
            a.root_rel[k] = rootpos[k] / g->range[l];
        }
        a.range = g->range[l];
        if (l + 1 < depth) {
            uint32_t* base = g->upper.as<uint32_t>() + ud.off[l + 1];
            const uint32_t w = ud.words[l + 1];
            a.pd = BitRank{base, base + 2 * w, w};
            a.px = BitRank{base + w, base + 3 * w, w};
            a.pucount = Ul[l + 1];
        }
        a.nodes = g->nodes[l].as<GvxNode>();
        a.pclist = g->clist[l + 1].as<uint64_t>();
        a.leaf_key = nullptr;
        const uint32_t cnt = Ul[l] + Xl[l];
        if (cnt) {
            k_write_nodes<<<blocks_for(cnt, 256), 256, 0, st>>>(a);
            g->launches++;
        }
    }

    // ---- leaf lookup, neighbours, point ranges
    g->lookup.ks = ks;
    g->lookup.a = d0;
    g->lookup.b = x0;
    g->lookup.b_offset = U0;
    g->lookup.remap = nullptr;
    g->lookup.b_offset_p = nullptr;
    g->lookup.cap = 0;
    g->lookup_valid = true;
    const uint32_t L0 = U0 + X0;
    GVX_CK(gvx_ensure(g->nbr, (size_t)std::max<uint32_t>(L0, 1u) * 27 * sizeof(int)));
    if (L0) {
        k_neighbors<<<blocks_for((uint64_t)L0 * 27, 256), 256, 0, st>>>(g->leaf_key.as<uint32_t>(), dc_host(L0), g->lookup,
                                                                        g->nbr.as<int>());
        g->launches++;
    }
    g->nbr_valid = true;
    rc = fill_leaf_ranges(g, L0);
    if (rc) return rc;
    g->group_valid = true;
    g->group_pos = g->pts.pos;
    g->group_n = n;
    for (int a = 0; a < 3; a++) g->group_trans[a] = o[a];

    g->root_level = depth;
    for (int a = 0; a < 3; a++) g->root_pos[a] = rootpos[a];
    g->used_leaves = L0;
    g->atlas_valid = false;
    GVX_CK(cudaGetLastError());
    return GVX_OK;
}

static gvx_status topo_full(gvx_grid* g, int n, float radius, const float o[3], int depth, const int rootpos[3],
                            const float mn[3], const float mx[3])
{
    FullBuild fb{};
    gvx_status rc = topo_full_launch(g, n, radius, o, depth, rootpos, mn, mx, fb);
    if (rc == GVX_OK) rc = topo_full_complete(g, fb);
    // recorded for a plan (gvx_topo_plan_make)
    if (!g->staged) g->staged = new gvx_topo_staged();
    g->staged->fb = fb;
    g->staged->last_full = rc == GVX_OK;
    g->staged->last_gen = g->topo_gen;
    return rc;
}

// slots of d_counts read back by the incremental build
enum { kCntNew = 0, kCntD0 = 20, kCntActive = 48 };

// grows a pool buffer keeping its first `keep` bytes (PoolAlloc "preserve
// existing on expand", VG.cpp:1096)
static gvx_status grow_keep(gvx_grid* g, DevBuf& b, size_t bytes, size_t keep)
{
    if (b.p && bytes <= b.cap) return GVX_OK;
    DevBuf nb;
    GVX_CK(gvx_ensure(nb, bytes));
    cudaError_t e = cudaSuccess;
    if (b.p && keep) e = cudaMemcpyAsync(nb.p, b.p, keep, cudaMemcpyDeviceToDevice, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) {
        gvx_free(nb);
        return gvx_cuda_fail(e, "pool growth");
    }
    gvx_free(b);
    b = nb;
    return GVX_OK;
}

// leaf lookup over the ACTIVE leaves in key space `ks` (bitmap + rank -> pool
// index), the per-leaf keys, the neighbour table and the point ranges of the
// grouping made in `ks`.  readback: kReadUsed = the active count becomes
// used_leaves (one synchronisation, with the device error word); kReadError =
// the device error word only; kReadNone = no synchronisation (the caller knows
// the active count; a device error stays in the word for the next readback)
enum { kReadNone = 0, kReadError = 1, kReadUsed = 2 };
static gvx_status build_active_lookup(gvx_grid* g, const KeySpace& ks, uint32_t words0, int readback)
{
    cudaStream_t st = g->stream;
    const uint32_t L0 = (uint32_t)g->count[0];
    GVX_CK(gvx_ensure(g->lk_bits, (size_t)words0 * 4));
    GVX_CK(gvx_ensure(g->lk_prefix, (size_t)words0 * 4));
    GVX_CK(gvx_ensure(g->remap, (size_t)L0 * 4 + 4));
    GVX_CK(gvx_ensure(g->leaf_key, (size_t)L0 * 4 + 4));
    GVX_CK(cudaMemsetAsync(g->lk_bits.p, 0, (size_t)words0 * 4, st));
    uint32_t* counts = g->d_counts.as<uint32_t>();
    if (L0) {
        k_node_bits<<<blocks_for(L0, 256), 256, 0, st>>>(g->nodes[0].as<GvxNode>(), L0, ks, 0, g->range[0],
                                                         kSetActive, g->lk_bits.as<uint32_t>(),
                                                         g->d_err.as<uint32_t>());
        g->launches++;
    }
    gvx_status rc = gvx_bitmap_prefix(g->lk_bits.as<uint32_t>(), g->lk_prefix.as<uint32_t>(), words0,
                                      counts + kCntActive, g->tmp_scan, st, &g->launches);
    if (rc) return rc;
    const BitRank lk{g->lk_bits.as<uint32_t>(), g->lk_prefix.as<uint32_t>(), words0};
    if (L0) {
        k_node_remap<<<blocks_for(L0, 256), 256, 0, st>>>(g->nodes[0].as<GvxNode>(), L0, ks, 0, g->range[0],
                                                          kSetActive, lk, g->remap.as<int>(),
                                                          g->leaf_key.as<uint32_t>());
        g->launches++;
    }
    g->lookup.ks = ks;
    g->lookup.a = lk;
    g->lookup.b = BitRank{nullptr, nullptr, 0u};
    g->lookup.b_offset = 0u;
    g->lookup.remap = g->remap.as<int>();
    g->lookup.b_offset_p = nullptr;
    g->lookup.cap = 0;
    g->lookup_valid = true;
    GVX_CK(gvx_ensure(g->nbr, (size_t)std::max<uint32_t>(L0, 1u) * 27 * sizeof(int)));
    if (L0) {
        k_neighbors<<<blocks_for((uint64_t)L0 * 27, 256), 256, 0, st>>>(g->leaf_key.as<uint32_t>(), dc_host(L0), g->lookup,
                                                                        g->nbr.as<int>());
        g->launches++;
    }
    g->nbr_valid = true;
    rc = fill_leaf_ranges(g, L0);
    if (rc) return rc;
    if (readback == kReadUsed) {
        uint32_t used = 0;
        gvx_status rc = readback_checked(g, &used, counts + kCntActive, 4, "RebuildTopology");
        if (rc) return rc;
        g->used_leaves = used;
        return GVX_OK;
    }
    if (readback == kReadNone) {
        GVX_CK(cudaGetLastError());
        return GVX_OK;
    }
    return gvx_check_device_error(g, "RebuildTopology");
}

// Incremental rebuild (ActivateIncreBricksGPU, VG.cpp:1020-1156) of the tree
// rooted at g->root_level over levels 0..depth-1; AccumulateTopology
// (VG.cpp:1158-1178) may pass a depth below the root's level.  act[6] is the
// box of the active leaves (voxels, max exclusive; empty when min > max).
static gvx_status topo_incremental(gvx_grid* g, int n, float radius, const float o[3], int depth, bool accum,
                                   const float mn[3], const float mx[3], const int act[6])
{
    cudaStream_t st = g->stream;
    const int b = g->brick, R = g->root_level;
    if (g->count[0] == 0) return GVX_OK;  // no leaf: the reference returns at once (VG.cpp:1022)
    if (radius > (float)(b - 1)) {
        gvx_set_error("RebuildTopology: incremental radius %g exceeds brick-1 = %d (box beyond the 26 neighbours)",
                      radius, b - 1);
        return GVX_ERR_UNSUPPORTED;
    }
    if (depth > R) {
        gvx_set_error("AccumulateTopology: points need %d levels, the tree's root is at level %d", depth + 1, R);
        return GVX_ERR_DEPTH;
    }
    const int top = depth < R ? depth : depth - 1;  // highest level whose linked set is needed
    uint32_t old[GVX_MAXLEV] = {};
    for (int l = 0; l <= R; l++) old[l] = (uint32_t)g->count[l];

    // ---- key space: the points' boxes and the active leaves, inside the root
    KeySpace ks;
    const int root_span = g->range[R] / b;
    const int align = 1 << g->tshift[top];
    int64_t total_bits = 0;
    for (int a = 0; a < 3; a++) {
        const int rl = g->root_pos[a] / b;
        const float lo_v = mn[a] > 0.f ? mn[a] : 0.f;
        int lo = (int)floorf((lo_v - radius - 2.0f) / (float)b);
        int hi = mx[a] < 0.f ? rl : (int)floorf((mx[a] + radius + 2.0f) / (float)b);
        if (act[a] < act[3 + a]) {
            lo = std::min(lo, act[a] / b);
            hi = std::max(hi, act[3 + a] / b - 1);
        }
        lo = std::max(lo, rl);
        hi = std::min(hi, rl + root_span - 1);
        if (hi < lo) hi = lo;
        lo = rl + ((lo - rl) / align) * align;
        ks.lo[a] = lo;
        ks.bits[a] = ceil_log2((int64_t)hi - lo + 1);
        total_bits += ks.bits[a];
    }
    if (total_bits > 30) {
        gvx_set_error("RebuildTopology: points and active bricks span 2^%lld leaf cells; the key space holds 2^30",
                      (long long)total_bits);
        return GVX_ERR_UNSUPPORTED;
    }
    ks.total_bits = (int)total_bits;
    const uint32_t words0 = std::max<uint32_t>(1u, (uint32_t)((1ull << total_bits) / 32ull));
    const uint32_t invalid_key = 1u << ks.total_bits;

    // ---- scratch: D0 / X0 (touched level-0 cells), L0 / N0 (linked / new), upper levels
    GVX_CK(gvx_ensure(g->d0_bits, (size_t)words0 * 4));
    GVX_CK(gvx_ensure(g->d0_prefix, (size_t)words0 * 4));
    GVX_CK(gvx_ensure(g->x0_bits, (size_t)words0 * 4));
    GVX_CK(gvx_ensure(g->inc0, (size_t)words0 * 16));
    GVX_CK(gvx_ensure(g->masks, (size_t)std::max(n, 1) * 4));
    GVX_CK(gvx_ensure(g->lists, (size_t)std::max(n, 1) * 4));
    GVX_CK(cudaMemsetAsync(g->d0_bits.p, 0, (size_t)words0 * 4, st));
    GVX_CK(cudaMemsetAsync(g->x0_bits.p, 0, (size_t)words0 * 4, st));
    GVX_CK(cudaMemsetAsync(g->inc0.p, 0, (size_t)words0 * 16, st));
    GVX_CK(cudaMemsetAsync(g->d_counts.p, 0, 64 * sizeof(uint32_t), st));
    // per upper level: D (touched via direct leaves), A (via box leaves), L bits, L prefix, N bits, N prefix
    UpperDesc ud;
    memset(&ud, 0, sizeof(ud));
    ud.nlev = depth - 1;
    uint32_t upper_words = 0;
    for (int l = 1; l <= top; l++) {
        ud.tshift[l] = g->tshift[l];
        ud.words[l] = std::max<uint32_t>(1u, (uint32_t)((1ull << ks_bits_at(ks, g->tshift[l])) / 32ull));
        ud.off[l] = upper_words;
        upper_words += 6u * ud.words[l];
    }
    GVX_CK(gvx_ensure(g->upper, (size_t)std::max<uint32_t>(upper_words, 1u) * 4));
    if (upper_words) GVX_CK(cudaMemsetAsync(g->upper.p, 0, (size_t)upper_words * 4, st));
    uint32_t* upper = g->upper.as<uint32_t>();
    uint32_t* counts = g->d_counts.as<uint32_t>();
    uint32_t* err = g->d_err.as<uint32_t>();

    // ---- touched cells: the points' leaves (D0) and their boxes [int(p)-r, int(p)+r] (X0), PT.cuh:420-465
    gvx_status rc = sort_points(g, n, o, ks, true);
    if (rc) return rc;
    const uint32_t* skeys = g->keys[g->sorted_buf].as<uint32_t>();
    const uint32_t* svals = g->vals[g->sorted_buf].as<uint32_t>();
    k_mark_runs<<<blocks_for(n, 256), 256, 0, st>>>(skeys, (uint32_t)n, g->key_shift, invalid_key,
                                                    g->d0_bits.as<uint32_t>());
    g->launches++;
    rc = gvx_bitmap_prefix(g->d0_bits.as<uint32_t>(), g->d0_prefix.as<uint32_t>(), words0, counts + kCntD0,
                           g->tmp_scan, st, &g->launches);
    if (rc) return rc;
    const BitRank d0{g->d0_bits.as<uint32_t>(), g->d0_prefix.as<uint32_t>(), words0};
    uint32_t* dlist = g->lists.as<uint32_t>();
    k_select<<<blocks_for(words0, 256), 256, 0, st>>>(d0.bits, d0.prefix, words0, dlist, 0xFFFFFFFFu);
    g->launches++;
    if (radius > 0.f) {
        GVX_CK(cudaMemsetAsync(g->masks.p, 0, (size_t)n * 4, st));
        k_point_masks<<<blocks_for(n, 256), 256, 0, st>>>(skeys, svals, (uint32_t)n, g->key_shift, invalid_key, d0, g->pts.pos,
                                                          g->pts.pos_off, g->pts.pos_stride, o[0], o[1], o[2],
                                                          radius, 1.0f, b, g->masks.as<uint32_t>());
        k_dilate<<<std::min(blocks_for(n, 256), 152u * 8u), 256, 0, st>>>(
            dlist, counts + kCntD0, ks, dilate_limit(ks, g->root_pos, b, g->range[R] / b), g->masks.as<uint32_t>(), d0,
            g->x0_bits.as<uint32_t>(), err);
        g->launches += 2;
    }
    if (ud.nlev > 0) {
        k_upper_direct<<<std::min(blocks_for(n, 256), 152u * 8u), 256, 0, st>>>(dlist, counts + kCntD0, ks, ud, upper);
        k_upper_extra<<<blocks_for(words0, 256), 256, 0, st>>>(g->x0_bits.as<uint32_t>(), words0, ks, ud, upper);
        g->launches += 2;
    }

    // ---- linked sets L_l with rank -> pool index, levels 0..top
    size_t roff[GVX_MAXLEV] = {}, rtotal = 0;
    for (int l = 0; l <= top; l++) {
        roff[l] = rtotal;
        rtotal += old[l];
    }
    GVX_CK(gvx_ensure(g->inc_remap, rtotal * 4 + 4));
    BitRank Lb[GVX_MAXLEV] = {}, Nb[GVX_MAXLEV] = {};
    for (int l = 0; l <= top; l++) {
        uint32_t* base = l == 0 ? g->inc0.as<uint32_t>() : upper + ud.off[l] + 2u * ud.words[l];
        const uint32_t w = l == 0 ? words0 : ud.words[l];
        Lb[l] = BitRank{base, base + w, w};
        Nb[l] = BitRank{base + 2u * w, base + 3u * w, w};
        if (old[l]) {
            k_node_bits<<<blocks_for(old[l], 256), 256, 0, st>>>(g->nodes[l].as<GvxNode>(), old[l], ks,
                                                                 g->tshift[l], g->range[l], kSetLinked, Lb[l].bits,
                                                                 err);
            g->launches++;
        }
        rc = gvx_bitmap_prefix(Lb[l].bits, Lb[l].prefix, w, nullptr, g->tmp_scan, st, &g->launches);
        if (rc) return rc;
        if (old[l]) {
            k_node_remap<<<blocks_for(old[l], 256), 256, 0, st>>>(g->nodes[l].as<GvxNode>(), old[l], ks,
                                                                  g->tshift[l], g->range[l], kSetLinked, Lb[l],
                                                                  g->inc_remap.as<int>() + roff[l], nullptr);
            g->launches++;
        }
    }
    // ---- new nodes N_l = T_l & ~L_l, levels 0..depth-1
    for (int l = 0; l < depth; l++) {
        const uint32_t* D = l == 0 ? d0.bits : upper + ud.off[l];
        const uint32_t* A = l == 0 ? g->x0_bits.as<uint32_t>() : upper + ud.off[l] + ud.words[l];
        k_new_bits<<<blocks_for(Nb[l].words, 256), 256, 0, st>>>(D, A, Lb[l].bits, Nb[l].bits, Nb[l].words);
        g->launches++;
        rc = gvx_bitmap_prefix(Nb[l].bits, Nb[l].prefix, Nb[l].words, counts + kCntNew + l, g->tmp_scan, st,
                               &g->launches);
        if (rc) return rc;
    }
    GVX_CK(cudaGetLastError());

    // ---- new-node counts to the host
    uint32_t hc[64];
    rc = readback_checked(g, hc, counts, sizeof(hc), "RebuildTopology");
    if (rc) return rc;
    uint32_t nnew[GVX_MAXLEV] = {};
    uint64_t total_new = 0;
    for (int l = 0; l < depth; l++) {
        nnew[l] = hc[kCntNew + l];
        total_new += nnew[l];
    }
    g->group_valid = false;  // the grouping now follows `ks`
    if (total_new == 0) {
        // no new node: the reference returns before it applies the markers (VG.cpp:1066)
        rc = build_active_lookup(g, ks, words0, accum ? kReadNone : kReadError);
        if (rc) return rc;
        g->last_rebuild = 0;
    } else {
        k_apply_markers<<<blocks_for(old[0], 256), 256, 0, st>>>(g->nodes[0].as<GvxNode>(), old[0], ks, g->range[0],
                                                                 d0.bits, g->x0_bits.as<uint32_t>(), accum ? 1 : 0);
        g->launches++;
        // ---- pools grow, keeping their nodes and child lists; new lists start empty
        for (int l = 0; l < depth; l++) {
            if (!nnew[l]) continue;
            const size_t cnt = (size_t)old[l] + nnew[l];
            rc = grow_keep(g, g->nodes[l], cnt * sizeof(GvxNode), (size_t)old[l] * sizeof(GvxNode));
            if (rc) return rc;
            if (l > 0) {
                const size_t vb = (size_t)g->res[l] * g->res[l] * g->res[l] * sizeof(uint64_t);
                rc = grow_keep(g, g->clist[l], cnt * vb, (size_t)old[l] * vb);
                if (rc) return rc;
                GVX_CK(cudaMemsetAsync((char*)g->clist[l].p + (size_t)old[l] * vb, 0xFF, (size_t)nnew[l] * vb, st));
            }
        }
        // ---- sorted keys of the new nodes
        GVX_CK(gvx_ensure(g->lists, (size_t)(total_new + 1) * 4));
        const uint32_t* nl[GVX_MAXLEV] = {};
        uint32_t* lp = g->lists.as<uint32_t>();
        for (int l = 0; l < depth; l++) {
            if (!nnew[l]) continue;
            k_select<<<blocks_for(Nb[l].words, 256), 256, 0, st>>>(Nb[l].bits, Nb[l].prefix, Nb[l].words, lp, 0xFFFFFFFFu);
            g->launches++;
            nl[l] = lp;
            lp += nnew[l];
        }
        // ---- new nodes and their links (gvdbLinkBricks top-down, VG.cpp:1121-1129)
        for (int l = depth - 1; l >= 0; l--) {
            if (!nnew[l]) continue;
            IncNodeArgs a;
            memset(&a, 0, sizeof(a));
            a.lev = l;
            a.count = nnew[l];
            a.base = old[l];
            a.keys = nl[l];
            a.ks = ks;
            a.tshift = g->tshift[l];
            a.range = g->range[l];
            for (int k = 0; k < 3; k++) {
                a.lo[k] = ks.lo[k] >> g->tshift[l];
                a.root_rel[k] = g->root_pos[k] / g->range[l];
            }
            a.nodes = g->nodes[l].as<GvxNode>();
            a.parent_root = l + 1 == R;
            if (!a.parent_root) {
                a.pl = Lb[l + 1];
                a.premap = g->inc_remap.as<int>() + roff[l + 1];
                if (l + 1 < depth && nnew[l + 1]) a.pn = Nb[l + 1];
                a.pbase = old[l + 1];
            }
            a.logdim_parent = g->logdim[l + 1];
            a.res_parent = g->res[l + 1];
            a.tshift_parent = g->tshift[l + 1];
            a.pclist = g->clist[l + 1].as<uint64_t>();
            a.err = err;
            k_inc_write_nodes<<<blocks_for(nnew[l], 256), 256, 0, st>>>(a);
            g->launches++;
        }
        for (int l = 0; l < depth; l++) g->count[l] = (int64_t)old[l] + nnew[l];
        // ---- delink, bottom-up (VG.cpp:1131-1140)
        const uint32_t L0 = (uint32_t)g->count[0];
        k_delink_leaves<<<blocks_for(L0, 256), 256, 0, st>>>(g->nodes[0].as<GvxNode>(), L0,
                                                             g->nodes[1].as<GvxNode>(), (uint32_t)g->count[1],
                                                             g->clist[1].as<uint64_t>(), g->res[1], g->range[0], err);
        g->launches++;
        for (int l = 1; l < depth; l++) {
            const uint32_t cnt = (uint32_t)g->count[l];
            const uint32_t vc = (uint32_t)(g->res[l] * g->res[l] * g->res[l]);
            k_delink_upper<<<blocks_for((uint64_t)cnt * 32u, 256), 256, 0, st>>>(
                g->nodes[l].as<GvxNode>(), cnt, g->clist[l].as<uint64_t>(), vc, g->nodes[l + 1].as<GvxNode>(),
                (uint32_t)g->count[l + 1], g->clist[l + 1].as<uint64_t>(), g->res[l + 1], g->range[l], err);
            g->launches++;
        }
        GVX_CK(cudaGetLastError());
        // accumulating, no leaf is delinked and a dead one stays dead (its parent reference is
        // gone, k_apply_markers): the active count grows by the new leaves, known on the host
        rc = build_active_lookup(g, ks, words0, accum ? kReadNone : kReadUsed);
        if (rc) return rc;
        if (accum) g->used_leaves += nnew[0];
        g->atlas_valid = false;
        g->last_rebuild = 2;
    }
    g->group_valid = true;
    g->group_pos = g->pts.pos;
    g->group_n = n;
    for (int a = 0; a < 3; a++) g->group_trans[a] = o[a];
    return GVX_OK;
}

// the incremental build checks its limits (UNSUPPORTED, DEPTH) before it
// touches anything; any later failure leaves no usable tree
static gvx_status incremental_status(gvx_grid* g, gvx_status rc)
{
    if (rc == GVX_OK) g->pools_appended = true;  // the pools kept their nodes, new ones appended
    if (rc == GVX_OK || rc == GVX_ERR_UNSUPPORTED || rc == GVX_ERR_DEPTH) return rc;
    g->rebuild_topo = true;
    g->root_level = -1;
    g->lookup_valid = false;
    g->group_valid = false;
    return rc;
}

// the grid's state after a full build: a failed one leaves no usable tree
static gvx_status full_status(gvx_grid* g, gvx_status rc)
{
    if (rc) {
        g->root_level = -1;
        g->lookup_valid = false;
        g->group_valid = false;
        return rc;
    }
    g->rebuild_topo = false;
    g->last_rebuild = 1;
    return GVX_OK;
}

// GetBoundingBox's box read back (hb[0..5], order-preserving float bits) -> the points' box
// (mn, mx), bbox_min/max with the reference's margins (VG.cpp:5452-5460), and DetermineDepth:
// the lowest level whose node covers posMin and posMax, and that node's position (depth -1: none)
static void bbox_depth(gvx_grid* g, const uint32_t* hb, float mn[3], float mx[3], int* depth, int rootpos[3])
{
    int pmin[3], pmax[3];
    for (int a = 0; a < 3; a++) {
        mn[a] = ord2f(hb[a]);
        mx[a] = ord2f(hb[3 + a]);
        float lo = mn[a] - 1.0f, hi = mx[a] + 2.0f;
        lo = 0 > lo ? 0 : lo;
        hi = 0 > hi ? 0 : hi;
        g->bbox_min[a] = lo;
        g->bbox_max[a] = hi;
        pmin[a] = (int)lo;
        pmax[a] = (int)hi;
    }
    *depth = -1;
    for (int l = 0; l < g->levels; l++) {
        const int r = g->range[l];
        if (pmin[0] / r == pmax[0] / r && pmin[1] / r == pmax[1] / r && pmin[2] / r == pmax[2] / r) {
            *depth = l;
            for (int a = 0; a < 3; a++) rootpos[a] = pmin[a] / r * r;
            break;
        }
    }
}

// RebuildTopology up to GetBoundingBox's readback, which is queued
static gvx_status rebuild_begin(gvx_grid* g, int n, float radius, const float orig[3], int mode)
{
    if (!g->configured) {
        gvx_set_error("RebuildTopology: Configure was not called");
        return GVX_ERR_NOT_CONFIGURED;
    }
    if (n <= 0 || n > g->pts.n || !g->pts.pos) {
        gvx_set_error("RebuildTopology: %d points requested, %d bound by SetPoints", n, g->pts.n);
        return GVX_ERR_INVALID_ARG;
    }
    if (!(radius >= 0.f)) {
        gvx_set_error("RebuildTopology: radius must be >= 0");
        return GVX_ERR_INVALID_ARG;
    }
    gvx_status rc = ensure_grid_scratch(g);
    if (rc) return rc;
    g->sc_valid = false;
    g->pools_appended = false;
    const float o[3] = {orig ? orig[0] : 0.f, orig ? orig[1] : 0.f, orig ? orig[2] : 0.f};
    cudaStream_t st = g->stream;
    // (the device error word is not cleared here: an error left by the unchecked tail of an
    // accumulating build is reported by this build's first readback)

    // ---- GetBoundingBox: one reduction, 24 bytes to the host
    uint32_t init[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
    GVX_CK(cudaMemcpyAsync(g->d_bbox.p, init, sizeof(init), cudaMemcpyHostToDevice, st));
    // a multiple of 3 blocks (of 256 threads): the packed path needs the thread count divisible by 3
    const unsigned bb = (std::min(blocks_for(n, 256), 152u * 8u) + 2u) / 3u * 3u;
    k_bbox<<<bb, 256, 0, st>>>(g->pts.pos, g->pts.pos_off, g->pts.pos_stride, (uint32_t)n, o[0], o[1], o[2],
                               g->d_bbox.as<uint32_t>(), g->d_err.as<uint32_t>());
    g->launches++;
    // an incremental build also needs the box of the active leaves: same readback
    const bool maybe_incremental = g->root_level >= 0 && !g->rebuild_topo && mode != GVX_TOPO_FULL;
    int* act_dev = g->d_bbox.as<int>() + 8;
    k_bounds_init<<<1, 32, 0, st>>>(act_dev);
    g->launches++;
    if (maybe_incremental && g->count[0] > 0) {
        k_leaf_bounds<<<blocks_for(g->count[0], 256), 256, 0, st>>>(g->nodes[0].as<GvxNode>(),
                                                                     (uint32_t)g->count[0], g->range[0], act_dev);
        g->launches++;
    }
    return readback_start(g, g->d_bbox.p, 14 * sizeof(uint32_t), "GetBoundingBox");
}

// the rest of RebuildTopology, from the bounding box (and active-leaf box) read
// back; a full build with `fb` stops after queueing its counts readback (*pending),
// for topo_full_complete
static gvx_status rebuild_after_bbox(gvx_grid* g, int n, float radius, const float orig[3], int mode, int min_depth,
                                     const uint32_t hb[14], FullBuild* fb, bool* pending)
{
    gvx_status rc = GVX_OK;
    const float o[3] = {orig ? orig[0] : 0.f, orig ? orig[1] : 0.f, orig ? orig[2] : 0.f};
    if (pending) *pending = false;
    float mn[3], mx[3];
    int depth = -1, rootpos[3] = {0, 0, 0};
    bbox_depth(g, hb, mn, mx, &depth, rootpos);
    int act[6];
    memcpy(act, hb + 8, sizeof(act));
    if (mode == GVX_TOPO_ACCUMULATE && !g->rebuild_topo) {
        // AccumulateTopology (VG.cpp:1158-1178): depth raised to min_depth, no depth-change check
        int d = depth;
        if (d >= 0 && d < min_depth) d = min_depth;
        if (d <= 0 || d >= g->levels) {
            gvx_set_error("AccumulateTopology: depth %d outside 1..%d", d, g->levels - 1);
            return GVX_ERR_DEPTH;
        }
        g->topo_gen++;
        return incremental_status(g, topo_incremental(g, n, radius, o, d, true, mn, mx, act));
    }
    if (depth <= 0) {
        gvx_set_error(depth == 0 ? "RebuildTopology: point extents smaller than 1 brick"
                                 : "RebuildTopology: point extents exceed the configured levels");
        return GVX_ERR_DEPTH;
    }
    if (depth >= g->levels) {
        gvx_set_error("RebuildTopology: point extents need %d levels, %d configured", depth + 1, g->levels);
        return GVX_ERR_DEPTH;
    }
    // ---- state machine of RebuildTopology (VG.cpp:1195-1217)
    if (mode == GVX_TOPO_FULL) g->rebuild_topo = true;
    if (!g->rebuild_topo && depth != g->curr_depth) {
        g->rebuild_topo = true;  // "Depth change in rebuild": Clear + full rebuild
        g->curr_depth = depth;
    }
    g->topo_gen++;  // the device tree changes (or is rebuilt) from here on
    if (!g->rebuild_topo) return incremental_status(g, topo_incremental(g, n, radius, o, depth, false, mn, mx, act));
    g->atlas_prefix = -1;  // the pools are rebuilt from scratch
    if (fb) {
        rc = topo_full_launch(g, n, radius, o, depth, rootpos, mn, mx, *fb);
        if (rc == GVX_OK) {
            *pending = true;
            return GVX_OK;
        }
    } else {
        rc = topo_full(g, n, radius, o, depth, rootpos, mn, mx);
    }
    return full_status(g, rc);
}


// Staged RebuildTopology for batches of grids (gvx_batch_topology): stage 1
// queues GetBoundingBox and its readback; stage 2, once the grid's stream has
// passed it, reads the box and queues a full build up to its node counts (any
// other kind of build runs to its end here); stage 3 reads the counts and
// finishes the full build.  The host waits on a grid only where its stream
// has had the time of the other grids' stages to get there.

gvx_status gvx_topo_stage1(gvx_grid* g, int n, float radius, int mode, int min_depth)
{
    if (!g->staged) g->staged = new gvx_topo_staged();
    gvx_topo_staged& S = *g->staged;
    S.n = n;
    S.radius = radius;
    S.mode = mode;
    S.min_depth = min_depth;
    S.pending = false;
    S.last_full = false;
    return rebuild_begin(g, n, radius, nullptr, mode);
}

gvx_status gvx_topo_stage2(gvx_grid* g)
{
    gvx_topo_staged& S = *g->staged;
    uint32_t hb[14];
    gvx_status rc = readback_finish(g, hb, sizeof(hb), "GetBoundingBox");
    if (rc) return rc;
    return rebuild_after_bbox(g, S.n, S.radius, nullptr, S.mode, S.min_depth, hb, &S.fb, &S.pending);
}

gvx_status gvx_topo_stage3(gvx_grid* g)
{
    gvx_topo_staged& S = *g->staged;
    if (!S.pending) return GVX_OK;
    S.pending = false;
    gvx_status rc = full_status(g, topo_full_complete(g, S.fb));
    S.last_full = rc == GVX_OK;
    S.last_gen = g->topo_gen;
    return rc;
}

void gvx_topo_staged_free(gvx_grid* g)
{
    delete g->staged;
    g->staged = nullptr;
}

// ---------------------------------------------------------------------------
// Planned full builds, for batches of grids rebuilt every frame (gvx_batch_frame).
// A full build waits on the host twice: for the bounding box, from which the
// host takes the depth, the root and the compact key space, and for the node
// counts, which size the pools.  A plan fixes both from the grid's last full
// build: the key space (that build's, widened on every side by an eighth of its
// extent and a leaf), the depth and root, and every pool's capacity (its count + 25% + 64).
// A planned build then queues GetBoundingBox, the full RebuildTopology, UpdateAtlas
// and the octant/attribute pass of InsertPoints with no host wait and no
// allocation, so that a batch of them can be captured in one CUDA graph: its
// kernels take the counts from device memory (DevCount) and clamp every write to
// the capacities.  The counts, the bounding box and the device error word go to
// pinned memory at the end.  Once the stream has passed them, gvx_topo_plan_finish
// checks that the plan held: the frame's own DetermineDepth gives the plan's root,
// the frame's own key space lies inside the plan's, and every count fits its
// capacity.  Then the pools, lists and atlas are those of an unplanned build --
// the pool order is the order of the leaf coordinates (x, y, z lexicographic),
// the same in every key space that holds them -- and the host state is set as an
// unplanned build sets it.  Otherwise the planned build is void and the caller
// builds the grid again without a plan.

enum { kRecCounts = 0, kRecBbox = 64, kRecErr = 80, kRecWords = 96 };
enum { kCntSlots = 56 };  // d_counts slot of a planned UpdateAtlas's slot count

struct gvx_topo_plan {
    FullBuild fb;                      // key space, depth, root, points, radius (words0, ud after enqueue)
    uint32_t cap[GVX_MAXLEV] = {};     // node capacity of levels 0 .. depth-1
    uint32_t* rec = nullptr;           // pinned: counts, bounding box, error word of the last build
    int sorted_buf = 0;                // where the planned sort leaves the keys
    uint64_t id = 0;
    bool enqueued = false;
};

static std::atomic<uint64_t> g_plan_ids{0};

void gvx_topo_plan_free(gvx_grid* g)
{
    if (!g->plan) return;
    if (g->plan->rec) cudaFreeHost(g->plan->rec);
    delete g->plan;
    g->plan = nullptr;
}

// (a plan fixes sizes, not addresses: any points of the same count may be built under it)
bool gvx_topo_plan_ready(const gvx_grid* g)
{
    return g->plan && g->plan->id && g->pts.pos && g->pts.n == g->plan->fb.n;
}

uint64_t gvx_topo_plan_id(const gvx_grid* g) { return g->plan ? g->plan->id : 0; }

const uint32_t* gvx_topo_plan_slots(const gvx_grid* g, uint32_t* cap)
{
    *cap = g->plan ? g->plan->cap[0] : 0u;
    return g->d_counts.as<uint32_t>() + kCntSlots;
}

gvx_status gvx_topo_plan_make(gvx_grid* g)
{
    const gvx_topo_staged* S = g->staged;
    if (!S || !S->last_full || S->last_gen != g->topo_gen || g->root_level < 0 || !g->lookup_valid) {
        gvx_set_error("plan: the grid's tree is not the result of a staged full build");
        return GVX_ERR_STATE;
    }
    if (!g->plan) g->plan = new gvx_topo_plan();
    gvx_topo_plan& P = *g->plan;
    P.id = 0;
    P.enqueued = false;
    if (!P.rec) GVX_CK(cudaMallocHost(&P.rec, kRecWords * sizeof(uint32_t)));
    const FullBuild& last = S->fb;
    KeySpace ks;
    // the widened key space, unless it would hold more than 8x the build's cells
    if (full_key_space(g, last.radius, last.depth, last.rootpos, last.mn, last.mx, ks, 8) != GVX_OK ||
        ks.total_bits > last.ks.total_bits + 3)
        ks = last.ks;
    P.fb = last;
    P.fb.ks = ks;
    for (int l = 0; l < GVX_MAXLEV; l++) P.cap[l] = 0;
    for (int l = 0; l < last.depth; l++) {
        const uint64_t c = (uint64_t)g->count[l];
        const uint64_t cap = c + c / 4 + 64;
        if (cap >= (1ull << 31)) {
            gvx_set_error("plan: level %d holds %llu nodes", l, (unsigned long long)c);
            return GVX_ERR_CAPACITY;
        }
        P.cap[l] = (uint32_t)cap;
    }
    P.id = ++g_plan_ids;
    return GVX_OK;
}

// pools, child lists, leaf keys, lookup, neighbours and point ranges of a planned build (the
// part of topo_full_complete after the counts), every launch over the capacities
static gvx_status plan_pools(gvx_grid* g, const gvx_topo_plan& P, const FullBuild& fb)
{
    cudaStream_t st = g->stream;
    const int depth = fb.depth;
    const KeySpace ks = fb.ks;
    const uint32_t words0 = fb.words0;
    const UpperDesc& ud = fb.ud;
    const uint32_t* dcnt = g->d_counts.as<uint32_t>();
    const uint32_t cap0 = P.cap[0];
    const BitRank d0{g->d0_bits.as<uint32_t>(), g->d0_prefix.as<uint32_t>(), words0};
    const BitRank x0{g->x0_bits.as<uint32_t>(), g->x0_prefix.as<uint32_t>(), words0};

    for (int l = 0; l < depth; l++) GVX_CK_STATUS(grow_nodes(g, l, P.cap[l]));
    GVX_CK_STATUS(grow_nodes(g, depth, 1));
    for (int l = 1; l <= depth; l++) {
        const size_t vc = (size_t)g->res[l] * g->res[l] * g->res[l];
        const size_t cnt = l < depth ? P.cap[l] : 1;
        GVX_CK(cudaMemsetAsync(g->clist[l].p, 0xFF, cnt * vc * sizeof(uint64_t), st));
    }
    // lists: X0 (cap0), then D_l and X_l (cap_l each) per upper level
    size_t list_words = cap0;
    for (int l = 1; l < depth; l++) list_words += 2 * (size_t)P.cap[l];
    GVX_CK(gvx_ensure(g->lists, list_words * 4 + 4));
    uint32_t* x0list = g->lists.as<uint32_t>();
    k_select<<<blocks_for(words0, 256), 256, 0, st>>>(x0.bits, x0.prefix, words0, x0list, cap0);
    g->launches++;
    uint32_t* lp = x0list + cap0;
    const uint32_t* dl[GVX_MAXLEV] = {};
    const uint32_t* xl[GVX_MAXLEV] = {};
    dl[0] = g->leaf_key.as<uint32_t>();  // the D0 list of the first half; level 0's nodes append X0 to it
    xl[0] = x0list;
    for (int l = 1; l < depth; l++) {
        uint32_t* base = g->upper.as<uint32_t>() + ud.off[l];
        const uint32_t w = ud.words[l];
        k_select<<<blocks_for(w, 256), 256, 0, st>>>(base, base + 2 * w, w, lp, P.cap[l]);
        dl[l] = lp;
        lp += P.cap[l];
        k_select<<<blocks_for(w, 256), 256, 0, st>>>(base + w, base + 3 * w, w, lp, P.cap[l]);
        xl[l] = lp;
        lp += P.cap[l];
        g->launches += 2;
    }

    // ---- nodes, parents and child lists, top-down, counts from d_counts
    k_write_root<<<1, 1, 0, st>>>(g->nodes[depth].as<GvxNode>(), depth, fb.rootpos[0], fb.rootpos[1],
                                  fb.rootpos[2]);
    g->launches++;
    for (int l = depth - 1; l >= 0; l--) {
        NodeLevelArgs a;
        memset(&a, 0, sizeof(a));
        a.lev = l;
        a.depth = depth;
        a.dlist = dl[l];
        a.xlist = xl[l];
        a.ks = ks;
        a.tshift = g->tshift[l];
        a.tshift_parent = g->tshift[l + 1];
        a.logdim_parent = g->logdim[l + 1];
        a.res_parent = g->res[l + 1];
        for (int k = 0; k < 3; k++) {
            a.lo[k] = ks.lo[k] >> g->tshift[l];
            a.root_rel[k] = fb.rootpos[k] / g->range[l];
        }
        a.range = g->range[l];
        a.ci_pu = -1;
        if (l + 1 < depth) {
            uint32_t* base = g->upper.as<uint32_t>() + ud.off[l + 1];
            const uint32_t w = ud.words[l + 1];
            a.pd = BitRank{base, base + 2 * w, w};
            a.px = BitRank{base + w, base + 3 * w, w};
            a.ci_pu = 2 + 2 * l;
            a.pcap = P.cap[l + 1];
        }
        a.nodes = g->nodes[l].as<GvxNode>();
        a.pclist = g->clist[l + 1].as<uint64_t>();
        a.leaf_key = l == 0 ? g->leaf_key.as<uint32_t>() : nullptr;
        a.dc = dcnt;
        a.ci_u = l == 0 ? 0 : 2 + 2 * (l - 1);
        a.ci_x = a.ci_u + 1;
        a.cap = P.cap[l];
        k_write_nodes<<<blocks_for(P.cap[l], 256), 256, 0, st>>>(a);
        g->launches++;
    }

    // ---- leaf lookup (X0 offset U0 from d_counts), neighbours, point ranges
    g->lookup.ks = ks;
    g->lookup.a = d0;
    g->lookup.b = x0;
    g->lookup.b_offset = 0u;
    g->lookup.remap = nullptr;
    g->lookup.b_offset_p = dcnt;
    g->lookup.cap = cap0;
    GVX_CK(gvx_ensure(g->nbr, (size_t)cap0 * 27 * sizeof(int)));
    k_neighbors<<<blocks_for((uint64_t)cap0 * 27, 256), 256, 0, st>>>(g->leaf_key.as<uint32_t>(),
                                                                      dc_dev(dcnt, 0, 1, cap0), g->lookup,
                                                                      g->nbr.as<int>());
    g->launches++;
    return fill_leaf_ranges(g, cap0);
}

// UpdateAtlas of a planned build: slots in pool order over the leaf capacity, the slot count
// to d_counts[kCntSlots]
static gvx_status plan_atlas(gvx_grid* g, const gvx_topo_plan& P)
{
    cudaStream_t st = g->stream;
    const uint32_t cap0 = P.cap[0];
    const DevCount nl = dc_dev(g->d_counts.as<uint32_t>(), 0, 1, cap0);
    GVX_CK_STATUS(gvx_grow_atlas(g, cap0));
    const int64_t slots = (int64_t)g->sub[0] * g->sub[1] * g->sub[2];
    const uint32_t fw = cap0 / 32u + 1u;
    GVX_CK(gvx_ensure(g->amap, (size_t)slots * sizeof(int4)));
    GVX_CK(cudaMemsetAsync(g->amap.p, 0xFF, (size_t)slots * sizeof(int4), st));
    GVX_CK(gvx_ensure(g->leaf_slot, (size_t)cap0 * 4));
    GVX_CK(gvx_ensure(g->slot_leaf, (size_t)std::max<int64_t>(slots, 1) * 4));
    GVX_CK(gvx_ensure(g->bm_a, (size_t)fw * 4));
    GVX_CK(gvx_ensure(g->bm_a_prefix, (size_t)fw * 4));
    GVX_CK(cudaMemsetAsync(g->bm_a.p, 0, (size_t)fw * 4, st));
    k_flag_bits<<<blocks_for(cap0, 256), 256, 0, st>>>(g->nodes[0].as<GvxNode>(), nl, g->bm_a.as<uint32_t>());
    g->launches++;
    GVX_CK_STATUS(gvx_bitmap_prefix(g->bm_a.as<uint32_t>(), g->bm_a_prefix.as<uint32_t>(), fw,
                                    g->d_counts.as<uint32_t>() + kCntSlots, g->tmp_scan, st, &g->launches));
    k_atlas_assign<<<blocks_for(cap0, 256), 256, 0, st>>>(
        g->nodes[0].as<GvxNode>(), nl, g->bm_a.as<uint32_t>(), g->bm_a_prefix.as<uint32_t>(), g->sub[0], g->sub[1],
        g->P, g->apron, g->leaf_slot.as<int>(), g->slot_leaf.as<int>(), g->amap.as<int4>());
    g->launches++;
    return GVX_OK;
}

gvx_status gvx_topo_plan_enqueue(gvx_grid* g, const GvxSortedAttr* attr, bool frame)
{
    if (!gvx_topo_plan_ready(g)) {
        gvx_set_error("planned build: no plan for the grid's points");
        return GVX_ERR_STATE;
    }
    gvx_topo_plan& P = *g->plan;
    cudaStream_t st = g->stream;
    const int n = P.fb.n, depth = P.fb.depth;
    const uint32_t cap0 = P.cap[0];
    const float o[3] = {0.f, 0.f, 0.f};
    GVX_CK_STATUS(ensure_grid_scratch(g));
    P.enqueued = false;

    // ---- GetBoundingBox (read by gvx_topo_plan_finish)
    k_bbox_reset<<<1, 32, 0, st>>>(g->d_bbox.as<uint32_t>());
    const unsigned bb = (std::min(blocks_for(n, 256), 152u * 8u) + 2u) / 3u * 3u;
    k_bbox<<<bb, 256, 0, st>>>(g->pts.pos, g->pts.pos_off, g->pts.pos_stride, (uint32_t)n, 0.f, 0.f, 0.f,
                               g->d_bbox.as<uint32_t>(), g->d_err.as<uint32_t>());
    g->launches += 2;

    // ---- the full build in the plan's key space, sized by the capacities
    GVX_CK(gvx_ensure(g->leaf_key, ((size_t)std::max<uint32_t>(cap0, (uint32_t)n) + 1) * 4));
    FullBuild fb{};
    GVX_CK_STATUS(topo_full_launch_ks(g, n, P.fb.radius, o, depth, P.fb.rootpos, P.fb.ks, fb, false));
    P.fb.words0 = fb.words0;
    P.fb.ud = fb.ud;
    gvx_status rc = plan_pools(g, P, fb);
    if (rc == GVX_OK && frame) rc = plan_atlas(g, P);
    // ---- InsertPoints: octant order and the sorted attributes over the leaf capacity
    if (rc == GVX_OK && frame) {
        g->oct_count = dc_dev(g->d_counts.as<uint32_t>(), 0, 1, cap0);
        g->oct_valid = false;
        rc = gvx_topo_octants(g, attr);
    }
    // the kernels took the device counts by value: the host state goes back to host counts
    g->oct_count = DevCount{};
    g->lookup.b_offset_p = nullptr;
    g->lookup.cap = 0;
    g->lookup_valid = false;
    if (rc) return rc;
    GVX_CK(cudaMemcpyAsync(P.rec + kRecCounts, g->d_counts.p, 64 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GVX_CK(cudaMemcpyAsync(P.rec + kRecBbox, g->d_bbox.p, 6 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    if (!frame) GVX_CK_STATUS(gvx_topo_plan_record_error(g, st));  // (a frame records it after its splat)
    GVX_CK(cudaGetLastError());
    P.sorted_buf = g->sorted_buf;
    P.enqueued = true;
    return GVX_OK;
}

// a captured planned build queued again (its graph launched)
void gvx_topo_plan_replayed(gvx_grid* g)
{
    if (g->plan) g->plan->enqueued = true;
}

// the device error word into the plan's record, on `st` after the work that may set it (the
// caller's: after the splat of the frame)
gvx_status gvx_topo_plan_record_error(gvx_grid* g, cudaStream_t st)
{
    GVX_CK(cudaMemcpyAsync(g->plan->rec + kRecErr, g->d_err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    return GVX_OK;
}

// a void planned build: nothing of the grid's tree, atlas or grouping is usable
static void plan_void(gvx_grid* g)
{
    g->root_level = -1;
    g->rebuild_topo = true;
    g->lookup_valid = false;
    g->group_valid = false;
    g->nbr_valid = false;
    g->atlas_valid = false;
    g->atlas_prefix = -1;
    g->oct_valid = false;
    g->perm_valid = false;
    g->used_leaves = 0;
    for (int c = 0; c < GVX_MAXCH; c++) apron_invalidate(g->ch[c]);
}

gvx_status gvx_topo_plan_finish(gvx_grid* g, bool* held, bool frame)
{
    *held = false;
    if (!g->plan || !g->plan->enqueued) {
        gvx_set_error("planned build: nothing queued");
        return GVX_ERR_STATE;
    }
    gvx_topo_plan& P = *g->plan;
    P.enqueued = false;
    const uint32_t* rec = P.rec;
    const int depth = P.fb.depth;
    // as rebuild_begin / rebuild_after_bbox
    g->sc_valid = false;
    g->pools_appended = false;
    g->topo_gen++;
    g->atlas_gen++;
    gvx_status rc = report_device_error(g, rec[kRecErr], frame ? "BatchFrame" : "RebuildTopology");  // (clears it)
    if (rc) {
        plan_void(g);
        return rc;
    }
    // did the plan hold?
    float mn[3], mx[3];
    int fdepth = -1, rootpos[3] = {0, 0, 0};
    bbox_depth(g, rec + kRecBbox, mn, mx, &fdepth, rootpos);
    bool ok = fdepth == depth;
    for (int a = 0; a < 3; a++) ok = ok && rootpos[a] == P.fb.rootpos[a];
    if (ok) {
        KeySpace ks;
        int hi[3];
        if (full_key_space(g, P.fb.radius, depth, rootpos, mn, mx, ks, 0, hi) != GVX_OK) {
            ok = false;
        } else {
            for (int a = 0; a < 3; a++)
                ok = ok && ks.lo[a] >= P.fb.ks.lo[a] && (int64_t)hi[a] < (int64_t)P.fb.ks.lo[a] + (1ll << P.fb.ks.bits[a]);
        }
    }
    uint64_t cnt[GVX_MAXLEV] = {};
    for (int l = 0; l < depth && ok; l++) {
        const int ci = l == 0 ? 0 : 2 + 2 * (l - 1);
        cnt[l] = (uint64_t)rec[kRecCounts + ci] + rec[kRecCounts + ci + 1];
        ok = cnt[l] <= P.cap[l];
    }
    ok = ok && (!frame || rec[kRecCounts + kCntSlots] == cnt[0]);  // every leaf of a full build is active
    if (!ok) {
        plan_void(g);
        return GVX_OK;
    }
    // ---- the host state of a full build (topo_full_complete, full_status) ...
    const uint32_t U0 = rec[kRecCounts + 0];
    for (int l = 0; l < GVX_MAXLEV; l++) g->count[l] = 0;
    for (int l = 0; l < depth; l++) g->count[l] = (int64_t)cnt[l];
    g->count[depth] = 1;
    g->lookup.ks = P.fb.ks;
    g->lookup.a = BitRank{g->d0_bits.as<uint32_t>(), g->d0_prefix.as<uint32_t>(), P.fb.words0};
    g->lookup.b = BitRank{g->x0_bits.as<uint32_t>(), g->x0_prefix.as<uint32_t>(), P.fb.words0};
    g->lookup.b_offset = U0;
    g->lookup.remap = nullptr;
    g->lookup.b_offset_p = nullptr;
    g->lookup.cap = 0;
    g->lookup_valid = true;
    g->nbr_valid = true;
    g->sorted_buf = P.sorted_buf;
    g->n_sorted = (uint32_t)P.fb.n;
    for (int a = 0; a < 3; a++) {
        g->sort_trans[a] = 0.f;
        g->group_trans[a] = 0.f;
        g->root_pos[a] = P.fb.rootpos[a];
    }
    g->group_valid = true;
    g->group_pos = g->pts.pos;
    g->group_n = P.fb.n;
    g->root_level = depth;
    g->used_leaves = (int64_t)cnt[0];
    g->rebuild_topo = false;
    g->last_rebuild = 1;
    g->oct_leaves = (uint32_t)cnt[0];
    g->perm_valid = false;
    if (!frame) {  // the topology alone: UpdateAtlas and the octant pass are the caller's next calls
        g->atlas_valid = false;
        g->atlas_prefix = -1;
        g->oct_valid = false;
        *held = true;
        return GVX_OK;
    }
    // ... of UpdateAtlas (gvx_topo_update_atlas: every brick in a new slot) ...
    g->atlas_used = (int64_t)cnt[0];
    g->atlas_valid = true;
    for (int c = 0; c < GVX_MAXCH; c++) apron_invalidate(g->ch[c]);
    g->atlas_prefix = g->atlas_used;
    // ... and of the octant pass of InsertPoints (the attributes: the caller)
    g->oct_valid = true;
    *held = true;
    return GVX_OK;
}

// A full RebuildTopology under the plan of the grid's last full build (same point count and
// radius, no origin): the whole build queued at once and one host wait at its end, for the
// counts, the bounding box and the error word, instead of a wait for the bounding box and
// another for the counts.  *done false: the plan did not hold (or there is none), nothing of
// the grid's tree is left, and the caller builds without it.
static gvx_status rebuild_planned(gvx_grid* g, int n, float radius, const float orig[3], int mode, bool* done)
{
    *done = false;
    const bool no_orig = !orig || (orig[0] == 0.f && orig[1] == 0.f && orig[2] == 0.f);
    if (mode != GVX_TOPO_FULL || !no_orig || !g->configured || !gvx_topo_plan_ready(g) || n != g->plan->fb.n ||
        radius != g->plan->fb.radius)
        return GVX_OK;
    gvx_status rc = gvx_topo_plan_enqueue(g, nullptr, false);
    if (rc == GVX_OK) GVX_CK(cudaStreamSynchronize(g->stream));
    bool held = false;
    if (rc == GVX_OK) rc = gvx_topo_plan_finish(g, &held, false);
    if (rc) {
        plan_void(g);
        return rc;
    }
    *done = held;
    if (held) {
        g->staged->last_full = false;  // (the plan stays: it is not remade from its own builds)
        g->planned_builds++;
    }
    return GVX_OK;
}

gvx_status gvx_topo_rebuild(gvx_grid* g, int n, float radius, const float orig[3], int mode, int min_depth)
{
    bool done = false;
    gvx_status rc = rebuild_planned(g, n, radius, orig, mode, &done);
    if (rc || done) return rc;
    rc = rebuild_begin(g, n, radius, orig, mode);
    if (rc) return rc;
    uint32_t hb[14];
    rc = readback_finish(g, hb, sizeof(hb), "GetBoundingBox");
    if (rc) return rc;
    rc = rebuild_after_bbox(g, n, radius, orig, mode, min_depth, hb, nullptr, nullptr);
    // a full build plans the next ones (any points of the same count and radius)
    if (rc == GVX_OK && mode == GVX_TOPO_FULL) (void)gvx_topo_plan_make(g);
    return rc;
}



// A tree given as node pools and child lists (LoadVBX, VG.cpp:507-686: Configure, PoolRead per level,
// FinishTopology).  The pools are taken as they are; the leaf lookup, leaf keys and neighbour table
// are derived from the level-0 pool as after a build, over a compact key space spanning the leaves;
// the next RebuildTopology is a full one (Clear, VG.cpp:2487-2503, sets mRebuildTopo).
gvx_status gvx_topo_import(gvx_grid* g, int root_level, const int64_t* counts, const GvxNode* const* nodes,
                           const uint64_t* const* clists)
{
    if (!g->configured) {
        gvx_set_error("topology import: Configure was not called");
        return GVX_ERR_NOT_CONFIGURED;
    }
    if (root_level < 1 || root_level >= g->levels || counts[root_level] < 1) {
        gvx_set_error("topology import: root level %d of a %d-level tree", root_level, g->levels);
        return GVX_ERR_INVALID_ARG;
    }
    gvx_status rc = ensure_grid_scratch(g);
    if (rc) return rc;
    cudaStream_t st = g->stream;
    const int b = g->brick, R = root_level;
    // ---- compact key space over the leaves, aligned as a build aligns it inside the root
    const GvxNode& root = nodes[R][0];
    KeySpace ks;
    const int root_span = g->range[R] / b;
    const int align = 1 << g->tshift[R - 1];
    int64_t total_bits = 0;
    for (int a = 0; a < 3; a++) {
        const int rl = root.pos[a] / b;
        int lo = rl + root_span - 1, hi = rl;
        for (int64_t i = 0; i < counts[0]; i++) {
            const int c = nodes[0][i].pos[a] / b;
            lo = std::min(lo, c);
            hi = std::max(hi, c);
        }
        lo = std::max(lo, rl);
        hi = std::min(hi, rl + root_span - 1);
        if (hi < lo) hi = lo;
        lo = rl + ((lo - rl) / align) * align;
        ks.lo[a] = lo;
        ks.bits[a] = ceil_log2((int64_t)hi - lo + 1);
        total_bits += ks.bits[a];
    }
    if (total_bits > 30) {
        gvx_set_error("topology import: the leaves span 2^%lld leaf cells; the compact key space holds 2^30",
                      (long long)total_bits);
        return GVX_ERR_UNSUPPORTED;
    }
    ks.total_bits = (int)total_bits;
    // ---- pools
    for (int l = 0; l < g->levels; l++) {
        const int64_t c = l <= R ? counts[l] : 0;
        g->count[l] = c;
        if (c == 0) continue;
        rc = grow_nodes(g, l, c);
        if (rc) return rc;
        GVX_CK(cudaMemcpyAsync(g->nodes[l].p, nodes[l], (size_t)c * sizeof(GvxNode), cudaMemcpyHostToDevice, st));
        if (l > 0) {
            const size_t vc = (size_t)g->res[l] * g->res[l] * g->res[l];
            GVX_CK(cudaMemcpyAsync(g->clist[l].p, clists[l], (size_t)c * vc * sizeof(uint64_t),
                                   cudaMemcpyHostToDevice, st));
        }
    }
    g->root_level = R;
    g->topo_gen++;
    g->pools_appended = false;
    g->atlas_prefix = -1;
    for (int a = 0; a < 3; a++) g->root_pos[a] = root.pos[a];
    g->rebuild_topo = true;
    g->last_rebuild = 1;
    g->n_sorted = 0;
    g->group_valid = false;
    g->perm_valid = false;
    g->sc_valid = false;
    g->atlas_valid = false;
    GVX_CK(cudaMemsetAsync(g->d_err.p, 0, 4, st));
    const uint32_t words0 = std::max<uint32_t>(1u, (uint32_t)((1ull << total_bits) / 32ull));
    return build_active_lookup(g, ks, words0, kReadUsed);
}

gvx_status gvx_topo_update_atlas(gvx_grid* g)
{
    if (g->root_level < 0) {
        gvx_set_error("UpdateAtlas: no topology");
        return GVX_ERR_STATE;
    }
    if (!g->have_atlas) {
        gvx_set_error("UpdateAtlas: no channel added");
        return GVX_ERR_STATE;
    }
    cudaStream_t st = g->stream;
    const int64_t used = g->used_leaves;
    // Slots go to the active leaves in pool order.  When the last UpdateAtlas gave every leaf
    // below atlas_prefix its own index as slot and the build since only appended leaves, all of
    // them active (AccumulateTopology), those leaves keep their slots and values: the aprons stay
    // copies except in the new bricks and around them.
    const int64_t from = g->pools_appended && g->atlas_prefix >= 0 && g->atlas_prefix <= used &&
                                 used == g->count[0]
                             ? g->atlas_prefix
                             : -1;
    gvx_status rc = gvx_grow_atlas(g, used);
    if (rc) return rc;
    const int64_t slots = (int64_t)g->sub[0] * g->sub[1] * g->sub[2];
    const uint32_t L0 = (uint32_t)g->count[0];
    const uint32_t fw = std::max<uint32_t>(1u, (L0 + 31u) / 32u);
    GVX_CK(gvx_ensure(g->amap, (size_t)slots * sizeof(int4)));
    GVX_CK(cudaMemsetAsync(g->amap.p, 0xFF, (size_t)slots * sizeof(int4), st));
    GVX_CK(gvx_ensure(g->leaf_slot, (size_t)std::max<uint32_t>(L0, 1u) * 4));
    GVX_CK(gvx_ensure(g->slot_leaf, (size_t)std::max<int64_t>(slots, 1) * 4));
    GVX_CK(gvx_ensure(g->bm_a, (size_t)fw * 4));
    GVX_CK(gvx_ensure(g->bm_a_prefix, (size_t)fw * 4));
    GVX_CK(cudaMemsetAsync(g->bm_a.p, 0, (size_t)fw * 4, st));
    if (L0) {
        k_flag_bits<<<blocks_for(L0, 256), 256, 0, st>>>(g->nodes[0].as<GvxNode>(), dc_host(L0), g->bm_a.as<uint32_t>());
        g->launches++;
        rc = gvx_bitmap_prefix(g->bm_a.as<uint32_t>(), g->bm_a_prefix.as<uint32_t>(), fw, nullptr, g->tmp_scan, st,
                               &g->launches);
        if (rc) return rc;
        k_atlas_assign<<<blocks_for(L0, 256), 256, 0, st>>>(
            g->nodes[0].as<GvxNode>(), dc_host(L0), g->bm_a.as<uint32_t>(), g->bm_a_prefix.as<uint32_t>(), g->sub[0],
            g->sub[1], g->P, g->apron, g->leaf_slot.as<int>(), g->slot_leaf.as<int>(), g->amap.as<int4>());
        g->launches++;
    }
    GVX_CK(cudaGetLastError());
    g->atlas_used = used;
    g->atlas_valid = true;
    g->sc_valid = false;  // subcell indices follow the atlas slots
    for (int c = 0; c < GVX_MAXCH; c++) {
        GvxChannel& ch = g->ch[c];
        if (from < 0 || !(ch.apron_valid || ch.apron_partial_from >= 0)) {
            apron_invalidate(ch);  // bricks moved to new slots
        } else if (from < used) {
            ch.apron_partial_from = ch.apron_valid ? from : std::min(ch.apron_partial_from, from);
            ch.apron_valid = false;
        }
    }
    g->atlas_prefix = used == g->count[0] ? used : -1;
    g->atlas_gen++;
    return GVX_OK;
}

// ComputeBounds (VG.cpp:1792-1816) runs on the device: min and max both start
// at level-0 pool node 0's position whatever its flags (a delinked node 0
// still seeds them), then the active leaves lower the minimum to their
// positions and raise the maximum to position + range.  mVoxResMax (the
// largest max - min per axis since Configure) is kept on the device beside
// them.  The result is read when the host asks for it (gvx_get_info), so
// FinishTopology adds no synchronisation.  host_stage: ints [0..2] min,
// [3..5] max, [6..8] res max.
__global__ void k_bounds_seed(const GvxNode* __restrict__ nodes, uint32_t n, int* out, int reset_res_max)
{
    const int a = threadIdx.x;
    if (a < 3) {
        out[a] = n ? nodes[0].pos[a] : 0x7FFFFFFF;
        out[3 + a] = n ? nodes[0].pos[a] : (int)0x80000000;
        if (reset_res_max) out[6 + a] = 0;
    }
}

__global__ void k_bounds_res_max(int* out, uint32_t n)
{
    const int a = threadIdx.x;
    if (a < 3 && n) out[6 + a] = max(out[6 + a], out[3 + a] - out[a]);
}

gvx_status gvx_topo_compute_bounds(gvx_grid* g)
{
    if (g->root_level < 0) return GVX_OK;
    gvx_status rc = ensure_grid_scratch(g);
    if (rc) return rc;
    const uint32_t L0 = (uint32_t)g->count[0];
    GVX_CK(gvx_ensure(g->host_stage, 64));
    k_bounds_seed<<<1, 32, 0, g->stream>>>(g->nodes[0].as<GvxNode>(), L0, g->host_stage.as<int>(),
                                          g->vox_res_max_reset ? 1 : 0);
    g->launches++;
    g->vox_res_max_reset = false;
    if (L0) {
        k_leaf_bounds<<<blocks_for(L0, 256), 256, 0, g->stream>>>(g->nodes[0].as<GvxNode>(), L0, g->range[0],
                                                                   g->host_stage.as<int>());
        k_bounds_res_max<<<1, 32, 0, g->stream>>>(g->host_stage.as<int>(), L0);
        g->launches += 2;
    }
    GVX_CK(cudaGetLastError());
    g->bounds_pending = true;
    return GVX_OK;
}

gvx_status gvx_topo_read_bounds(gvx_grid* g)
{
    if (!g->bounds_pending) return GVX_OK;
    int hb[9];
    GVX_CK(cudaMemcpyAsync(hb, g->host_stage.p, sizeof(hb), cudaMemcpyDeviceToHost, g->stream));
    GVX_CK(cudaStreamSynchronize(g->stream));
    const bool any = g->count[0] > 0;
    for (int a = 0; a < 3; a++) {
        g->obj_min[a] = any ? (float)hb[a] : 0.f;
        g->obj_max[a] = any ? (float)hb[3 + a] : 0.f;
        g->vox_res_max[a] = (float)hb[6 + a];
    }
    g->bounds_pending = false;
    return GVX_OK;
}

// InsertPoints: group the points by leaf for positions + trans, reusing the
// grouping of the topology build when it was made from the same points
gvx_status gvx_topo_group_points(gvx_grid* g, int n, const float trans[3])
{
    if (!g->lookup_valid) {
        gvx_set_error("InsertPoints: no topology");
        return GVX_ERR_STATE;
    }
    if (n <= 0 || n > g->pts.n || !g->pts.pos) {
        gvx_set_error("InsertPoints: %d points requested, %d bound", n, g->pts.n);
        return GVX_ERR_INVALID_ARG;
    }
    const float t[3] = {trans ? trans[0] : 0.f, trans ? trans[1] : 0.f, trans ? trans[2] : 0.f};
    if (g->group_valid && g->group_pos == g->pts.pos && g->group_n == n && t[0] == g->group_trans[0] &&
        t[1] == g->group_trans[1] && t[2] == g->group_trans[2])
        return GVX_OK;
    gvx_status rc = ensure_grid_scratch(g);
    if (rc) return rc;
    rc = sort_points(g, n, t, g->lookup.ks, true);
    if (rc) return rc;
    rc = fill_leaf_ranges(g, (uint32_t)g->count[0]);
    if (rc) return rc;
    g->group_valid = true;
    g->group_pos = g->pts.pos;
    g->group_n = n;
    for (int a = 0; a < 3; a++) g->group_trans[a] = t[a];
    return GVX_OK;
}
