// gvx_apron.cu -- UpdateApron.
//
// Reference: VolumeGVDB::UpdateApron (gvdb_volume_gvdb.cpp:4418-4457) and the
// UpdateApron<T> kernels (cuda_gvdb_operators.cuh:73-146): every apron voxel of
// every brick (faces, edges and corners) receives the value of the interior
// voxel at the same index-space position in whichever brick holds it, or the
// boundary value when no brick does.  The reference finds that brick with a
// full root-to-leaf descent per apron voxel; here the 26 neighbours of every
// leaf are resolved once per topology (gvx_topology.cu, k_neighbors) and one
// warp copies a brick's 6P^2-12P+8 apron voxels with loads/stores of the
// channel's native element (float4 for FLOAT3/FLOAT4 channels).  The warp
// first resolves the brick's 26 neighbour slots into shared memory; the
// voxels then come from a table, built once per brick shape, of (apron voxel,
// neighbour, source voxel in that neighbour).
#include <string.h>

#include <vector>

#include "gvx_grid.cuh"

namespace {
constexpr int kApronWarps = 8;
}

struct ApronArgs {
    int brick, P;
    uint32_t nslots;
    const int* slot_leaf;
    const int* leaf_slot;
    const int* nbr;
    const uint2* tab;  // per apron voxel: padded index | neighbour << 24, source index in the neighbour
    int napron;
    void* data;
    const unsigned char* only;  // optional per-slot mark: bricks whose aprons are copied (others kept)
};

template <class T>
__global__ void __launch_bounds__(kApronWarps * 32) k_apron(ApronArgs a, T boundval)
{
    __shared__ int s_ns[kApronWarps][27];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t wglobal = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const int P3 = a.P * a.P * a.P;
    T* data = (T*)a.data;
    for (uint32_t s = wglobal; s < a.nslots; s += nwarps) {
        if (a.only && !a.only[s]) continue;  // warp-uniform: one brick per warp
        const int leaf = a.slot_leaf[s];
        if (lane < 27) {
            const int nl = a.nbr[(size_t)leaf * 27 + lane];
            s_ns[wid][lane] = nl >= 0 ? a.leaf_slot[nl] : -1;
        }
        __syncwarp();
        T* dst = data + (size_t)s * P3;
        // U values per lane are loaded before any is stored: the sources (neighbours' interiors)
        // and the destinations (this brick's apron) are the same array, so a load-store loop
        // would keep one load in flight per lane
        constexpr int U = sizeof(T) <= 4 ? 16 : 4;
        for (int e0 = 0; e0 < a.napron; e0 += 32 * U) {
            T v[U];
            uint32_t di[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int e = e0 + u * 32 + lane;
                v[u] = boundval;
                di[u] = 0xFFFFFFFFu;
                if (e < a.napron) {
                    const uint2 t = a.tab[e];
                    const int ns = s_ns[wid][t.x >> 24];
                    if (ns >= 0) v[u] = data[(size_t)ns * P3 + t.y];
                    di[u] = t.x & 0xFFFFFFu;
                }
            }
#pragma unroll
            for (int u = 0; u < U; u++)
                if (di[u] != 0xFFFFFFFFu) dst[di[u]] = v[u];
        }
        __syncwarp();
    }
}

// the table of k_apron for padded bricks of side P (apron 1)
static std::vector<uint2> apron_table(int P, int b)
{
    const int napron = 6 * P * P - 12 * P + 8;
    std::vector<uint2> t((size_t)napron);
    for (int e = 0; e < napron; e++) {
        int x, y, z;
        const int P2 = P * P;
        if (e < 2 * P2) {
            z = e < P2 ? 0 : P - 1;
            y = (e % P2) / P;
            x = (e % P2) % P;
        } else {
            const int ring = 4 * P - 4, j = e - 2 * P2, r = j % ring;
            z = 1 + j / ring;
            if (r < 2 * P) {
                y = r < P ? 0 : P - 1;
                x = r % P;
            } else {
                y = 1 + (r - 2 * P) / 2;
                x = ((r - 2 * P) & 1) ? P - 1 : 0;
            }
        }
        const int dx = x == 0 ? -1 : (x == P - 1 ? 1 : 0);
        const int dy = y == 0 ? -1 : (y == P - 1 ? 1 : 0);
        const int dz = z == 0 ? -1 : (z == P - 1 ? 1 : 0);
        const int k = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1);
        const int sx = x - dx * b, sy = y - dy * b, sz = z - dz * b;  // padded coords in the neighbour
        t[e] = make_uint2((uint32_t)((z * P + y) * P + x) | ((uint32_t)k << 24), (uint32_t)((sz * P + sy) * P + sx));
    }
    return t;
}

// UpdateApronFaces (VG.cpp:4461-4496, gvdbUpdateApronFacesF OP.cuh:27-63): per active brick and
// each of its -x, -y, -z face neighbours, the b^2 voxel pairs across the shared face: the
// neighbour's +side apron takes the brick's first interior layer, the brick's -side apron the
// neighbour's last.  Every apron voxel has one writer and only interior voxels are read.
__global__ void __launch_bounds__(kApronWarps * 32) k_apron_faces(ApronArgs a)
{
    const int lane = threadIdx.x & 31;
    const uint32_t wglobal = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const int P = a.P, b = a.brick, P3 = P * P * P;
    float* data = (float*)a.data;
    for (uint32_t s = wglobal; s < a.nslots; s += nwarps) {
        const int leaf = a.slot_leaf[s];
#pragma unroll 1
        for (int side = 0; side < 3; side++) {
            const int k = side == 0 ? 12 : (side == 1 ? 10 : 4);  // (-1,0,0), (0,-1,0), (0,0,-1) in the 27 table
            const int nl = a.nbr[(size_t)leaf * 27 + k];
            const int ns = nl >= 0 ? a.leaf_slot[nl] : -1;
            if (ns < 0) continue;
            float* self = data + (size_t)s * P3;
            float* nbr = data + (size_t)ns * P3;
            const int st[3] = {1, P, P * P};  // padded strides of x, y, z
            const int ax = side, au = side == 0 ? 1 : 0, av = side == 2 ? 1 : 2;
            for (int e = lane; e < b * b; e += 32) {
                const int u = 1 + e % b, v = 1 + e / b;
                const int base = u * st[au] + v * st[av];
                const float v1 = self[base + 1 * st[ax]];  // the brick's first interior layer
                const float v2 = nbr[base + b * st[ax]];   // the neighbour's last interior layer
                nbr[base + (b + 1) * st[ax]] = v1;
                self[base] = v2;
            }
        }
    }
}

gvx_status gvx_apron_faces_run(gvx_grid* g, int chan)
{
    if (chan < 0 || chan >= GVX_MAXCH || !g->ch[chan].used) {
        gvx_set_error("UpdateApronFaces: channel %d does not exist", chan);
        return GVX_ERR_INVALID_ARG;
    }
    if (g->apron == 0) return GVX_OK;  // VG.cpp:4463
    if (g->ch[chan].type != GVX_T_FLOAT) {
        gvx_set_error("UpdateApronFaces: float channels only (the reference's one kernel, OP.cuh:27)");
        return GVX_ERR_UNSUPPORTED;
    }
    if (g->root_level < 0 || !g->atlas_valid || !g->nbr_valid) {
        gvx_set_error("UpdateApronFaces: no topology/atlas");
        return GVX_ERR_STATE;
    }
    ApronArgs a;
    memset(&a, 0, sizeof(a));
    a.brick = g->brick;
    a.P = g->P;
    a.nslots = (uint32_t)g->atlas_used;
    a.slot_leaf = g->slot_leaf.as<int>();
    a.leaf_slot = g->leaf_slot.as<int>();
    a.nbr = g->nbr.as<int>();
    a.data = g->ch[chan].data.p;
    if (a.nslots == 0) return GVX_OK;
    const unsigned blocks = (unsigned)std::min<uint64_t>((a.nslots + kApronWarps - 1) / kApronWarps, 152ull * 16ull);
    k_apron_faces<<<blocks, kApronWarps * 32, 0, g->stream>>>(a);
    g->launches++;
    GVX_CK(cudaGetLastError());
    apron_invalidate(g->ch[chan]);  // edges and corners are not updated
    return GVX_OK;
}

// marks the bricks of slots >= from (added by an appending topology build) and their 26
// neighbours: the bricks whose aprons may differ from the neighbours' interiors
__global__ void k_apron_mark(uint32_t from, uint32_t nslots, const int* __restrict__ slot_leaf,
                             const int* __restrict__ leaf_slot, const int* __restrict__ nbr, unsigned char* mark)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t s = from + i / 27;
    if (s >= nslots) return;
    const int k = (int)(i % 27);
    const int leaf = slot_leaf[s];
    if (k == 13) {
        mark[s] = 1;
        return;
    }
    const int nl = nbr[(size_t)leaf * 27 + k];
    if (nl < 0) return;
    const int ns = leaf_slot[nl];
    if (ns >= 0) mark[ns] = 1;
}

static gvx_status apron_launch(gvx_grid* g, int chan, float boundval, const unsigned char* only);

gvx_status gvx_apron_run(gvx_grid* g, int chan, float boundval) { return apron_launch(g, chan, boundval, nullptr); }

gvx_status gvx_apron_run_partial(gvx_grid* g, int chan, float boundval, int64_t from)
{
    if (g->apron == 0) return GVX_OK;
    const int64_t used = g->atlas_used;
    if (from >= used) return GVX_OK;  // no new brick: every apron holds its copies
    if (g->apron_mark_from != from || g->apron_mark_gen != g->atlas_gen) {
        // the marks are shared by the channels of one UpdateAtlas
        GVX_CK(gvx_ensure(g->apron_mark, (size_t)used));
        GVX_CK(cudaMemsetAsync(g->apron_mark.p, 0, (size_t)used, g->stream));
        const uint64_t work = (uint64_t)(used - from) * 27u;
        k_apron_mark<<<(unsigned)((work + 255) / 256), 256, 0, g->stream>>>(
            (uint32_t)from, (uint32_t)used, g->slot_leaf.as<int>(), g->leaf_slot.as<int>(), g->nbr.as<int>(),
            g->apron_mark.as<unsigned char>());
        g->launches++;
        g->apron_mark_from = from;
        g->apron_mark_gen = g->atlas_gen;
    }
    return apron_launch(g, chan, boundval, g->apron_mark.as<unsigned char>());
}

static gvx_status apron_launch(gvx_grid* g, int chan, float boundval, const unsigned char* only)
{
    if (chan < 0 || chan >= GVX_MAXCH || !g->ch[chan].used) {
        gvx_set_error("UpdateApron: channel %d does not exist", chan);
        return GVX_ERR_INVALID_ARG;
    }
    if (g->apron == 0) return GVX_OK;  // VG.cpp:4420
    if (g->root_level < 0 || !g->atlas_valid || !g->nbr_valid) {
        gvx_set_error("UpdateApron: no topology/atlas");
        return GVX_ERR_STATE;
    }
    const int P = g->P;
    if (g->apron_tab_P != P) {  // (P^3 < 2^24 for bricks up to 2^6: the packing holds)
        const std::vector<uint2> tab = apron_table(P, g->brick);
        GVX_CK(gvx_ensure(g->apron_tab, tab.size() * sizeof(uint2)));
        GVX_CK(cudaMemcpy(g->apron_tab.p, tab.data(), tab.size() * sizeof(uint2), cudaMemcpyHostToDevice));
        g->apron_tab_P = P;
    }
    ApronArgs a;
    a.brick = g->brick;
    a.P = g->P;
    a.tab = g->apron_tab.as<uint2>();
    a.napron = 6 * P * P - 12 * P + 8;
    a.nslots = (uint32_t)g->atlas_used;
    a.slot_leaf = g->slot_leaf.as<int>();
    a.leaf_slot = g->leaf_slot.as<int>();
    a.nbr = g->nbr.as<int>();
    a.data = g->ch[chan].data.p;
    a.only = only;
    if (a.nslots == 0) return GVX_OK;
    const unsigned threads = kApronWarps * 32;
    const uint64_t warps_needed = a.nslots;
    unsigned blocks = (unsigned)std::min<uint64_t>((warps_needed + kApronWarps - 1) / kApronWarps, 152ull * 16ull);
    switch (g->ch[chan].type) {
    case GVX_T_FLOAT:
        k_apron<float><<<blocks, threads, 0, g->stream>>>(a, boundval);
        break;
    case GVX_T_FLOAT3:
    case GVX_T_FLOAT4:
        k_apron<float4><<<blocks, threads, 0, g->stream>>>(a, make_float4(boundval, boundval, boundval, boundval));
        break;
    case GVX_T_UCHAR: {
        const unsigned char bv = (unsigned char)boundval;
        k_apron<unsigned char><<<blocks, threads, 0, g->stream>>>(a, bv);
        break;
    }
    case GVX_T_UCHAR4: {
        const unsigned char bv = (unsigned char)boundval;
        k_apron<uchar4><<<blocks, threads, 0, g->stream>>>(a, make_uchar4(bv, bv, bv, bv));
        break;
    }
    default:
        gvx_set_error("UpdateApron: channel type %d", g->ch[chan].type);
        return GVX_ERR_UNSUPPORTED;
    }
    g->launches++;
    GVX_CK(cudaGetLastError());
    return GVX_OK;
}
