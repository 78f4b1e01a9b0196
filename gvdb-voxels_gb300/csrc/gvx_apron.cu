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
// channel's native element (float4 for FLOAT3/FLOAT4 channels).
#include "gvx_grid.cuh"

struct ApronArgs {
    int brick, P;
    uint32_t nslots;
    const int* slot_leaf;
    const int* leaf_slot;
    const int* nbr;
    void* data;
};

// apron voxel number e of a padded brick (apron 1) -> padded coordinates
__device__ __forceinline__ void apron_voxel(int e, int P, int& x, int& y, int& z)
{
    const int P2 = P * P;
    if (e < 2 * P2) {
        z = e < P2 ? 0 : P - 1;
        const int r = e % P2;
        y = r / P;
        x = r % P;
        return;
    }
    const int ring = 4 * P - 4;
    const int j = e - 2 * P2;
    z = 1 + j / ring;
    const int r = j % ring;
    if (r < 2 * P) {
        y = r < P ? 0 : P - 1;
        x = r % P;
    } else {
        const int r2 = r - 2 * P;
        y = 1 + r2 / 2;
        x = (r2 & 1) ? P - 1 : 0;
    }
}

template <class T>
__global__ void k_apron(ApronArgs a, T boundval)
{
    const int lane = threadIdx.x & 31;
    const uint32_t wglobal = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const int P = a.P, b = a.brick, P3 = P * P * P;
    const int napron = 6 * P * P - 12 * P + 8;
    T* data = (T*)a.data;
    for (uint32_t s = wglobal; s < a.nslots; s += nwarps) {
        const int leaf = a.slot_leaf[s];
        const int* nb = a.nbr + (size_t)leaf * 27;
        T* dst = data + (size_t)s * P3;
        for (int e = lane; e < napron; e += 32) {
            int x, y, z;
            apron_voxel(e, P, x, y, z);
            const int dx = x == 0 ? -1 : (x == P - 1 ? 1 : 0);
            const int dy = y == 0 ? -1 : (y == P - 1 ? 1 : 0);
            const int dz = z == 0 ? -1 : (z == P - 1 ? 1 : 0);
            const int nl = nb[(dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)];
            const int ns = nl >= 0 ? a.leaf_slot[nl] : -1;
            T v = boundval;
            if (ns >= 0) {
                const int sx = x - dx * b, sy = y - dy * b, sz = z - dz * b;  // padded coords in the neighbour
                v = data[(size_t)ns * P3 + (sz * P + sy) * P + sx];
            }
            dst[(z * P + y) * P + x] = v;
        }
    }
}

gvx_status gvx_apron_run(gvx_grid* g, int chan, float boundval)
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
    ApronArgs a;
    a.brick = g->brick;
    a.P = g->P;
    a.nslots = (uint32_t)g->atlas_used;
    a.slot_leaf = g->slot_leaf.as<int>();
    a.leaf_slot = g->leaf_slot.as<int>();
    a.nbr = g->nbr.as<int>();
    a.data = g->ch[chan].data.p;
    if (a.nslots == 0) return GVX_OK;
    const unsigned threads = 256;
    const uint64_t warps_needed = a.nslots;
    unsigned blocks = (unsigned)std::min<uint64_t>((warps_needed + 7) / 8, 152ull * 16ull);
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
