// gvx_compute.cu -- Compute(effect, channel, iterations, params, bUpdateApron,
// skipOverAprons, boundval) over the brick atlas (VG.cpp:4532-4558) for the
// operators of the point path's samples: FUNC_FILL_F / FILL_C / FILL_C4
// (gvdbOpFill*, OP.cuh:352-380) and FUNC_SMOOTH (gvdbOpSmooth, OP.cuh:383-400).
//
// The reference launches 8^3-thread blocks over T = skipOverAprons ?
// getAtlasPackres : getAtlasRes threads per axis, and each operator's own
// index macro picks the voxels it writes (OP.cuh:189-223):
//  - the fills (GVDB_VOXUNPACKED) write atlas voxel blockIdx*8 + threadIdx + 1,
//    i.e. every voxel whose coordinates all lie in [1, min(8 ceil(T/8) + 1, R));
//  - FUNC_SMOOTH (GVDB_VOXPACKED) writes every brick interior voxel whatever T
//    is, from the six face neighbours read before any write.  With an apron
//    those are the brick's own apron voxels: one block here takes one atlas
//    slot, its padded block in shared memory, so slots are independent.  With
//    no apron they lie in other bricks, which the reference's blocks may be
//    writing meanwhile; here the iteration reads a snapshot of the atlas
//    (Jacobi, the ordering in which every read comes first) and 0 outside
//    the atlas.  The channel's device pointer never moves.
#include "gvx_grid.cuh"

namespace {
constexpr int kComputeThreads = 256;
inline unsigned blocks_for(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

struct AtlasShape {
    int P, sx, sy, sz;
};

// atlas slot element i -> atlas voxel coordinates
__device__ __forceinline__ void atlas_coords(const AtlasShape& s, size_t i, int& X, int& Y, int& Z)
{
    const int P = s.P, P3 = P * P * P;
    const size_t slot = i / (size_t)P3;
    const int r = (int)(i - slot * (size_t)P3);
    const int bx = (int)(slot % (size_t)s.sx), by = (int)((slot / (size_t)s.sx) % (size_t)s.sy),
              bz = (int)(slot / ((size_t)s.sx * s.sy));
    X = bx * P + r % P;
    Y = by * P + (r / P) % P;
    Z = bz * P + r / (P * P);
}

// atlas voxel (X, Y, Z) -> element index in the brick-major channel
__device__ __forceinline__ size_t atlas_index(const AtlasShape& s, int X, int Y, int Z)
{
    const int bx = X / s.P, by = Y / s.P, bz = Z / s.P;
    const size_t slot = ((size_t)bz * s.sy + by) * s.sx + bx;
    return ((slot * s.P + (Z - bz * s.P)) * s.P + (Y - by * s.P)) * s.P + (X - bx * s.P);
}

// v / (p1 + 6) + p2 after the float sum.  The reference divides in double
// (OP.cuh:397: a double literal); FP32 here, correctly rounded, is within one
// float rounding of it and keeps the FP64 units (a small fraction of GB300's
// throughput) off the stencil
__device__ __forceinline__ float smooth_value(float v, float p1, float p2)
{
    return __fadd_rn(__fdiv_rn(v, __fadd_rn(p1, 6.0f)), p2);
}

}  // namespace

// FUNC_FILL_F / FILL_C / FILL_C4 over the atlas voxels in [1, hi) per axis,
// one thread per atlas voxel
__global__ void k_fill_op(unsigned char* data, AtlasShape s, int3 hi, int effect, float p1, float p2, float p3,
                          size_t nvox)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nvox; i += (size_t)gridDim.x * blockDim.x) {
        int X, Y, Z;
        atlas_coords(s, i, X, Y, Z);
        if (X < 1 || Y < 1 || Z < 1 || X >= hi.x || Y >= hi.y || Z >= hi.z) continue;
        if (effect == GVX_FUNC_FILL_F) {
            float v = p1;
            if (p3 < 0.0f)  // the reference's test pattern (OP.cuh:356-361)
                v = sinf((float)((double)(X * 12) / (3.141592 * 30.0))) +
                    sinf((float)((double)(Y * 12) / (3.141592 * 30.0))) +
                    sinf((float)((double)(Z * 12) / (3.141592 * 30.0)));
            ((float*)data)[i] = v;
        } else if (effect == GVX_FUNC_FILL_C) {
            data[i] = (unsigned char)(unsigned)fminf(fmaxf(p1, 0.0f), 255.0f);  // truncated, saturating
        } else {  // FILL_C4: CLR2INT(p1, p2, p3, 1) (OP.cuh:20), the components * 255 ORed unmasked
            const uint32_t c = (255u << 24) | ((uint32_t)(p3 * 255.0f) << 16) | ((uint32_t)(p2 * 255.0f) << 8) |
                               (uint32_t)(p1 * 255.0f);
            ((uint32_t*)data)[i] = c;
        }
    }
}

// FUNC_SMOOTH with an apron: one block per atlas slot, the slot's padded block
// staged in shared memory, its interior written back in place
__global__ void k_smooth_slots(float* data, int P, int apron, size_t nslots, float p1, float p2)
{
    extern __shared__ __align__(16) float sb[];
    const int P3 = P * P * P;
    const int b = P - 2 * apron;
    for (size_t s = blockIdx.x; s < nslots; s += gridDim.x) {
        float* g = data + s * (size_t)P3;
        if ((P3 & 3) == 0) {  // slots of P^3 floats, P even: 16-byte aligned, moved as float4
            const float4* g4 = (const float4*)g;
            for (int i = threadIdx.x; i < P3 / 4; i += blockDim.x) ((float4*)sb)[i] = g4[i];
        } else {
            for (int i = threadIdx.x; i < P3; i += blockDim.x) sb[i] = g[i];
        }
        __syncthreads();
        for (int i = threadIdx.x; i < b * b * b; i += blockDim.x) {
            const int x = apron + i % b, y = apron + (i / b) % b, z = apron + i / (b * b);
            const int c = (z * P + y) * P + x;
            float v = p1 * sb[c];
            v += sb[c - 1];
            v += sb[c + 1];
            v += sb[c - P];
            v += sb[c + P];
            v += sb[c - P * P];
            v += sb[c + P * P];
            g[c] = smooth_value(v, p1, p2);
        }
        __syncthreads();
    }
}

// FUNC_SMOOTH without an apron: every voxel from its atlas neighbours in the
// snapshot `src` (0 outside the atlas) into `dst`
__global__ void k_smooth_atlas(const float* __restrict__ src, float* __restrict__ dst, AtlasShape s, float p1,
                               float p2, size_t nvox)
{
    const int rx = s.sx * s.P, ry = s.sy * s.P, rz = s.sz * s.P;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nvox; i += (size_t)gridDim.x * blockDim.x) {
        int X, Y, Z;
        atlas_coords(s, i, X, Y, Z);
        float v = p1 * src[i];
        if (X > 0) v += src[atlas_index(s, X - 1, Y, Z)];
        if (X + 1 < rx) v += src[atlas_index(s, X + 1, Y, Z)];
        if (Y > 0) v += src[atlas_index(s, X, Y - 1, Z)];
        if (Y + 1 < ry) v += src[atlas_index(s, X, Y + 1, Z)];
        if (Z > 0) v += src[atlas_index(s, X, Y, Z - 1)];
        if (Z + 1 < rz) v += src[atlas_index(s, X, Y, Z + 1)];
        dst[i] = smooth_value(v, p1, p2);
    }
}

extern "C" gvx_status gvx_compute(gvx_grid* g, int effect, int chan, int iterations, const float params[3],
                                  int update_apron, int skip_over_aprons, float boundval)
{
    if (!g) {
        gvx_set_error("null grid handle");
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(cudaSetDevice(g->device));
    if (chan < 0 || chan >= GVX_MAXCH || !g->ch[chan].used || !params || iterations < 0) {
        gvx_set_error("Compute: channel %d does not exist (or no parameters)", chan);
        return GVX_ERR_INVALID_ARG;
    }
    GvxChannel& ch = g->ch[chan];
    const int type = ch.type;
    const bool ok = (effect == GVX_FUNC_FILL_F && type == GVX_T_FLOAT) ||
                    (effect == GVX_FUNC_FILL_C && type == GVX_T_UCHAR) ||
                    (effect == GVX_FUNC_FILL_C4 && type == GVX_T_UCHAR4) ||
                    (effect == GVX_FUNC_SMOOTH && type == GVX_T_FLOAT);
    if (!ok) {
        gvx_set_error("Compute: operator %d is not available for channel type %d", effect, type);
        return GVX_ERR_UNSUPPORTED;
    }
    if (!g->have_atlas || ch.slots == 0) return GVX_OK;
    const int P = g->P, b = g->brick;
    const size_t nslots = (size_t)ch.slots;
    const size_t nvox = nslots * (size_t)P * P * P;
    const AtlasShape s{P, g->sub[0], g->sub[1], g->sub[2]};
    int hi[3];
    for (int k = 0; k < 3; k++) {
        const int R = g->sub[k] * P;
        const int T = skip_over_aprons ? g->sub[k] * b : R;
        hi[k] = std::min((T + 7) / 8 * 8 + 1, R);
    }
    cudaStream_t st = g->stream;
    const unsigned flat_grid = std::min(blocks_for(nvox, kComputeThreads), 152u * 64u);
    for (int it = 0; it < iterations; it++) {
        if (effect == GVX_FUNC_SMOOTH && g->apron > 0) {
            const size_t smem = (size_t)P * P * P * sizeof(float);
            if (smem > 48 * 1024)
                GVX_CK(cudaFuncSetAttribute(k_smooth_slots, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            const unsigned grid = (unsigned)std::min<size_t>(nslots, 152u * 32u);
            k_smooth_slots<<<grid, kComputeThreads, smem, st>>>(ch.data.as<float>(), P, g->apron, nslots, params[0],
                                                                params[1]);
        } else if (effect == GVX_FUNC_SMOOTH) {
            GVX_CK(gvx_ensure(g->atlas_tmp, nvox * sizeof(float)));
            GVX_CK(cudaMemcpyAsync(g->atlas_tmp.p, ch.data.p, nvox * sizeof(float), cudaMemcpyDeviceToDevice, st));
            k_smooth_atlas<<<flat_grid, kComputeThreads, 0, st>>>(g->atlas_tmp.as<float>(), ch.data.as<float>(), s,
                                                                  params[0], params[1], nvox);
        } else {
            k_fill_op<<<flat_grid, kComputeThreads, 0, st>>>(ch.data.as<unsigned char>(), s,
                                                             make_int3(hi[0], hi[1], hi[2]), effect, params[0],
                                                             params[1], params[2], nvox);
        }
        g->launches++;
        GVX_CK(cudaGetLastError());
        apron_invalidate(ch);
        if (update_apron) {
            gvx_status rc = gvx_update_apron(g, chan, boundval);
            if (rc) return rc;
        }
    }
    return GVX_OK;
}
