// gvx_gather.cu -- InsertPointsSubcell, GatherDensity and GatherLevelSet.
//
// Reference path (paths relative to the reference project):
//   VolumeGVDB::InsertPointsSubcell     gvdb_volume_gvdb.cpp:4971-5092
//   gvdbSetFlagSubcell                  cuda_gvdb_particles.cuh:109-118
//   gvdbInsertSubcell / gvdbCountSubcell cuda_gvdb_particles.cuh:218-315
//   gvdbCalcSubcellPos                  cuda_gvdb_particles.cuh:677-694
//   VolumeGVDB::GatherDensity / GatherLevelSet   gvdb_volume_gvdb.cpp:5318-5373
//   gvdbGatherDensity / gvdbGatherLevelSet       cuda_gvdb_particles.cuh:696-773
//   VolumeGVDB::InsertPointsSubcell_FP16         gvdb_volume_gvdb.cpp:5094-5190
//   gvdbInsertSubcell_fp16                       cuda_gvdb_particles.cuh:154-216
//   VolumeGVDB::GatherLevelSet_FP16              gvdb_volume_gvdb.cpp:5375-5401
//   gvdbGatherLevelSet_fp16                      cuda_gvdb_particles.cuh:775-813
//
// Every point adds itself to each subcell (size s) of an existing leaf that
// its box [(int(p-r)/s)s, (int(p+1+r)/s)s] touches; every voxel of every
// subcell then takes max(R - |p_j - v|) (density) or min(|p_j - v| - R)
// (level set) over the subcell's points.  The reference counts the entries
// with global atomics, scans, and copies the points in arrival order.  Here
// each point writes its entries at a scanned offset, one stable radix sort by
// subcell index groups them (each list then holds its points in index order,
// so colour sums are deterministic), and a permute pass stores the translated
// positions contiguously per subcell: the gather streams each list once, one
// warp per subcell, with broadcast loads.
//
// Subcell index = atlas slot * (b/s)^3 + local subcell.  The reference's
// sc_mapping is the rank of the leaf among the linked leaves (parent set),
// which in every tree the topology builds make is the rank among the active
// leaves, i.e. the atlas slot.
#include <math.h>
#include <string.h>

#include "gvx_grid.cuh"

namespace {

inline unsigned blocks_for(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

inline int ceil_log2(int64_t v)
{
    int b = 0;
    while ((int64_t(1) << b) < v) b++;
    return b;
}

struct ScPointArgs {
    const char* pos;
    int off, stride;
    uint32_t n;
    float t[3];
    float rins;
    int sc, scdim, spb, brick;
    LeafLookup L;
    const int* leaf_slot;
    uint32_t* cnt;   // count pass: entries per point; emit pass: their offsets
    uint32_t* keys;  // emit pass: subcell index per entry
    uint32_t* vals;  // emit pass: point index per entry
    uint32_t* err;
};

}  // namespace

// per point: the subcells of existing leaves its box touches (gvdbCountSubcell /
// gvdbInsertSubcell); EMIT writes them at the point's offset, in loop order
template <bool EMIT>
__global__ void k_sc_points(ScPointArgs a)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const float* p = (const float*)(a.pos + (size_t)i * (size_t)a.stride + a.off);
    const float raw[3] = {p[0], p[1], p[2]};
    uint32_t c = 0u;
    const uint32_t o = EMIT ? a.cnt[i] : 0u;
    bool degen = false;
    if (raw[2] != GVX_NOHIT) {
        float w[3];
        for (int k = 0; k < 3; k++) w[k] = raw[k] + a.t[k];
        if (w[0] >= 0.f && w[1] >= 0.f && w[2] >= 0.f) {
            int lo[3], hi[3];
            for (int k = 0; k < 3; k++) {
                lo[k] = ((int)(w[k] - a.rins) / a.sc) * a.sc;
                hi[k] = ((int)((w[k] + 1.0f) + a.rins) / a.sc) * a.sc;
            }
            for (int sx = lo[0]; sx <= hi[0]; sx += a.sc)
                for (int sy = lo[1]; sy <= hi[1]; sy += a.sc)
                    for (int sz = lo[2]; sz <= hi[2]; sz += a.sc) {
                        if (sx < 0 || sy < 0 || sz < 0) {
                            degen = true;  // the reference descends from a negative position here
                            continue;
                        }
                        const int cx = sx / a.brick, cy = sy / a.brick, cz = sz / a.brick;
                        const int leaf = ll_find(a.L, cx - a.L.ks.lo[0], cy - a.L.ks.lo[1], cz - a.L.ks.lo[2]);
                        if (leaf < 0) continue;
                        const int slot = a.leaf_slot[leaf];
                        if (slot < 0) continue;
                        const int px = (sx - cx * a.brick) / a.sc, py = (sy - cy * a.brick) / a.sc,
                                  pz = (sz - cz * a.brick) / a.sc;
                        if (EMIT) {
                            a.keys[o + c] = (uint32_t)slot * (uint32_t)a.spb + (uint32_t)((pz * a.scdim + py) * a.scdim + px);
                            a.vals[o + c] = i;
                        }
                        c++;
                    }
        }
    }
    if (!EMIT) a.cnt[i] = c;
    if (degen) atomicOr(a.err, GVX_DERR_DEGENERATE);
}

// sorted entries -> translated positions (colour bits in .w) contiguous per
// subcell, and each subcell's [beg, end)
__global__ void k_sc_copy(const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ svals, uint32_t m,
                          const char* pos, int off, int stride, const char* clr, int clr_off, int clr_stride, float tx,
                          float ty, float tz, float4* pts, uint32_t* beg, uint32_t* end)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    const uint32_t i = svals[k];
    const float* p = (const float*)(pos + (size_t)i * (size_t)stride + off);
    const uint32_t c = clr ? *(const uint32_t*)(clr + (size_t)i * (size_t)clr_stride + clr_off) : 0u;
    pts[k] = make_float4(p[0] + tx, p[1] + ty, p[2] + tz, __uint_as_float(c));
    const uint32_t key = skeys[k];
    if (k == 0 || skeys[k - 1] != key) beg[key] = k;
    if (k + 1 == m || skeys[k + 1] != key) end[key] = k + 1;
}

// FP16 lists (gvdbInsertSubcell_fp16, PT.cuh:204-207): each entry's translated
// position as 16-bit fractions of the last GetBoundingBox's box,
// (w - mPosMin) / mPosRange * 65535 truncated, each float step rounded on its own
__global__ void k_sc_copy_q(const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ svals, uint32_t m,
                            const char* pos, int off, int stride, const char* clr, int clr_off, int clr_stride,
                            float3 t, float3 qmin, float3 qrange, uint2* q, uint32_t* qclr, uint32_t* beg,
                            uint32_t* end)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    const uint32_t i = svals[k];
    const float* p = (const float*)(pos + (size_t)i * (size_t)stride + off);
    const float w[3] = {__fadd_rn(p[0], t.x), __fadd_rn(p[1], t.y), __fadd_rn(p[2], t.z)};
    const float mn[3] = {qmin.x, qmin.y, qmin.z}, rg[3] = {qrange.x, qrange.y, qrange.z};
    uint32_t u[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float f = __fmul_rn(__fdiv_rn(__fsub_rn(w[a], mn[a]), rg[a]), 65535.0f);
        u[a] = f > 0.0f ? (f >= 65535.0f ? 65535u : __float2uint_rz(f)) : 0u;  // saturating, NaN -> 0
    }
    q[k] = make_uint2(u[0] | (u[1] << 16), u[2]);
    if (qclr) qclr[k] = clr ? *(const uint32_t*)(clr + (size_t)i * (size_t)clr_stride + clr_off) : 0u;
    const uint32_t key = skeys[k];
    if (k == 0 || skeys[k - 1] != key) beg[key] = k;
    if (k + 1 == m || skeys[k + 1] != key) end[key] = k + 1;
}

namespace {

struct GatherArgs {
    uint32_t nsub;
    int sc, scdim, spb, P, apron;
    const int* slot_leaf;
    const GvxNode* nodes0;
    const uint32_t* beg;
    const uint32_t* end;
    const float4* pts;
    float radius;
    int levelset, accum;
    float* out;         // T_FLOAT channel, brick-major padded
    uint32_t* clr_out;  // T_UCHAR4 channel or null
    uint32_t* next;     // subcell counter (zeroed before the launch)
};

__device__ __forceinline__ uint32_t clr_to_char(const float c[4])
{
    uint32_t u = 0u;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        // uchar(c * 255): truncation, saturated to [0, 255] (NaN -> 0)
        const float v = fminf(fmaxf(c[k] * 255.0f, 0.0f), 255.0f);
        u |= (uint32_t)__float2uint_rz(v) << (8 * k);
    }
    return u;
}

struct GatherQArgs {
    uint32_t nsub;
    int sc, scdim, spb, P, apron;
    const int* slot_leaf;
    const GvxNode* nodes0;
    const uint32_t* beg;
    const uint32_t* end;
    const uint2* q;
    const uint32_t* qclr;  // null: no colours
    float qmin[3], qrange[3];
    float radius;
    float* out;           // T_FLOAT channel
    uint32_t* clr_out;    // any 4-byte channel, or null
    uint32_t* next;       // subcell counter (zeroed before the launch)
};

// float -> uint32 as the GPU's conversion does: truncation, saturating, NaN -> 0
__device__ __forceinline__ uint32_t f2u_sat(float v)
{
    return v > 0.0f ? (v >= 4294967296.0f ? 0xFFFFFFFFu : __float2uint_rz(v)) : 0u;
}

}  // namespace

// GatherLevelSet_FP16 (PT.cuh:775-813): one warp per subcell, VPL voxels per
// lane.  Every voxel of every subcell: dist from 3, min(|p - v| - R) over the
// list, positions read back as q / 65535 * range + min; with colours, the sum
// of INT2CLR(c) / |p - v| from 0 (uninitialised in the reference) written as
// particles.cuh's CLR2INT (components * 255 added, carries included).  Every
// float step is rounded on its own, as the oracle restates them.
// SHARE: what a lane's VPL voxels have in common (voxel v + 32 q): 2 = x and y (sc^2 divides 32),
// 1 = x (sc divides 32), 0 = nothing
template <int VPL, int SHARE>
__global__ void __launch_bounds__(256) k_gather_fp16(GatherQArgs a)
{
    const int lane = threadIdx.x & 31;
    const int sc = a.sc, nv = sc * sc * sc;
    // the decoded entries of the current 32, read back by every lane (broadcast loads)
    __shared__ float4 s_ent[8][32];
    float4* ent = s_ent[threadIdx.x >> 5];
    // subcells from a counter (WarpUnits): their lists differ widely in length
    WarpUnits wu(a.next, lane);
    uint32_t s;
    while (wu.next(a.next, a.nsub, lane, s)) {
        const uint32_t slot = s / (uint32_t)a.spb;
        const int loc = (int)(s - slot * (uint32_t)a.spb);
        const GvxNode& nd = a.nodes0[a.slot_leaf[slot]];
        const int so[3] = {(loc % a.scdim) * sc, ((loc / a.scdim) % a.scdim) * sc, (loc / a.scdim / a.scdim) * sc};
        const uint32_t jb = a.beg[s], je = a.end[s];
        for (int v0 = 0; v0 < nv; v0 += 32 * VPL) {
            float m2[VPL], wx[VPL], wy[VPL], wz[VPL], c4[VPL][4];
            size_t idx[VPL];
#pragma unroll
            for (int q = 0; q < VPL; q++) {
                const int v = v0 + q * 32 + lane;
                const int vv = v < nv ? v : 0;
                const int lx = so[0] + vv % sc, ly = so[1] + (vv / sc) % sc, lz = so[2] + vv / (sc * sc);
                wx[q] = (float)(nd.pos[0] + lx);
                wy[q] = (float)(nd.pos[1] + ly);
                wz[q] = (float)(nd.pos[2] + lz);
                idx[q] = (((size_t)slot * a.P + (lz + a.apron)) * a.P + (ly + a.apron)) * a.P + (lx + a.apron);
                m2[q] = __int_as_float(0x7f800000);  // +inf: the smallest squared distance so far
                c4[q][0] = c4[q][1] = c4[q][2] = c4[q][3] = 0.0f;
            }
            for (uint32_t j0 = jb; j0 < je; j0 += 32u) {
                // 32 entries at a time: lane k reads back entry j0 + k once, the warp shares it
                float4 mine = make_float4(0.f, 0.f, 0.f, 0.f);
                if (j0 + lane < je) {
                    const uint2 qq = a.q[j0 + lane];
                    const uint32_t u[3] = {qq.x & 0xFFFFu, qq.x >> 16, qq.y};
                    float p[3];
#pragma unroll
                    for (int k = 0; k < 3; k++)
                        p[k] = __fadd_rn(__fmul_rn(__fdiv_rn((float)u[k], 65535.0f), a.qrange[k]), a.qmin[k]);
                    mine = make_float4(p[0], p[1], p[2], __uint_as_float(a.clr_out ? a.qclr[j0 + lane] : 0u));
                }
                const int cnt = (int)min(32u, je - j0);
                __syncwarp();  // the last chunk's reads are done
                ent[lane] = mine;
                __syncwarp();
                for (int e = 0; e < cnt; e++) {
                const float4 pe = ent[e];
                const float p[3] = {pe.x, pe.y, pe.z};
                const uint32_t cu = __float_as_uint(pe.w);
                // dx^2 (+ dy^2) once per entry where the lane's voxels share them; the squared
                // distance is summed in the same order either way
                const float dx0 = __fsub_rn(p[0], wx[0]), dx20 = __fmul_rn(dx0, dx0);
                const float dy0 = __fsub_rn(p[1], wy[0]), dxy0 = __fadd_rn(dx20, __fmul_rn(dy0, dy0));
#pragma unroll
                for (int q = 0; q < VPL; q++) {
                    float dxy = dxy0;
                    if (q > 0 && SHARE < 2) {
                        float dx2 = dx20;
                        if (SHARE < 1) {
                            const float dx = __fsub_rn(p[0], wx[q]);
                            dx2 = __fmul_rn(dx, dx);
                        }
                        const float dy = __fsub_rn(p[1], wy[q]);
                        dxy = __fadd_rn(dx2, __fmul_rn(dy, dy));
                    }
                    const float dz = __fsub_rn(p[2], wz[q]);
                    const float s2 = __fadd_rn(dxy, __fmul_rn(dz, dz));
                    m2[q] = fminf(m2[q], s2);
                    if (a.clr_out) {
                        const float c = __fsqrt_rn(s2);
#pragma unroll
                        for (int k = 0; k < 4; k++)
                            c4[q][k] = __fadd_rn(c4[q][k], __fdiv_rn(__fdiv_rn((float)((cu >> (8 * k)) & 255u), 255.0f), c));
                    }
                }
                }
            }
#pragma unroll
            for (int q = 0; q < VPL; q++) {
                if (v0 + q * 32 + lane >= nv) continue;
                // min_j (sqrt(s2_j) - R) = sqrt(min_j s2_j) - R: rounded sqrt and subtraction are monotone
                a.out[idx[q]] = fminf(3.0f, __fsub_rn(__fsqrt_rn(m2[q]), a.radius));
                if (!a.clr_out) continue;
                uint32_t u = 0u;
#pragma unroll
                for (int k = 0; k < 4; k++) u += f2u_sat(__fmul_rn(c4[q][k], 255.0f)) << (8 * k);
                a.clr_out[idx[q]] = u;
            }
        }
    }
}

// one warp per subcell; VPL voxels per lane per pass over the subcell's list
template <int VPL>
__global__ void k_gather(GatherArgs a)
{
    const int lane = threadIdx.x & 31;
    const int sc = a.sc, nv = sc * sc * sc;
    // subcells from a counter (WarpUnits): their lists differ widely in length
    WarpUnits wu(a.next, lane);
    uint32_t s;
    while (wu.next(a.next, a.nsub, lane, s)) {
        const uint32_t slot = s / (uint32_t)a.spb;
        const int loc = (int)(s - slot * (uint32_t)a.spb);
        const GvxNode& nd = a.nodes0[a.slot_leaf[slot]];
        const int so[3] = {(loc % a.scdim) * sc, ((loc / a.scdim) % a.scdim) * sc, (loc / a.scdim / a.scdim) * sc};
        const uint32_t jb = a.beg[s], je = a.end[s];
        // the colour sum of the list: lane-strided, then a fixed butterfly (deterministic)
        float csum[4] = {0.f, 0.f, 0.f, 0.f};
        if (a.clr_out) {
            for (uint32_t j = jb + lane; j < je; j += 32u) {
                const uint32_t u = __float_as_uint(a.pts[j].w);
                for (int k = 0; k < 4; k++) csum[k] += (float)((u >> (8 * k)) & 255u) / 255.0f;
            }
            for (int k = 0; k < 4; k++)
                for (int o = 16; o > 0; o >>= 1) csum[k] += __shfl_xor_sync(0xFFFFFFFFu, csum[k], o);
        }
        for (int v0 = 0; v0 < nv; v0 += 32 * VPL) {
            float val[VPL], wx[VPL], wy[VPL], wz[VPL];
            size_t idx[VPL];
#pragma unroll
            for (int q = 0; q < VPL; q++) {
                const int v = v0 + q * 32 + lane;
                const int vv = v < nv ? v : 0;
                const int lx = so[0] + vv % sc, ly = so[1] + (vv / sc) % sc, lz = so[2] + vv / (sc * sc);
                wx[q] = (float)(nd.pos[0] + lx);
                wy[q] = (float)(nd.pos[1] + ly);
                wz[q] = (float)(nd.pos[2] + lz);
                idx[q] = (((size_t)slot * a.P + (lz + a.apron)) * a.P + (ly + a.apron)) * a.P + (lx + a.apron);
                val[q] = a.levelset ? 3.0f : 0.0f;
                if (a.accum && v < nv) val[q] = a.out[idx[q]];
            }
            // the nearest listed point decides: min_j (c_j - R) and max_j (R - c_j) are the values at the
            // smallest squared distance, rounded sqrt and subtraction being monotone
            float m2[VPL];
#pragma unroll
            for (int q = 0; q < VPL; q++) m2[q] = __int_as_float(0x7f800000);
            for (uint32_t j = jb; j < je; j++) {
                const float4 p = a.pts[j];
#pragma unroll
                for (int q = 0; q < VPL; q++) {
                    const float dx = p.x - wx[q], dy = p.y - wy[q], dz = p.z - wz[q];
                    m2[q] = fminf(m2[q], dx * dx + dy * dy + dz * dz);
                }
            }
#pragma unroll
            for (int q = 0; q < VPL; q++) {
                const float c = sqrtf(m2[q]);  // +inf without points: the start value stays
                val[q] = a.levelset ? fminf(val[q], c - a.radius) : fmaxf(val[q], a.radius - c);
            }
#pragma unroll
            for (int q = 0; q < VPL; q++) {
                if (v0 + q * 32 + lane >= nv) continue;
                a.out[idx[q]] = val[q];
                if (!a.clr_out) continue;
                float c4[4] = {0.f, 0.f, 0.f, 1.f};
                if (a.accum) {
                    const uint32_t u = a.clr_out[idx[q]];
                    for (int k = 0; k < 4; k++) c4[k] = (float)((u >> (8 * k)) & 255u) / 255.0f;
                }
                const float den = (float)(je - jb + (a.accum ? 1u : 0u));
                for (int k = 0; k < 4; k++) c4[k] = (c4[k] + csum[k]) / den;
                a.clr_out[idx[q]] = clr_to_char(c4);
            }
        }
    }
}

// InsertPointsSubcell and InsertPointsSubcell_FP16: the same lists, FP32
// translated positions or 16-bit fractions of the bounding box
static gvx_status insert_subcell(gvx_grid* g, int subcell, int n, float radius, const float trans[3], int* sc_len,
                                 bool fp16)
{
    if (!g) {
        gvx_set_error("null grid handle");
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(cudaSetDevice(g->device));
    if (!g->lookup_valid || g->root_level < 0) {
        gvx_set_error("InsertPointsSubcell: no topology");
        return GVX_ERR_STATE;
    }
    if (!g->atlas_valid) {
        gvx_set_error("InsertPointsSubcell: UpdateAtlas must follow the topology build");
        return GVX_ERR_STATE;
    }
    if (subcell <= 0 || g->brick % subcell) {
        gvx_set_error("InsertPointsSubcell: subcell size %d does not divide the brick size %d", subcell, g->brick);
        return GVX_ERR_INVALID_ARG;
    }
    if (n < 0 || n > g->pts.n || (n > 0 && !g->pts.pos) || !(radius >= 0.f)) {
        gvx_set_error("InsertPointsSubcell: %d points requested, %d bound (radius %g)", n, g->pts.n, radius);
        return GVX_ERR_INVALID_ARG;
    }
    g->sc_valid = false;
    const int64_t used = g->used_leaves;
    if (used == 0) return GVX_OK;  // "InsertPointsSubcell yet no bricks exist" (VG.cpp:4974-4977)
    const int scdim = g->brick / subcell, spb = scdim * scdim * scdim;
    const int64_t nsub = (int64_t)spb * used;
    const int64_t per_axis = (int64_t)floor((2.0 * radius + 1.0) / subcell) + 2;
    if (nsub >= (int64_t(1) << 31) || (int64_t)n * per_axis * per_axis * per_axis >= (int64_t(1) << 31)) {
        gvx_set_error("InsertPointsSubcell: %d points x up to %lld subcells each exceed 2^31 entries", n,
                      (long long)(per_axis * per_axis * per_axis));
        return GVX_ERR_CAPACITY;
    }
    cudaStream_t st = g->stream;
    GVX_CK(gvx_ensure(g->d_err, 64));
    GVX_CK(gvx_ensure(g->d_counts, 64 * sizeof(uint32_t)));
    GVX_CK(cudaMemsetAsync(g->d_err.p, 0, 4, st));
    GVX_CK(gvx_ensure(g->sc_cnt, (size_t)n * 4 + 4));
    GVX_CK(gvx_ensure(g->sc_off, (size_t)n * 4 + 4));
    GVX_CK(gvx_ensure(g->sc_beg, (size_t)nsub * 4));
    GVX_CK(gvx_ensure(g->sc_end, (size_t)nsub * 4));
    GVX_CK(cudaMemsetAsync(g->sc_beg.p, 0, (size_t)nsub * 4, st));
    GVX_CK(cudaMemsetAsync(g->sc_end.p, 0, (size_t)nsub * 4, st));
    const float t[3] = {trans ? trans[0] : 0.f, trans ? trans[1] : 0.f, trans ? trans[2] : 0.f};
    // mPosMin / mPosRange of the last GetBoundingBox (VG.cpp:5452-5462), host floats as the reference's
    float qmin[3], qrange[3];
    for (int k = 0; k < 3; k++) {
        qmin[k] = g->bbox_min[k];
        qrange[k] = g->bbox_max[k] - g->bbox_min[k];
    }

    ScPointArgs a;
    memset(&a, 0, sizeof(a));
    a.pos = g->pts.pos;
    a.off = g->pts.pos_off;
    a.stride = g->pts.pos_stride;
    a.n = (uint32_t)n;
    for (int k = 0; k < 3; k++) a.t[k] = t[k];
    a.rins = radius;
    a.sc = subcell;
    a.scdim = scdim;
    a.spb = spb;
    a.brick = g->brick;
    a.L = g->lookup;
    a.leaf_slot = g->leaf_slot.as<int>();
    a.err = g->d_err.as<uint32_t>();
    uint32_t m = 0;
    if (n > 0) {
        a.cnt = g->sc_cnt.as<uint32_t>();
        k_sc_points<false><<<blocks_for(n, 256), 256, 0, st>>>(a);
        g->launches++;
        uint32_t* total = g->d_counts.as<uint32_t>() + 60;
        gvx_status rc = gvx_scan_u32(g->sc_cnt.as<uint32_t>(), g->sc_off.as<uint32_t>(), (uint32_t)n, total,
                                     g->tmp_scan, st, &g->launches);
        if (rc) return rc;
        GVX_CK(cudaMemcpyAsync(&m, total, 4, cudaMemcpyDeviceToHost, st));
        GVX_CK(cudaStreamSynchronize(st));
    }
    if (m > 0) {
        GVX_CK(gvx_ensure(g->sc_keys[0], (size_t)m * 4));
        GVX_CK(gvx_ensure(g->sc_keys[1], (size_t)m * 4));
        GVX_CK(gvx_ensure(g->sc_vals[0], (size_t)m * 4));
        GVX_CK(gvx_ensure(g->sc_vals[1], (size_t)m * 4));
        if (fp16) {
            GVX_CK(gvx_ensure(g->sc_q, (size_t)m * sizeof(uint2)));
            if (g->pts.clr) GVX_CK(gvx_ensure(g->sc_qclr, (size_t)m * 4));
        } else {
            GVX_CK(gvx_ensure(g->sc_pts, (size_t)m * sizeof(float4)));
        }
        a.cnt = g->sc_off.as<uint32_t>();
        a.keys = g->sc_keys[0].as<uint32_t>();
        a.vals = g->sc_vals[0].as<uint32_t>();
        k_sc_points<true><<<blocks_for(n, 256), 256, 0, st>>>(a);
        g->launches++;
        uint32_t* kk[2] = {g->sc_keys[0].as<uint32_t>(), g->sc_keys[1].as<uint32_t>()};
        uint32_t* vv[2] = {g->sc_vals[0].as<uint32_t>(), g->sc_vals[1].as<uint32_t>()};
        int res = 0;
        gvx_status rc = gvx_sort_pairs(kk, vv, m, std::max(1, ceil_log2(nsub)), g->sort, false, st,
                                       g->d_err.as<uint32_t>(), &res, &g->launches);
        if (rc) return rc;
        if (fp16) {
            k_sc_copy_q<<<blocks_for(m, 256), 256, 0, st>>>(
                kk[res], vv[res], m, g->pts.pos, g->pts.pos_off, g->pts.pos_stride, g->pts.clr, g->pts.clr_off,
                g->pts.clr_stride, make_float3(t[0], t[1], t[2]), make_float3(qmin[0], qmin[1], qmin[2]),
                make_float3(qrange[0], qrange[1], qrange[2]), g->sc_q.as<uint2>(),
                g->pts.clr ? g->sc_qclr.as<uint32_t>() : nullptr, g->sc_beg.as<uint32_t>(),
                g->sc_end.as<uint32_t>());
        } else {
            k_sc_copy<<<blocks_for(m, 256), 256, 0, st>>>(kk[res], vv[res], m, g->pts.pos, g->pts.pos_off,
                                                          g->pts.pos_stride, g->pts.clr, g->pts.clr_off,
                                                          g->pts.clr_stride, t[0], t[1], t[2],
                                                          g->sc_pts.as<float4>(), g->sc_beg.as<uint32_t>(),
                                                          g->sc_end.as<uint32_t>());
        }
        g->launches++;
    }
    GVX_CK(cudaGetLastError());
    gvx_status rc = gvx_check_device_error(g, "InsertPointsSubcell");
    if (rc) return rc;
    g->sc_size = subcell;
    g->sc_len = m;
    g->sc_nsub = (uint32_t)nsub;
    g->sc_has_clr = g->pts.clr != nullptr;
    g->sc_fp16 = fp16;
    for (int k = 0; k < 3; k++) {
        g->sc_qmin[k] = qmin[k];
        g->sc_qrange[k] = qrange[k];
    }
    g->sc_valid = true;
    if (sc_len) *sc_len = (int)m;
    return GVX_OK;
}

extern "C" {

gvx_status gvx_insert_points_subcell(gvx_grid* g, int subcell, int n, float radius, const float trans[3], int* sc_len)
{
    if (g) {
        gvx_status rc = gvx_wait_positions(g);
        if (rc) return rc;
    }
    return insert_subcell(g, subcell, n, radius, trans, sc_len, false);
}

gvx_status gvx_insert_points_subcell_fp16(gvx_grid* g, int subcell, int n, float radius, const float trans[3],
                                          int* sc_len)
{
    if (g) {
        gvx_status rc = gvx_wait_positions(g);
        if (rc) return rc;
    }
    return insert_subcell(g, subcell, n, radius, trans, sc_len, true);
}

// GatherLevelSet_FP16 (VG.cpp:5375-5401): no accumulation, no entry-count test,
// the colour (when the lists hold colours) into any 4-byte channel, after the
// level set (the same channel may take both: the colour then stays)
gvx_status gvx_gather_levelset_fp16(gvx_grid* g, int subcell, int n, float radius, const float trans[3], int sc_len,
                                    int chan_levelset, int chan_clr)
{
    if (!g) {
        gvx_set_error("null grid handle");
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(cudaSetDevice(g->device));
    (void)n;      // the lists hold the points
    (void)trans;  // stored translated by the insert
    (void)sc_len;
    if (g->root_level < 0 || g->used_leaves == 0) return GVX_OK;  // num_brick == 0 (VG.cpp:5378)
    const int cl = chan_levelset;
    if (cl < 0 || cl >= GVX_MAXCH || !g->ch[cl].used || g->ch[cl].type != GVX_T_FLOAT) {
        gvx_set_error("GatherLevelSet_FP16: channel %d is not a T_FLOAT channel", cl);
        return GVX_ERR_INVALID_ARG;
    }
    const bool want_clr = g->sc_has_clr && chan_clr >= 0;
    if (want_clr && (chan_clr >= GVX_MAXCH || !g->ch[chan_clr].used || g->ch[chan_clr].elem_bytes != 4)) {
        gvx_set_error("GatherLevelSet_FP16: colour channel %d is not a 4-byte channel", chan_clr);
        return GVX_ERR_INVALID_ARG;
    }
    if (!g->sc_valid || !g->sc_fp16 || g->sc_size != subcell || !g->atlas_valid) {
        gvx_set_error("GatherLevelSet_FP16: no FP16 subcell lists of size %d for this topology "
                      "(call InsertPointsSubcell_FP16 first)", subcell);
        return GVX_ERR_STATE;
    }
    GatherQArgs a;
    memset(&a, 0, sizeof(a));
    a.nsub = g->sc_nsub;
    a.sc = subcell;
    a.scdim = g->brick / subcell;
    a.spb = a.scdim * a.scdim * a.scdim;
    a.P = g->P;
    a.apron = g->apron;
    a.slot_leaf = g->slot_leaf.as<int>();
    a.nodes0 = g->nodes[0].as<GvxNode>();
    a.beg = g->sc_beg.as<uint32_t>();
    a.end = g->sc_end.as<uint32_t>();
    a.q = g->sc_q.as<uint2>();
    a.qclr = want_clr ? g->sc_qclr.as<uint32_t>() : nullptr;
    for (int k = 0; k < 3; k++) {
        a.qmin[k] = g->sc_qmin[k];
        a.qrange[k] = g->sc_qrange[k];
    }
    a.radius = radius;
    a.out = g->ch[cl].data.as<float>();
    a.clr_out = want_clr ? g->ch[chan_clr].data.as<uint32_t>() : nullptr;
    GVX_CK(gvx_ensure(g->d_next, sizeof(uint32_t)));
    GVX_CK(cudaMemsetAsync(g->d_next.p, 0, sizeof(uint32_t), g->stream));
    a.next = g->d_next.as<uint32_t>();
    const unsigned blocks = std::min<unsigned>(blocks_for((uint64_t)a.nsub * 32u, 256), 152u * 16u);
    if (subcell * subcell * subcell <= 64)
        k_gather_fp16<2, 2><<<blocks, 256, 0, g->stream>>>(a);  // sc <= 4: sc^2 divides 32
    else if (32 % subcell == 0)
        k_gather_fp16<8, 1><<<blocks, 256, 0, g->stream>>>(a);
    else
        k_gather_fp16<8, 0><<<blocks, 256, 0, g->stream>>>(a);
    g->launches++;
    GVX_CK(cudaGetLastError());
    apron_invalidate(g->ch[cl]);
    if (a.clr_out) apron_invalidate(g->ch[chan_clr]);
    return GVX_OK;
}

}  // extern "C"

// GatherDensity / GatherLevelSet over the lists of the last InsertPointsSubcell
gvx_status gvx_gather_run(gvx_grid* g, int levelset, int subcell, float radius, int sc_len, int chan, int chan_clr,
                          int accum)
{
    const char* what = levelset ? "GatherLevelSet" : "GatherDensity";
    if (g->root_level < 0 || g->used_leaves == 0) return GVX_OK;  // num_brick == 0: nothing (VG.cpp:5320-5322)
    if (!levelset && sc_len == 0) return GVX_OK;                   // pSCPntsLength == 0 (VG.cpp:5321)
    if (chan < 0 || chan >= GVX_MAXCH || !g->ch[chan].used || g->ch[chan].type != GVX_T_FLOAT) {
        gvx_set_error("%s: channel %d is not a T_FLOAT channel", what, chan);
        return GVX_ERR_INVALID_ARG;
    }
    if (chan_clr >= 0 && (chan_clr >= GVX_MAXCH || !g->ch[chan_clr].used || g->ch[chan_clr].type != GVX_T_UCHAR4)) {
        gvx_set_error("%s: colour channel %d is not a T_UCHAR4 channel", what, chan_clr);
        return GVX_ERR_INVALID_ARG;
    }
    if (!g->sc_valid || g->sc_fp16 || g->sc_size != subcell || !g->atlas_valid) {
        gvx_set_error("%s: no FP32 subcell lists of size %d for this topology (call InsertPointsSubcell first)",
                      what, subcell);
        return GVX_ERR_STATE;
    }
    GatherArgs a;
    memset(&a, 0, sizeof(a));
    a.nsub = g->sc_nsub;
    a.sc = subcell;
    a.scdim = g->brick / subcell;
    a.spb = a.scdim * a.scdim * a.scdim;
    a.P = g->P;
    a.apron = g->apron;
    a.slot_leaf = g->slot_leaf.as<int>();
    a.nodes0 = g->nodes[0].as<GvxNode>();
    a.beg = g->sc_beg.as<uint32_t>();
    a.end = g->sc_end.as<uint32_t>();
    a.pts = g->sc_pts.as<float4>();
    a.radius = radius;
    a.levelset = levelset;
    a.accum = accum ? 1 : 0;
    a.out = g->ch[chan].data.as<float>();
    a.clr_out = (chan_clr >= 0 && g->sc_has_clr) ? g->ch[chan_clr].data.as<uint32_t>() : nullptr;
    GVX_CK(gvx_ensure(g->d_next, sizeof(uint32_t)));
    GVX_CK(cudaMemsetAsync(g->d_next.p, 0, sizeof(uint32_t), g->stream));
    a.next = g->d_next.as<uint32_t>();
    const unsigned blocks = std::min<unsigned>(blocks_for((uint64_t)a.nsub * 32u, 256), 152u * 16u);
    if (subcell * subcell * subcell <= 64)
        k_gather<2><<<blocks, 256, 0, g->stream>>>(a);
    else
        k_gather<8><<<blocks, 256, 0, g->stream>>>(a);
    g->launches++;
    GVX_CK(cudaGetLastError());
    apron_invalidate(g->ch[chan]);  // the gathers write interior voxels only
    if (a.clr_out) apron_invalidate(g->ch[chan_clr]);
    return GVX_OK;
}
