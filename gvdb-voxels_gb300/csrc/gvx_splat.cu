// gvx_splat.cu -- point -> brick-atlas splats.
//
// Modes
//   TRILINEAR, CUBIC (no reference counterpart): every active brick PULLS the
//     points of its 27-brick neighbourhood (points are grouped by brick by the
//     topology sort), keeps those whose footprint reaches its interior, and
//     accumulates them in a shared-memory copy of the whole padded brick.  The
//     brick then leaves shared memory in one bulk (TMA) store per channel, so
//     there are no global atomics and every brick is written exactly once.
//   REF_SCATTER: ScatterDensity semantics (gvdb_volume_gvdb.cpp:5624-5660,
//     cuda_gvdb_particles.cuh:516-573): (1 - d^2/r^2)^3 at the point's voxel
//     and its 6 face neighbours, inside the point's own padded brick, summed
//     in shared memory instead of the reference's racy surface read-modify-write.
//
// Sample convention of all modes: voxel v of the index space is sampled at the
// integer coordinate v (as gvdbGatherDensity, cuda_gvdb_particles.cuh:705).
#include <math.h>

#include "gvx_grid.cuh"
#include "gvx_ptx.cuh"

namespace {
constexpr int kSplatThreads = 256;
constexpr int kListCap = 1024;
constexpr float kInvPi = 0.318309886183790671538f;
}  // namespace

// sorted point attributes: (x, y, z, weight) and (vx, vy, vz, radius)
__global__ void k_permute(const uint32_t* __restrict__ svals, uint32_t n, const char* pos, int poff, int pstride,
                          const char* vel, int voff, int vstride, const float* __restrict__ weight,
                          const float* __restrict__ radius, float tx, float ty, float tz, float4* spos,
                          float4* svel)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t j = svals[i];
    const float* p = (const float*)(pos + (size_t)j * pstride + poff);
    spos[i] = make_float4(p[0] + tx, p[1] + ty, p[2] + tz, weight ? weight[j] : 1.0f);
    if (svel) {
        float4 v = make_float4(0.f, 0.f, 0.f, radius ? radius[j] : 0.f);
        if (vel) {
            const float* q = (const float*)(vel + (size_t)j * vstride + voff);
            v.x = q[0];
            v.y = q[1];
            v.z = q[2];
        }
        svel[i] = v;
    }
}

struct SplatArgs {
    int mode;
    int brick, P, apron;
    uint32_t nslots;
    const int* slot_leaf;
    const GvxNode* nodes0;
    const int* nbr;
    const int2* leaf_range;
    const float4* spos;
    const float4* svel;  // nullptr when no velocity and no per-point radius
    bool per_point_radius;
    float radius;
    float* den;          // channel data (slot-major, P^3 per slot) or nullptr
    float4* vel;         // or nullptr
    bool accum;
    uint32_t* err;
};

// M4 cubic spline (Monaghan & Lattanzio 1985) without the 1/(pi h^3) factor,
// for a voxel at offset (dx, dy, dz) from a point of support R = 2h.  Near the
// edge of the support the outer branch 0.25 (2-q)^3 loses all precision if
// 2-q is formed in FP32, so it is evaluated as (R^2 - d^2) / (h (R + d)) with
// R^2 - d^2 computed from error-free products and sums (fmaf two-product,
// Knuth two-sum): the result keeps FP32 relative accuracy up to q -> 2.
__device__ __forceinline__ float m4_offset(float dx, float dy, float dz, float R, float inv_h)
{
    const float px = dx * dx, ex = fmaf(dx, dx, -px);
    const float py = dy * dy, ey = fmaf(dy, dy, -py);
    const float pz = dz * dz, ez = fmaf(dz, dz, -pz);
    const float s1 = px + py;
    float bv = s1 - px;
    const float e1 = (px - (s1 - bv)) + (py - bv);
    const float s = s1 + pz;
    bv = s - s1;
    const float e2 = (s1 - (s - bv)) + (pz - bv);
    const float lo = ((ex + ey) + ez) + (e1 + e2);
    const float r2h = R * R, r2l = fmaf(R, R, -r2h);
    const float t = (r2h - s) + (r2l - lo);  // R^2 - d^2
    if (t <= 0.0f) return 0.0f;
    const float d = sqrtf(s);
    const float q = d * inv_h;
    if (q < 1.0f) return 1.0f - 1.5f * q * q + 0.75f * q * q * q;
    const float u = t / (0.5f * R * (R + d));  // 2 - q
    return 0.25f * u * u * u;
}

template <bool HAS_DEN, bool HAS_VEL>
__global__ void __launch_bounds__(kSplatThreads) k_splat(SplatArgs a)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const int P = a.P, P3 = P * P * P, b = a.brick, ap = a.apron;
    float4* tvel = (float4*)smem;                                     // P^3 float4
    float* tden = (float*)(smem + (HAS_VEL ? (size_t)P3 * 16 : 0));  // P^3 float
    __shared__ int s_list[kListCap];
    __shared__ int s_nlist;
    __shared__ int2 s_rng[27];
    __shared__ int s_off[28];
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ int s_total;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t den_bytes = (uint32_t)P3 * 4u, vel_bytes = (uint32_t)P3 * 16u;
    if (tid == 0) {
        mbar_init(&s_bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    uint32_t phase = 0;

    for (uint32_t s = blockIdx.x; s < a.nslots; s += gridDim.x) {
        const int leaf = a.slot_leaf[s];
        const GvxNode& nd = a.nodes0[leaf];
        const int B0x = nd.pos[0], B0y = nd.pos[1], B0z = nd.pos[2];

        // ---- tile init: previous values (accumulate) or zeros
        if (a.accum) {
            if (tid == 0) {
                mbar_expect_tx(&s_bar, (HAS_DEN ? den_bytes : 0u) + (HAS_VEL ? vel_bytes : 0u));
                if (HAS_DEN) bulk_g2s(tden, a.den + (size_t)s * P3, den_bytes, &s_bar);
                if (HAS_VEL) bulk_g2s(tvel, a.vel + (size_t)s * P3, vel_bytes, &s_bar);
            }
            if (!mbar_wait_bounded(&s_bar, phase)) atomicOr(a.err, GVX_DERR_TIMEOUT);
            phase ^= 1u;
        } else {
            for (int i = tid; i < P3; i += kSplatThreads) {
                if (HAS_DEN) tden[i] = 0.f;
                if (HAS_VEL) tvel[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
        if (tid < 27) {
            const int nl = a.nbr[(size_t)leaf * 27 + tid];
            s_rng[tid] = nl >= 0 ? a.leaf_range[nl] : make_int2(0, 0);
        }
        __syncthreads();
        if (tid == 0) {
            int acc = 0;
            for (int k = 0; k < 27; k++) {
                s_off[k] = acc;
                acc += max(0, s_rng[k].y - s_rng[k].x);
            }
            s_off[27] = acc;
            s_total = acc;
        }
        __syncthreads();
        const int total = s_total;

        // ---- candidates in rounds: filter into the list, then splat the list
        for (int base = 0; base < total; base += kListCap) {
            if (tid == 0) s_nlist = 0;
            __syncthreads();
            for (int v = base + tid; v < min(total, base + kListCap); v += kSplatThreads) {
                int k = 0;
                while (k < 26 && s_off[k + 1] <= v) k++;
                const int i = s_rng[k].x + (v - s_off[k]);
                const float4 p = a.spos[i];
                float R = a.radius;
                if (a.per_point_radius) R = a.svel[i].w;
                int lo[3], hi[3];
                const float pc[3] = {p.x, p.y, p.z};
                const int B0[3] = {B0x, B0y, B0z};
                bool hit = true;
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    if (a.mode == GVX_SPLAT_TRILINEAR) {
                        lo[c] = (int)floorf(pc[c]);
                        hi[c] = lo[c] + 1;
                    } else {
                        lo[c] = (int)floorf(pc[c] - R);
                        hi[c] = (int)ceilf(pc[c] + R);
                    }
                    if (hi[c] < B0[c] || lo[c] >= B0[c] + b) hit = false;
                }
                if (hit) {
                    const int slot = atomicAdd(&s_nlist, 1);
                    s_list[slot] = i;
                }
            }
            __syncthreads();
            const int nlist = s_nlist;
            if (a.mode == GVX_SPLAT_TRILINEAR) {
                for (int e = tid; e < nlist; e += kSplatThreads) {
                    const int i = s_list[e];
                    const float4 p = a.spos[i];
                    float4 u = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (HAS_VEL) u = a.svel[i];
                    const float fx0 = floorf(p.x), fy0 = floorf(p.y), fz0 = floorf(p.z);
                    const float f[3] = {p.x - fx0, p.y - fy0, p.z - fz0};
                    const int i0[3] = {(int)fx0 - B0x, (int)fy0 - B0y, (int)fz0 - B0z};
#pragma unroll
                    for (int c = 0; c < 8; c++) {
                        const int dx = c & 1, dy = (c >> 1) & 1, dz = c >> 2;
                        const int lx = i0[0] + dx, ly = i0[1] + dy, lz = i0[2] + dz;
                        if (lx < 0 || ly < 0 || lz < 0 || lx >= b || ly >= b || lz >= b) continue;
                        const float wgt = p.w * (dx ? f[0] : 1.f - f[0]) * (dy ? f[1] : 1.f - f[1]) *
                                          (dz ? f[2] : 1.f - f[2]);
                        const int t = ((lz + ap) * P + (ly + ap)) * P + (lx + ap);
                        if (HAS_DEN) atomicAdd(&tden[t], wgt);
                        if (HAS_VEL) {
                            atomicAdd(&tvel[t].x, wgt * u.x);
                            atomicAdd(&tvel[t].y, wgt * u.y);
                            atomicAdd(&tvel[t].z, wgt * u.z);
                        }
                    }
                }
            } else {
                // one point per warp, lanes over the footprint box clipped to the brick
                for (int e = warp; e < nlist; e += kSplatThreads / 32) {
                    const int i = s_list[e];
                    const float4 p = a.spos[i];
                    float4 u = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (HAS_VEL || a.per_point_radius) u = a.svel[i];
                    const float R = a.per_point_radius ? u.w : a.radius;
                    const float h = 0.5f * R, inv_h = 1.0f / h;
                    const float norm = kInvPi * inv_h * inv_h * inv_h * p.w;
                    const int lx0 = max((int)floorf(p.x - R), B0x), lx1 = min((int)ceilf(p.x + R), B0x + b - 1);
                    const int ly0 = max((int)floorf(p.y - R), B0y), ly1 = min((int)ceilf(p.y + R), B0y + b - 1);
                    const int lz0 = max((int)floorf(p.z - R), B0z), lz1 = min((int)ceilf(p.z + R), B0z + b - 1);
                    const int nx = lx1 - lx0 + 1, ny = ly1 - ly0 + 1, nz = lz1 - lz0 + 1;
                    if (nx <= 0 || ny <= 0 || nz <= 0) continue;
                    const int ncell = nx * ny * nz;
                    for (int c = lane; c < ncell; c += 32) {
                        const int cx = c % nx, cy = (c / nx) % ny, cz = c / (nx * ny);
                        const int vx = lx0 + cx, vy = ly0 + cy, vz = lz0 + cz;
                        const float m = m4_offset((float)vx - p.x, (float)vy - p.y, (float)vz - p.z, R, inv_h);
                        if (m == 0.0f) continue;
                        const float wgt = norm * m;
                        const int t = ((vz - B0z + ap) * P + (vy - B0y + ap)) * P + (vx - B0x + ap);
                        if (HAS_DEN) atomicAdd(&tden[t], wgt);
                        if (HAS_VEL) {
                            atomicAdd(&tvel[t].x, wgt * u.x);
                            atomicAdd(&tvel[t].y, wgt * u.y);
                            atomicAdd(&tvel[t].z, wgt * u.z);
                        }
                    }
                }
            }
            __syncthreads();
        }

        // ---- one bulk store per channel for the whole padded brick
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            if (HAS_DEN) bulk_s2g(a.den + (size_t)s * P3, tden, den_bytes);
            if (HAS_VEL) bulk_s2g(a.vel + (size_t)s * P3, tvel, vel_bytes);
            bulk_commit();
            bulk_wait_read_all();
        }
        __syncthreads();
    }
    if (tid == 0) bulk_wait_all();
}

// ScatterDensity, race-free: own points only, into the own padded tile
struct ScatterArgs {
    int brick, P, apron;
    uint32_t nslots;
    const int* slot_leaf;
    const GvxNode* nodes0;
    const int2* leaf_range;
    const float4* spos;
    float radius;
    int expand;
    float* den;
    uint32_t* err;
};

__global__ void __launch_bounds__(kSplatThreads) k_scatter_ref(ScatterArgs a)
{
    extern __shared__ __align__(128) unsigned char smem[];
    float* tden = (float*)smem;
    __shared__ __align__(8) uint64_t s_bar;
    const int P = a.P, P3 = P * P * P, b = a.brick, ap = a.apron, tid = threadIdx.x;
    const uint32_t bytes = (uint32_t)P3 * 4u;
    if (tid == 0) {
        mbar_init(&s_bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    uint32_t phase = 0;
    const float r2 = a.radius * a.radius;
    for (uint32_t s = blockIdx.x; s < a.nslots; s += gridDim.x) {
        const int leaf = a.slot_leaf[s];
        const GvxNode& nd = a.nodes0[leaf];
        const int2 rg = a.leaf_range[leaf];
        if (rg.y <= rg.x) continue;  // no point: the brick is left as it is
        if (tid == 0) {
            mbar_expect_tx(&s_bar, bytes);
            bulk_g2s(tden, a.den + (size_t)s * P3, bytes, &s_bar);
        }
        if (!mbar_wait_bounded(&s_bar, phase)) atomicOr(a.err, GVX_DERR_TIMEOUT);
        phase ^= 1u;
        const float vx = (float)nd.pos[0], vy = (float)nd.pos[1], vz = (float)nd.pos[2];
        const int cnt = a.expand ? 7 : 1;
        for (int e = rg.x + tid; e < rg.y; e += kSplatThreads) {
            const float4 w = a.spos[e];
            const float px = w.x - vx, py = w.y - vy, pz = w.z - vz;
            const float pix = (float)(int)px, piy = (float)(int)py, piz = (float)(int)pz;
            if (pix < 0 || piy < 0 || piz < 0 || pix >= b || piy >= b || piz >= b) continue;
            for (int k = 0; k < cnt; k++) {
                const int ox = (k == 1) ? -1 : (k == 2) ? 1 : 0;
                const int oy = (k == 3) ? -1 : (k == 4) ? 1 : 0;
                const int oz = (k == 5) ? -1 : (k == 6) ? 1 : 0;
                const float bx = pix + ox - px, by = piy + oy - py, bz = piz + oz - pz;
                const float c = (bx * bx + by * by + bz * bz) / r2;
                const float v = 1.0f + c * (-3.0f + c * (3.0f - c));
                const int lx = (int)pix + ox + ap, ly = (int)piy + oy + ap, lz = (int)piz + oz + ap;
                if (lx < 0 || ly < 0 || lz < 0 || lx >= P || ly >= P || lz >= P) continue;
                atomicAdd(&tden[(lz * P + ly) * P + lx], v);
            }
        }
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            bulk_s2g(a.den + (size_t)s * P3, tden, bytes);
            bulk_commit();
            bulk_wait_read_all();
        }
        __syncthreads();
    }
    if (tid == 0) bulk_wait_all();
}

// ---------------------------------------------------------------------------

static inline unsigned blocks_for(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

// InsertPoints (VG.cpp:5219-5267): group the points by brick (topology sort,
// reused when the points and translation are those of the rebuild) and write
// the sorted float4 attribute arrays the splat kernels stream through
gvx_status gvx_prepare_points(gvx_grid* g, int n, const float trans[3], bool need_svel)
{
    const float t[3] = {trans ? trans[0] : 0.f, trans ? trans[1] : 0.f, trans ? trans[2] : 0.f};
    gvx_status rc = gvx_topo_group_points(g, n, t);
    if (rc) return rc;
    if (g->perm_valid && (g->perm_has_svel || !need_svel) && g->perm_vel == g->pts.vel &&
        g->perm_w == g->pts.weight && g->perm_r == g->pts.radius)
        return GVX_OK;
    need_svel = need_svel || g->pts.vel || g->pts.radius;
    const uint32_t m = g->n_sorted;
    GVX_CK(gvx_ensure(g->spos, (size_t)std::max<uint32_t>(m, 1u) * sizeof(float4)));
    if (need_svel) GVX_CK(gvx_ensure(g->svel, (size_t)std::max<uint32_t>(m, 1u) * sizeof(float4)));
    if (m) {
        k_permute<<<blocks_for(m, 256), 256, 0, g->stream>>>(
            g->vals[g->sorted_buf].as<uint32_t>(), m, g->pts.pos, g->pts.pos_off, g->pts.pos_stride, g->pts.vel,
            g->pts.vel_off, g->pts.vel_stride, g->pts.weight, g->pts.radius, t[0], t[1], t[2], g->spos.as<float4>(),
            need_svel ? g->svel.as<float4>() : nullptr);
        g->launches++;
    }
    GVX_CK(cudaGetLastError());
    g->perm_valid = true;
    g->perm_has_svel = need_svel;
    g->perm_vel = g->pts.vel;
    g->perm_w = g->pts.weight;
    g->perm_r = g->pts.radius;
    return GVX_OK;
}

static gvx_status check_splat_state(gvx_grid* g, const char* what)
{
    if (g->root_level < 0 || !g->lookup_valid) {
        gvx_set_error("%s: no topology", what);
        return GVX_ERR_STATE;
    }
    if (!g->atlas_valid) {
        gvx_set_error("%s: UpdateAtlas was not called after the topology changed", what);
        return GVX_ERR_STATE;
    }
    return GVX_OK;
}

static int sm_count(gvx_grid* g)
{
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, g->device);
    return v > 0 ? v : 152;
}

gvx_status gvx_splat_run(gvx_grid* g, int mode, int n, float radius, const float trans[3], int chan_d, int chan_v,
                         int accum)
{
    gvx_status rc = check_splat_state(g, "Splat");
    if (rc) return rc;
    if (mode != GVX_SPLAT_TRILINEAR && mode != GVX_SPLAT_CUBIC) {
        gvx_set_error("Splat: unknown mode %d", mode);
        return GVX_ERR_INVALID_ARG;
    }
    const bool has_d = chan_d >= 0, has_v = chan_v >= 0;
    if (!has_d && !has_v) {
        gvx_set_error("Splat: no output channel");
        return GVX_ERR_INVALID_ARG;
    }
    if (has_d && (chan_d >= GVX_MAXCH || !g->ch[chan_d].used || g->ch[chan_d].type != GVX_T_FLOAT)) {
        gvx_set_error("Splat: density channel %d must be a T_FLOAT channel", chan_d);
        return GVX_ERR_INVALID_ARG;
    }
    if (has_v && (chan_v >= GVX_MAXCH || !g->ch[chan_v].used || g->ch[chan_v].elem_bytes != 16)) {
        gvx_set_error("Splat: velocity channel %d must be a T_FLOAT3/T_FLOAT4 channel", chan_v);
        return GVX_ERR_INVALID_ARG;
    }
    const bool ppr = mode == GVX_SPLAT_CUBIC && g->pts.radius != nullptr;
    if (mode == GVX_SPLAT_CUBIC && !ppr && !(radius > 0.f)) {
        gvx_set_error("Splat: cubic splat needs a radius > 0");
        return GVX_ERR_INVALID_ARG;
    }
    const bool need_svel = has_v || ppr;
    rc = gvx_prepare_points(g, n, trans, need_svel);
    if (rc) return rc;

    const int P = g->P, P3 = P * P * P;
    const size_t smem = (has_v ? (size_t)P3 * 16 : 0) + (has_d ? (size_t)P3 * 4 : 0);
    if (smem > 200 * 1024) {
        gvx_set_error("Splat: a %d^3 padded brick of these channels needs %zu bytes of shared memory", P, smem);
        return GVX_ERR_UNSUPPORTED;
    }
    SplatArgs a;
    a.mode = mode;
    a.brick = g->brick;
    a.P = P;
    a.apron = g->apron;
    a.nslots = (uint32_t)g->atlas_used;
    a.slot_leaf = g->slot_leaf.as<int>();
    a.nodes0 = g->nodes[0].as<GvxNode>();
    a.nbr = g->nbr.as<int>();
    a.leaf_range = g->leaf_range.as<int2>();
    a.spos = g->spos.as<float4>();
    a.svel = need_svel ? g->svel.as<float4>() : nullptr;
    a.per_point_radius = ppr;
    a.radius = radius;
    a.den = has_d ? g->ch[chan_d].data.as<float>() : nullptr;
    a.vel = has_v ? g->ch[chan_v].data.as<float4>() : nullptr;
    a.accum = accum != 0;
    a.err = g->d_err.as<uint32_t>();
    if (a.nslots == 0) return GVX_OK;
    void (*kern)(SplatArgs) = has_d ? (has_v ? k_splat<true, true> : k_splat<true, false>)
                                    : k_splat<false, true>;
    GVX_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    GVX_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSplatThreads, smem));
    const uint32_t grid = std::min<uint32_t>(a.nslots, (uint32_t)(sm_count(g) * std::max(per_sm, 1)));
    kern<<<grid, kSplatThreads, smem, g->stream>>>(a);
    g->launches++;
    GVX_CK(cudaGetLastError());
    return GVX_OK;
}

gvx_status gvx_scatter_ref(gvx_grid* g, int n, float radius, const float trans[3], int expand)
{
    gvx_status rc = check_splat_state(g, "ScatterDensity");
    if (rc) return rc;
    if (!g->ch[0].used || g->ch[0].type != GVX_T_FLOAT) {
        gvx_set_error("ScatterDensity: channel 0 must be a T_FLOAT channel");
        return GVX_ERR_INVALID_ARG;
    }
    if (!(radius != 0.f)) {
        gvx_set_error("ScatterDensity: radius must be nonzero");
        return GVX_ERR_INVALID_ARG;
    }
    rc = gvx_prepare_points(g, n, trans, false);
    if (rc) return rc;
    const int P = g->P, P3 = P * P * P;
    const size_t smem = (size_t)P3 * 4;
    ScatterArgs a;
    a.brick = g->brick;
    a.P = P;
    a.apron = g->apron;
    a.nslots = (uint32_t)g->atlas_used;
    a.slot_leaf = g->slot_leaf.as<int>();
    a.nodes0 = g->nodes[0].as<GvxNode>();
    a.leaf_range = g->leaf_range.as<int2>();
    a.spos = g->spos.as<float4>();
    a.radius = radius;
    a.expand = expand;
    a.den = g->ch[0].data.as<float>();
    a.err = g->d_err.as<uint32_t>();
    if (a.nslots == 0) return GVX_OK;
    GVX_CK(cudaFuncSetAttribute(k_scatter_ref, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    GVX_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_scatter_ref, kSplatThreads, smem));
    const uint32_t grid = std::min<uint32_t>(a.nslots, (uint32_t)(sm_count(g) * std::max(per_sm, 1)));
    k_scatter_ref<<<grid, kSplatThreads, smem, g->stream>>>(a);
    g->launches++;
    GVX_CK(cudaGetLastError());
    return GVX_OK;
}
