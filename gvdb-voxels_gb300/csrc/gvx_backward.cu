// gvx_backward.cu -- adjoint of the TRILINEAR / CUBIC density splat (no
// reference counterpart).
//
// Forward (gvx_splat.cu): rho_v = sum_i w_i W(v - p_i; R_i) over the interior
// voxels v of the active bricks, W the CIC weight or the M4 cubic spline
// norm(h) M4(|v - p| / h), norm = 1 / (pi h^3), h = R / 2, support R.
// Backward: with G_v = dL/drho_v,
//   dL/dw_i = sum_v G_v W
//   dL/dp_i = sum_v G_v w_i dW/dp
//   dL/dR_i = sum_v G_v w_i dW/dR,   dW/dR = -(3 M4 + q M4') / (2 pi h^4)
// gathered per point, one warp per point over its support, in the sorted
// order of the forward's grouping (re-keyed and re-sorted when the points
// changed), reduced by a fixed butterfly: deterministic, no atomics.  Only
// interior voxels are read: an apron voxel is a copy of its owner's interior.
#include <math.h>

#include "gvx_grid.cuh"

namespace {

constexpr float kInvPi = 0.318309886183790671538f;
constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr int kBackThreads = 256;

inline unsigned blocks_for(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

struct BackArgs {
    int brick, lb, P, apron;  // lb = log2(brick)
    bool ppr;
    float radius;
    uint32_t n;               // sorted points
    const uint32_t* skeys;    // compact level-0 keys, sorted
    const uint32_t* svals;    // sorted -> original point index
    int kshift;               // the sort keys are leaf key << kshift | octant
    uint32_t invalid_key;
    const float4* spos;       // (x, y, z, w), sorted
    const float4* svel;       // (., ., ., R), sorted (per-point radius) or null
    LeafLookup L;
    const int* leaf_slot;
    const float* G;           // dL/drho, density channel layout
    float* gpos;              // 3 per original point
    float* gw;
    float* gr;                // or null
    uint32_t* err;
    uint32_t* next;           // point counter (zeroed before the launch)
};

}  // namespace

template <int MODE>
__global__ void __launch_bounds__(kBackThreads) k_splat_backward(BackArgs a)
{
    const int lane = threadIdx.x & 31;
    const int P = a.P, P3 = P * P * P, ap = a.apron, b = a.brick, lb = a.lb;
    // points one at a time from a counter (their supports differ in size), the next one claimed
    // while the current one runs
    uint32_t in = lane == 0 ? atomicAdd(a.next, 1u) : 0u;
    for (;;) {
        const uint32_t i = __shfl_sync(0xFFFFFFFFu, in, 0);
        if (i >= a.n) break;
        if (lane == 0) in = atomicAdd(a.next, 1u);
        const uint32_t key = a.skeys[i] >> a.kshift;
        const uint32_t orig = a.svals[i];
        // the point takes part iff its own brick is in the lookup (as in the forward)
        int own = -1;
        if (key < a.invalid_key) {
            int c[3];
            ks_unpack(a.L.ks, key, 0, c);
            own = ll_find(a.L, c[0], c[1], c[2]);
        }
        float gx = 0.f, gy = 0.f, gz = 0.f, gwv = 0.f, grv = 0.f;
        if (own >= 0) {
            const float4 p = a.spos[i];
            const float R = a.ppr ? a.svel[i].w : a.radius;
            if (MODE == GVX_SPLAT_CUBIC && R > (float)(b - 1)) {
                if (lane == 0) atomicOr(a.err, GVX_DERR_RADIUS);
            }
            // support box (world voxels) and the bricks it spans (at most 3 per axis)
            int lo[3], hi[3];
            const float pc[3] = {p.x, p.y, p.z};
            for (int k = 0; k < 3; k++) {
                if (MODE == GVX_SPLAT_CUBIC) {
                    lo[k] = (int)floorf(pc[k] - R) + 1;
                    hi[k] = (int)ceilf(pc[k] + R) - 1;
                } else {
                    lo[k] = (int)floorf(pc[k]);
                    hi[k] = lo[k] + 1;
                }
                lo[k] = max(lo[k], 0);
            }
            const int bx0 = lo[0] >> lb, by0 = lo[1] >> lb, bz0 = lo[2] >> lb;
            const int nbx = (max(hi[0], lo[0]) >> lb) - bx0 + 1, nby = (max(hi[1], lo[1]) >> lb) - by0 + 1;
            // lane k < nbx*nby*nbz holds the atlas slot of brick k (-1 if none)
            int myslot = -1;
            {
                const int nbz = (max(hi[2], lo[2]) >> lb) - bz0 + 1;
                if (lane < nbx * nby * nbz) {
                    const int kx = lane % nbx, ky = (lane / nbx) % nby, kz = lane / (nbx * nby);
                    const int leaf = ll_find(a.L, bx0 + kx - a.L.ks.lo[0], by0 + ky - a.L.ks.lo[1],
                                             bz0 + kz - a.L.ks.lo[2]);
                    myslot = leaf >= 0 ? a.leaf_slot[leaf] : -1;
                }
            }
            const int nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
            const int ncell = (nx > 0 && ny > 0 && nz > 0) ? nx * ny * nz : 0;
            float h = 0.f, inv_h = 0.f, norm = 0.f, r2h = 0.f, r2l = 0.f;
            if (MODE == GVX_SPLAT_CUBIC) {
                h = 0.5f * R;
                inv_h = 1.0f / h;
                norm = kInvPi * inv_h * inv_h * inv_h;
                r2h = R * R;
                r2l = fmaf(R, R, -r2h);
            }
            const float fx0 = floorf(p.x), fy0 = floorf(p.y), fz0 = floorf(p.z);
            for (int c0 = 0; c0 < ncell; c0 += 32) {
                const int c = c0 + lane;
                const int cc = c < ncell ? c : 0;
                const int vx = lo[0] + cc % nx, vy = lo[1] + (cc / nx) % ny, vz = lo[2] + cc / (nx * ny);
                const int kb = ((vx >> lb) - bx0) + nbx * (((vy >> lb) - by0) + nby * ((vz >> lb) - bz0));
                const int slot = __shfl_sync(kFull, myslot, kb & 31);
                if (c >= ncell || slot < 0) continue;
                const int lx = vx & (b - 1), ly = vy & (b - 1), lz = vz & (b - 1);
                const float Gv = a.G[(size_t)slot * P3 + ((size_t)(lz + ap) * P + (ly + ap)) * P + (lx + ap)];
                if (Gv == 0.0f) continue;
                const float dx = (float)vx - p.x, dy = (float)vy - p.y, dz = (float)vz - p.z;
                if (MODE == GVX_SPLAT_TRILINEAR) {
                    const float fx = p.x - fx0, fy = p.y - fy0, fz = p.z - fz0;
                    const bool ux = (float)vx == fx0, uy = (float)vy == fy0, uz = (float)vz == fz0;
                    const float wx = ux ? 1.f - fx : fx, wy = uy ? 1.f - fy : fy, wz = uz ? 1.f - fz : fz;
                    const float gwx = Gv * p.w;
                    gwv += Gv * wx * wy * wz;
                    gx += gwx * (ux ? -1.f : 1.f) * wy * wz;
                    gy += gwx * wx * (uy ? -1.f : 1.f) * wz;
                    gz += gwx * wx * wy * (uz ? -1.f : 1.f);
                } else {
                    // R^2 - d^2 error-free, as in the forward
                    const float qy = dy * dy, ey = fmaf(dy, dy, -qy);
                    const float qz = dz * dz, ez = fmaf(dz, dz, -qz);
                    const float syz = qy + qz;
                    float bv = syz - qy;
                    const float e1 = (qy - (syz - bv)) + (qz - bv);
                    const float c1 = r2h - syz;
                    bv = c1 - r2h;
                    const float e2 = (r2h - (c1 - bv)) + (-syz - bv);
                    const float cl = e2 + r2l - ((ey + ez) + e1);
                    const float t = fmaf(-dx, dx, c1) + cl;  // R^2 - d^2
                    if (t <= 0.0f) continue;
                    const float d = sqrtf(fmaf(dx, dx, syz));
                    const float q = d * inv_h;
                    float m4, dm_over_hd, qdm;  // M4(q), M4'(q) / (h d), q M4'(q)
                    if (q < 1.0f) {
                        m4 = fmaf(q * q, fmaf(0.75f, q, -1.5f), 1.0f);
                        const float dm_over_q = fmaf(2.25f, q, -3.0f);  // M4'(q) / q
                        dm_over_hd = dm_over_q * inv_h * inv_h;
                        qdm = dm_over_q * q * q;
                    } else {
                        const float uu = t / (h * (R + d));  // 2 - q
                        m4 = 0.25f * uu * uu * uu;
                        const float dm = -0.75f * uu * uu;
                        dm_over_hd = dm / (h * d);
                        qdm = q * dm;
                    }
                    const float gnw = Gv * norm;
                    gwv += gnw * m4;
                    // dW/dp = norm M4'(q) / (h d) (p - v)
                    const float s = gnw * p.w * dm_over_hd;
                    gx -= s * dx;
                    gy -= s * dy;
                    gz -= s * dz;
                    // dW/dR = -(3 M4 + q M4') / (2 pi h^4) = -norm (3 M4 + q M4') / (2 h)
                    grv -= gnw * p.w * (3.0f * m4 + qdm) * (0.5f * inv_h);
                }
            }
        }
        // fixed butterfly: the same sum order on every run
        for (int o = 16; o > 0; o >>= 1) {
            gx += __shfl_xor_sync(kFull, gx, o);
            gy += __shfl_xor_sync(kFull, gy, o);
            gz += __shfl_xor_sync(kFull, gz, o);
            gwv += __shfl_xor_sync(kFull, gwv, o);
            grv += __shfl_xor_sync(kFull, grv, o);
        }
        if (lane == 0) {
            a.gpos[(size_t)orig * 3 + 0] = gx;
            a.gpos[(size_t)orig * 3 + 1] = gy;
            a.gpos[(size_t)orig * 3 + 2] = gz;
            a.gw[orig] = gwv;
            if (a.gr) a.gr[orig] = grv;
        }
    }
}

extern "C" gvx_status gvx_splat_backward_ex(gvx_grid* g, int mode, int n, float radius, const float trans[3],
                                            const float* dL_drho, float* grad_pos, float* grad_w, float* grad_r,
                                            int flags)
{
    if (!g) {
        gvx_set_error("null grid handle");
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(cudaSetDevice(g->device));
    if (g->root_level < 0 || !g->lookup_valid || !g->atlas_valid) {
        gvx_set_error("SplatBackward: no topology / atlas");
        return GVX_ERR_STATE;
    }
    if (mode != GVX_SPLAT_TRILINEAR && mode != GVX_SPLAT_CUBIC) {
        gvx_set_error("SplatBackward: mode %d has no adjoint", mode);
        return GVX_ERR_INVALID_ARG;
    }
    if (!dL_drho || !grad_pos || !grad_w) {
        gvx_set_error("SplatBackward: dL_drho, grad_pos and grad_w are required");
        return GVX_ERR_INVALID_ARG;
    }
    const bool ppr = mode == GVX_SPLAT_CUBIC && g->pts.radius != nullptr;
    if (mode == GVX_SPLAT_CUBIC && !ppr && !(radius > 0.f && radius <= (float)(g->brick - 1))) {
        gvx_set_error("SplatBackward: cubic radius %g outside (0, brick-1]", radius);
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(cudaMemsetAsync(g->d_err.p, 0, 4, g->stream));
    // the grouping of the forward: reused when valid, else re-keyed and re-sorted.
    // GVX_BWD_RECOMPUTE drops it first, so the permutation is recomputed from the
    // positions (keys with their octants, radix sort, the sorted attributes)
    // rather than taken from the forward; the sort is deterministic, so the new
    // grouping equals the forward's and the gradients are the same bit for bit.
    if (flags & GVX_BWD_RECOMPUTE) {
        g->group_valid = false;
        g->oct_valid = false;
        g->perm_valid = false;
    }
    gvx_status rc = gvx_prepare_points(g, n, trans, ppr);
    if (rc) return rc;
    BackArgs a;
    a.brick = g->brick;
    a.lb = 0;
    while ((1 << a.lb) < g->brick) a.lb++;
    a.P = g->P;
    a.apron = g->apron;
    a.ppr = ppr;
    a.radius = radius;
    a.n = g->n_sorted;
    a.skeys = g->keys[g->sorted_buf].as<uint32_t>();
    a.svals = g->vals[g->sorted_buf].as<uint32_t>();
    a.kshift = g->key_shift;
    a.invalid_key = 1u << g->lookup.ks.total_bits;
    a.spos = g->spos.as<float4>();
    a.svel = ppr ? g->svel.as<float4>() : nullptr;
    a.L = g->lookup;
    a.leaf_slot = g->leaf_slot.as<int>();
    a.G = dL_drho;
    a.gpos = grad_pos;
    a.gw = grad_w;
    a.gr = grad_r;
    a.err = g->d_err.as<uint32_t>();
    if (a.n) {
        GVX_CK(gvx_ensure(g->d_next, sizeof(uint32_t)));
        GVX_CK(cudaMemsetAsync(g->d_next.p, 0, sizeof(uint32_t), g->stream));
        a.next = g->d_next.as<uint32_t>();
        const unsigned blocks = std::min<unsigned>(blocks_for((uint64_t)a.n * 32u, kBackThreads), 152u * 16u);
        if (mode == GVX_SPLAT_CUBIC)
            k_splat_backward<GVX_SPLAT_CUBIC><<<blocks, kBackThreads, 0, g->stream>>>(a);
        else
            k_splat_backward<GVX_SPLAT_TRILINEAR><<<blocks, kBackThreads, 0, g->stream>>>(a);
        g->launches++;
    }
    GVX_CK(cudaGetLastError());
    return GVX_OK;
}

extern "C" gvx_status gvx_splat_backward(gvx_grid* g, int mode, int n, float radius, const float trans[3],
                                         const float* dL_drho, float* grad_pos, float* grad_w, float* grad_r)
{
    return gvx_splat_backward_ex(g, mode, n, radius, trans, dL_drho, grad_pos, grad_w, grad_r, 0);
}
