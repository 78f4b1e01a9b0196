// gvx_splat.cu -- point -> brick-atlas splats.
//
// Modes
//   TRILINEAR, CUBIC (no reference counterpart): one warp per z-slab of an
//     active PADDED brick PULLS the points of the brick's 27-neighbourhood
//     (points are grouped by brick by the topology sort), keeps those whose
//     footprint reaches its slab, and adds them into a shared-memory copy of
//     the slab in their global sorted order, one point at a time across the
//     warp's lanes.  Every voxel is therefore the same sum, added in the same
//     order, in the brick that owns it and in the bricks that hold it as an
//     apron voxel: the splat writes interior and apron together, the apron
//     bit-identical to the neighbours' interior (UpdateApron's copy
//     semantics), with no atomics, deterministically, and one bulk (TMA) store
//     per channel and slab.
//   REF_SCATTER: ScatterDensity semantics (gvdb_volume_gvdb.cpp:5624-5660,
//     cuda_gvdb_particles.cuh:516-573): (1 - d^2/r^2)^3 at the point's voxel
//     and its 6 face neighbours, inside the point's own padded brick, summed
//     in shared memory instead of the reference's racy surface read-modify-write.
//
// Sample convention of all modes: voxel v of the index space is sampled at the
// integer coordinate v (as gvdbGatherDensity, cuda_gvdb_particles.cuh:705).
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <map>
#include <atomic>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include "gvx_grid.cuh"
#include "gvx_ptx.cuh"

namespace {
constexpr int kSplatThreads = 256;
constexpr int kSlabWarps = 4;        // warps (brick slabs) per block of the splat
constexpr int kSlabMinBlocks = 6;    // resident blocks per SM the register budget is sized for
constexpr size_t kSlabTileMax = 48 * 1024;  // shared tile bytes of one warp at most
constexpr int kBatchMaxGrids = 256;         // grids of one batched launch
constexpr int kMaxRanges = 27 * 4;          // candidate ranges of a slab: at most 4 octant runs per neighbour
constexpr float kInvPi = 0.318309886183790671538f;
constexpr uint32_t kFull = 0xFFFFFFFFu;
}  // namespace

// apron voxel number e of a padded brick (apron 1) -> padded coordinates:
// the two z faces, then per inner z layer the two y rows and the two x ends
__device__ __forceinline__ void apron_voxel_coords(int e, int P, int& x, int& y, int& z)
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

// sorted point attributes: (x, y, z, weight) and (vx, vy, vz, radius); with
// per-point radii also the largest radius (float bits, NaN counted as huge)
__global__ void k_permute(const uint32_t* __restrict__ svals, uint32_t n, const char* pos, int poff, int pstride,
                          const char* vel, int voff, int vstride, const float* __restrict__ weight,
                          const float* __restrict__ radius, float tx, float ty, float tz, float4* spos,
                          float4* svel, unsigned int* rmax)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (radius && rmax) {
        float r = i < n ? radius[svals[i]] : 0.0f;
        r = r != r ? 3.0e38f : fmaxf(r, 0.0f);
        const unsigned int m = __reduce_max_sync(0xFFFFFFFFu, __float_as_uint(r));
        if ((threadIdx.x & 31) == 0 && m && m > *(volatile unsigned int*)rmax) atomicMax(rmax, m);
    }
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
    int brick, P, apron;
    uint32_t nslots;
    const int* slot_leaf;
    const int* leaf_slot;
    const GvxNode* nodes0;
    const int* nbr;
    const int2* leaf_range;
    const int* leaf_oct;  // 8 per leaf: first sorted index of each octant of its points
    const float4* spos;
    const float4* svel;  // nullptr when no velocity and no per-point radius
    bool per_point_radius;
    float radius;
    float* den;          // channel data (slot-major, P^3 per slot) or nullptr
    float4* vel;         // or nullptr
    int slabs, slab_layers;  // z-slabs per brick, layers per slab
    // push (apron 1, not accumulating): a tile covers the interior rows and layers only (x with
    // its apron), and the slab's boundary rows go to the neighbours' y/z aprons; else the whole
    // padded brick.  tile_rows: rows of a tile layer (the brick, or the padded brick)
    bool push;
    int tile_rows;
    int lb;              // log2(brick)
    int reach;           // voxels a point's footprint reaches beyond its own voxel (neighbour pruning)
    const unsigned int* rmax;  // per-point radii: float bits of the largest (bounds `reach` on the device)
    float max_radius;    // per-point radii above this reach past the 26 neighbours
    bool accum;
    float boundval;
    uint32_t* err;
    uint32_t* next;  // work-unit counter of the single-grid launch
    // an accumulating single-grid splat may visit only the slots whose bricks some point can
    // reach (unit_slots[0 .. *unit_count), in no particular order); null: every slot
    const uint32_t* unit_slots;
    const uint32_t* unit_count;
};

// Shared-memory tile of one padded brick.  Density only: float per voxel.
// Velocity (with or without density): float4 per voxel (vx, vy, vz, density),
// so a contribution is one 16-byte shared read-modify-write.
template <bool HAS_DEN, bool HAS_VEL>
struct Tile {
    static constexpr bool VEC = HAS_VEL;
    static __host__ __device__ size_t bytes(int P3) { return (size_t)P3 * (VEC ? 16 : 4); }
    // The velocity sums are explicit fused multiply-adds: left to the compiler,
    // `o.x += wgt * ux` may be fused in one kernel (or one unrolled copy) and not
    // in another, and every brick must add a voxel's terms with the same rounding.
    __device__ static void add(unsigned char* t, int i, float wgt, float ux, float uy, float uz)
    {
        if (VEC) {
            float4* v = (float4*)t;
            float4 o = v[i];
            o.x = __fmaf_rn(wgt, ux, o.x);
            o.y = __fmaf_rn(wgt, uy, o.y);
            o.z = __fmaf_rn(wgt, uz, o.z);
            if (HAS_DEN) o.w += wgt;
            v[i] = o;
        } else {
            ((float*)t)[i] += wgt;
        }
    }
    __device__ static void set(unsigned char* t, int i, float val)
    {
        if (VEC)
            ((float4*)t)[i] = make_float4(val, val, val, val);
        else
            ((float*)t)[i] = val;
    }
};

// The footprint cells of a batch of hit points (lane i holds the i-th point of
// the batch in sorted order; lanes without a point have ncell 0), dealt to the
// lanes 32 at a time.  Lanes whose cells share a row apply their updates one
// after another in lane order, which is the points' sorted order (the cells of
// one point lie in distinct rows or distinct chunks of a row); rows apart apply
// together.  So every voxel sums its contributions in the same order in every
// brick that holds it.
//
// SMALL footprints (trilinear, and cubic of a uniform radius <= 2) span at most
// 4 voxels on every axis: a cell is one row of the box, and of a cubic box
// only the rows that can reach the sphere are dealt.  Their decode is a table
// of 5 bits per layer k of the box, at bit 5k: the first row (2 bits, counted
// from yl) and the number of rows (3 bits).  Other footprints deal every row
// of the box in chunks of up to 4 voxels, decoded by division with multipliers
// m = ceil(2^32 / n) (umulhi(c, m) == c / n for every c < 2^32 / n; 0 stands
// for n = 1).
template <bool HAS_DEN, bool HAS_VEL, int MODE, bool PPR, bool SMALL>
__device__ __forceinline__ void deal_cells(unsigned char* tile, const float4 p, const float4 uv, uint32_t box0,
                                           const uint32_t box1, int ncell, const int P, const int TY, const int yoff,
                                           const int Ox, const int Oy, const int Zlo, const float R0,
                                           const float h0, const float inv_h0, const float norm0, const float r2h0,
                                           const float r2l0, const int lane)
{
    using T = Tile<HAS_DEN, HAS_VEL>;
    constexpr bool CUBIC = MODE == GVX_SPLAT_CUBIC;
    uint32_t aux1 = 0u, aux2 = 0u;  // SMALL: the row table; else the multipliers of the chunk and row counts
    if (ncell > 0) {
        const int yl = (int)((box0 >> 16) & 255u), yh = (int)(box0 >> 24);
        if (SMALL) {
            const int zl = (int)(box1 & 255u), zh = (int)((box1 >> 8) & 255u);
            // A row whose float dy, dz give dy^2 + dz^2 < R^2 (1 + 1e-6) in float holds every row
            // with R^2 - dy^2 - dz^2 > 0 exactly (the rows the weights below can reach), with a
            // margin of several roundings; the rows of one layer that pass form one run.
            const float lim = r2h0 * 1.000001f;
            int cnt = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                if (zl + k > zh) break;
                int first = 0, n = yh - yl + 1;
                if (CUBIC) {
                    const float dz = (float)(zl + k + Zlo) - p.z;
                    const float dz2 = dz * dz;
                    first = -1;
                    n = 0;
#pragma unroll
                    for (int yy = 0; yy < 4; yy++) {
                        if (yl + yy > yh) break;
                        const float dy = (float)(yl + yy + Oy) - p.y;
                        if (dy * dy + dz2 < lim) {
                            if (first < 0) first = yy;
                            n++;
                        }
                    }
                    first = max(first, 0);
                }
                aux1 |= (uint32_t)(first | (n << 2)) << (5 * k);
                cnt += n;
            }
            // a point whose box reaches the slab but whose sphere does not keeps one (empty) row,
            // so that every point of the batch owns a cell
            if (cnt == 0) {
                aux1 = 1u << 2;
                cnt = 1;
            }
            ncell = cnt;
            box0 = (box0 & 0x00FFFFFFu) | ((uint32_t)zl << 24);  // xl, xh, yl, zl
        } else {
            const uint32_t nch = (((box0 >> 8) & 255u) - (box0 & 255u) + 4u) >> 2;
            const uint32_t ny = (uint32_t)(yh - yl + 1);
            aux1 = nch > 1u ? 0xFFFFFFFFu / nch + 1u : 0u;
            aux2 = ny > 1u ? 0xFFFFFFFFu / ny + 1u : 0u;
        }
    }
    // inclusive scan of the cell counts over the lanes
    int cend = ncell;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(kFull, cend, o);
        if (lane >= o) cend += t;
    }
    const int ctot = __shfl_sync(kFull, cend, 31);
    const int cstart = cend - ncell;
    for (int g0 = 0; g0 < ctot; g0 += 32) {
        const int g = g0 + lane;
        const bool act = g < ctot;
        // the point dealing this cell: the points are lanes 0 .. nb-1, each with a cell at least,
        // so it is the number of points that start at or before g, less one
        const bool own = ncell > 0;
        const uint32_t starts =
            __reduce_or_sync(kFull, own && cstart >= g0 && cstart < g0 + 32 ? 1u << (cstart - g0) : 0u);
        const int before = __popc(__ballot_sync(kFull, own && cstart < g0));
        const int j = before - 1 + __popc(starts & (kFull >> (31 - lane)));
        const float px = __shfl_sync(kFull, p.x, j), py = __shfl_sync(kFull, p.y, j);
        const float pz = __shfl_sync(kFull, p.z, j), pw = __shfl_sync(kFull, p.w, j);
        float ux = 0.f, uy = 0.f, uz = 0.f;
        if (HAS_VEL) {
            ux = __shfl_sync(kFull, uv.x, j);
            uy = __shfl_sync(kFull, uv.y, j);
            uz = __shfl_sync(kFull, uv.z, j);
        }
        const uint32_t b0 = __shfl_sync(kFull, box0, j);
        const uint32_t a1 = __shfl_sync(kFull, aux1, j);
        const int cell = g - __shfl_sync(kFull, cstart, j);
        const float pR = PPR ? __shfl_sync(kFull, uv.w, j) : 0.0f;
        const int xl = (int)(b0 & 255u), xh = (int)((b0 >> 8) & 255u), yl = (int)((b0 >> 16) & 255u);
        int lx, ly, lz;
        if (SMALL) {
            const int s1 = (int)((a1 >> 2) & 7u), s2 = s1 + (int)((a1 >> 7) & 7u), s3 = s2 + (int)((a1 >> 12) & 7u);
            const int k = (cell >= s1) + (cell >= s2) + (cell >= s3);
            const int pre = k == 0 ? 0 : (k == 1 ? s1 : (k == 2 ? s2 : s3));
            lx = xl;
            ly = yl + (int)((a1 >> (5 * k)) & 3u) + (cell - pre);
            lz = (int)(b0 >> 24) + k;
        } else {
            const uint32_t b1 = __shfl_sync(kFull, box1, j), m2 = __shfl_sync(kFull, aux2, j);
            const int zl = (int)(b1 & 255u);
            const int nch = (xh - xl + 4) >> 2, ny = (int)(b0 >> 24) - yl + 1;
            const int r = a1 ? (int)__umulhi((uint32_t)cell, a1) : cell;  // cell / nch
            const int zz = m2 ? (int)__umulhi((uint32_t)r, m2) : r;       // r / ny
            lx = xl + 4 * (cell - r * nch);
            ly = yl + (r - zz * ny);
            lz = zl + zz;
        }
        // the lane's voxels lx .. min(lx + 3, xh) of row (ly, lz): values, and a bit per voxel touched
        float w[4] = {0.f, 0.f, 0.f, 0.f};
        uint32_t vm = 0u;
        const int t0 = (lz * TY + (ly - yoff)) * P + lx;  // (the tile's rows start at padded y = yoff)
        if (act) {
            if (!CUBIC) {
                const float fx0 = floorf(px), fy0 = floorf(py), fz0 = floorf(pz);
                const float fx = px - fx0, fy = py - fy0, fz = pz - fz0;
                const float wyz = ((float)(ly + Oy) == fy0 ? 1.f - fy : fy) * ((float)(lz + Zlo) == fz0 ? 1.f - fz : fz);
                const float wxa = (float)(lx + Ox) == fx0 ? 1.f - fx : fx;
                w[0] = pw * wxa * wyz;
                vm = 1u;
                if (lx + 1 <= xh) {
                    w[1] = pw * fx * wyz;  // lx + 1 is floor(px) + 1 here
                    vm |= 2u;
                }
            } else {
                // M4 cubic spline (Monaghan & Lattanzio 1985), 3D normalisation 1/(pi h^3),
                // support R = 2h.  Along the row R^2 - d^2 is formed from an error-free
                // c = R^2 - dy^2 - dz^2 (two-product, two-sum) so that the outer branch
                // 0.25 (2-q)^3 = 0.25 ((R^2-d^2) / (h (R+d)))^3 keeps FP32 relative
                // accuracy up to the edge of the support.
                float R = R0, h = h0, inv_h = inv_h0, norm = norm0, r2h = r2h0, r2l = r2l0;
                if (PPR) {
                    R = pR;
                    h = 0.5f * R;
                    inv_h = 1.0f / h;
                    norm = kInvPi * inv_h * inv_h * inv_h;
                    r2h = R * R;
                    r2l = fmaf(R, R, -r2h);
                }
                norm *= pw;
                const float dy = (float)(ly + Oy) - py, dz = (float)(lz + Zlo) - pz;
                const float qy = dy * dy, ey = fmaf(dy, dy, -qy);
                const float qz = dz * dz, ez = fmaf(dz, dz, -qz);
                const float syz = qy + qz;
                float bv = syz - qy;
                const float e1 = (qy - (syz - bv)) + (qz - bv);
                const float c1 = r2h - syz;
                bv = c1 - r2h;
                const float e2 = (r2h - (c1 - bv)) + (-syz - bv);
                const float cl = e2 + r2l - ((ey + ez) + e1);
                if (c1 + cl > 0.0f) {
                    // the four voxels without branches (a slot outside the row or the support
                    // is computed and masked), so that their independent chains interleave
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        const float dx = (float)(lx + k + Ox) - px;
                        const float t = fmaf(-dx, dx, c1) + cl;  // R^2 - d^2
                        const float d2 = fmaf(dx, dx, syz);
                        const float d = d2 > 0.0f ? d2 * rsqrtf(d2) : 0.0f;
                        const float q = d * inv_h;
                        const float wi = fmaf(q * q, fmaf(0.75f, q, -1.5f), 1.0f);  // q < 1
                        const float uu = __fdividef(t, h * (R + d));               // 2 - q
                        const float wk = norm * (q < 1.0f ? wi : 0.25f * uu * uu * uu);
                        const bool ok = lx + k <= xh && t > 0.0f;
                        w[k] = ok ? wk : 0.0f;
                        vm |= ok ? 1u << k : 0u;
                    }
                }
            }
        }
        // lanes sharing a row apply in lane order (the cells of one point lie in distinct rows
        // or distinct chunks of a row); rows apart apply together
        const int key = act ? (lz * P + ly) : -1 - lane;
        const uint32_t grp = __match_any_sync(kFull, key);
        const int rank = __popc(grp & ((1u << lane) - 1u));
        const int nph = (int)__reduce_max_sync(kFull, (uint32_t)rank) + 1;
        for (int ph = 0; ph < nph; ph++) {
            if (rank == ph && vm) {
#pragma unroll
                for (int k = 0; k < 4; k++)
                    if ((vm >> k) & 1u) T::add(tile, t0 + k, w[k], ux, uy, uz);
            }
            __syncwarp();
        }
    }
}

// one voxel out: the tile's (density in .w with velocity), or the boundary value
template <bool HAS_DEN, bool HAS_VEL>
__device__ __forceinline__ void put_voxel(const SplatArgs& a, const unsigned char* tile, int ti, size_t gi)
{
    if (HAS_VEL) {
        const float4 o = ((const float4*)tile)[ti];
        if (HAS_DEN) {
            a.den[gi] = o.w;
            a.vel[gi] = make_float4(o.x, o.y, o.z, 0.0f);
        } else {
            a.vel[gi] = o;
        }
    } else {
        a.den[gi] = ((const float*)tile)[ti];
    }
}
template <bool HAS_DEN, bool HAS_VEL>
__device__ __forceinline__ void put_bound(const SplatArgs& a, size_t gi)
{
    const float v = a.boundval;
    if (HAS_DEN) a.den[gi] = v;
    if (HAS_VEL) a.vel[gi] = make_float4(v, v, v, HAS_DEN ? 0.0f : v);
}

// The slab of a push tile to HBM (apron 1).  The tile holds the brick's interior rows and
// layers of the slab, x with its apron (computed from the points, exact copies of the
// x-neighbours' interiors by the canonical sums).  Every voxel of the padded atlas has one
// writer, the brick whose interior holds it:
//  - the tile's rows go to the brick's own slot;
//  - its boundary rows go to the y/z aprons of the neighbours B + (0, dy, dz) that exist,
//    whole rows, x aprons included (the receiver's apron row in direction -(dy, dz) holds,
//    x apart, this brick's voxels, and at its two ends the voxels of B -/+ x, which this
//    brick's x apron holds);
//  - where that neighbour B + (0, dy, dz) is missing, the end voxels of its would-be row go
//    from the bricks B + (-1|+1, dy, dz) that exist, one voxel a row (this brick's first or
//    last interior column), to B + (+1|-1, ...)'s row ends: with receiver offset (dx, dy, dz),
//    dx != 0, this brick sends when B + (dx, 0, 0) is missing;
//  - the brick's own y/z apron rows facing a missing B + (0, dy, dz) take the boundary value
//    (their end voxels too where B + (-1|+1, dy, dz) is missing as well).
// Rows of a receiver direction: dy = -1: the first interior row (to the receiver's last padded
// row), +1: the last (to its row 0), 0: every row; likewise in z, where only the slab holding
// the first (last) interior layer sends.  nbs: lane r < 27 holds the slot of neighbour r,
// r = (dx+1)*9 + (dy+1)*3 + (dz+1).
template <bool HAS_DEN, bool HAS_VEL>
__device__ __forceinline__ void push_out(const SplatArgs& a, const unsigned char* tile, uint32_t s, int z0, int nl,
                                         int nbs, int lane)
{
    const int P = a.P, P3 = P * P * P, b = a.brick, lb = a.lb, TY = b;
    const uint32_t mP = 0xFFFFFFFFu / (uint32_t)P + 1u;  // e / P == umulhi(e, mP) for e < 2^16
    // the brick's own rows: a tile layer is contiguous in the slot from padded (y 1, z)
    const size_t own = (size_t)s * P3;
    const int lay = TY * P, nvox = nl * lay;
    const uint32_t mL = 0xFFFFFFFFu / (uint32_t)lay + 1u;
    for (int e = lane; e < nvox; e += 32) {
        const int lz = (int)__umulhi((uint32_t)e, mL);
        put_voxel<HAS_DEN, HAS_VEL>(a, tile, e, own + (uint32_t)((z0 + lz) * P * P + P + (e - lz * lay)));
    }
    const bool xm = __shfl_sync(kFull, nbs, 4) >= 0, xp = __shfl_sync(kFull, nbs, 22) >= 0;  // B -/+ x
#pragma unroll 1
    for (int q = 0; q < 9; q++) {
        const int dy = q / 3 - 1, dz = q % 3 - 1;
        if (dy == 0 && dz == 0) continue;
        // the sending rows (ly in [ly0, ly0 + nry), lz in [lz0, lz0 + nrz)) of direction (., dy, dz)
        int ly0 = 0, nry = TY, lz0 = 0, nrz = nl;
        if (dy != 0) {
            ly0 = dy < 0 ? 0 : TY - 1;
            nry = 1;
        }
        if (dz != 0) {
            lz0 = dz < 0 ? 1 - z0 : P - 2 - z0;  // the first (last) interior layer
            if (lz0 < 0 || lz0 >= nl) continue;
            nrz = 1;
        }
        const int nrows = nry * nrz;
        const int d0 = 9 + (dy + 1) * 3 + (dz + 1);  // (0, dy, dz); (-1|+1, dy, dz) at d0 -/+ 9
        const int r0 = __shfl_sync(kFull, nbs, d0);
        const int rm = __shfl_sync(kFull, nbs, d0 - 9), rp = __shfl_sync(kFull, nbs, d0 + 9);
        // row r of the direction: tile row, and its padded (y, z) in a receiver (-1 -> P-1, +1 -> 0)
        auto row = [&](int r, int& ti, int& yr, int& zr) {
            const int ly = ly0 + (nry == 1 ? 0 : (r & (TY - 1))), lz = lz0 + (nry == 1 ? r : (r >> lb));
            ti = (lz * TY + ly) * P;
            yr = dy < 0 ? P - 1 : (dy > 0 ? 0 : ly + 1);
            zr = dz < 0 ? P - 1 : (dz > 0 ? 0 : z0 + lz);
        };
        if (r0 >= 0) {  // whole rows to B + (0, dy, dz)
            const size_t rb = (size_t)r0 * P3;
            for (int e = lane; e < nrows * P; e += 32) {
                const int r = (int)__umulhi((uint32_t)e, mP), x = e - r * P;
                int ti, yr, zr;
                row(r, ti, yr, zr);
                put_voxel<HAS_DEN, HAS_VEL>(a, tile, ti + x, rb + (uint32_t)((zr * P + yr) * P + x));
            }
        } else if (!a.accum) {  // the brick's own apron rows facing the missing B + (0, dy, dz)
            // (their end voxels too where B -/+ x + (0, dy, dz) is missing as well)
            const bool lo = rm < 0, hi = rp < 0;
            for (int e = lane; e < nrows * P; e += 32) {
                const int r = (int)__umulhi((uint32_t)e, mP), x = e - r * P;
                if ((x == 0 && !lo) || (x == P - 1 && !hi)) continue;
                int ti, yr, zr;
                row(r, ti, yr, zr);
                const int yB = dy == 0 ? yr : P - 1 - yr, zB = dz == 0 ? zr : P - 1 - zr;  // the own side
                put_bound<HAS_DEN, HAS_VEL>(a, own + (uint32_t)((zB * P + yB) * P + x));
            }
        }
        // one voxel a row to B -/+ x + (0, dy, dz), whose row source B -/+ x is missing
        if (!xm && rm >= 0) {
            const size_t rb = (size_t)rm * P3;
            for (int r = lane; r < nrows; r += 32) {
                int ti, yr, zr;
                row(r, ti, yr, zr);
                put_voxel<HAS_DEN, HAS_VEL>(a, tile, ti + 1, rb + (uint32_t)((zr * P + yr) * P + P - 1));
            }
        }
        if (!xp && rp >= 0) {
            const size_t rb = (size_t)rp * P3;
            for (int r = lane; r < nrows; r += 32) {
                int ti, yr, zr;
                row(r, ti, yr, zr);
                put_voxel<HAS_DEN, HAS_VEL>(a, tile, ti + P - 2, rb + (uint32_t)((zr * P + yr) * P));
            }
        }
    }
}

// One warp per (brick, z-slab): the padded brick's layers are split into
// slabs of a.slab_layers layers, each with its own shared tile, so a warp's
// tile is a fraction of the brick and more warps stay resident.  Every slab
// sees the same candidate points in the same order, so a voxel's sum does not
// depend on the split.  splat_unit processes work unit u = slot * slabs + slab.
template <bool HAS_DEN, bool HAS_VEL, int MODE, bool PPR, bool SMALL>
__device__ __forceinline__ void splat_unit(const SplatArgs& a, const uint32_t u, unsigned char* tile, uint64_t* bar,
                                           int* s_rs_w, int* s_ro_w, uint32_t& phase,
                                           const int lane)
{
    using T = Tile<HAS_DEN, HAS_VEL>;
    constexpr bool CUBIC = MODE == GVX_SPLAT_CUBIC;
    // single-channel tiles go to HBM in one bulk (TMA) copy; the combined
    // density+velocity tile is split into the two channels by vector stores
    constexpr bool BULK = !(HAS_DEN && HAS_VEL);
    // cubic constants of a uniform radius (per point with PPR)
    const float R0 = a.radius, h0 = 0.5f * R0, inv_h0 = CUBIC && !PPR ? 1.0f / h0 : 0.0f;
    const float norm0 = kInvPi * inv_h0 * inv_h0 * inv_h0, r2h0 = R0 * R0, r2l0 = fmaf(R0, R0, -r2h0);
    const int P = a.P, P2 = P * P, P3 = P2 * P, ap = a.apron, b = a.brick;
    const int L = a.slab_layers, S = a.slabs;
    // the tile: rows [yoff, yoff + TY) of layers [z0, z0 + nl) of the padded brick, x whole
    constexpr bool PUSHABLE = HAS_DEN && HAS_VEL;  // the host sets push for these kernels only
    const bool push = PUSHABLE && a.push;
    const int TY = push ? a.tile_rows : P, yoff = push ? ap : 0, zend = push ? P - ap : P;
    const uint32_t ui = u / (uint32_t)S;  // the unit's brick in the unit order, its slab u - ui * S
    const uint32_t s = a.unit_slots ? a.unit_slots[ui] : ui;
    const int z0 = yoff + (int)(u - ui * (uint32_t)S) * L;  // first padded layer of the slab
    const int nl = min(L, zend - z0);
    const int nvox = nl * TY * P;
    const size_t gofs = (size_t)s * P3 + (size_t)z0 * P2;  // slab start in the channel (no push)
    const int leaf = a.slot_leaf[s];
    const GvxNode* nd = a.nodes0 + leaf;
    const int Ox = nd->pos[0] - ap, Oy = nd->pos[1] - ap, Oz = nd->pos[2] - ap;  // padded origin
    const int Zlo = Oz + z0, Zhi = Oz + z0 + nl - 1;                          // world z of the slab

    // ---- candidate ranges: the octants of the 27 neighbours (the brick itself included) whose
    // points can reach the slab, in the sorted order of the points -- neighbours by key, i.e. by
    // (dx, dy, dz), and inside a brick by octant 4 hx + 2 hy + hz.  Lane r < 27 takes the
    // neighbour (dx, dy, dz) = (r / 9, r / 3 % 3, r % 3) - 1.  Along each axis a half of a brick
    // (floor coordinates [c, c + b/2)) is read when its points, whose footprints reach `reach`
    // voxels from their own, can touch the tile's extent.  A lane's octants are merged
    // into runs of adjacent octants: at most 4 ranges a lane.
    // with per-point radii the reach is that of the largest radius (ceil R voxels, at most brick - 1)
    const int reach = PPR && a.rmax ? min(a.reach, (int)ceilf(__uint_as_float(*a.rmax))) : a.reach;
    bool has_nb = false;
    int nbs = -1;        // lane r < 27: the atlas slot of neighbour r (-1: none)
    uint32_t need = 0u;  // octants to read
    int oc[9];           // first index of each octant, and the end of the brick's points
#pragma unroll
    for (int o = 0; o < 9; o++) oc[o] = 0;
    if (lane < 27) {
        const int dx = lane / 9 - 1, dy = (lane / 3) % 3 - 1, dz = lane % 3 - 1;
        const int nl_ = a.nbr[(size_t)leaf * 27 + (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)];
        if (nl_ >= 0) {
            nbs = a.leaf_slot[nl_];
            has_nb = nbs >= 0;
            const int hb = b >> 1;
            const int cx = nd->pos[0] + dx * b, cy = nd->pos[1] + dy * b, cz = nd->pos[2] + dz * b;
            uint32_t mx = 0u, my = 0u, mz = 0u;
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int x0 = cx + h * hb, y0 = cy + h * hb, z0h = cz + h * hb;
                mx |= (uint32_t)(x0 - reach <= Ox + P - 1 && x0 + hb - 1 + reach >= Ox) << h;
                my |= (uint32_t)(y0 - reach <= Oy + yoff + TY - 1 && y0 + hb - 1 + reach >= Oy + yoff) << h;
                mz |= (uint32_t)(z0h - reach <= Zhi && z0h + hb - 1 + reach >= Zlo) << h;
            }
#pragma unroll
            for (int o = 0; o < 8; o++) need |= ((mx >> (o >> 2)) & (my >> ((o >> 1) & 1)) & (mz >> (o & 1)) & 1u) << o;
            if (need) {
                const int4* q = (const int4*)(a.leaf_oct + (size_t)nl_ * 8);
                const int4 q0 = q[0], q1 = q[1];
                oc[0] = q0.x, oc[1] = q0.y, oc[2] = q0.z, oc[3] = q0.w;
                oc[4] = q1.x, oc[5] = q1.y, oc[6] = q1.z, oc[7] = q1.w;
                oc[8] = a.leaf_range[nl_].y;
            }
        }
    }
    const uint32_t nbmask = __ballot_sync(kFull, has_nb);  // bit r: neighbour r (key order) is active
    // runs of needed octants: their count and points
    int nr = 0, len = 0;
    {
        bool in = false;
        int rs0 = 0;
#pragma unroll
        for (int o = 0; o <= 8; o++) {
            const bool nd_o = o < 8 && ((need >> o) & 1u);
            if (nd_o && !in) {
                rs0 = oc[o];
                in = true;
            } else if (!nd_o && in) {
                if (oc[o] > rs0) {
                    nr++;
                    len += oc[o] - rs0;
                }
                in = false;
            }
        }
    }
    int incl = len, rincl = nr;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(kFull, incl, o), u = __shfl_up_sync(kFull, rincl, o);
        if (lane >= o) {
            incl += t;
            rincl += u;
        }
    }
    const int total = __shfl_sync(kFull, incl, 31);
    const int m = __shfl_sync(kFull, rincl, 31);
    {
        int rank = rincl - nr, off = incl - len;
        bool in = false;
        int rs0 = 0;
#pragma unroll
        for (int o = 0; o <= 8; o++) {
            const bool nd_o = o < 8 && ((need >> o) & 1u);
            if (nd_o && !in) {
                rs0 = oc[o];
                in = true;
            } else if (!nd_o && in) {
                if (oc[o] > rs0) {
                    s_rs_w[rank] = rs0;
                    s_ro_w[rank] = off;
                    rank++;
                    off += oc[o] - rs0;
                }
                in = false;
            }
        }
    }
    if (lane == 0) s_ro_w[m] = total;
    // an accumulating splat leaves a slab that no point reaches as it is: no load, no store
    if (a.accum && total == 0) return;

    // ---- tile: previous values (accumulate) or zeros, once the bulk store of the warp's last
    // slab has read it (the wait is deferred to here: that read overlaps the ranges above)
    if (BULK) {
        if (lane == 0) bulk_wait_read_all();
        __syncwarp();
    }
    if (a.accum) {
        if (BULK) {
            if (lane == 0) {
                const uint32_t nb = (uint32_t)T::bytes(nvox);
                mbar_expect_tx(bar, nb);
                if (HAS_DEN) bulk_g2s(tile, a.den + gofs, nb, bar);
                else bulk_g2s(tile, a.vel + gofs, nb, bar);
            }
            if (!mbar_wait_bounded(bar, phase)) atomicOr(a.err, GVX_DERR_TIMEOUT);
            phase ^= 1u;
        } else {
            float4* tv = (float4*)tile;
            for (int i = lane; i < nvox; i += 32) {
                const float4 v = a.vel[gofs + i];
                tv[i] = make_float4(v.x, v.y, v.z, a.den[gofs + i]);
            }
        }
    } else {
        // zeros in 16-byte stores (a slab holds a multiple of 4 voxels: P is even)
        const int n16 = (int)(T::bytes(nvox) / 16);
        for (int i = lane; i < n16; i += 32) ((float4*)tile)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncwarp();

    // ---- candidates, 32 at a time, in sorted order.  Each lane tests one
    // candidate and sizes the cells of its footprint in the slab (a cell = up
    // to 4 consecutive x voxels of one (y, z) row).  Most candidates miss the
    // slab, so the hits are first gathered, in order, into a batch of up to 32
    // points (lane i holds the i-th); a batch that the next round's hits would
    // overflow, and the last one, has its cells dealt (deal_cells).  Batches
    // are dealt in order, so the order of every voxel's sum is the points'
    // sorted order.
    float4 bp = make_float4(0.f, 0.f, 0.f, 0.f), buv = make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t bb0 = 0u, bb1 = 0u;
    int bnc = 0, nb = 0;  // this lane's cell count; points in the batch (warp-uniform)
    // the regions of the padded slab (bit (dx+1)*9 + (dy+1)*3 + (dz+1): below, inside or above
    // the interior on each axis) that this lane's hits reach
    uint32_t touched = 0u;
    for (int base = 0;; base += 32) {
        const bool done = base >= total;  // one more pass deals the last batch
        const int v = base + lane;
        int idx = -1;
        if (v < total) {
            int lo = 0, hi = m - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s_ro_w[mid] <= v)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            idx = s_rs_w[lo] + (v - s_ro_w[lo]);
        }
        float4 p = make_float4(0.f, 0.f, 0.f, 0.f), uv = make_float4(0.f, 0.f, 0.f, 0.f);
        uint32_t box0 = 0u, box1 = 0u;  // footprint in slab-tile coordinates, 8 bits a bound
        int ncell = 0;
        if (idx >= 0) {
            p = a.spos[idx];
            if (HAS_VEL || PPR) uv = a.svel[idx];
            int xl, xh, yl, yh, zl, zh;
            if (!CUBIC) {
                const int x0 = (int)floorf(p.x) - Ox, y0 = (int)floorf(p.y) - Oy, zb = (int)floorf(p.z) - Zlo;
                xl = max(x0, 0), xh = min(x0 + 1, P - 1);
                yl = max(y0, yoff), yh = min(y0 + 1, yoff + TY - 1);
                zl = max(zb, 0), zh = min(zb + 1, nl - 1);
            } else {
                // voxels strictly inside (p - R, p + R) on every axis
                const float R = PPR ? uv.w : R0;
                if (PPR && R > a.max_radius) atomicOr(a.err, GVX_DERR_RADIUS);
                xl = max((int)floorf(p.x - R) + 1 - Ox, 0), xh = min((int)ceilf(p.x + R) - 1 - Ox, P - 1);
                yl = max((int)floorf(p.y - R) + 1 - Oy, yoff);
                yh = min((int)ceilf(p.y + R) - 1 - Oy, yoff + TY - 1);
                zl = max((int)floorf(p.z - R) + 1 - Zlo, 0), zh = min((int)ceilf(p.z + R) - 1 - Zlo, nl - 1);
            }
            if (xl <= xh && yl <= yh && zl <= zh) {
                const int nch = (xh - xl + 4) >> 2, ny = yh - yl + 1;
                ncell = nch * ny * (zh - zl + 1);
                box0 = (uint32_t)xl | ((uint32_t)xh << 8) | ((uint32_t)yl << 16) | ((uint32_t)yh << 24);
                box1 = (uint32_t)zl | ((uint32_t)zh << 8);
                // per axis: 1 = reaches below the interior, 2 = the interior, 4 = above it; the
                // product of the three spread sets has one bit per region reached (no carries)
                const int zpl = z0 + zl, zph = z0 + zh;
                const uint32_t tx = (uint32_t)(xl < ap) | (uint32_t)(xl <= P - 1 - ap && xh >= ap) << 1 |
                                    (uint32_t)(xh > P - 1 - ap) << 2;
                const uint32_t ty = (uint32_t)(yl < ap) | (uint32_t)(yl <= P - 1 - ap && yh >= ap) << 1 |
                                    (uint32_t)(yh > P - 1 - ap) << 2;
                const uint32_t tz = (uint32_t)(zpl < ap) | (uint32_t)(zpl <= P - 1 - ap && zph >= ap) << 1 |
                                    (uint32_t)(zph > P - 1 - ap) << 2;
                touched |= ((tx & 1u) | (tx & 2u) << 8 | (tx & 4u) << 16) *
                           ((ty & 1u) | (ty & 2u) << 2 | (ty & 4u) << 4) * tz;
            }
        }
        const uint32_t hm = __ballot_sync(kFull, ncell > 0);
        const int h = __popc(hm);
        if (done ? nb > 0 : nb + h > 32) {
            deal_cells<HAS_DEN, HAS_VEL, MODE, PPR, SMALL>(tile, bp, buv, bb0, bb1, bnc, P, TY, yoff, Ox, Oy, Zlo, R0,
                                                           h0, inv_h0, norm0, r2h0, r2l0, lane);
            bnc = 0;
            nb = 0;
        }
        if (done) break;
        if (h == 0) continue;
        // lane nb + i takes the i-th hit of this round: the lane of the (i+1)-th set bit of hm
        const int d = lane - nb;
        const bool take = d >= 0 && d < h;
        int src = lane;
        if (take) {
            int lo = 0, hi = 31;
#pragma unroll
            for (int it = 0; it < 5; it++) {
                const int mid = (lo + hi) >> 1;
                if (__popc(hm & (kFull >> (31 - mid))) > d)
                    hi = mid;
                else
                    lo = mid + 1;
            }
            src = lo;
        }
        const float4 np = make_float4(__shfl_sync(kFull, p.x, src), __shfl_sync(kFull, p.y, src),
                                      __shfl_sync(kFull, p.z, src), __shfl_sync(kFull, p.w, src));
        float4 nuv = make_float4(0.f, 0.f, 0.f, 0.f);
        if (HAS_VEL || PPR)
            nuv = make_float4(__shfl_sync(kFull, uv.x, src), __shfl_sync(kFull, uv.y, src),
                              __shfl_sync(kFull, uv.z, src), __shfl_sync(kFull, uv.w, src));
        const uint32_t n0 = __shfl_sync(kFull, box0, src), n1 = __shfl_sync(kFull, box1, src);
        const int nn = __shfl_sync(kFull, ncell, src);
        if (take) {
            bp = np;
            buv = nuv;
            bb0 = n0;
            bb1 = n1;
            bnc = nn;
        }
        nb += h;
    }

    // ---- apron voxels with no neighbouring brick take the boundary value (0):
    // the apron region facing each missing neighbour (apron 1), clipped to the slab.  The tile
    // was zeroed, so with the boundary value 0 only the regions that some hit reached are reset.
    uint32_t reset = ~nbmask & 0x7FFFFFFu & ~(1u << 13);
    if (a.boundval == 0.0f) reset &= __reduce_or_sync(kFull, touched);
    if (push) reset &= (1u << 4) | (1u << 22);  // the tile's only apron voxels: the two x faces
    if (ap && reset && !a.accum) {
#pragma unroll 1
        for (int k = 0; k < 27; k++) {
            if (!((reset >> k) & 1u)) continue;
            const int dx = k / 9 - 1, dy = (k / 3) % 3 - 1, dz = k % 3 - 1;
            const int xb = dx < 0 ? 0 : (dx > 0 ? P - 1 : 1), yb = dy < 0 ? 0 : (dy > 0 ? P - 1 : 1);
            const int bx = dx == 0 ? a.lb : 0, by = dy == 0 ? a.lb : 0;  // log2 of the region's x, y extents
            const int zlo = max(dz < 0 ? 0 : (dz > 0 ? P - 1 : 1), z0);
            const int zhi = min(dz < 0 ? 0 : (dz > 0 ? P - 1 : P - 2), z0 + nl - 1);
            const int cnt = zhi >= zlo ? (zhi - zlo + 1) << (bx + by) : 0;
            for (int c = lane; c < cnt; c += 32) {
                const int x = xb + (c & ((1 << bx) - 1)), y = yb + ((c >> bx) & ((1 << by) - 1));
                const int z = zlo + (c >> (bx + by));
                T::set(tile, ((z - z0) * TY + (y - yoff)) * P + x, a.boundval);
            }
        }
        __syncwarp();
    }

    // ---- out to HBM
    if (push) {
        if (PUSHABLE) push_out<HAS_DEN, HAS_VEL>(a, tile, s, z0, nl, nbs, lane);
    } else if (BULK) {
        fence_async_smem();
        __syncwarp();
        if (lane == 0) {
            if (HAS_DEN) bulk_s2g(a.den + gofs, tile, (uint32_t)T::bytes(nvox));
            else bulk_s2g(a.vel + gofs, tile, (uint32_t)T::bytes(nvox));
            bulk_commit();  // (its read of the tile is waited for before the tile's next write)
        }
    } else {
        const float4* tv = (const float4*)tile;
        float* dg = a.den + gofs;
        float4* vg = a.vel + gofs;
        for (int i = lane; i < nvox; i += 32) {
            const float4 o = tv[i];
            dg[i] = o.w;
            vg[i] = make_float4(o.x, o.y, o.z, 0.0f);
        }
        __syncwarp();
    }
}

// resident blocks per SM the registers are budgeted for: 8 for the trilinear splats without
// velocity (a few bytes of spill; sparse batched clouds, 2 points a brick: 2.30 -> 2.02 ms on
// 800k bricks, the memory latency of a brick's short candidate chain hidden by more warps), 6 for
// the others, whose registers would spill tens of bytes at 8
template <bool HAS_DEN, bool HAS_VEL, int MODE>
constexpr int splat_min_blocks()
{
    return !HAS_VEL && MODE == GVX_SPLAT_TRILINEAR ? 8 : kSlabMinBlocks;
}

template <bool HAS_DEN, bool HAS_VEL, int MODE, bool PPR, bool SMALL>
__global__ void __launch_bounds__(kSlabWarps * 32, splat_min_blocks<HAS_DEN, HAS_VEL, MODE>()) k_splat_slab(SplatArgs a)
{
    using T = Tile<HAS_DEN, HAS_VEL>;
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned char* tile = smem + (size_t)wid * T::bytes(a.slab_layers * a.tile_rows * a.P);
    __shared__ __align__(8) uint64_t s_bar[kSlabWarps];
    __shared__ int s_rs[kSlabWarps][kMaxRanges + 1];
    __shared__ int s_ro[kSlabWarps][kMaxRanges + 1];
    if (lane == 0) {
        mbar_init(&s_bar[wid], 1);
        mbar_fence_init();
    }
    __syncthreads();
    uint32_t phase = 0;
    const uint32_t units = (a.unit_count ? min(*a.unit_count, a.nslots) : a.nslots) * (uint32_t)a.slabs;
    // units one at a time from a counter (zeroed before the launch), the next one claimed while
    // the current one runs (its atomic's latency hidden: the 4M frame's splat 3.10 -> 3.04 ms):
    // bricks differ widely in cost and the costly ones cluster (dense regions, the surface of an
    // accumulating frame), so claims of several units leave warps idle at the end (measured: the
    // batched clouds' splats 16.7 -> 23.2 ms with claims of 4)
    uint32_t un = lane == 0 ? atomicAdd(a.next, 1u) : 0u;
    for (;;) {
        const uint32_t u = __shfl_sync(kFull, un, 0);
        if (u >= units) break;
        if (lane == 0) un = atomicAdd(a.next, 1u);  // the next unit, claimed while this one runs
        splat_unit<HAS_DEN, HAS_VEL, MODE, PPR, SMALL>(a, u, tile, &s_bar[wid], s_rs[wid], s_ro[wid], phase, lane);
    }
    if (!(HAS_DEN && HAS_VEL) && lane == 0) bulk_wait_all();
}

// The same work over many grids in one persistent launch: the units of grid
// k are [ustart[k], ustart[k+1]) of one global range, taken by the warps from
// a counter; every grid has the same brick and tile shape (slab_layers, P).
template <bool HAS_DEN, bool HAS_VEL, int MODE, bool PPR, bool SMALL>
__global__ void __launch_bounds__(kSlabWarps * 32, splat_min_blocks<HAS_DEN, HAS_VEL, MODE>())
    k_splat_batch(const SplatArgs* __restrict__ args, uint32_t* __restrict__ ustart, int ngrids)
{
    using T = Tile<HAS_DEN, HAS_VEL>;
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned char* tile = smem + (size_t)wid * T::bytes(args[0].slab_layers * args[0].tile_rows * args[0].P);
    __shared__ __align__(8) uint64_t s_bar[kSlabWarps];
    __shared__ int s_rs[kSlabWarps][kMaxRanges + 1];
    __shared__ int s_ro[kSlabWarps][kMaxRanges + 1];
    __shared__ uint32_t s_us[kBatchMaxGrids + 1];
    for (int i = threadIdx.x; i <= ngrids; i += blockDim.x) s_us[i] = ustart[i];
    if (lane == 0) {
        mbar_init(&s_bar[wid], 1);
        mbar_fence_init();
    }
    __syncthreads();
    uint32_t phase = 0;
    const uint32_t total = s_us[ngrids];
    // units are taken one at a time from a counter (ustart[ngrids + 1], zeroed before every
    // launch), the next claimed while the current runs: a brick of a dense cloud costs many times
    // a sparse one, and a fixed stride would leave the warps that drew the dense ones running
    // alone at the end
    uint32_t* next = ustart + ngrids + 1;
    uint32_t un = lane == 0 ? atomicAdd(next, 1u) : 0u;
    for (;;) {
        const uint32_t u = __shfl_sync(kFull, un, 0);
        if (u >= total) break;
        if (lane == 0) un = atomicAdd(next, 1u);  // the next unit, claimed while this one runs
        int lo = 0, hi = ngrids - 1;  // the grid k with ustart[k] <= u < ustart[k+1]
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_us[mid] <= u)
                lo = mid;
            else
                hi = mid - 1;
        }
        splat_unit<HAS_DEN, HAS_VEL, MODE, PPR, SMALL>(args[lo], u - s_us[lo], tile, &s_bar[wid], s_rs[wid],
                                                       s_ro[wid], phase, lane);
    }
    if (!(HAS_DEN && HAS_VEL) && lane == 0) bulk_wait_all();
}

// ScatterDensity, race-free: own points only, into the own padded tile.  With
// point colours (PT.cuh:555-571, 610-642) each point also colours the interior
// voxel it lies in: clr_mode 1 (avgColor) = integer mean of the voxel's
// points' r, g, b with alpha 255, into channel 1; clr_mode 2 = the colour of
// the voxel's highest-index point (the reference's writers race), channel 3.
// Both are counted with shared-memory integer atomics: deterministic.
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
    int clr_mode;             // 0 none, 1 average, 2 one point's colour
    const uint32_t* perm;     // sorted position -> point index
    const char* clr;
    int clr_off, clr_stride;
    uint32_t* clr_out;        // 4-byte channel, brick-major padded
};

__global__ void __launch_bounds__(kSplatThreads) k_scatter_ref(ScatterArgs a)
{
    extern __shared__ __align__(128) unsigned char smem[];
    float* tden = (float*)smem;
    __shared__ __align__(8) uint64_t s_bar;
    const int P = a.P, P3 = P * P * P, b = a.brick, ap = a.apron, tid = threadIdx.x, b3 = b * b * b;
    const uint32_t bytes = (uint32_t)P3 * 4u;
    // colour tables after the tile: average = count, r, g, b per interior voxel; one point = its index
    uint32_t* tclr = (uint32_t*)(smem + (((size_t)P3 * 4 + 15) & ~(size_t)15));
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
        if (a.clr_mode) {
            const int words = a.clr_mode == 1 ? 4 * b3 : b3;
            const uint32_t init = a.clr_mode == 1 ? 0u : 0xFFFFFFFFu;
            for (int i = tid; i < words; i += kSplatThreads) tclr[i] = init;
        }
        if (!mbar_wait_bounded(&s_bar, phase)) atomicOr(a.err, GVX_DERR_TIMEOUT);
        phase ^= 1u;
        if (a.clr_mode) __syncthreads();
        const float vx = (float)nd.pos[0], vy = (float)nd.pos[1], vz = (float)nd.pos[2];
        const int cnt = a.expand ? 7 : 1;
        for (int e = rg.x + tid; e < rg.y; e += kSplatThreads) {
            const float4 w = a.spos[e];
            const float px = w.x - vx, py = w.y - vy, pz = w.z - vz;
            const float pix = (float)(int)px, piy = (float)(int)py, piz = (float)(int)pz;
            if (pix < 0 || piy < 0 || piz < 0 || pix >= b || piy >= b || piz >= b) continue;
            if (a.clr_mode) {
                const int v = ((int)piz * b + (int)piy) * b + (int)pix;
                const uint32_t pt = a.perm[e];
                if (a.clr_mode == 1) {
                    const uint32_t c = *(const uint32_t*)(a.clr + (size_t)pt * (size_t)a.clr_stride + a.clr_off);
                    atomicAdd(&tclr[v], 1u);
                    atomicAdd(&tclr[b3 + v], c & 255u);
                    atomicAdd(&tclr[2 * b3 + v], (c >> 8) & 255u);
                    atomicAdd(&tclr[3 * b3 + v], (c >> 16) & 255u);
                } else {
                    atomicMax((int*)&tclr[v], (int)pt);  // the highest point index; -1 = none
                }
            }
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
        }
        if (a.clr_mode) {
            uint32_t* out = a.clr_out + (size_t)s * P3;
            for (int v = tid; v < b3; v += kSplatThreads) {
                const int o = (((v / (b * b)) + ap) * P + ((v / b) % b + ap)) * P + (v % b + ap);
                if (a.clr_mode == 1) {
                    const uint32_t n = tclr[v];
                    if (n == 0u) continue;
                    out[o] = (tclr[b3 + v] / n & 255u) | ((tclr[2 * b3 + v] / n & 255u) << 8) |
                             ((tclr[3 * b3 + v] / n & 255u) << 16) | (255u << 24);
                } else {
                    const int pt = (int)tclr[v];
                    if (pt < 0) continue;
                    out[o] = *(const uint32_t*)(a.clr + (size_t)pt * (size_t)a.clr_stride + a.clr_off);
                }
            }
        }
        if (tid == 0) bulk_wait_read_all();
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
    gvx_status rc = gvx_wait_attributes(g);
    if (rc) return rc;
    rc = gvx_topo_group_points(g, n, t);
    if (rc) return rc;
    const bool want_svel = need_svel || g->pts.vel || g->pts.radius;
    const uint32_t m = g->n_sorted;
    auto attr_buffers = [&](unsigned int** rmax) -> gvx_status {
        GVX_CK(gvx_ensure(g->spos, (size_t)std::max<uint32_t>(m, 1u) * sizeof(float4)));
        if (want_svel) GVX_CK(gvx_ensure(g->svel, (size_t)std::max<uint32_t>(m, 1u) * sizeof(float4)));
        *rmax = nullptr;
        if (g->pts.radius && want_svel) {
            GVX_CK(gvx_ensure(g->d_rmax, sizeof(unsigned int)));
            GVX_CK(cudaMemsetAsync(g->d_rmax.p, 0, sizeof(unsigned int), g->stream));
            *rmax = g->d_rmax.as<unsigned int>();
        }
        return GVX_OK;
    };
    auto mark_permuted = [&]() {
        g->perm_valid = true;
        g->perm_has_svel = want_svel;
        g->perm_vel = g->pts.vel;
        g->perm_w = g->pts.weight;
        g->perm_r = g->pts.radius;
    };
    if (!g->oct_valid) {
        // a new grouping: the octant pass (the sorted attributes; the octant order itself where the
        // sort keys could not carry it)
        unsigned int* rmax = nullptr;
        rc = attr_buffers(&rmax);
        if (rc) return rc;
        GvxSortedAttr A;
        A.vel = g->pts.vel;
        A.vel_off = g->pts.vel_off;
        A.vel_stride = g->pts.vel_stride;
        A.weight = g->pts.weight;
        A.radius = g->pts.radius;
        A.spos = g->spos.as<float4>();
        A.svel = want_svel ? g->svel.as<float4>() : nullptr;
        A.rmax = rmax;
        rc = gvx_topo_octants(g, &A);
        if (rc) return rc;
        mark_permuted();
        return GVX_OK;
    }
    if (g->perm_valid && (g->perm_has_svel || !need_svel) && g->perm_vel == g->pts.vel &&
        g->perm_w == g->pts.weight && g->perm_r == g->pts.radius)
        return GVX_OK;
    // the same grouping with other attributes: the permute alone
    unsigned int* rmax = nullptr;
    rc = attr_buffers(&rmax);
    if (rc) return rc;
    if (m) {
        k_permute<<<blocks_for(m, 256), 256, 0, g->stream>>>(
            g->vals[g->sorted_buf].as<uint32_t>(), m, g->pts.pos, g->pts.pos_off, g->pts.pos_stride, g->pts.vel,
            g->pts.vel_off, g->pts.vel_stride, g->pts.weight, g->pts.radius, t[0], t[1], t[2], g->spos.as<float4>(),
            want_svel ? g->svel.as<float4>() : nullptr, rmax);
        g->launches++;
    }
    GVX_CK(cudaGetLastError());
    mark_permuted();
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

static int sm_count(int device)
{
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device);
    return v > 0 ? v : 152;
}

// kernel variant: channel set x mode x per-point radius
struct SplatKind {
    bool has_d, has_v, ppr;
    int mode;
    bool small;  // footprint within 4 voxels a side: trilinear, or cubic of a uniform radius <= 2
    bool operator==(const SplatKind& o) const
    {
        return has_d == o.has_d && has_v == o.has_v && ppr == o.ppr && mode == o.mode && small == o.small;
    }
};

template <bool D, bool V>
static void* pick_kernel(const SplatKind& k, bool batch)
{
    if (k.mode == GVX_SPLAT_TRILINEAR)
        return batch ? (void*)k_splat_batch<D, V, GVX_SPLAT_TRILINEAR, false, true>
                     : (void*)k_splat_slab<D, V, GVX_SPLAT_TRILINEAR, false, true>;
    if (k.ppr)
        return batch ? (void*)k_splat_batch<D, V, GVX_SPLAT_CUBIC, true, false>
                     : (void*)k_splat_slab<D, V, GVX_SPLAT_CUBIC, true, false>;
    if (k.small)
        return batch ? (void*)k_splat_batch<D, V, GVX_SPLAT_CUBIC, false, true>
                     : (void*)k_splat_slab<D, V, GVX_SPLAT_CUBIC, false, true>;
    return batch ? (void*)k_splat_batch<D, V, GVX_SPLAT_CUBIC, false, false>
                 : (void*)k_splat_slab<D, V, GVX_SPLAT_CUBIC, false, false>;
}

static void* splat_kernel(const SplatKind& k, bool batch)
{
    return k.has_d ? (k.has_v ? pick_kernel<true, true>(k, batch) : pick_kernel<true, false>(k, batch))
                   : pick_kernel<false, true>(k, batch);
}

// Tile geometry of a grid's splat: a push tile (apron 1, not accumulating) covers the interior
// rows and layers of the padded brick, else the whole padded brick; `span` layers to cover,
// `rows` rows a layer
struct SlabShape {
    bool push;
    int span, rows;
};
static SlabShape slab_shape(const gvx_grid* g, int accum, bool dense, bool den_vel)
{
    const bool push = g->apron == 1 && !accum && dense && den_vel;
    return SlabShape{push, push ? g->brick : g->P, push ? g->brick : g->P};
}

// Points per active brick from which the push tile is used (and only by the splat of density
// with velocity, the only kernels compiled with it: the others keep their registers): its
// scattered apron stores cost a slab several hundred more instructions, which the
// interior-only dealing repays on dense clouds (4M SPH frame, 14 a brick: 3.04 -> 2.95 ms)
// and not on sparse ones (the batched clouds, 4.6 a brick: 15.3 -> 18.8 ms with it)
constexpr uint64_t kPushPointsPerBrick = 8;
static bool dense_cloud(uint64_t points, uint64_t bricks)
{
    return bricks > 0 && points >= kPushPointsPerBrick * bricks;
}

// the largest slab (in layers) whose tile fits the per-warp budget, at most `want`
static int clamp_layers(const SlabShape& sh, int P, size_t eb, int want)
{
    const int fit = (int)(kSlabTileMax / ((size_t)sh.rows * P * eb));
    return std::min(std::min(want, sh.span), fit);
}

// validation of one grid's splat and its kernel kind; *layers in: the wanted slab height (<= 0:
// half the padded brick), out: clamped to the tile budget
static gvx_status splat_check(gvx_grid* g, int mode, float radius, int chan_d, int chan_v, int accum,
                              bool dense, int* layers, SplatKind* kind)
{
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
    if (mode == GVX_SPLAT_CUBIC && !ppr && radius > (float)(g->brick - 1)) {
        gvx_set_error("Splat: radius %g reaches beyond the 26 neighbouring bricks", radius);
        return GVX_ERR_UNSUPPORTED;
    }
    if (g->brick < 2) {
        gvx_set_error("Splat: bricks of 1 voxel are not supported (tiles are moved in 16-byte units)");
        return GVX_ERR_UNSUPPORTED;
    }
    const int P = g->P;
    const SlabShape sh = slab_shape(g, accum, dense, has_d && has_v);
    // a push tile takes the brick's whole interior (one unit a brick: the candidate ranges and the z
    // pushes once; 4M frame 2.80 -> 2.54 ms against two 4-layer slabs), else half the padded brick
    *layers = clamp_layers(sh, P, has_v ? 16 : 4, *layers > 0 ? *layers : (sh.push ? sh.span : (sh.span + 1) / 2));
    if (*layers < 1) {
        gvx_set_error("Splat: a %d^2 layer of the padded brick exceeds the shared tile budget", P);
        return GVX_ERR_UNSUPPORTED;
    }
    kind->has_d = has_d;
    kind->has_v = has_v;
    kind->ppr = ppr;
    kind->mode = mode;
    kind->small = mode == GVX_SPLAT_TRILINEAR || (!ppr && radius <= 2.0f);
    return GVX_OK;
}

// the kernel arguments of one grid's splat over its current grouping and atlas
static void splat_fill(gvx_grid* g, const SplatKind& k, float radius, int chan_d, int chan_v, int accum, bool dense,
                       int layers, SplatArgs* out)
{
    const bool need_svel = k.has_v || k.ppr;
    const int P = g->P;
    SplatArgs& a = *out;
    memset(&a, 0, sizeof(a));
    a.brick = g->brick;
    a.P = P;
    a.apron = g->apron;
    a.nslots = (uint32_t)g->atlas_used;
    a.slot_leaf = g->slot_leaf.as<int>();
    a.leaf_slot = g->leaf_slot.as<int>();
    a.nodes0 = g->nodes[0].as<GvxNode>();
    a.nbr = g->nbr.as<int>();
    a.leaf_range = g->leaf_range.as<int2>();
    a.leaf_oct = g->leaf_oct.as<int>();
    a.spos = g->spos.as<float4>();
    a.svel = need_svel ? g->svel.as<float4>() : nullptr;
    a.per_point_radius = k.ppr;
    a.radius = radius;
    a.den = k.has_d ? g->ch[chan_d].data.as<float>() : nullptr;
    a.vel = k.has_v ? g->ch[chan_v].data.as<float4>() : nullptr;
    const SlabShape sh = slab_shape(g, accum, dense, k.has_d && k.has_v);
    a.push = sh.push;
    a.tile_rows = sh.rows;
    a.slab_layers = layers;
    a.slabs = (sh.span + layers - 1) / layers;
    a.lb = 0;
    while ((1 << a.lb) < g->brick) a.lb++;
    a.max_radius = (float)(g->brick - 1);
    a.reach = k.mode == GVX_SPLAT_TRILINEAR ? 1 : (k.ppr ? g->brick - 1 : (int)ceilf(radius));
    a.rmax = k.ppr && g->n_sorted ? g->d_rmax.as<unsigned int>() : nullptr;
    a.accum = accum != 0;
    a.boundval = 0.0f;
    a.err = g->d_err.as<uint32_t>();
}

// validation, InsertPoints grouping and the kernel arguments of one grid's splat;
// layers <= 0 picks the default slab height (see splat_check); dense < 0: the tile shape from the
// grid's own points per brick, else as given (a batch decides for all its grids)
static gvx_status splat_prepare(gvx_grid* g, int mode, int n, float radius, const float trans[3], int chan_d,
                                int chan_v, int accum, int layers, int dense, SplatArgs* out, SplatKind* kind)
{
    gvx_status rc = check_splat_state(g, "Splat");
    if (rc) return rc;
    const bool dn = dense < 0 ? dense_cloud((uint64_t)n, (uint64_t)g->atlas_used) : dense != 0;
    rc = splat_check(g, mode, radius, chan_d, chan_v, accum, dn, &layers, kind);
    if (rc) return rc;
    rc = gvx_prepare_points(g, n, trans, kind->has_v || kind->ppr);
    if (rc) return rc;
    splat_fill(g, *kind, radius, chan_d, chan_v, accum, dn, layers, out);
    return GVX_OK;
}

// one tile shape for the grids of a batch: from their points and bricks together
static bool batch_dense(const gvx_batch* b);

// apron state after the splat: exact copies with boundary value 0, unless an
// accumulating splat started from an apron that was not a valid copy
static void splat_finish(gvx_grid* g, int chan_d, int chan_v, int accum)
{
    for (int c : {chan_d, chan_v}) {
        if (c < 0) continue;
        GvxChannel& ch = g->ch[c];
        if (!accum) {
            ch.apron_valid = true;  // every apron voxel is the neighbour's sum, or 0 where no brick is
            ch.apron_partial_from = -1;
        } else if (ch.apron_bv != 0.0f) {
            apron_invalidate(ch);
        }
        // accumulating onto copies (all of them, or all but those near new bricks) adds the same
        // sums to both sides of every copy: the state is kept
        ch.apron_bv = 0.0f;
    }
}

static size_t splat_smem(const SplatArgs& a, const SplatKind& k)
{
    return (size_t)a.slab_layers * a.tile_rows * a.P * (k.has_v ? 16 : 4) * kSlabWarps;
}

// The slots whose brick has points of the current grouping in itself or one of its 26 neighbours:
// the only bricks an accumulating splat changes (the others it leaves as they are, loading and
// storing nothing).  A warp per slot, lane r < 27 testing neighbour r; compacted by an atomic
// counter (each unit writes its own brick only, so their order does not matter).
__global__ void k_touched_slots(const int* __restrict__ slot_leaf, uint32_t nslots, const int* __restrict__ nbr,
                                const int2* __restrict__ leaf_range, uint32_t* __restrict__ out,
                                uint32_t* __restrict__ count)
{
    const uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= nslots) return;  // whole warps
    const int leaf = slot_leaf[s];
    bool has = false;
    if (lane < 27 && leaf >= 0) {
        const int nl = nbr[(size_t)leaf * 27 + lane];
        if (nl >= 0) {
            const int2 r = leaf_range[nl];
            has = r.y > r.x;
        }
    }
    if (__ballot_sync(0xFFFFFFFFu, has) && lane == 0) out[atomicAdd(count, 1u)] = s;
}

gvx_status gvx_splat_run(gvx_grid* g, int mode, int n, float radius, const float trans[3], int chan_d, int chan_v,
                         int accum)
{
    SplatArgs a;
    SplatKind kind;
    gvx_status rc = splat_prepare(g, mode, n, radius, trans, chan_d, chan_v, accum, 0, -1, &a, &kind);
    if (rc) return rc;
    if (a.nslots) {
        const size_t smem = splat_smem(a, kind);
        void* kern = splat_kernel(kind, false);
        GVX_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int per_sm = 0;
        GVX_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSlabWarps * 32, smem));
        const uint64_t units = (uint64_t)a.nslots * a.slabs;
        const uint64_t ctas_needed = (units + kSlabWarps - 1) / kSlabWarps;
        const uint32_t grid =
            (uint32_t)std::min<uint64_t>(ctas_needed, (uint64_t)sm_count(g->device) * std::max(per_sm, 1));
        GVX_CK(gvx_ensure(g->d_next, 2 * sizeof(uint32_t)));
        GVX_CK(cudaMemsetAsync(g->d_next.p, 0, 2 * sizeof(uint32_t), g->stream));
        a.next = g->d_next.as<uint32_t>();
        if (accum) {
            // only the bricks that this grouping's points can reach (accumulating frames of a growing
            // scene touch a small part of it: the fusion frames, about a tenth of 129k bricks)
            GVX_CK(gvx_ensure(g->touched, (size_t)a.nslots * sizeof(uint32_t)));
            a.unit_count = g->d_next.as<uint32_t>() + 1;
            a.unit_slots = g->touched.as<uint32_t>();
            k_touched_slots<<<blocks_for((uint64_t)a.nslots * 32u, 256), 256, 0, g->stream>>>(
                a.slot_leaf, a.nslots, a.nbr, a.leaf_range, g->touched.as<uint32_t>(), g->d_next.as<uint32_t>() + 1);
            g->launches++;
        }
        void* args[] = {&a};
        GVX_CK(cudaLaunchKernel(kern, dim3(grid), dim3(kSlabWarps * 32), args, smem, g->stream));
        g->launches++;
    }
    splat_finish(g, chan_d, chan_v, accum);
    return GVX_OK;
}

// ---------------------------------------------------------------------------
// Batched multi-grid splat: the splats of many grids (same brick shape and
// channel kinds) in ONE persistent launch, optionally captured in a CUDA graph
// and replayed while the grids' buffers stay where they are, with an
// autotuner over the slab height and the CTAs per SM (cached per GPU).

struct BatchTuning {
    int layers = 0, blocks_per_sm = 0;
    float ms = 0.f;
};

static std::mutex g_tune_mu;
static std::map<std::string, BatchTuning> g_tune_cache;

struct gvx_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::vector<gvx_grid*> grids;
    DevBuf d_args, d_ustart;
    std::vector<SplatArgs> cap_args;   // arguments of the captured graph
    std::vector<uint32_t> cap_ustart;
    SplatKind cap_kind{};
    int cap_blocks = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev = nullptr;
    BatchTuning tuning;
    int64_t launches = 0;
    // gvx_batch_frame: the grids' planned builds and the splat, captured in one graph
    DevBuf f_args, f_ustart, f_cnt, f_caps;
    cudaEvent_t f_fork = nullptr;
    std::vector<cudaEvent_t> f_join;     // one per grid
    cudaGraph_t f_graph = nullptr;
    cudaGraphExec_t f_exec = nullptr;
    std::vector<uint64_t> f_key, f_failed_key;
    bool f_warm = false;                 // a planned frame ran without a graph since the plans were made
    float f_topo_radius = -1.f;          // the radius the plans were made for
    int64_t f_launches = 0;              // batch-stream launches of one replay
    std::vector<int64_t> f_grid_launches;
    int f_path = 0, f_void = 0;          // how the last frame ran, its grids built again without a plan
};

static bool batch_dense(const gvx_batch* b)
{
    uint64_t pts = 0, bricks = 0;
    for (const gvx_grid* g : b->grids) {
        pts += (uint64_t)(g->group_valid ? g->group_n : g->pts.n);
        bricks += (uint64_t)g->atlas_used;
    }
    return dense_cloud(pts, bricks);
}

static void frame_drop_graph(gvx_batch* b)
{
    if (b->f_exec) cudaGraphExecDestroy(b->f_exec);
    if (b->f_graph) cudaGraphDestroy(b->f_graph);
    b->f_exec = nullptr;
    b->f_graph = nullptr;
    b->f_key.clear();
}

static void batch_drop_graph(gvx_batch* b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->cap_args.clear();
}

static std::string tune_key(int device, const SplatArgs& a, const SplatKind& k)
{
    cudaDeviceProp prop;
    memset(&prop, 0, sizeof(prop));
    cudaGetDeviceProperties(&prop, device);
    char buf[512];
    snprintf(buf, sizeof(buf), "%s|%d|P%d|p%d|m%d|d%d|v%d|r%d|s%d", prop.name, device, a.P, (int)a.push, k.mode,
             (int)k.has_d, (int)k.has_v, (int)k.ppr, (int)k.small);
    return buf;
}

// one launch of the batch kernel over args/ustart already on the device
static gvx_status batch_launch(gvx_batch* b, const SplatKind& k, const SplatArgs& a0, int ngrids, int blocks)
{
    const size_t smem = splat_smem(a0, k);
    void* kern = splat_kernel(k, true);
    const SplatArgs* dargs = b->d_args.as<SplatArgs>();
    uint32_t* dus = b->d_ustart.as<uint32_t>();
    GVX_CK(cudaMemsetAsync(dus + ngrids + 1, 0, sizeof(uint32_t), b->stream));  // the unit counter
    void* args[] = {(void*)&dargs, (void*)&dus, (void*)&ngrids};
    GVX_CK(cudaLaunchKernel(kern, dim3(blocks), dim3(kSlabWarps * 32), args, smem, b->stream));
    b->launches++;
    return GVX_OK;
}

// argument table of every grid for a slab height, and the unit ranges
static gvx_status batch_tables(gvx_batch* b, int mode, float radius, int chan_d, int chan_v, int accum, int layers,
                               std::vector<SplatArgs>& args, std::vector<uint32_t>& ustart, SplatKind& kind)
{
    args.resize(b->grids.size());
    ustart.assign(b->grids.size() + 1, 0u);
    uint64_t tot = 0;
    const int dense = batch_dense(b) ? 1 : 0;
    for (size_t i = 0; i < b->grids.size(); i++) {
        gvx_grid* g = b->grids[i];
        const int n = g->group_valid ? g->group_n : g->pts.n;
        const float* t = g->group_valid ? g->group_trans : nullptr;
        SplatKind k;
        gvx_status rc = splat_prepare(g, mode, n, radius, t, chan_d, chan_v, accum, layers, dense, &args[i], &k);
        if (rc) return rc;
        if (i == 0) {
            kind = k;
        } else if (!(k == kind) || args[i].P != args[0].P || args[i].slab_layers != args[0].slab_layers ||
                   args[i].push != args[0].push) {
            gvx_set_error("BatchSplat: grid %zu differs from grid 0 in brick shape, channels or radius kind", i);
            return GVX_ERR_INVALID_ARG;
        }
        ustart[i] = (uint32_t)tot;
        tot += (uint64_t)args[i].nslots * args[i].slabs;
        if (tot >= (1ull << 31)) {
            gvx_set_error("BatchSplat: more than 2^31 work units");
            return GVX_ERR_CAPACITY;
        }
    }
    ustart[b->grids.size()] = (uint32_t)tot;
    return GVX_OK;
}

static gvx_status batch_upload(gvx_batch* b, const std::vector<SplatArgs>& args, const std::vector<uint32_t>& ustart)
{
    GVX_CK(gvx_ensure(b->d_args, args.size() * sizeof(SplatArgs)));
    GVX_CK(gvx_ensure(b->d_ustart, (ustart.size() + 1) * sizeof(uint32_t)));  // + the unit counter
    GVX_CK(cudaMemcpyAsync(b->d_args.p, args.data(), args.size() * sizeof(SplatArgs), cudaMemcpyHostToDevice,
                           b->stream));
    GVX_CK(cudaMemcpyAsync(b->d_ustart.p, ustart.data(), ustart.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                           b->stream));
    return GVX_OK;
}

static gvx_status batch_max_blocks(gvx_batch* b, const SplatKind& k, const SplatArgs& a0, int* per_sm)
{
    void* kern = splat_kernel(k, true);
    const size_t smem = splat_smem(a0, k);
    GVX_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    GVX_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, kern, kSlabWarps * 32, smem));
    *per_sm = std::max(*per_sm, 1);
    return GVX_OK;
}

// tries the candidate (slab height, CTAs per SM) pairs on the live batch and
// keeps the fastest; each candidate: one warm-up, then the mean of two timed runs
static gvx_status batch_tune(gvx_batch* b, int mode, float radius, int chan_d, int chan_v, BatchTuning* best)
{
    // (the tuning splat does not accumulate)
    const int span = slab_shape(b->grids[0], 0, batch_dense(b), chan_d >= 0 && chan_v >= 0).span;
    const int cand_layers[3] = {(span + 1) / 2, span, (span + 2) / 3};
    cudaEvent_t e0, e1;
    GVX_CK(cudaEventCreate(&e0));
    GVX_CK(cudaEventCreate(&e1));
    best->ms = 1e30f;
    gvx_status rc = GVX_OK;
    for (int li = 0; li < 3 && rc == GVX_OK; li++) {
        std::vector<SplatArgs> args;
        std::vector<uint32_t> us;
        SplatKind k;
        rc = batch_tables(b, mode, radius, chan_d, chan_v, 0, cand_layers[li], args, us, k);
        if (rc) break;
        if (li > 0 && args[0].slab_layers == best->layers) continue;  // clamped to a height already tried
        rc = batch_upload(b, args, us);
        if (rc) break;
        int per_sm = 1;
        rc = batch_max_blocks(b, k, args[0], &per_sm);
        if (rc) break;
        const int sms = sm_count(b->device);
        for (int bp : {per_sm, std::max(1, (per_sm + 1) / 2)}) {
            const int blocks = sms * bp;
            float ms = 0.f;
            for (int it = 0; it < 3 && rc == GVX_OK; it++) {
                if (it == 1) cudaEventRecord(e0, b->stream);
                rc = batch_launch(b, k, args[0], (int)args.size(), blocks);
            }
            if (rc) break;
            cudaEventRecord(e1, b->stream);
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                rc = gvx_cuda_fail(cudaGetLastError(), "autotune");
                break;
            }
            cudaEventElapsedTime(&ms, e0, e1);
            ms *= 0.5f;
            if (ms < best->ms) {
                best->ms = ms;
                best->layers = args[0].slab_layers;
                best->blocks_per_sm = bp;
            }
            if (bp == 1) break;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

// ---------------------------------------------------------------------------
// A whole frame of a batch (gvx_batch_frame): every grid's full RebuildTopology,
// UpdateAtlas and InsertPoints, then the batched splat.  Once every grid has a
// plan (gvx_topo_plan_make, from a staged full build), the builds are planned --
// no host wait, no allocation -- and, with GVX_BATCH_GRAPH, the grids' builds
// (forked onto their own streams) and the splat are captured in one CUDA graph,
// replayed every frame while no buffer has moved.  The splat's unit ranges come
// from the builds' slot counts on the device (k_batch_ustart).

// unit ranges of a batch whose slot counts are in device memory: ustart[k] = slabs * the sum
// of the slot counts of grids < k (each clamped to its capacity); the unit counter
// ustart[ngrids + 1] zeroed
__global__ void k_batch_ustart(const uint32_t* const* __restrict__ counts, const uint32_t* __restrict__ caps,
                               int ngrids, int slabs, uint32_t* __restrict__ ustart)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    uint32_t t = 0;
    for (int k = 0; k < ngrids; k++) {
        ustart[k] = t;
        t += min(*counts[k], caps[k]) * (uint32_t)slabs;
    }
    ustart[ngrids] = t;
    ustart[ngrids + 1] = 0u;
}

// the sorted attributes InsertPoints writes, then the planned build (whose octant pass writes them)
static gvx_status frame_build(gvx_grid* g, bool want_svel)
{
    const size_t m = (size_t)std::max(g->pts.n, 1);
    GVX_CK(gvx_ensure(g->spos, m * sizeof(float4)));
    if (want_svel) GVX_CK(gvx_ensure(g->svel, m * sizeof(float4)));
    unsigned int* rmax = nullptr;
    if (g->pts.radius && want_svel) {
        GVX_CK(gvx_ensure(g->d_rmax, sizeof(unsigned int)));
        GVX_CK(cudaMemsetAsync(g->d_rmax.p, 0, sizeof(unsigned int), g->stream));
        rmax = g->d_rmax.as<unsigned int>();
    }
    GvxSortedAttr A;
    A.vel = g->pts.vel;
    A.vel_off = g->pts.vel_off;
    A.vel_stride = g->pts.vel_stride;
    A.weight = g->pts.weight;
    A.radius = g->pts.radius;
    A.spos = g->spos.as<float4>();
    A.svel = want_svel ? g->svel.as<float4>() : nullptr;
    A.rmax = rmax;
    return gvx_topo_plan_enqueue(g, &A, true);
}

// every grid's planned build on its own stream, forked from and joined back into the batch
// stream (a grid whose build fails is joined all the same, so that a capture stays whole)
static gvx_status frame_builds(gvx_batch* b, const std::vector<char>& want_svel)
{
    gvx_status first = GVX_OK;
    GVX_CK(cudaEventRecord(b->f_fork, b->stream));
    for (size_t i = 0; i < b->grids.size(); i++) {
        gvx_grid* g = b->grids[i];
        const bool own = g->stream != b->stream;
        if (own) GVX_CK(cudaStreamWaitEvent(g->stream, b->f_fork, 0));
        gvx_status rc = frame_build(g, want_svel[i] != 0);
        if (rc != GVX_OK && first == GVX_OK) {
            const std::string m = gvx_last_error();
            gvx_set_error("BatchFrame: grid %zu: %s", i, m.c_str());
            first = rc;
        }
        if (own) {
            GVX_CK(cudaEventRecord(b->f_join[i], g->stream));
            GVX_CK(cudaStreamWaitEvent(b->stream, b->f_join[i], 0));
        }
    }
    return first;
}

// the splat arguments and the slot-count table of every grid to the device (before a capture,
// or after the builds of a frame without a graph)
static gvx_status frame_upload(gvx_batch* b, const SplatKind& kind, float radius, int chan_d, int chan_v,
                               int layers)
{
    const size_t ng = b->grids.size();
    std::vector<SplatArgs> args(ng);
    std::vector<const uint32_t*> cnt(ng);
    std::vector<uint32_t> caps(ng);
    for (size_t i = 0; i < ng; i++) {
        splat_fill(b->grids[i], kind, radius, chan_d, chan_v, 0, batch_dense(b), layers, &args[i]);
        cnt[i] = gvx_topo_plan_slots(b->grids[i], &caps[i]);
    }
    GVX_CK(cudaMemcpyAsync(b->f_args.p, args.data(), ng * sizeof(SplatArgs), cudaMemcpyHostToDevice, b->stream));
    GVX_CK(cudaMemcpyAsync(b->f_cnt.p, cnt.data(), ng * sizeof(void*), cudaMemcpyHostToDevice, b->stream));
    GVX_CK(cudaMemcpyAsync(b->f_caps.p, caps.data(), ng * sizeof(uint32_t), cudaMemcpyHostToDevice, b->stream));
    return GVX_OK;
}

// the unit ranges from the slot counts, then the batched splat
static gvx_status frame_splat(gvx_batch* b, const SplatKind& kind, const SplatArgs& a0, int blocks)
{
    const int ng = (int)b->grids.size();
    k_batch_ustart<<<1, 32, 0, b->stream>>>(b->f_cnt.as<const uint32_t*>(), b->f_caps.as<uint32_t>(), ng, a0.slabs,
                                            b->f_ustart.as<uint32_t>());
    const size_t smem = splat_smem(a0, kind);  // (the shared-memory limit set by batch_max_blocks)
    void* kern = splat_kernel(kind, true);
    const SplatArgs* dargs = b->f_args.as<SplatArgs>();
    uint32_t* dus = b->f_ustart.as<uint32_t>();
    int n = ng;
    void* kargs[] = {(void*)&dargs, (void*)&dus, (void*)&n};
    GVX_CK(cudaLaunchKernel(kern, dim3(blocks), dim3(kSlabWarps * 32), kargs, smem, b->stream));
    b->launches += 2;
    // every grid's device error word (topology and splat) into its plan's record
    for (gvx_grid* g : b->grids) GVX_CK_STATUS(gvx_topo_plan_record_error(g, b->stream));
    return GVX_OK;
}

// what a captured frame depends on: buffer addresses (the allocation epoch), the plans, the
// points and attributes bound, the streams and the splat's parameters
static std::vector<uint64_t> frame_key(gvx_batch* b, float topo_radius, int mode, float radius, int chan_d,
                                       int chan_v, int layers, int blocks)
{
    auto fb = [](float f) {
        uint32_t u;
        memcpy(&u, &f, 4);
        return (uint64_t)u;
    };
    std::vector<uint64_t> k = {gvx_alloc_epoch(), fb(topo_radius), (uint64_t)mode, fb(radius), (uint64_t)chan_d,
                               (uint64_t)chan_v, (uint64_t)layers, (uint64_t)blocks, (uint64_t)(uintptr_t)b->stream,
                               (uint64_t)batch_dense(b)};
    for (gvx_grid* g : b->grids) {
        const GvxPoints& p = g->pts;
        for (uint64_t v : {gvx_topo_plan_id(g), (uint64_t)(uintptr_t)g->stream, (uint64_t)(uintptr_t)p.pos,
                           (uint64_t)p.pos_off, (uint64_t)p.pos_stride, (uint64_t)p.n, (uint64_t)(uintptr_t)p.vel,
                           (uint64_t)p.vel_off, (uint64_t)p.vel_stride, (uint64_t)(uintptr_t)p.weight,
                           (uint64_t)(uintptr_t)p.radius})
            k.push_back(v);
    }
    return k;
}

// the planned builds and the splat captured in b->f_exec (nothing allocated meanwhile)
static gvx_status frame_capture(gvx_batch* b, const std::vector<char>& want_svel, const SplatKind& kind,
                                const SplatArgs& a0, int blocks)
{
    const size_t ng = b->grids.size();
    std::vector<int64_t> l0(ng);
    for (size_t i = 0; i < ng; i++) l0[i] = b->grids[i]->launches;
    const int64_t b0 = b->launches;
    gvx_status rc;
    cudaGraph_t graph = nullptr;
    cudaError_t e;
    {
        GvxNoAllocScope no_alloc;
        GVX_CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        rc = frame_builds(b, want_svel);
        if (rc == GVX_OK) rc = frame_splat(b, kind, a0, blocks);
        e = cudaStreamEndCapture(b->stream, &graph);
    }
    (void)cudaGetLastError();
    b->f_grid_launches.assign(ng, 0);
    for (size_t i = 0; i < ng; i++) {
        b->f_grid_launches[i] = b->grids[i]->launches - l0[i];
        b->grids[i]->launches = l0[i];  // counted when the graph runs
    }
    b->f_launches = b->launches - b0;
    b->launches = b0;
    if (rc != GVX_OK || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return rc != GVX_OK ? rc : gvx_cuda_fail(e, "BatchFrame capture");
    }
    e = cudaGraphInstantiate(&b->f_exec, graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        b->f_exec = nullptr;
        return gvx_cuda_fail(e, "BatchFrame graph instantiation");
    }
    b->f_graph = graph;
    return GVX_OK;
}

// a frame without plans: the staged batch topology and the batched splat, then every grid's
// plan from its build
static gvx_status frame_unplanned(gvx_batch* b, float topo_radius, int mode, float radius, int chan_d, int chan_v,
                                  int flags)
{
    frame_drop_graph(b);
    b->f_warm = false;
    b->f_topo_radius = -1.f;
    b->f_path = 0;
    gvx_status rc = gvx_batch_topology(b, topo_radius, GVX_TOPO_FULL, 0);
    if (rc) return rc;
    rc = gvx_batch_splat(b, mode, radius, chan_d, chan_v, 0, flags & GVX_BATCH_TUNE);
    if (rc) return rc;
    GVX_CK(cudaStreamSynchronize(b->stream));
    bool all = true;
    for (gvx_grid* g : b->grids) all = gvx_topo_plan_make(g) == GVX_OK && all;
    if (all) b->f_topo_radius = topo_radius;
    return GVX_OK;
}

// one grid of a planned frame whose plan did not hold: built and splatted again without one,
// and planned anew
static gvx_status frame_rebuild(gvx_grid* g, float topo_radius, int mode, float radius, int chan_d, int chan_v)
{
    gvx_status rc = gvx_topo_stage1(g, g->pts.n, topo_radius, GVX_TOPO_FULL, 1);
    if (rc == GVX_OK) rc = gvx_topo_stage2(g);
    if (rc == GVX_OK) rc = gvx_topo_stage3(g);
    if (rc == GVX_OK) rc = gvx_topo_update_atlas(g);
    if (rc == GVX_OK) rc = gvx_splat_run(g, mode, g->pts.n, radius, nullptr, chan_d, chan_v, 0);
    if (rc == GVX_OK) GVX_CK(cudaStreamSynchronize(g->stream));
    if (rc == GVX_OK) (void)gvx_topo_plan_make(g);  // (without a plan the next frame runs unplanned)
    return rc;
}

extern "C" {

gvx_status gvx_batch_create(int device, gvx_batch** out)
{
    if (!out) {
        gvx_set_error("gvx_batch_create: null output");
        return GVX_ERR_INVALID_ARG;
    }
    *out = nullptr;
    GVX_CK(cudaSetDevice(device));
    gvx_batch* b = new gvx_batch();
    b->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        if (b->stream) cudaStreamDestroy(b->stream);
        delete b;
        return gvx_cuda_fail(e, "gvx_batch_create");
    }
    b->own_stream = true;
    *out = b;
    return GVX_OK;
}

gvx_status gvx_batch_destroy(gvx_batch* b)
{
    if (!b) return GVX_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    batch_drop_graph(b);
    frame_drop_graph(b);
    gvx_free(b->d_args);
    gvx_free(b->d_ustart);
    for (DevBuf* d : {&b->f_args, &b->f_ustart, &b->f_cnt, &b->f_caps}) gvx_free(*d);
    if (b->f_fork) cudaEventDestroy(b->f_fork);
    for (cudaEvent_t e : b->f_join) cudaEventDestroy(e);
    if (b->ev) cudaEventDestroy(b->ev);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return GVX_OK;
}

gvx_status gvx_batch_set_stream(gvx_batch* b, void* stream)
{
    if (!b) {
        gvx_set_error("null batch handle");
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(cudaSetDevice(b->device));
    GVX_CK(cudaStreamSynchronize(b->stream));
    if (b->own_stream) cudaStreamDestroy(b->stream);
    b->stream = (cudaStream_t)stream;
    b->own_stream = false;
    batch_drop_graph(b);
    frame_drop_graph(b);
    return GVX_OK;
}

gvx_status gvx_batch_set_grids(gvx_batch* b, gvx_grid* const* grids, int count)
{
    if (!b || (count > 0 && !grids) || count < 0 || count > kBatchMaxGrids) {
        gvx_set_error("BatchSetGrids: need 0..%d grids", kBatchMaxGrids);
        return GVX_ERR_INVALID_ARG;
    }
    for (int i = 0; i < count; i++) {
        if (!grids[i] || grids[i]->device != b->device) {
            gvx_set_error("BatchSetGrids: grid %d is null or on another device", i);
            return GVX_ERR_INVALID_ARG;
        }
    }
    b->grids.assign(grids, grids + count);
    batch_drop_graph(b);
    frame_drop_graph(b);
    b->f_warm = false;
    b->f_topo_radius = -1.f;
    return GVX_OK;
}

// Topology of every grid from a pool of host threads: each grid is driven by one
// thread at a time (a grid handle is not shared between threads), and builds of
// grids on different streams overlap on the GPU.  A build is mostly small kernels
// and two host readbacks, so one thread alone leaves the GPU idle most of the time.
gvx_status gvx_batch_topology(gvx_batch* b, float radius, int mode, int threads)
{
    if (!b) {
        gvx_set_error("null batch handle");
        return GVX_ERR_INVALID_ARG;
    }
    if (mode < GVX_TOPO_AUTO || mode > GVX_TOPO_ACCUMULATE) {
        gvx_set_error("BatchTopology: mode %d", mode);
        return GVX_ERR_INVALID_ARG;
    }
    const size_t n = b->grids.size();
    if (n == 0) return GVX_OK;
    if (threads <= 0) {
        // staged, from this thread: every grid's GetBoundingBox, then (one wait per grid, by
        // then mostly passed) every grid's build up to its node counts, then every grid's
        // pools, UpdateAtlas and InsertPoints; the grids' streams overlap on the GPU
        GVX_CK(cudaSetDevice(b->device));
        const char* what[3] = {"GetBoundingBox", "RebuildTopology", "pools/UpdateAtlas/InsertPoints"};
        for (int stage = 0; stage < 3; stage++) {
            for (size_t i = 0; i < n; i++) {
                gvx_grid* g = b->grids[i];
                gvx_status r = GVX_OK;
                if (stage == 0) {
                    r = gvx_wait_positions(g);
                    if (r == GVX_OK) r = gvx_topo_stage1(g, g->pts.n, radius, mode, 1);
                } else if (stage == 1) {
                    r = gvx_topo_stage2(g);
                } else {
                    r = gvx_topo_stage3(g);
                    if (r == GVX_OK) r = gvx_wait_attributes(g);
                    if (r == GVX_OK) r = gvx_topo_update_atlas(g);
                    if (r == GVX_OK) r = gvx_prepare_points(g, g->pts.n, nullptr, false);
                }
                if (r != GVX_OK) {
                    const std::string m = gvx_last_error();
                    gvx_set_error("BatchTopology: grid %zu (%s): %s", i, what[stage], m.c_str());
                    return r;
                }
            }
        }
        return GVX_OK;
    }
    const size_t nt = std::min<size_t>(n, (size_t)threads);
    std::atomic<size_t> next{0};
    std::vector<gvx_status> st(n, GVX_OK);
    std::vector<std::string> msg(n);
    const int device = b->device;
    auto work = [&]() {
        if (cudaSetDevice(device) != cudaSuccess) return;
        for (;;) {
            const size_t i = next.fetch_add(1);
            if (i >= n) break;
            gvx_grid* g = b->grids[i];
            gvx_status r = gvx_rebuild_topology(g, g->pts.n, radius, nullptr, mode, 1);
            if (r == GVX_OK) r = gvx_update_atlas(g);
            if (r == GVX_OK) r = gvx_insert_points(g, g->pts.n, nullptr, nullptr);
            st[i] = r;
            if (r != GVX_OK) msg[i] = gvx_last_error();
        }
    };
    std::vector<std::thread> pool;
    for (size_t t = 1; t < nt; t++) pool.emplace_back(work);
    work();
    for (std::thread& t : pool) t.join();
    for (size_t i = 0; i < n; i++)
        if (st[i] != GVX_OK) {
            gvx_set_error("BatchTopology: grid %zu: %s", i, msg[i].c_str());
            return st[i];
        }
    return GVX_OK;
}

gvx_status gvx_batch_splat(gvx_batch* b, int mode, float radius, int chan_density, int chan_vel, int accum, int flags)
{
    if (!b) {
        gvx_set_error("null batch handle");
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(cudaSetDevice(b->device));
    if (b->grids.empty()) return GVX_OK;
    // the grids' own streams first (their InsertPoints work), then the batch
    for (gvx_grid* g : b->grids) {
        if (g->stream == b->stream) continue;
        GVX_CK(cudaEventRecord(b->ev, g->stream));
        GVX_CK(cudaStreamWaitEvent(b->stream, b->ev, 0));
    }
    int layers = 0, bps = 0;
    std::vector<SplatArgs> args;
    std::vector<uint32_t> us;
    SplatKind kind;
    gvx_status rc = batch_tables(b, mode, radius, chan_density, chan_vel, accum, 0, args, us, kind);
    if (rc) return rc;
    const std::string key = tune_key(b->device, args[0], kind);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) b->tuning = it->second;
    }
    if ((flags & GVX_BATCH_TUNE) && !accum && b->tuning.layers == 0) {
        // the grids' streams must not run during the timing
        for (gvx_grid* g : b->grids) GVX_CK(cudaStreamSynchronize(g->stream));
        batch_drop_graph(b);
        rc = batch_tune(b, mode, radius, chan_density, chan_vel, &b->tuning);
        if (rc) return rc;
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = b->tuning;
    }
    layers = b->tuning.layers;
    bps = b->tuning.blocks_per_sm;
    if (layers > 0 && layers != args[0].slab_layers) {
        rc = batch_tables(b, mode, radius, chan_density, chan_vel, accum, layers, args, us, kind);
        if (rc) return rc;
    }
    int per_sm = 1;
    rc = batch_max_blocks(b, kind, args[0], &per_sm);
    if (rc) return rc;
    if (bps <= 0 || bps > per_sm) bps = per_sm;
    const uint64_t ctas_needed = ((uint64_t)us.back() + kSlabWarps - 1) / kSlabWarps;
    const int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>(ctas_needed, (uint64_t)sm_count(b->device) * bps));
    const bool same = b->exec && b->cap_args.size() == args.size() && b->cap_kind == kind &&
                      b->cap_blocks == blocks &&
                      memcmp(b->cap_args.data(), args.data(), args.size() * sizeof(SplatArgs)) == 0 &&
                      b->cap_ustart == us;
    if (us.back() > 0) {
        if (flags & GVX_BATCH_GRAPH) {
            if (!same) {
                batch_drop_graph(b);
                rc = batch_upload(b, args, us);
                if (rc) return rc;
                GVX_CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
                rc = batch_launch(b, kind, args[0], (int)args.size(), blocks);
                cudaGraph_t graph = nullptr;
                cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
                if (rc) {
                    if (graph) cudaGraphDestroy(graph);
                    return rc;
                }
                if (e != cudaSuccess) return gvx_cuda_fail(e, "cudaStreamEndCapture");
                b->graph = graph;
                e = cudaGraphInstantiate(&b->exec, b->graph, 0);
                if (e != cudaSuccess) {
                    batch_drop_graph(b);
                    return gvx_cuda_fail(e, "cudaGraphInstantiate");
                }
                b->cap_args = args;
                b->cap_ustart = us;
                b->cap_kind = kind;
                b->cap_blocks = blocks;
                b->launches--;  // the captured launch runs with the graph below
            }
            GVX_CK(cudaGraphLaunch(b->exec, b->stream));
            b->launches++;
        } else {
            rc = batch_upload(b, args, us);
            if (rc) return rc;
            rc = batch_launch(b, kind, args[0], (int)args.size(), blocks);
            if (rc) return rc;
        }
    }
    // the grids' streams see the splat before their next work
    GVX_CK(cudaEventRecord(b->ev, b->stream));
    for (gvx_grid* g : b->grids) {
        if (g->stream != b->stream) GVX_CK(cudaStreamWaitEvent(g->stream, b->ev, 0));
        g->launches++;
        splat_finish(g, chan_density, chan_vel, accum);
    }
    return GVX_OK;
}

gvx_status gvx_batch_get_tuning(gvx_batch* b, int* slab_layers, int* blocks_per_sm, float* ms)
{
    if (!b) {
        gvx_set_error("null batch handle");
        return GVX_ERR_INVALID_ARG;
    }
    if (slab_layers) *slab_layers = b->tuning.layers;
    if (blocks_per_sm) *blocks_per_sm = b->tuning.blocks_per_sm;
    if (ms) *ms = b->tuning.ms;
    return GVX_OK;
}

gvx_status gvx_batch_kernel_launches(gvx_batch* b, int64_t* out)
{
    if (!b || !out) {
        gvx_set_error("null batch handle");
        return GVX_ERR_INVALID_ARG;
    }
    *out = b->launches;
    return GVX_OK;
}


gvx_status gvx_batch_frame(gvx_batch* b, float topo_radius, int mode, float radius, int chan_density, int chan_vel,
                           int flags)
{
    if (!b) {
        gvx_set_error("null batch handle");
        return GVX_ERR_INVALID_ARG;
    }
    if (!(topo_radius >= 0.f)) {
        gvx_set_error("BatchFrame: topology radius must be >= 0");
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(cudaSetDevice(b->device));
    const size_t ng = b->grids.size();
    b->f_void = 0;
    if (ng == 0) return GVX_OK;
    bool planned = b->f_topo_radius == topo_radius;
    for (gvx_grid* g : b->grids) planned = planned && gvx_topo_plan_ready(g);
    if (!planned) return frame_unplanned(b, topo_radius, mode, radius, chan_density, chan_vel, flags);

    // the splat's kind and slab height, the same for every grid
    SplatKind kind{};
    int layers = 0;
    std::vector<char> want_svel(ng);
    for (size_t i = 0; i < ng; i++) {
        gvx_grid* g = b->grids[i];
        int l = b->tuning.layers;
        SplatKind k;
        gvx_status rc = splat_check(g, mode, radius, chan_density, chan_vel, 0, batch_dense(b), &l, &k);
        if (rc) return rc;
        if (i == 0) {
            kind = k;
            layers = l;
        } else if (!(k == kind) || g->P != b->grids[0]->P || l != layers) {
            gvx_set_error("BatchFrame: grid %zu differs from grid 0 in brick shape, channels or radius kind", i);
            return GVX_ERR_INVALID_ARG;
        }
        want_svel[i] = k.has_v || k.ppr || g->pts.vel || g->pts.radius;
    }
    SplatArgs a0;
    memset(&a0, 0, sizeof(a0));
    const SlabShape sh0 = slab_shape(b->grids[0], 0, batch_dense(b), kind.has_d && kind.has_v);
    a0.P = b->grids[0]->P;
    a0.push = sh0.push;
    a0.tile_rows = sh0.rows;
    a0.slab_layers = layers;
    a0.slabs = (sh0.span + layers - 1) / layers;
    uint64_t units = 0;
    for (gvx_grid* g : b->grids) {
        uint32_t cap = 0;
        (void)gvx_topo_plan_slots(g, &cap);
        units += (uint64_t)cap * a0.slabs;
    }
    if (units >= (1ull << 31)) {
        gvx_set_error("BatchFrame: more than 2^31 work units");
        return GVX_ERR_CAPACITY;
    }
    int per_sm = 1;
    gvx_status rc = batch_max_blocks(b, kind, a0, &per_sm);
    if (rc) return rc;
    int bps = b->tuning.blocks_per_sm;
    if (bps <= 0 || bps > per_sm) bps = per_sm;
    const int blocks = sm_count(b->device) * bps;

    // the grids' queued work (point uploads included) before the frame
    if (!b->f_fork) GVX_CK(cudaEventCreateWithFlags(&b->f_fork, cudaEventDisableTiming));
    while (b->f_join.size() < ng) {
        cudaEvent_t e;
        GVX_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        b->f_join.push_back(e);
    }
    for (size_t i = 0; i < ng; i++) {
        gvx_grid* g = b->grids[i];
        rc = gvx_wait_positions(g);
        if (rc == GVX_OK) rc = gvx_wait_attributes(g);
        if (rc) return rc;
        if (g->stream != b->stream) {
            GVX_CK(cudaEventRecord(b->f_join[i], g->stream));
            GVX_CK(cudaStreamWaitEvent(b->stream, b->f_join[i], 0));
        }
    }
    GVX_CK(gvx_ensure(b->f_args, ng * sizeof(SplatArgs)));
    GVX_CK(gvx_ensure(b->f_ustart, (ng + 2) * sizeof(uint32_t)));
    GVX_CK(gvx_ensure(b->f_cnt, ng * sizeof(void*)));
    GVX_CK(gvx_ensure(b->f_caps, ng * sizeof(uint32_t)));

    bool use_graph = (flags & GVX_BATCH_GRAPH) && b->f_warm;
    if (use_graph) {
        const std::vector<uint64_t> key = frame_key(b, topo_radius, mode, radius, chan_density, chan_vel, layers, blocks);
        if (!(b->f_exec && key == b->f_key)) {
            frame_drop_graph(b);
            use_graph = key != b->f_failed_key;
            if (use_graph) {
                rc = frame_upload(b, kind, radius, chan_density, chan_vel, layers);
                if (rc) return rc;
                if (frame_capture(b, want_svel, kind, a0, blocks) == GVX_OK) {
                    b->f_key = key;
                } else {
                    b->f_failed_key = key;  // the frame runs without a graph; no new attempt with this key
                    use_graph = false;
                }
            }
        }
    }
    if (use_graph) {
        GVX_CK(cudaGraphLaunch(b->f_exec, b->stream));
        b->launches += b->f_launches;
        for (size_t i = 0; i < ng; i++) {
            b->grids[i]->launches += b->f_grid_launches[i];
            gvx_topo_plan_replayed(b->grids[i]);
        }
        b->f_path = 2;
    } else {
        rc = frame_builds(b, want_svel);
        if (rc == GVX_OK) rc = frame_upload(b, kind, radius, chan_density, chan_vel, layers);
        if (rc == GVX_OK) rc = frame_splat(b, kind, a0, blocks);
        if (rc) {
            cudaStreamSynchronize(b->stream);
            return rc;
        }
        b->f_path = 1;
    }
    GVX_CK(cudaStreamSynchronize(b->stream));

    // which plans held: the grids whose did not are built again without one
    gvx_status first = GVX_OK;
    std::vector<size_t> redo;
    for (size_t i = 0; i < ng; i++) {
        gvx_grid* g = b->grids[i];
        bool held = false;
        rc = gvx_topo_plan_finish(g, &held, true);
        if (rc != GVX_OK) {
            if (first == GVX_OK) {
                const std::string m = gvx_last_error();
                gvx_set_error("BatchFrame: grid %zu: %s", i, m.c_str());
                first = rc;
            }
            continue;
        }
        if (!held) {
            redo.push_back(i);
            continue;
        }
        g->perm_valid = true;  // as gvx_prepare_points leaves it
        g->perm_has_svel = want_svel[i] != 0;
        g->perm_vel = g->pts.vel;
        g->perm_w = g->pts.weight;
        g->perm_r = g->pts.radius;
        splat_finish(g, chan_density, chan_vel, 0);
    }
    if (first != GVX_OK) {
        frame_drop_graph(b);
        b->f_warm = false;
        b->f_topo_radius = -1.f;
        return first;
    }
    if (b->f_path == 1) b->f_warm = true;
    if (!redo.empty()) {
        frame_drop_graph(b);
        b->f_warm = false;
        b->f_void = (int)redo.size();
        for (size_t i : redo) {
            rc = frame_rebuild(b->grids[i], topo_radius, mode, radius, chan_density, chan_vel);
            if (rc) {
                const std::string m = gvx_last_error();
                gvx_set_error("BatchFrame: grid %zu: %s", i, m.c_str());
                b->f_topo_radius = -1.f;
                return rc;
            }
        }
    }
    return GVX_OK;
}

gvx_status gvx_batch_frame_path(gvx_batch* b, int* path, int* rebuilt)
{
    if (!b) {
        gvx_set_error("null batch handle");
        return GVX_ERR_INVALID_ARG;
    }
    if (path) *path = b->f_path;
    if (rebuilt) *rebuilt = b->f_void;
    return GVX_OK;
}

}  // extern "C"

gvx_status gvx_scatter_ref(gvx_grid* g, int n, float radius, const float trans[3], int expand, int avg_color)
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
    // the colour half (VG.cpp:5638-5655): with point colours, avgColor averages into channel 1; without,
    // each voxel takes a point's colour in channel 3, unless an avgColor call ever ran on this grid
    // (the reference's colour buffer then exists and silently takes the sums)
    int clr_mode = 0;
    if (g->pts.clr) {
        if (avg_color) clr_mode = 1;
        else if (!g->colavg_seen) clr_mode = 2;
    }
    const int clr_chan = clr_mode == 1 ? 1 : 3;
    if (clr_mode && (!g->ch[clr_chan].used || g->ch[clr_chan].elem_bytes != 4)) {
        gvx_set_error("ScatterDensity: point colours go to channel %d, which must be a 4-byte channel", clr_chan);
        return GVX_ERR_INVALID_ARG;
    }
    rc = gvx_prepare_points(g, n, trans, false);
    if (rc) return rc;
    if (clr_mode == 1) g->colavg_seen = true;
    const int P = g->P, P3 = P * P * P, b3 = g->brick * g->brick * g->brick;
    const size_t smem = (((size_t)P3 * 4 + 15) & ~(size_t)15) + (clr_mode == 1 ? 16 : clr_mode == 2 ? 4 : 0) * (size_t)b3;
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
    a.clr_mode = clr_mode;
    a.perm = g->vals[g->sorted_buf].as<uint32_t>();
    a.clr = g->pts.clr;
    a.clr_off = g->pts.clr_off;
    a.clr_stride = g->pts.clr_stride;
    a.clr_out = clr_mode ? g->ch[clr_chan].data.as<uint32_t>() : nullptr;
    apron_invalidate(g->ch[0]);
    if (clr_mode) apron_invalidate(g->ch[clr_chan]);
    if (a.nslots == 0) return GVX_OK;
    GVX_CK(cudaFuncSetAttribute(k_scatter_ref, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    GVX_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_scatter_ref, kSplatThreads, smem));
    const uint32_t grid = std::min<uint32_t>(a.nslots, (uint32_t)(sm_count(g->device) * std::max(per_sm, 1)));
    k_scatter_ref<<<grid, kSplatThreads, smem, g->stream>>>(a);
    g->launches++;
    GVX_CK(cudaGetLastError());
    return GVX_OK;
}
