// ref_harness.cu -- runs the REFERENCE's own CUDA kernels for parity pinning.
//
// TEST INFRASTRUCTURE ONLY.  Loads the PTX that oracle/ref_build.py compiles
// from the reference's kernel sources (cuda_gvdb_module.cu) and drives those
// kernels with a restatement of the reference's host orchestration, so that the
// oracle (gvx_oracle.c) and libgvx can be compared with what the reference
// itself computes on the same GPU.  Host steps are restated from
// (paths relative to the reference project):
//   RebuildTopology / AccumulateTopology   gvdb_volume_gvdb.cpp:1158-1218
//   GetBoundingBox / DetermineDepth        gvdb_volume_gvdb.cpp:5404-5467, 821-837
//   ActivateBricksGPU                      gvdb_volume_gvdb.cpp:1229-1413
//   ActivateExtraBricksGPU                 gvdb_volume_gvdb.cpp:931-1016
//   ActivateIncreBricksGPU                 gvdb_volume_gvdb.cpp:1020-1156
//   PrepareVDB / PrepareVDBPartially       gvdb_volume_gvdb.cpp:3946-4020
//   UpdateAtlas                            gvdb_volume_gvdb.cpp:2630-2704
//   InsertPoints / ScatterDensity          gvdb_volume_gvdb.cpp:5219-5267, 5624-5660
//   InsertPointsSubcell / Gather*          gvdb_volume_gvdb.cpp:4971-5092, 5318-5373
//   UpdateApron                            gvdb_volume_gvdb.cpp:4418-4457
// Departures (none changes a result on the inputs the tests use):
//   - the reference sorts keys with thrust::sort (CU.cu:11-16) and finds unique
//     keys with its FindUnique/PrefixSum/Compact kernels; here thrust::sort
//     and thrust::unique on the device give the same total order and unique
//     list, which are copied to the host for the allocation loop as the
//     reference copies AUX_UNIQUE_LEVXYZ;
//   - the min/max of the bounding box: thrust::min_element / max_element on
//     the device per axis, as gvdbDeviceMin/MaxElementF (gvdb_cutils.cu:22-39),
//     then one copy of the 6 floats (RetrieveData of AUX_BOUNDING_BOX);
//   - key buffers are sized generously (the reference's N*depth buffer can overflow);
//   - ScatterDensity is launched with the kernel's own argument list (the
//     reference host call omits the VDBInfo pointer, VG.cpp:5645);
//   - float channels are cleared by the reference's own kernelFillTex (AtlasFill);
//     channels of wider voxels by a device copy of zeros (kernelFillTex writes 4
//     bytes per voxel); the atlas grows by a device array-to-array copy as
//     AllocateTextureGPU preserves its data.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <thrust/device_ptr.h>
#include <thrust/extrema.h>
#include <thrust/sort.h>
#include <thrust/unique.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

namespace {

thread_local std::string t_err;

#define RH_CK(call)                                                          \
    do {                                                                     \
        CUresult _r = (call);                                                \
        if (_r != CUDA_SUCCESS) {                                            \
            const char* _s = nullptr;                                        \
            cuGetErrorString(_r, &_s);                                       \
            t_err = std::string(#call) + ": " + (_s ? _s : "?");             \
            return -1;                                                       \
        }                                                                    \
    } while (0)

constexpr uint64_t UNDEFL = 0xFFFFFFFFull;
constexpr uint64_t UNDEF64 = 0xFFFFFFFFFFFFFFFFull;
constexpr float NOHIT = 1.0e10f;

// Node (gvdb_node.h:27-40) and VDBInfo (cuda_gvdb_nodes.cuh:42-67): the layout
// the reference kernels read, declared field for field
struct __align__(16) RNode {
    uint8_t lev, flags, prio, pad;
    int32_t pos[3];
    int32_t value[3];
    float vrange[3];
    uint64_t parent;
    uint64_t childlist;
    uint64_t mask;
};
static_assert(sizeof(RNode) == 64, "node");

struct __align__(16) RAtlasNode {
    int32_t pos[3];
    int32_t leaf;
};

struct __align__(16) RVDBInfo {
    int dim[10];
    int res[10];
    float3 vdel[10];
    int3 noderange[10];
    int nodecnt[10];
    int nodewid[10];
    int childwid[10];
    char* nodelist[10];
    char* childlist[10];
    RAtlasNode* atlas_map;
    int3 atlas_cnt;
    int3 atlas_res;
    int atlas_apron;
    int brick_res;
    int apron_table[8];
    int top_lev;
    int max_iter;
    float epsilon;
    bool update;
    unsigned char clr_chan;
    float3 bmin;
    float3 bmax;
    unsigned long long volIn[32];
    unsigned long long volOut[32];
};

struct Mod {
    bool loaded = false;
    CUmodule m = nullptr;
    CUfunction splitpos, calcbrick, link, extra, increextra, delinkleaf, delink, insertpts, scatter, setflag,
        countsc, insertsc, scpos, gatherd, gatherl, apronf, apronf4, insertsc16, gatherl16, convxform;
    CUmodule mcopy = nullptr;  // cuda_gvdb_copydata.ptx: kernelFillTex (Allocator::AtlasFill)
    CUfunction filltex = nullptr;
} g_mod;

struct DBuf {
    CUdeviceptr p = 0;
    size_t cap = 0;
};
int dens(DBuf& b, size_t bytes)
{
    if (bytes <= b.cap && b.p) return 0;
    if (b.p) cuMemFree(b.p);
    b.p = 0;
    b.cap = 0;
    size_t want = bytes < 256 ? 256 : bytes;
    RH_CK(cuMemAlloc(&b.p, want));
    b.cap = want;
    return 0;
}

}  // namespace

struct rh_grid {
    int levels = 0, logdim[10] = {}, res[10] = {}, range[10] = {};
    int apron = 1, brick = 8, P = 10;
    int defsub[3] = {16, 16, 1};
    std::vector<RNode> nodes[10];
    std::vector<uint64_t> clist[10];
    int used0 = 0;
    DBuf dnodes[10], dclist[10];
    bool rebuild = true;
    int curr_depth = -1;
    int root_level = -1;
    int last_mode = 0;
    // atlas
    int sub[3] = {0, 0, 0};
    bool have_atlas = false;
    struct Chan {
        bool used = false;
        int type = 0, elem = 4;
        CUarray arr = nullptr;
        CUsurfObject surf = 0;
    } ch[32];
    std::vector<RAtlasNode> amap;
    DBuf damap;
    RVDBInfo info;
    DBuf dinfo;
    float3 objmin{0, 0, 0}, objmax{0, 0, 0};
    // points
    int n = 0;
    DBuf dpos;
    // aux
    DBuf range_res, keys, cnt, markers, splitx, splity, splitz;
    DBuf pnode, poff, gcnt;
    DBuf zero;  // zero-filled source of device-side clears of array regions
    DBuf scflag, scmap, sccnt, scoff, scpts, scpos, scnid;
    int sc_len = 0, num_sc = 0;
    float3 pos_min{0, 0, 0}, pos_range{0, 0, 0};  // mPosMin, mPosRange of GetBoundingBox (VG.cpp:5452-5462)
};

namespace {

int vc(const rh_grid* g, int l) { return g->res[l] * g->res[l] * g->res[l]; }

int top_lev(const rh_grid* g)
{
    int t = 1;
    for (int n = g->levels - 1; n >= 0; n--)
        if ((int)g->nodes[n].size() == 1) t = n;
    return t;
}

// PoolAlloc (AL.cpp:158-188) + SetupNode (VG.cpp:2512-2524) + child list 0xFF
int alloc_node(rh_grid* g, int lev, int x, int y, int z)
{
    RNode nd;
    memset(&nd, 0, sizeof(nd));
    nd.lev = (uint8_t)lev;
    nd.flags = 1;
    nd.pos[0] = x;
    nd.pos[1] = y;
    nd.pos[2] = z;
    nd.value[0] = nd.value[1] = nd.value[2] = -1;
    nd.parent = UNDEFL;
    nd.childlist = UNDEFL;
    int i = (int)g->nodes[lev].size();
    if (lev > 0) {
        nd.childlist = 1ull | ((uint64_t)lev << 8) | ((uint64_t)i << 16);
        g->clist[lev].resize((size_t)(i + 1) * vc(g, lev), UNDEF64);
    }
    g->nodes[lev].push_back(nd);
    if (lev == 0) g->used0++;
    return i;
}

int commit_pools(rh_grid* g)
{
    for (int l = 0; l < g->levels; l++) {
        size_t nb = g->nodes[l].size() * sizeof(RNode);
        if (dens(g->dnodes[l], nb ? nb : 64)) return -1;
        if (nb) RH_CK(cuMemcpyHtoD(g->dnodes[l].p, g->nodes[l].data(), nb));
        size_t cb = g->clist[l].size() * 8;
        if (dens(g->dclist[l], cb ? cb : 64)) return -1;
        if (cb) RH_CK(cuMemcpyHtoD(g->dclist[l].p, g->clist[l].data(), cb));
    }
    return 0;
}

int fetch_pools(rh_grid* g)
{
    RH_CK(cuCtxSynchronize());
    for (int l = 0; l < g->levels; l++) {
        size_t nb = g->nodes[l].size() * sizeof(RNode);
        if (nb) RH_CK(cuMemcpyDtoH(g->nodes[l].data(), g->dnodes[l].p, nb));
        size_t cb = g->clist[l].size() * 8;
        if (cb) RH_CK(cuMemcpyDtoH(g->clist[l].data(), g->dclist[l].p, cb));
    }
    return 0;
}

// PrepareVDBPartially (VG.cpp:3996-4020) and PrepareVDB (VG.cpp:3946-3990)
int prepare(rh_grid* g, bool full)
{
    RVDBInfo& v = g->info;
    for (int n = 0; n < g->levels; n++) {
        v.dim[n] = g->logdim[n];
        v.res[n] = g->res[n];
        v.vdel[n] = make_float3((float)g->range[n] / g->res[n], (float)g->range[n] / g->res[n],
                                (float)g->range[n] / g->res[n]);
        v.noderange[n] = make_int3(g->range[n], g->range[n], g->range[n]);
        v.nodecnt[n] = (int)g->nodes[n].size();
        v.nodewid[n] = (int)sizeof(RNode);
        v.childwid[n] = n == 0 ? 0 : vc(g, n) * 8;
        v.nodelist[n] = (char*)g->dnodes[n].p;
        v.childlist[n] = (char*)g->dclist[n].p;
    }
    v.top_lev = top_lev(g);
    v.bmin = g->objmin;
    v.bmax = g->objmax;
    if (full) {
        v.atlas_map = (RAtlasNode*)g->damap.p;
        v.atlas_apron = g->apron;
        v.atlas_cnt = make_int3(g->sub[0], g->sub[1], g->sub[2]);
        v.atlas_res = make_int3(g->sub[0] * g->P, g->sub[1] * g->P, g->sub[2] * g->P);
        v.brick_res = g->P;
        v.top_lev = top_lev(g);
        for (int c = 0; c < 32; c++) v.volOut[c] = g->ch[c].used ? g->ch[c].surf : 0;
    }
    if (dens(g->dinfo, sizeof(RVDBInfo))) return -1;
    RH_CK(cuMemcpyHtoD(g->dinfo.p, &v, sizeof(RVDBInfo)));
    return 0;
}

int launch(CUfunction f, unsigned gx, unsigned gy, unsigned gz, unsigned bx, unsigned by, unsigned bz, void** args)
{
    RH_CK(cuLaunchKernel(f, gx, gy, gz, bx, by, bz, 0, nullptr, args, nullptr));
    return 0;
}

int link_levels(rh_grid* g, int depth, unsigned grid_override)
{
    for (int lev = depth - 1; lev >= 0; lev--) {
        unsigned pblks = grid_override ? grid_override : (unsigned)(g->nodes[lev].size() / 512 + 1);
        CUdeviceptr info = g->dinfo.p;
        void* args[] = {&info, &lev};
        if (launch(g_mod.link, pblks, 1, 1, 512, 1, 1, args)) return -1;
    }
    return 0;
}

// the first `count` device keys -> sorted unique keys on the host and per-level
// counts (RadixSortByByte + FindUniqueBrick, VG.cpp:843-928)
int sort_unique(rh_grid* g, size_t count, int depth, int* levcnt, std::vector<uint64_t>& k)
{
    RH_CK(cuCtxSynchronize());
    thrust::device_ptr<uint64_t> d((uint64_t*)g->keys.p);
    thrust::sort(d, d + count);
    const size_t u = (size_t)(thrust::unique(d, d + count) - d);
    k.resize(u);
    if (u) RH_CK(cuMemcpyDtoH(k.data(), g->keys.p, u * 8));
    for (int l = 0; l < depth; l++) levcnt[l] = 0;
    for (uint64_t key : k) {
        int lev = (int)((key >> 48) & 0xFF);
        if (lev != 255 && lev < depth) levcnt[lev]++;
    }
    return 0;
}

void alloc_from_keys(rh_grid* g, const std::vector<uint64_t>& k, const int* levcnt, int depth)
{
    size_t pre = 0;
    for (int lev = 0; lev < depth; lev++) {
        int r = g->range[lev];
        for (size_t n = pre; n < pre + levcnt[lev]; n++)
            alloc_node(g, lev, (int)((k[n] >> 32) & 0xFFFF) * r, (int)((k[n] >> 16) & 0xFFFF) * r,
                       (int)(k[n] & 0xFFFF) * r);
        pre += levcnt[lev];
    }
}

int upload_range_res(rh_grid* g, int depth)
{
    std::vector<int> rr(depth);
    for (int l = 0; l < depth; l++) rr[l] = g->range[l];
    if (dens(g->range_res, depth * 4)) return -1;
    RH_CK(cuMemcpyHtoD(g->range_res.p, rr.data(), depth * 4));
    return 0;
}

int activate_bricks(rh_grid* g, float3 orig, int depth, const int* rootpos)
{
    alloc_node(g, depth, rootpos[0], rootpos[1], rootpos[2]);
    g->root_level = depth;
    if (upload_range_res(g, depth)) return -1;
    size_t nk = (size_t)g->n * depth;
    if (dens(g->keys, nk * 8)) return -1;
    int n = g->n, ld = depth, off = 0, stride = 12;
    CUdeviceptr rr = g->range_res.p, pos = g->dpos.p, keys = g->keys.p;
    void* args[] = {&n, &ld, &rr, &pos, &off, &stride, &orig, &keys};
    if (launch(g_mod.calcbrick, n / 512 + 1, 1, 1, 512, 1, 1, args)) return -1;
    std::vector<uint64_t> k;
    int levcnt[10];
    if (sort_unique(g, nk, depth, levcnt, k)) return -1;
    alloc_from_keys(g, k, levcnt, depth);
    if (commit_pools(g) || prepare(g, false) || link_levels(g, depth, 0) || fetch_pools(g)) return -1;
    return 0;
}

int activate_extra(rh_grid* g, float radius, float3 orig, int depth)
{
    size_t cap = (size_t)g->n * depth * 64 + 64;
    if (dens(g->keys, cap * 8) || dens(g->cnt, 4)) return -1;
    RH_CK(cuMemsetD8(g->cnt.p, 0, 4));
    int n = g->n, ld = depth, off = 0, stride = 12;
    CUdeviceptr info = g->dinfo.p, rr = g->range_res.p, pos = g->dpos.p, keys = g->keys.p, cnt = g->cnt.p;
    void* args[] = {&info, &radius, &n, &ld, &rr, &pos, &off, &stride, &orig, &keys, &cnt};
    if (launch(g_mod.extra, n / 512 + 1, 1, 1, 512, 1, 1, args)) return -1;
    RH_CK(cuCtxSynchronize());
    int count = 0;
    RH_CK(cuMemcpyDtoH(&count, g->cnt.p, 4));
    if ((size_t)count > cap) {
        t_err = "extra key buffer overflow";
        return -1;
    }
    std::vector<uint64_t> k;
    int levcnt[10];
    if (sort_unique(g, (size_t)count, depth, levcnt, k)) return -1;
    alloc_from_keys(g, k, levcnt, depth);
    if (commit_pools(g) || prepare(g, false) || link_levels(g, depth, 0) || fetch_pools(g)) return -1;
    return 0;
}

int activate_incremental(rh_grid* g, float radius, float3 orig, int depth, bool accum)
{
    int total = (int)g->nodes[0].size();
    if (total == 0) return 0;
    std::vector<int> marker(total, 0);
    if (accum)
        for (int i = 0; i < total; i++) marker[i] = g->nodes[0][i].flags;
    if (dens(g->markers, (size_t)total * 4)) return -1;
    RH_CK(cuMemcpyHtoD(g->markers.p, marker.data(), (size_t)total * 4));
    if (upload_range_res(g, depth)) return -1;
    size_t cap = (size_t)g->n * depth * 64 + 64;
    if (dens(g->keys, cap * 8) || dens(g->cnt, 4)) return -1;
    RH_CK(cuMemsetD8(g->cnt.p, 0, 4));
    if (commit_pools(g) || prepare(g, false)) return -1;
    int n = g->n, ld = depth, off = 0, stride = 12;
    CUdeviceptr info = g->dinfo.p, rr = g->range_res.p, pos = g->dpos.p, keys = g->keys.p, cnt = g->cnt.p,
                mk = g->markers.p;
    void* args[] = {&info, &radius, &n, &ld, &rr, &pos, &off, &stride, &orig, &keys, &cnt, &mk};
    if (launch(g_mod.increextra, n / 512 + 1, 1, 1, 512, 1, 1, args)) return -1;
    RH_CK(cuCtxSynchronize());
    int count = 0;
    RH_CK(cuMemcpyDtoH(&count, g->cnt.p, 4));
    if (count == 0) {
        g->last_mode = 0;
        return 0;
    }
    std::vector<uint64_t> k;
    int levcnt[10];
    if (sort_unique(g, (size_t)count, depth, levcnt, k)) return -1;
    RH_CK(cuMemcpyDtoH(marker.data(), g->markers.p, (size_t)total * 4));
    for (int i = 0; i < total; i++) g->nodes[0][i].flags = (uint8_t)marker[i];
    alloc_from_keys(g, k, levcnt, depth);
    if (commit_pools(g) || prepare(g, false)) return -1;
    unsigned pblks = (unsigned)(g->nodes[0].size() / 512 + 1);
    if (link_levels(g, depth, pblks)) return -1;
    CUdeviceptr info2 = g->dinfo.p;
    void* a1[] = {&info2};
    if (launch(g_mod.delinkleaf, pblks, 1, 1, 512, 1, 1, a1)) return -1;
    for (int lev = 1; lev < depth; lev++) {
        void* a2[] = {&info2, &lev};
        if (launch(g_mod.delink, pblks, 1, 1, 512, 1, 1, a2)) return -1;
    }
    if (fetch_pools(g)) return -1;
    int used = (int)g->nodes[0].size();
    for (auto& nd : g->nodes[0])
        if (!nd.flags) used--;
    g->used0 = used;
    g->last_mode = 2;
    return 0;
}

void clear_tree(rh_grid* g)
{
    for (int l = 0; l < 10; l++) {
        g->nodes[l].clear();
        g->clist[l].clear();
    }
    g->used0 = 0;
    g->root_level = -1;
    g->rebuild = true;
}

int make_array(rh_grid* g, int c, int sx, int sy, int sz, CUarray* out, CUsurfObject* surf)
{
    CUDA_ARRAY3D_DESCRIPTOR d;
    memset(&d, 0, sizeof(d));
    d.Format = CU_AD_FORMAT_FLOAT;
    d.NumChannels = g->ch[c].type == 3 ? 1 : 4;
    d.Width = (size_t)sx * g->P;
    d.Height = (size_t)sy * g->P;
    d.Depth = (size_t)sz * g->P;
    d.Flags = CUDA_ARRAY3D_SURFACE_LDST;
    RH_CK(cuArray3DCreate(out, &d));
    CUDA_RESOURCE_DESC rd;
    memset(&rd, 0, sizeof(rd));
    rd.resType = CU_RESOURCE_TYPE_ARRAY;
    rd.res.array.hArray = *out;
    RH_CK(cuSurfObjectCreate(surf, &rd));
    return 0;
}

int copy_host_array(rh_grid* g, int c, const void* src, void* dst, bool to_array)
{
    CUDA_MEMCPY3D cp;
    memset(&cp, 0, sizeof(cp));
    size_t W = (size_t)g->sub[0] * g->P, H = (size_t)g->sub[1] * g->P, D = (size_t)g->sub[2] * g->P;
    if (to_array) {
        cp.srcMemoryType = CU_MEMORYTYPE_HOST;
        cp.srcHost = src;
        cp.srcPitch = W * g->ch[c].elem;
        cp.srcHeight = H;
        cp.dstMemoryType = CU_MEMORYTYPE_ARRAY;
        cp.dstArray = g->ch[c].arr;
    } else {
        cp.srcMemoryType = CU_MEMORYTYPE_ARRAY;
        cp.srcArray = g->ch[c].arr;
        cp.dstMemoryType = CU_MEMORYTYPE_HOST;
        cp.dstHost = dst;
        cp.dstPitch = W * g->ch[c].elem;
        cp.dstHeight = H;
    }
    cp.WidthInBytes = W * g->ch[c].elem;
    cp.Height = H;
    cp.Depth = D;
    RH_CK(cuMemcpy3D(&cp));
    return 0;
}

// voxel slices [z0, z1) of channel c's array set to zero on the device (a copy from a
// zero-filled linear buffer; the array has sub[0] x sub[1] bricks per slice)
int zero_array_slices(rh_grid* g, int c, CUarray arr, size_t z0, size_t z1)
{
    if (z1 <= z0) return 0;
    const size_t W = (size_t)g->sub[0] * g->P, H = (size_t)g->sub[1] * g->P;
    const size_t bytes = W * H * (z1 - z0) * g->ch[c].elem;
    if (dens(g->zero, bytes)) return -1;
    RH_CK(cuMemsetD8(g->zero.p, 0, bytes));
    CUDA_MEMCPY3D cp;
    memset(&cp, 0, sizeof(cp));
    cp.srcMemoryType = CU_MEMORYTYPE_DEVICE;
    cp.srcDevice = g->zero.p;
    cp.srcPitch = W * g->ch[c].elem;
    cp.srcHeight = H;
    cp.dstMemoryType = CU_MEMORYTYPE_ARRAY;
    cp.dstArray = arr;
    cp.dstZ = z0;
    cp.WidthInBytes = W * g->ch[c].elem;
    cp.Height = H;
    cp.Depth = z1 - z0;
    RH_CK(cuMemcpy3D(&cp));
    return 0;
}

// AtlasResize (AL.cpp:622-650): a new array; the old content is kept by a
// device array-to-array copy, as AllocateTextureGPU's "preserve" does
// (AL.cpp:428-448); the new slices are zero
int resize_atlas(rh_grid* g, int nz)
{
    int old[3] = {g->sub[0], g->sub[1], g->sub[2]};
    for (int c = 0; c < 32; c++) {
        if (!g->ch[c].used) continue;
        CUarray na = nullptr;
        CUsurfObject ns = 0;
        if (make_array(g, c, old[0], old[1], nz, &na, &ns)) return -1;
        const size_t W = (size_t)old[0] * g->P, H = (size_t)old[1] * g->P;
        const size_t keep_z = (size_t)std::min(old[2], nz) * g->P;
        if (keep_z) {
            CUDA_MEMCPY3D cp;
            memset(&cp, 0, sizeof(cp));
            cp.srcMemoryType = CU_MEMORYTYPE_ARRAY;
            cp.srcArray = g->ch[c].arr;
            cp.dstMemoryType = CU_MEMORYTYPE_ARRAY;
            cp.dstArray = na;
            cp.WidthInBytes = W * g->ch[c].elem;
            cp.Height = H;
            cp.Depth = keep_z;
            RH_CK(cuMemcpy3D(&cp));
        }
        if (zero_array_slices(g, c, na, keep_z, (size_t)nz * g->P)) return -1;
        cuSurfObjectDestroy(g->ch[c].surf);
        cuArrayDestroy(g->ch[c].arr);
        g->ch[c].arr = na;
        g->ch[c].surf = ns;
    }
    g->sub[2] = nz;
    return 0;
}

}  // namespace

extern "C" {

const char* rh_error(void) { return t_err.c_str(); }

int rh_load(const char* module_ptx)
{
    if (g_mod.loaded) return 0;
    if (cudaFree(0) != cudaSuccess) {
        t_err = "no CUDA device";
        return -1;
    }
    RH_CK(cuInit(0));
    RH_CK(cuModuleLoad(&g_mod.m, module_ptx));
    struct {
        CUfunction* f;
        const char* name;
    } fs[] = {{&g_mod.splitpos, "gvdbSplitPos"},          {&g_mod.calcbrick, "gvdbCalcBrickId"},
              {&g_mod.link, "gvdbLinkBricks"},            {&g_mod.extra, "gvdbCalcExtraBrickId"},
              {&g_mod.increextra, "gvdbCalcIncreExtraBrickId"}, {&g_mod.delinkleaf, "gvdbDelinkLeafBricks"},
              {&g_mod.delink, "gvdbDelinkBricks"},        {&g_mod.insertpts, "gvdbInsertPoints"},
              {&g_mod.scatter, "gvdbScatterPointDensity"}, {&g_mod.setflag, "gvdbSetFlagSubcell"},
              {&g_mod.countsc, "gvdbCountSubcell"},       {&g_mod.insertsc, "gvdbInsertSubcell"},
              {&g_mod.scpos, "gvdbCalcSubcellPos"},       {&g_mod.gatherd, "gvdbGatherDensity"},
              {&g_mod.gatherl, "gvdbGatherLevelSet"},     {&g_mod.apronf, "gvdbUpdateApronF"},
              {&g_mod.apronf4, "gvdbUpdateApronF4"},      {&g_mod.insertsc16, "gvdbInsertSubcell_fp16"},
              {&g_mod.gatherl16, "gvdbGatherLevelSet_fp16"}, {&g_mod.convxform, "gvdbConvAndTransform"}};
    for (auto& e : fs) RH_CK(cuModuleGetFunction(e.f, g_mod.m, e.name));
    // the copy-data module beside it (ClearChannel's fill kernel), when it was built
    std::string cp = module_ptx;
    const size_t at = cp.rfind("cuda_gvdb_module.ptx");
    if (at != std::string::npos) {
        cp.replace(at, strlen("cuda_gvdb_module.ptx"), "cuda_gvdb_copydata.ptx");
        if (cuModuleLoad(&g_mod.mcopy, cp.c_str()) == CUDA_SUCCESS)
            RH_CK(cuModuleGetFunction(&g_mod.filltex, g_mod.mcopy, "kernelFillTex"));
    }
    g_mod.loaded = true;
    return 0;
}

rh_grid* rh_create(int levels, const int* logdim, int apron, int cx, int cy, int cz)
{
    if (!g_mod.loaded || levels < 2 || levels > 10) return nullptr;
    rh_grid* g = new rh_grid();
    g->levels = levels;
    int r = 1;
    for (int l = 0; l < levels; l++) {
        g->logdim[l] = logdim[l];
        g->res[l] = 1 << logdim[l];
        r = l == 0 ? g->res[0] : r * g->res[l];
        g->range[l] = r;
    }
    g->apron = apron;
    g->brick = g->res[0];
    g->P = g->brick + 2 * apron;
    g->defsub[0] = cx;
    g->defsub[1] = cy;
    g->defsub[2] = cz;
    memset(&g->info, 0, sizeof(g->info));
    return g;
}

void rh_destroy(rh_grid* g)
{
    if (!g) return;
    cuCtxSynchronize();
    for (int c = 0; c < 32; c++)
        if (g->ch[c].used) {
            cuSurfObjectDestroy(g->ch[c].surf);
            cuArrayDestroy(g->ch[c].arr);
        }
    DBuf* bufs[] = {&g->damap, &g->dinfo, &g->dpos, &g->range_res, &g->keys, &g->cnt, &g->markers, &g->splitx,
                    &g->splity, &g->splitz, &g->pnode, &g->poff, &g->gcnt, &g->scflag, &g->scmap, &g->sccnt,
                    &g->scoff, &g->scpts, &g->scpos, &g->scnid, &g->zero};
    for (DBuf* b : bufs)
        if (b->p) cuMemFree(b->p);
    for (int l = 0; l < 10; l++) {
        if (g->dnodes[l].p) cuMemFree(g->dnodes[l].p);
        if (g->dclist[l].p) cuMemFree(g->dclist[l].p);
    }
    delete g;
}

int rh_add_channel(rh_grid* g, int c, int type)
{
    if (!g || c < 0 || c >= 32 || (type != 3 && type != 4)) return -1;
    if (!g->have_atlas) {
        g->sub[0] = g->defsub[0];
        g->sub[1] = g->defsub[1];
        g->sub[2] = g->defsub[2];
        g->have_atlas = true;
    }
    g->ch[c].used = true;
    g->ch[c].type = type;
    g->ch[c].elem = type == 3 ? 4 : 16;
    if (make_array(g, c, g->sub[0], g->sub[1], g->sub[2], &g->ch[c].arr, &g->ch[c].surf)) return -1;
    std::vector<unsigned char> z((size_t)g->sub[0] * g->P * g->sub[1] * g->P * g->sub[2] * g->P * g->ch[c].elem, 0);
    return copy_host_array(g, c, z.data(), nullptr, true);
}

int rh_set_points(rh_grid* g, int n, const float* pos)
{
    if (!g || n <= 0) return -1;
    g->n = n;
    if (dens(g->dpos, (size_t)n * 12)) return -1;
    RH_CK(cuMemcpyHtoD(g->dpos.p, pos, (size_t)n * 12));
    return 0;
}

// RebuildTopology / AccumulateTopology: mode 0 AUTO, 1 FULL, 2 ACCUMULATE
int rh_rebuild(rh_grid* g, float radius, const float* orig, int mode, int min_depth)
{
    float3 o = make_float3(orig[0], orig[1], orig[2]);
    // GetBoundingBox
    int n = g->n, off = 0, stride = 12;
    if (dens(g->splitx, (size_t)n * 4) || dens(g->splity, (size_t)n * 4) || dens(g->splitz, (size_t)n * 4))
        return -1;
    CUdeviceptr pos = g->dpos.p, xo = g->splitx.p, yo = g->splity.p, zo = g->splitz.p;
    void* args[] = {&n, &o, &pos, &off, &stride, &xo, &yo, &zo};
    if (launch(g_mod.splitpos, n / 256 + 1, 1, 1, 256, 1, 1, args)) return -1;
    RH_CK(cuCtxSynchronize());
    CUdeviceptr src[3] = {xo, yo, zo};
    float mn[3], mx[3];
    for (int a = 0; a < 3; a++) {
        thrust::device_ptr<float> d = thrust::device_pointer_cast((float*)src[a]);
        mn[a] = *thrust::min_element(d, d + n);
        mx[a] = *thrust::max_element(d, d + n);
    }
    int pmin[3], pmax[3];
    float plo[3], phi[3];
    for (int a = 0; a < 3; a++) {
        float lo = mn[a] - 1, hi = mx[a] + 2;
        lo = 0 > lo ? 0 : lo;
        hi = 0 > hi ? 0 : hi;
        plo[a] = lo;
        phi[a] = hi;
        pmin[a] = (int)lo;
        pmax[a] = (int)hi;
    }
    g->pos_min = make_float3(plo[0], plo[1], plo[2]);
    g->pos_range = make_float3(phi[0] - plo[0], phi[1] - plo[1], phi[2] - plo[2]);
    int depth = -1, rootpos[3] = {0, 0, 0};
    for (int lev = 0; lev < g->levels; lev++) {
        int r = g->range[lev];
        if (pmin[0] / r == pmax[0] / r && pmin[1] / r == pmax[1] / r && pmin[2] / r == pmax[2] / r) {
            depth = lev;
            for (int a = 0; a < 3; a++) rootpos[a] = pmin[a] / r * r;
            break;
        }
    }
    if (mode == 2 && !g->rebuild) {
        int d = depth < min_depth ? min_depth : depth;
        if (d <= 0 || d >= g->levels) {
            t_err = "depth";
            return 2;
        }
        return activate_incremental(g, radius, o, d, true);
    }
    if (depth <= 0 || depth >= g->levels) {
        t_err = "depth";
        return 2;
    }
    if (mode == 1) g->rebuild = true;
    if (g->rebuild) {
        clear_tree(g);
    } else if (depth != g->curr_depth) {
        clear_tree(g);
        g->curr_depth = depth;
    }
    if (g->rebuild) {
        if (activate_bricks(g, o, depth, rootpos)) return -1;
        if (radius >= 1 && activate_extra(g, radius, o, depth)) return -1;
        g->rebuild = false;
        g->last_mode = 1;
        return 0;
    }
    return activate_incremental(g, radius, o, depth, false);
}

int rh_update_atlas(rh_grid* g)
{
    if (!g->have_atlas || g->sub[0] * g->sub[1] <= 0) {
        t_err = "UpdateAtlas: the grid has no channel (no atlas to assign)";
        return -1;
    }
    int used = g->used0;
    int amax = g->sub[0] * g->sub[1] * g->sub[2];
    if (used > amax) {
        if (resize_atlas(g, (int)ceil(used / (float)(g->sub[0] * g->sub[1])))) return -1;
    }
    int last = 0;
    for (auto& nd : g->nodes[0]) {
        if (!nd.flags) continue;
        int id = last++;
        int a2 = g->sub[0] * g->sub[1];
        int z = id / a2, rem = id - z * a2, y = rem / g->sub[0], x = rem - y * g->sub[0];
        nd.value[0] = x * g->P + g->apron;
        nd.value[1] = y * g->P + g->apron;
        nd.value[2] = z * g->P + g->apron;
    }
    int slots = g->sub[0] * g->sub[1] * g->sub[2];
    g->amap.assign(slots, RAtlasNode{{(int)UNDEFL, (int)UNDEFL, (int)UNDEFL}, (int)UNDEFL});
    for (size_t i = 0; i < g->nodes[0].size(); i++) {
        RNode& nd = g->nodes[0][i];
        if (!nd.flags) continue;
        int bx = nd.value[0] / g->P, by = nd.value[1] / g->P, bz = nd.value[2] / g->P;
        RAtlasNode& an = g->amap[(bz * g->sub[1] + by) * g->sub[0] + bx];
        an.pos[0] = nd.pos[0];
        an.pos[1] = nd.pos[1];
        an.pos[2] = nd.pos[2];
        an.leaf = (int)i;
    }
    if (dens(g->damap, (size_t)slots * sizeof(RAtlasNode))) return -1;
    RH_CK(cuMemcpyHtoD(g->damap.p, g->amap.data(), (size_t)slots * sizeof(RAtlasNode)));
    return commit_pools(g);
}

// ClearChannel (VG.cpp:1596-1603) -> Allocator::AtlasFill (AL.cpp:813-822):
// kernelFillTex (cuda_gvdb_copydata.cu:21-27) over the atlas in 8^3 blocks.  That
// kernel writes one 4-byte zero per voxel, which clears float channels; wider
// voxels are cleared by a device copy of zeros instead (the reference's fill
// leaves their other components as they were).
int rh_clear_channel(rh_grid* g, int c)
{
    if (g_mod.filltex && g->ch[c].elem == 4) {
        int3 res = make_int3(g->sub[0] * g->P, g->sub[1] * g->P, g->sub[2] * g->P);
        int dsize = g->ch[c].elem;
        CUsurfObject so = g->ch[c].surf;
        void* args[] = {&res, &dsize, &so};
        if (launch(g_mod.filltex, res.x / 8 + 1, res.y / 8 + 1, res.z / 8 + 1, 8, 8, 8, args)) return -1;
        RH_CK(cuCtxSynchronize());
        return 0;
    }
    return zero_array_slices(g, c, g->ch[c].arr, 0, (size_t)g->sub[2] * g->P);
}

int rh_write_channel_dense(rh_grid* g, int c, const void* src) { return copy_host_array(g, c, src, nullptr, true); }
int rh_read_channel_dense(rh_grid* g, int c, void* dst)
{
    RH_CK(cuCtxSynchronize());
    return copy_host_array(g, c, nullptr, dst, false);
}
int64_t rh_channel_bytes(rh_grid* g, int c)
{
    return (int64_t)g->sub[0] * g->P * g->sub[1] * g->P * g->sub[2] * g->P * g->ch[c].elem;
}

// InsertPoints + ScatterDensity (kernel argument list of cuda_gvdb_particles.cuh:525)
int rh_scatter(rh_grid* g, float radius, const float* trans, int expand)
{
    float3 t = make_float3(trans[0], trans[1], trans[2]);
    if (prepare(g, true)) return -1;
    int n = g->n, off = 0, stride = 12;
    int bricks = (int)g->nodes[0].size();
    if (dens(g->pnode, (size_t)n * 4) || dens(g->poff, (size_t)n * 4) || dens(g->gcnt, (size_t)bricks * 4 + 4)) return -1;
    RH_CK(cuMemsetD8(g->gcnt.p, 0, (size_t)bricks * 4 + 4));
    CUdeviceptr info = g->dinfo.p, pos = g->dpos.p, pn = g->pnode.p, po = g->poff.p, gc = g->gcnt.p;
    void* a1[] = {&info, &n, &pos, &off, &stride, &pn, &po, &gc, &t};
    if (launch(g_mod.insertpts, n / 512 + 1, 1, 1, 512, 1, 1, a1)) return -1;
    float amp = 1.0f;
    CUdeviceptr clr = 0, cbuf = 0;
    int coff = 0, cstride = 0;
    bool ex = expand != 0;
    void* a2[] = {&info, &n, &radius, &amp, &pos, &off, &stride, &clr, &coff, &cstride, &pn, &t, &ex, &cbuf};
    if (launch(g_mod.scatter, n / 256 + 1, 1, 1, 256, 1, 1, a2)) return -1;
    RH_CK(cuCtxSynchronize());
    return 0;
}

// InsertPointsSubcell + GatherDensity / GatherLevelSet
int rh_gather(rh_grid* g, int levelset, int sc, float radius, float rins, const float* trans, int chan, int accum)
{
    float3 t = make_float3(trans[0], trans[1], trans[2]);
    if (prepare(g, true)) return -1;
    int numBrick = g->used0;
    int scdim = g->res[0] / sc;
    int spb = scdim * scdim * scdim;
    int numSC = spb * numBrick;
    int3 range = make_int3(g->range[0] / scdim, g->range[0] / scdim, g->range[0] / scdim);
    int M = (int)g->nodes[0].size();
    if (dens(g->scflag, (size_t)M * 4 + 4) || dens(g->scmap, (size_t)M * 4 + 4)) return -1;
    CUdeviceptr info = g->dinfo.p, fl = g->scflag.p;
    void* a1[] = {&info, &M, &fl};
    if (launch(g_mod.setflag, M / 512 + 1, 1, 1, 512, 1, 1, a1)) return -1;
    RH_CK(cuCtxSynchronize());
    std::vector<int> flag(M), map(M);
    RH_CK(cuMemcpyDtoH(flag.data(), g->scflag.p, (size_t)M * 4));
    int acc = 0;
    for (int i = 0; i < M; i++) {
        map[i] = acc;
        acc += flag[i];
    }
    RH_CK(cuMemcpyHtoD(g->scmap.p, map.data(), (size_t)M * 4));
    if (dens(g->sccnt, (size_t)numSC * 4 + 4) || dens(g->scoff, (size_t)numSC * 4 + 4)) return -1;
    RH_CK(cuMemsetD8(g->sccnt.p, 0, (size_t)numSC * 4 + 4));
    int n = g->n, off = 0, stride = 12;
    CUdeviceptr pos = g->dpos.p, cnt = g->sccnt.p, mp = g->scmap.p;
    void* a2[] = {&info, &sc, &spb, &n, &pos, &off, &stride, &cnt, &range, &t, &scdim, &rins, &numSC, &mp};
    if (launch(g_mod.countsc, n / 512 + 1, 1, 1, 512, 1, 1, a2)) return -1;
    RH_CK(cuCtxSynchronize());
    std::vector<int> c(numSC), o(numSC);
    RH_CK(cuMemcpyDtoH(c.data(), g->sccnt.p, (size_t)numSC * 4));
    int len = 0;
    for (int i = 0; i < numSC; i++) {
        o[i] = len;
        len += c[i];
    }
    g->sc_len = len;
    g->num_sc = numSC;
    if (len == 0) return 0;
    RH_CK(cuMemcpyHtoD(g->scoff.p, o.data(), (size_t)numSC * 4));
    RH_CK(cuMemsetD8(g->sccnt.p, 0, (size_t)numSC * 4));
    if (dens(g->scpts, (size_t)len * 12) || dens(g->scpos, (size_t)numSC * 12 + 12) || dens(g->scnid, (size_t)numSC * 4 + 4))
        return -1;
    CUdeviceptr offp = g->scoff.p, pts = g->scpts.p, zero = 0;
    int zi = 0;
    void* a3[] = {&info, &sc, &spb, &n, &cnt, &offp, &mp, &range, &t, &scdim, &rins, &pos, &off, &stride, &pts,
                  &zero, &zi, &zi, &zero, &zero, &zi, &zi, &zero};
    if (launch(g_mod.insertsc, n / 512 + 1, 1, 1, 512, 1, 1, a3)) return -1;
    CUdeviceptr nid = g->scnid.p, scp = g->scpos.p;
    void* a4[] = {&info, &nid, &scp, &M, &scdim, &spb, &sc, &mp};
    if (launch(g_mod.scpos, M / 512 + 1, 1, 1, 512, 1, 1, a4)) return -1;
    int chanc = 0;
    bool acc2 = accum != 0;
    void* a5[] = {&info, &n, &numSC, &radius, &nid, &cnt, &offp, &scp, &pts, &zero, &zero, &chan, &chanc, &acc2};
    if (launch(levelset ? g_mod.gatherl : g_mod.gatherd, numSC, 1, 1, sc, sc, sc, a5)) return -1;
    RH_CK(cuCtxSynchronize());
    return 0;
}

// InsertPointsSubcell_FP16 + GatherLevelSet_FP16 (VG.cpp:5094-5190, 5375-5401): the
// FP32 orchestration above with the reference's FP16 kernels (ushort3 entries, no
// velocities or colours)
int rh_gather_fp16(rh_grid* g, int sc, float radius, float rins, const float* trans, int chan)
{
    float3 t = make_float3(trans[0], trans[1], trans[2]);
    if (prepare(g, true)) return -1;
    int numBrick = g->used0;
    int scdim = g->res[0] / sc;
    int spb = scdim * scdim * scdim;
    int numSC = spb * numBrick;
    int3 range = make_int3(g->range[0] / scdim, g->range[0] / scdim, g->range[0] / scdim);
    int M = (int)g->nodes[0].size();
    if (dens(g->scflag, (size_t)M * 4 + 4) || dens(g->scmap, (size_t)M * 4 + 4)) return -1;
    CUdeviceptr info = g->dinfo.p, fl = g->scflag.p;
    void* a1[] = {&info, &M, &fl};
    if (launch(g_mod.setflag, M / 512 + 1, 1, 1, 512, 1, 1, a1)) return -1;
    RH_CK(cuCtxSynchronize());
    std::vector<int> flag(M), map(M);
    RH_CK(cuMemcpyDtoH(flag.data(), g->scflag.p, (size_t)M * 4));
    int acc = 0;
    for (int i = 0; i < M; i++) {
        map[i] = acc;
        acc += flag[i];
    }
    RH_CK(cuMemcpyHtoD(g->scmap.p, map.data(), (size_t)M * 4));
    if (dens(g->sccnt, (size_t)numSC * 4 + 4) || dens(g->scoff, (size_t)numSC * 4 + 4)) return -1;
    RH_CK(cuMemsetD8(g->sccnt.p, 0, (size_t)numSC * 4 + 4));
    int n = g->n, off = 0, stride = 12;
    CUdeviceptr pos = g->dpos.p, cnt = g->sccnt.p, mp = g->scmap.p;
    void* a2[] = {&info, &sc, &spb, &n, &pos, &off, &stride, &cnt, &range, &t, &scdim, &rins, &numSC, &mp};
    if (launch(g_mod.countsc, n / 512 + 1, 1, 1, 512, 1, 1, a2)) return -1;
    RH_CK(cuCtxSynchronize());
    std::vector<int> c(numSC), o(numSC);
    RH_CK(cuMemcpyDtoH(c.data(), g->sccnt.p, (size_t)numSC * 4));
    int len = 0;
    for (int i = 0; i < numSC; i++) {
        o[i] = len;
        len += c[i];
    }
    g->sc_len = len;
    g->num_sc = numSC;
    RH_CK(cuMemcpyHtoD(g->scoff.p, o.data(), (size_t)numSC * 4));
    RH_CK(cuMemsetD8(g->sccnt.p, 0, (size_t)numSC * 4));
    if (dens(g->scpts, (size_t)len * 6 + 8) || dens(g->scpos, (size_t)numSC * 12 + 12) ||
        dens(g->scnid, (size_t)numSC * 4 + 4))
        return -1;
    CUdeviceptr offp = g->scoff.p, pts = g->scpts.p, zero = 0;
    int zi = 0;
    float3 vmin = make_float3(0, 0, 0), vrange = make_float3(1, 1, 1);
    void* a3[] = {&info, &sc, &spb, &n, &cnt, &offp, &mp, &g->pos_min, &g->pos_range, &vmin, &vrange, &range, &t,
                  &scdim, &rins, &pos, &off, &stride, &pts, &zero, &zi, &zi, &zero, &zero, &zi, &zi, &zero};
    if (len > 0 && launch(g_mod.insertsc16, n / 512 + 1, 1, 1, 512, 1, 1, a3)) return -1;
    CUdeviceptr nid = g->scnid.p, scp = g->scpos.p;
    void* a4[] = {&info, &nid, &scp, &M, &scdim, &spb, &sc, &mp};
    if (launch(g_mod.scpos, M / 512 + 1, 1, 1, 512, 1, 1, a4)) return -1;
    int chanc = -1;
    void* a5[] = {&info, &n, &numSC, &radius, &g->pos_min, &g->pos_range, &vmin, &vrange, &nid, &cnt, &offp, &scp,
                  &pts, &zero, &zero, &chan, &chanc};
    if (launch(g_mod.gatherl16, numSC, 1, 1, sc, sc, sc, a5)) return -1;
    RH_CK(cuCtxSynchronize());
    return 0;
}

int rh_pos_bounds(rh_grid* g, float* out)
{
    out[0] = g->pos_min.x;
    out[1] = g->pos_min.y;
    out[2] = g->pos_min.z;
    out[3] = g->pos_range.x;
    out[4] = g->pos_range.y;
    out[5] = g->pos_range.z;
    return 0;
}

// ConvertAndTransform (VG.cpp:5668-5682) on host arrays through the reference's kernel
int rh_convert(int n, const void* src, int srcbits, float* dst, const float* wmin, const float* wdelta,
               const float* trans, const float* scal)
{
    CUdeviceptr ds = 0, dd = 0;
    const size_t sb = (size_t)n * (srcbits == 2 ? 6 : 12);
    RH_CK(cuMemAlloc(&ds, sb + 16));
    RH_CK(cuMemAlloc(&dd, (size_t)n * 12 + 16));
    RH_CK(cuMemcpyHtoD(ds, src, sb));
    char sbits = (char)srcbits, dbits = 4;
    float3 mn = make_float3(wmin[0], wmin[1], wmin[2]), dl = make_float3(wdelta[0], wdelta[1], wdelta[2]);
    float3 tr = make_float3(trans[0], trans[1], trans[2]), sc = make_float3(scal[0], scal[1], scal[2]);
    void* args[] = {&n, &ds, &sbits, &dd, &dbits, &mn, &dl, &tr, &sc};
    int rc = launch(g_mod.convxform, n / 512 + 1, 1, 1, 512, 1, 1, args);
    if (rc == 0) {
        RH_CK(cuCtxSynchronize());
        RH_CK(cuMemcpyDtoH(dst, dd, (size_t)n * 12));
    }
    cuMemFree(ds);
    cuMemFree(dd);
    return rc;
}

int rh_sc_len(rh_grid* g) { return g->sc_len; }

int rh_update_apron(rh_grid* g, int c, float boundval)
{
    if (g->apron == 0) return 0;
    if (prepare(g, true)) return -1;
    int bricks = (int)g->nodes[0].size();
    if (bricks == 0) return 0;
    unsigned char chan = (unsigned char)c;
    int brickres = g->P, brickwid = g->brick;
    CUdeviceptr info = g->dinfo.p;
    void* args[] = {&info, &chan, &bricks, &brickres, &brickwid, &boundval};
    unsigned gy = (unsigned)((brickres + 7) / 8);
    if (launch(g->ch[c].type == 3 ? g_mod.apronf : g_mod.apronf4, bricks, gy, gy, 6, 8, 8, args)) return -1;
    RH_CK(cuCtxSynchronize());
    return 0;
}

int rh_root_level(rh_grid* g) { return g->root_level; }
int rh_num_nodes(rh_grid* g, int l) { return (int)g->nodes[l].size(); }
int rh_used_leaves(rh_grid* g) { return g->used0; }
int rh_last_mode(rh_grid* g) { return g->last_mode; }
int rh_atlas_subdim(rh_grid* g, int* out)
{
    out[0] = g->sub[0];
    out[1] = g->sub[1];
    out[2] = g->sub[2];
    return 0;
}
int rh_get_nodes(rh_grid* g, int l, void* out, int cap)
{
    if (cap < (int)g->nodes[l].size()) return -1;
    if (!g->nodes[l].empty()) memcpy(out, g->nodes[l].data(), g->nodes[l].size() * sizeof(RNode));
    return 0;
}
int rh_get_childlist(rh_grid* g, int l, uint64_t* out, int64_t cap)
{
    if (cap < (int64_t)g->clist[l].size()) return -1;
    if (!g->clist[l].empty()) memcpy(out, g->clist[l].data(), g->clist[l].size() * 8);
    return 0;
}

}  // extern "C"
