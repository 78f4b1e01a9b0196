// gvx_api.cu -- extern "C" entry points of libgvx (declared in include/gvx.h).
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <vector>

#include "gvx_grid.cuh"

static thread_local char t_err[1024] = "";

void gvx_set_error(const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_err, sizeof(t_err), fmt, ap);
    va_end(ap);
}

gvx_status gvx_cuda_fail(cudaError_t e, const char* what)
{
    gvx_set_error("CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), what);
    // the runtime keeps the last error until it is read: read it here, so that a failure that
    // leaves the context usable (an allocation) is not reported again by a later call's launch check
    (void)cudaGetLastError();
    return GVX_ERR_DEVICE;
}

static std::atomic<uint64_t> g_alloc_epoch{0};
static thread_local bool t_no_alloc = false;

uint64_t gvx_alloc_epoch() { return g_alloc_epoch.load(); }

GvxNoAllocScope::GvxNoAllocScope() : prev(t_no_alloc) { t_no_alloc = true; }
GvxNoAllocScope::~GvxNoAllocScope() { t_no_alloc = prev; }

cudaError_t gvx_ensure(DevBuf& b, size_t bytes)
{
    if (bytes <= b.cap && b.p) return cudaSuccess;
    if (t_no_alloc) return cudaErrorNotPermitted;
    g_alloc_epoch++;
    if (b.p) {
        cudaError_t e = cudaFree(b.p);
        if (e != cudaSuccess) return e;
    }
    b.p = nullptr;
    b.cap = 0;
    const size_t want = bytes + bytes / 4 + 256;  // slack so that slowly growing sizes do not reallocate each call
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
        b.p = nullptr;
        return e;
    }
    b.cap = want;
    return cudaSuccess;
}

void gvx_free(DevBuf& b)
{
    if (b.p) {
        g_alloc_epoch++;
        cudaFree(b.p);
    }
    b.p = nullptr;
    b.cap = 0;
}

#define GVX_GUARD(g)                                \
    do {                                            \
        if (!(g)) {                                 \
            gvx_set_error("null grid handle");      \
            return GVX_ERR_INVALID_ARG;             \
        }                                           \
        cudaError_t _se = cudaSetDevice((g)->device); \
        if (_se != cudaSuccess) return gvx_cuda_fail(_se, "cudaSetDevice"); \
    } while (0)

static int type_bytes(int type, int* ncomp)
{
    switch (type) {
    case GVX_T_FLOAT: *ncomp = 1; return 4;
    case GVX_T_FLOAT3: *ncomp = 4; return 16;  // stored as 4 floats (AL.cpp:395)
    case GVX_T_FLOAT4: *ncomp = 4; return 16;
    case GVX_T_UCHAR: *ncomp = 1; return 1;
    case GVX_T_UCHAR4: *ncomp = 4; return 4;
    }
    return 0;
}

gvx_status gvx_grow_atlas(gvx_grid* g, int64_t need)
{
    const int64_t amax = (int64_t)g->sub[0] * g->sub[1] * g->sub[2];
    if (need <= amax) return GVX_OK;
    // AtlasResize (AL.cpp:622-650): Z grows to ceil(used / (sx*sy)); data kept, new bricks zero
    const int nz = (int)ceil((double)need / (double)((int64_t)g->sub[0] * g->sub[1]));
    const int64_t slots = (int64_t)g->sub[0] * g->sub[1] * nz;
    const int64_t P3 = (int64_t)g->P * g->P * g->P;
    for (int c = 0; c < GVX_MAXCH; c++) {
        GvxChannel& ch = g->ch[c];
        if (!ch.used) continue;
        const size_t old_bytes = (size_t)(ch.slots * P3 * ch.elem_bytes);
        const size_t new_bytes = (size_t)(slots * P3 * ch.elem_bytes);
        if (ch.data.p && new_bytes <= ch.data.cap) {
            // grows inside the allocation: only the new bricks are cleared
            GVX_CK(cudaMemsetAsync((char*)ch.data.p + old_bytes, 0, new_bytes - old_bytes, g->stream));
        } else {
            // a growing atlas (accumulating topologies) at least doubles its capacity, so that
            // it is reallocated and copied a logarithmic number of times
            DevBuf nb;
            GVX_CK(gvx_ensure(nb, ch.data.p ? std::max(new_bytes, 2 * ch.data.cap) : new_bytes));
            GVX_CK(cudaMemsetAsync((char*)nb.p + old_bytes, 0, new_bytes - old_bytes, g->stream));
            if (ch.data.p && ch.slots)
                GVX_CK(cudaMemcpyAsync(nb.p, ch.data.p, old_bytes, cudaMemcpyDeviceToDevice, g->stream));
            GVX_CK(cudaStreamSynchronize(g->stream));
            gvx_free(ch.data);
            ch.data = nb;
        }
        ch.slots = slots;  // the bricks keep their slots and values; UpdateAtlas settles the aprons' state
    }
    g->sub[2] = nz;
    return GVX_OK;
}

__global__ void k_fill(unsigned char* data, int64_t n, int eb, uint4 pattern)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned char* src = (const unsigned char*)&pattern;
        for (int k = 0; k < eb; k++) data[i * eb + k] = src[k];
    }
}

__global__ void k_pnode(const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ svals, uint32_t n,
                        int kshift, uint32_t invalid_key, LeafLookup L, int* pnode)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = skeys[i] >> kshift;
    int leaf = -1;
    if (k < invalid_key) {
        int c[3];
        ks_unpack(L.ks, k, 0, c);
        leaf = ll_find(L, c[0], c[1], c[2]);
    }
    pnode[svals[i]] = leaf;
}

// the grid's stream waits for the uploads of the last commit still in flight on the
// side stream: all of them (the attributes are copied after the positions) ...
gvx_status gvx_wait_attributes(gvx_grid* g)
{
    if (g->attr_pending) {
        GVX_CK(cudaStreamWaitEvent(g->stream, g->ev_attr_ready, 0));
        g->attr_pending = false;
        g->pos_pending = false;
    }
    return GVX_OK;
}

// ... or the positions alone (what the topology build and the subcell lists read)
gvx_status gvx_wait_positions(gvx_grid* g)
{
    if (g->pos_pending) {
        GVX_CK(cudaStreamWaitEvent(g->stream, g->ev_pos_ready, 0));
        g->pos_pending = false;
    }
    return GVX_OK;
}

extern "C" {

const char* gvx_last_error(void) { return t_err; }
const char* gvx_version(void) { return "gvx 0.1 (sm_103a)"; }

gvx_status gvx_create(int device, gvx_grid** out)
{
    if (!out) {
        gvx_set_error("gvx_create: null output");
        return GVX_ERR_INVALID_ARG;
    }
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        gvx_set_error("gvx_create: no CUDA device (%s)", e == cudaSuccess ? "count 0" : cudaGetErrorString(e));
        return GVX_ERR_DEVICE;
    }
    if (device < 0 || device >= ndev) {
        gvx_set_error("gvx_create: device %d of %d", device, ndev);
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(cudaSetDevice(device));
    gvx_grid* g = new gvx_grid();
    g->device = device;
    e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete g;
        return gvx_cuda_fail(e, "cudaStreamCreate");
    }
    g->own_stream = true;
    // the device error word starts clear; from then on it is cleared when it is read
    e = gvx_ensure(g->d_err, 64);
    if (e == cudaSuccess) e = cudaMemset(g->d_err.p, 0, 64);
    if (e != cudaSuccess) {
        cudaStreamDestroy(g->stream);
        gvx_free(g->d_err);
        delete g;
        return gvx_cuda_fail(e, "gvx_create: error word");
    }
    *out = g;
    return GVX_OK;
}

gvx_status gvx_destroy(gvx_grid* g)
{
    if (!g) return GVX_OK;
    cudaSetDevice(g->device);
    if (g->stream) cudaStreamSynchronize(g->stream);
    if (g->aux_stream) cudaStreamSynchronize(g->aux_stream);
    DevBuf* bufs[] = {&g->bm_a, &g->bm_a_prefix, &g->bm_b, &g->bm_b_prefix, &g->remap, &g->leaf_key, &g->leaf_range,
                      &g->leaf_oct,
                      &g->leaf_slot, &g->slot_leaf, &g->nbr, &g->amap, &g->own_pos[0], &g->own_vel[0],
                      &g->own_w[0], &g->own_r[0], &g->own_pos[1], &g->own_vel[1], &g->own_w[1], &g->own_r[1],
                      &g->keys[0], &g->keys[1], &g->vals[0], &g->vals[1], &g->spos, &g->svel,
                      &g->sort.hist, &g->sort.base, &g->sort.lookback, &g->sort.counter, &g->d0_bits,
                      &g->d0_prefix, &g->x0_bits, &g->x0_prefix, &g->masks, &g->upper, &g->lists, &g->tmp_scan,
                      &g->d_counts, &g->d_err, &g->d_bbox, &g->d_rmax, &g->d_next, &g->touched, &g->host_stage,
                      &g->api_keys[0], &g->api_keys[1], &g->api_vals[0], &g->api_vals[1], &g->lk_bits, &g->lk_prefix,
                      &g->inc0, &g->inc_remap, &g->sc_cnt, &g->sc_off, &g->sc_keys[0], &g->sc_keys[1],
                      &g->sc_vals[0], &g->sc_vals[1], &g->sc_pts, &g->sc_beg, &g->sc_end, &g->atlas_tmp,
                      &g->sc_q, &g->sc_qclr, &g->own_stage, &g->apron_tab, &g->apron_mark};
    for (DevBuf* b : bufs) gvx_free(*b);
    for (int l = 0; l < GVX_MAXLEV; l++) {
        gvx_free(g->nodes[l]);
        gvx_free(g->clist[l]);
    }
    for (int c = 0; c < GVX_MAXCH; c++) gvx_free(g->ch[c].data);
    gvx_host_tree_free(g);
    gvx_topo_staged_free(g);
    gvx_topo_plan_free(g);
    if (g->own_stream && g->stream) cudaStreamDestroy(g->stream);
    if (g->aux_stream) cudaStreamDestroy(g->aux_stream);
    if (g->h_pin) cudaFreeHost(g->h_pin);
    for (int k = 0; k < 2; k++)
        if (g->ev_set_free[k]) cudaEventDestroy(g->ev_set_free[k]);
    if (g->ev_pos_ready) cudaEventDestroy(g->ev_pos_ready);
    if (g->ev_attr_ready) cudaEventDestroy(g->ev_attr_ready);
    delete g;
    return GVX_OK;
}

gvx_status gvx_set_stream(gvx_grid* g, void* stream)
{
    GVX_GUARD(g);
    GVX_CK(cudaStreamSynchronize(g->stream));
    if (g->own_stream) cudaStreamDestroy(g->stream);
    g->stream = (cudaStream_t)stream;
    g->own_stream = false;
    return GVX_OK;
}

gvx_status gvx_sync(gvx_grid* g)
{
    GVX_GUARD(g);
    if (g->aux_stream) GVX_CK(cudaStreamSynchronize(g->aux_stream));
    GVX_CK(cudaStreamSynchronize(g->stream));
    return gvx_check_device_error(g, "sync");
}

gvx_status gvx_configure(gvx_grid* g, int levels, const int* logdim, const int* init_counts)
{
    GVX_GUARD(g);
    (void)init_counts;  // pools grow to the exact counts of each rebuild
    if (levels < 2 || levels > GVX_MAXLEV || !logdim) {
        gvx_set_error("Configure: levels must be 2..%d", GVX_MAXLEV);
        return GVX_ERR_INVALID_ARG;
    }
    int64_t range = 1;
    for (int l = 0; l < levels; l++) {
        const int r = logdim[l] == 0 ? 1 : logdim[l];  // VG.cpp:2397
        if (r < 1 || r > 6) {
            gvx_set_error("Configure: log2 resolution %d at level %d (1..6 supported)", logdim[l], l);
            return GVX_ERR_INVALID_ARG;
        }
        g->logdim[l] = r;
        g->res[l] = 1 << r;
        range = (l == 0) ? g->res[0] : range * g->res[l];
        if (range > (int64_t(1) << 30)) {
            gvx_set_error("Configure: index-space extent exceeds 2^30 voxels");
            return GVX_ERR_INVALID_ARG;
        }
        g->range[l] = (int)range;
        g->tshift[l] = l == 0 ? 0 : g->tshift[l - 1] + r;
    }
    g->levels = levels;
    g->brick = g->res[0];
    g->P = g->brick + 2 * g->apron;
    g->configured = true;
    g->topo_gen++;
    g->root_level = -1;
    gvx_topo_plan_free(g);  // a plan's depth and key space are in the old levels' terms
    g->vox_res_max_reset = true;  // VG.cpp:2428
    g->bounds_pending = false;
    for (int a = 0; a < 3; a++) g->obj_min[a] = g->obj_max[a] = g->vox_res_max[a] = 0.f;
    g->rebuild_topo = true;
    g->curr_depth = -1;
    g->lookup_valid = g->group_valid = g->atlas_valid = g->nbr_valid = false;
    for (int l = 0; l < GVX_MAXLEV; l++) g->count[l] = 0;
    g->used_leaves = 0;
    return GVX_OK;
}

gvx_status gvx_set_channel_default(gvx_grid* g, int cx, int cy, int cz)
{
    GVX_GUARD(g);
    if (cx <= 0 || cy <= 0 || cz <= 0) {
        gvx_set_error("SetChannelDefault: counts must be positive");
        return GVX_ERR_INVALID_ARG;
    }
    g->defsub[0] = cx;
    g->defsub[1] = cy;
    g->defsub[2] = cz;
    return GVX_OK;
}

gvx_status gvx_add_channel(gvx_grid* g, int chan, int type, int apron)
{
    GVX_GUARD(g);
    if (!g->configured) {
        gvx_set_error("AddChannel: Configure was not called");
        return GVX_ERR_NOT_CONFIGURED;
    }
    int ncomp = 0;
    const int eb = type_bytes(type, &ncomp);
    if (chan < 0 || chan >= GVX_MAXCH || eb == 0) {
        gvx_set_error("AddChannel: channel %d type %d", chan, type);
        return GVX_ERR_INVALID_ARG;
    }
    if (apron != 0 && apron != 1) {
        gvx_set_error("AddChannel: apron %d (the apron update supports 0 or 1, OP.cuh:102)", apron);
        return GVX_ERR_UNSUPPORTED;
    }
    bool any = false;
    for (int c = 0; c < GVX_MAXCH; c++) any |= g->ch[c].used;
    if (any && apron != g->apron) {
        gvx_set_error("AddChannel: all channels share one apron (%d)", g->apron);
        return GVX_ERR_INVALID_ARG;
    }
    g->apron = apron;
    g->P = g->brick + 2 * apron;
    if (!g->have_atlas) {
        g->sub[0] = g->defsub[0];
        g->sub[1] = g->defsub[1];
        g->sub[2] = g->defsub[2];
        g->have_atlas = true;
    }
    GvxChannel& ch = g->ch[chan];
    gvx_free(ch.data);
    ch.used = true;
    ch.type = type;
    ch.ncomp = ncomp;
    ch.elem_bytes = eb;
    apron_invalidate(ch);
    ch.slots = (int64_t)g->sub[0] * g->sub[1] * g->sub[2];
    const size_t bytes = (size_t)ch.slots * g->P * g->P * g->P * eb;
    GVX_CK(gvx_ensure(ch.data, bytes));
    GVX_CK(cudaMemsetAsync(ch.data.p, 0, bytes, g->stream));
    return GVX_OK;
}

gvx_status gvx_clear_channel(gvx_grid* g, int chan)
{
    GVX_GUARD(g);
    if (chan < 0 || chan >= GVX_MAXCH || !g->ch[chan].used) {
        gvx_set_error("ClearChannel: channel %d does not exist", chan);
        return GVX_ERR_INVALID_ARG;
    }
    GvxChannel& ch = g->ch[chan];
    GVX_CK(cudaMemsetAsync(ch.data.p, 0, (size_t)ch.slots * g->P * g->P * g->P * ch.elem_bytes, g->stream));
    apron_invalidate(ch);
    return GVX_OK;
}

gvx_status gvx_fill_channel(gvx_grid* g, int chan, const float value[4])
{
    GVX_GUARD(g);
    if (chan < 0 || chan >= GVX_MAXCH || !g->ch[chan].used || !value) {
        gvx_set_error("FillChannel: channel %d does not exist", chan);
        return GVX_ERR_INVALID_ARG;
    }
    GvxChannel& ch = g->ch[chan];
    apron_invalidate(ch);
    uint4 pat = make_uint4(0, 0, 0, 0);
    unsigned char* pb = (unsigned char*)&pat;
    if (ch.type == GVX_T_FLOAT) {
        memcpy(pb, value, 4);
    } else if (ch.elem_bytes == 16) {
        memcpy(pb, value, 16);
    } else {
        for (int k = 0; k < ch.elem_bytes; k++) pb[k] = (unsigned char)value[k];
    }
    const int64_t n = ch.slots * g->P * g->P * g->P;
    k_fill<<<1216, 256, 0, g->stream>>>((unsigned char*)ch.data.p, n, ch.elem_bytes, pat);
    g->launches++;
    GVX_CK(cudaGetLastError());
    return GVX_OK;
}

gvx_status gvx_set_points(gvx_grid* g, int n, const void* pos, int pos_offset, int pos_stride, const void* vel,
                          int vel_offset, int vel_stride, const void* clr, int clr_offset, int clr_stride)
{
    GVX_GUARD(g);
    if (n < 0 || (n > 0 && !pos) || pos_stride < 12 || (pos_offset & 3) || (pos_stride & 3) ||
        (vel && (vel_stride < 12 || (vel_stride & 3) || (vel_offset & 3)))) {
        gvx_set_error("SetPoints: need float3 positions with a stride >= 12 and 4-byte alignment");
        return GVX_ERR_INVALID_ARG;
    }
    if (((uintptr_t)pos & 3) || ((uintptr_t)vel & 3) ||
        (clr && (clr_stride < 4 || (clr_stride & 3) || (clr_offset & 3) || ((uintptr_t)clr & 3)))) {
        gvx_set_error("SetPoints: buffers must be 4-byte aligned, colours 4 bytes (uchar4) per point");
        return GVX_ERR_INVALID_ARG;
    }
    g->pts.n = n;
    g->pts.pos = (const char*)pos;
    g->pts.pos_off = pos_offset;
    g->pts.pos_stride = pos_stride;
    g->pts.vel = (const char*)vel;
    g->pts.vel_off = vel_offset;
    g->pts.vel_stride = vel_stride;
    g->pts.clr = (const char*)clr;
    g->pts.clr_off = clr_offset;
    g->pts.clr_stride = clr_stride;
    g->group_valid = false;
    g->perm_valid = false;
    return GVX_OK;
}

gvx_status gvx_set_point_attribs(gvx_grid* g, const float* weight, const float* radius)
{
    GVX_GUARD(g);
    g->pts.weight = weight;
    g->pts.radius = radius;
    g->perm_valid = false;
    return GVX_OK;
}

// strided float3 records (staged on the device as they are) -> packed float3
__global__ void k_pack_float3(const unsigned char* __restrict__ src, int stride, uint32_t n, float* __restrict__ dst)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* s = (const float*)(src + (size_t)i * stride);
        dst[3 * (size_t)i] = s[0];
        dst[3 * (size_t)i + 1] = s[1];
        dst[3 * (size_t)i + 2] = s[2];
    }
}

// one host -> device copy of n float3 records with a byte stride: packed records in one flat copy;
// strided ones as the raw bytes, packed by a kernel (a 2D copy of 12-byte rows is one DMA row a point)
static gvx_status upload_float3(gvx_grid* g, DevBuf& dst, const void* src, int stride, int n, cudaStream_t st)
{
    GVX_CK(gvx_ensure(dst, (size_t)n * 12));
    if (stride == 12) {
        GVX_CK(cudaMemcpyAsync(dst.p, src, (size_t)n * 12, cudaMemcpyHostToDevice, st));
        return GVX_OK;
    }
    if (stride & 3) {
        gvx_set_error("CommitData: the point stride %d is not a multiple of 4 bytes", stride);
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(gvx_ensure(g->own_stage, (size_t)n * stride));
    GVX_CK(cudaMemcpyAsync(g->own_stage.p, src, (size_t)(n - 1) * stride + 12, cudaMemcpyHostToDevice, st));
    k_pack_float3<<<std::min<unsigned>((unsigned)((n + 255) / 256), 152u * 16u), 256, 0, st>>>(
        g->own_stage.as<unsigned char>(), stride, (uint32_t)n, dst.as<float>());
    g->launches++;
    GVX_CK(cudaGetLastError());
    return GVX_OK;
}

gvx_status gvx_commit_points_host(gvx_grid* g, int n, const void* pos, int pos_stride, const void* vel,
                                  int vel_stride, const float* weight, const float* radius)
{
    GVX_GUARD(g);
    if (n <= 0 || !pos || pos_stride < 12 || (vel && vel_stride < 12)) {
        gvx_set_error("CommitData: invalid host points");
        return GVX_ERR_INVALID_ARG;
    }
    // Two sets of library-owned point buffers, filled in turn: this call fills the set the
    // previous call did not, on the side stream, after the work that was queued before the
    // previous call (the last work that read this set).  Its copies therefore overlap the work
    // queued since (a previous frame), and the calls that read points make the grid's stream
    // wait for them: the topology build and the subcell lists for the positions, the point
    // permute for everything (gvx_wait_positions, gvx_wait_attributes).
    if (!g->aux_stream) {
        GVX_CK(cudaStreamCreateWithFlags(&g->aux_stream, cudaStreamNonBlocking));
        for (int k = 0; k < 2; k++) GVX_CK(cudaEventCreateWithFlags(&g->ev_set_free[k], cudaEventDisableTiming));
        GVX_CK(cudaEventCreateWithFlags(&g->ev_pos_ready, cudaEventDisableTiming));
        GVX_CK(cudaEventCreateWithFlags(&g->ev_attr_ready, cudaEventDisableTiming));
    }
    const int cur = g->own_set, nxt = cur ^ 1;
    GVX_CK(cudaEventRecord(g->ev_set_free[cur], g->stream));  // everything queued so far reads set `cur`
    if (g->own_set_used[nxt]) GVX_CK(cudaStreamWaitEvent(g->aux_stream, g->ev_set_free[nxt], 0));
    cudaStream_t as = g->aux_stream;
    gvx_status rc0 = upload_float3(g, g->own_pos[nxt], pos, pos_stride, n, as);
    if (rc0) return rc0;
    GVX_CK(cudaEventRecord(g->ev_pos_ready, as));
    if (vel) {
        rc0 = upload_float3(g, g->own_vel[nxt], vel, vel_stride, n, as);
        if (rc0) return rc0;
    }
    if (weight) {
        GVX_CK(gvx_ensure(g->own_w[nxt], (size_t)n * 4));
        GVX_CK(cudaMemcpyAsync(g->own_w[nxt].p, weight, (size_t)n * 4, cudaMemcpyHostToDevice, as));
    }
    if (radius) {
        GVX_CK(gvx_ensure(g->own_r[nxt], (size_t)n * 4));
        GVX_CK(cudaMemcpyAsync(g->own_r[nxt].p, radius, (size_t)n * 4, cudaMemcpyHostToDevice, as));
    }
    GVX_CK(cudaEventRecord(g->ev_attr_ready, as));
    g->pos_pending = true;
    g->attr_pending = true;
    g->own_set = nxt;
    g->own_set_used[nxt] = true;
    gvx_status rc = gvx_set_points(g, n, g->own_pos[nxt].p, 0, 12, vel ? g->own_vel[nxt].p : nullptr, 0, 12, nullptr,
                                   0, 0);
    if (rc) return rc;
    return gvx_set_point_attribs(g, weight ? g->own_w[nxt].as<float>() : nullptr,
                                 radius ? g->own_r[nxt].as<float>() : nullptr);
}

gvx_status gvx_rebuild_topology(gvx_grid* g, int n, float radius, const float orig[3], int mode, int min_depth)
{
    GVX_GUARD(g);
    if (mode < GVX_TOPO_AUTO || mode > GVX_TOPO_ACCUMULATE) {
        gvx_set_error("RebuildTopology: mode %d", mode);
        return GVX_ERR_INVALID_ARG;
    }
    gvx_status rc = gvx_wait_positions(g);
    if (rc) return rc;
    rc = gvx_topo_rebuild(g, n, radius, orig, mode, min_depth);
    // the topology build is queued: from here the grid's stream also covers the attribute uploads
    gvx_status rw = gvx_wait_attributes(g);
    return rc ? rc : rw;
}

gvx_status gvx_request_full_rebuild(gvx_grid* g, int on)
{
    GVX_GUARD(g);
    g->rebuild_topo = on != 0;
    return GVX_OK;
}

gvx_status gvx_finish_topology_ex(gvx_grid* g, int commit_pool, int compute_bounds)
{
    GVX_GUARD(g);
    (void)commit_pool;  // the device pools are the tree: space activated on the host is always committed
    gvx_status rc = gvx_host_tree_commit(g);  // pools grown by ActivateSpace go to the device
    if (rc) return rc;
    return compute_bounds ? gvx_topo_compute_bounds(g) : GVX_OK;
}

gvx_status gvx_finish_topology(gvx_grid* g) { return gvx_finish_topology_ex(g, 1, 1); }

gvx_status gvx_clear(gvx_grid* g)
{
    GVX_GUARD(g);
    g->root_level = -1;
    for (int l = 0; l < GVX_MAXLEV; l++) g->count[l] = 0;
    g->used_leaves = 0;
    g->rebuild_topo = true;
    g->lookup_valid = g->group_valid = g->atlas_valid = g->nbr_valid = g->sc_valid = false;
    g->perm_valid = false;
    g->pools_appended = false;
    g->atlas_prefix = -1;
    g->topo_gen++;
    return GVX_OK;
}

gvx_status gvx_update_atlas(gvx_grid* g)
{
    GVX_GUARD(g);
    return gvx_topo_update_atlas(g);
}

gvx_status gvx_insert_points(gvx_grid* g, int n, const float trans[3], int32_t* pnode_out)
{
    GVX_GUARD(g);
    gvx_status rc = gvx_prepare_points(g, n, trans, false);
    if (rc || !pnode_out) return rc;
    DevBuf tmp;
    GVX_CK(gvx_ensure(tmp, (size_t)n * 4));
    k_pnode<<<(n + 255) / 256, 256, 0, g->stream>>>(g->keys[g->sorted_buf].as<uint32_t>(),
                                                    g->vals[g->sorted_buf].as<uint32_t>(), (uint32_t)n,
                                                    g->key_shift, 1u << g->lookup.ks.total_bits, g->lookup,
                                                    tmp.as<int>());
    g->launches++;
    cudaError_t e = cudaMemcpyAsync(pnode_out, tmp.p, (size_t)n * 4, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    gvx_free(tmp);
    if (e != cudaSuccess) return gvx_cuda_fail(e, "InsertPoints readback");
    return GVX_OK;
}

gvx_status gvx_scatter_density(gvx_grid* g, int n, float radius, float amp, const float trans[3], int expand,
                               int avg_color)
{
    GVX_GUARD(g);
    (void)amp;  // unused by the reference kernel as well (PT.cuh:525-573)
    return gvx_scatter_ref(g, n, radius, trans, expand, avg_color);
}

gvx_status gvx_gather_density(gvx_grid* g, int subcell, int n, float radius, const float trans[3], int sc_len,
                              int chan_density, int chan_clr, int accum)
{
    GVX_GUARD(g);
    (void)n;      // the lists of InsertPointsSubcell hold the points, as in the reference
    (void)trans;  // (VG.cpp:5318-5344 passes neither to the kernel)
    return gvx_gather_run(g, 0, subcell, radius, sc_len, chan_density, chan_clr, accum);
}

gvx_status gvx_gather_levelset(gvx_grid* g, int subcell, int n, float radius, const float trans[3], int sc_len,
                               int chan_levelset, int chan_clr, int accum)
{
    GVX_GUARD(g);
    (void)n;
    (void)trans;
    return gvx_gather_run(g, 1, subcell, radius, sc_len, chan_levelset, chan_clr, accum);
}

gvx_status gvx_splat(gvx_grid* g, int mode, int n, float radius, const float trans[3], int chan_density,
                     int chan_vel, int accum)
{
    GVX_GUARD(g);
    return gvx_splat_run(g, mode, n, radius, trans, chan_density, chan_vel, accum);
}

static gvx_status update_apron_one(gvx_grid* g, int chan, float boundval)
{
    const bool known = chan >= 0 && chan < GVX_MAXCH && g->ch[chan].used && g->atlas_valid &&
                       g->ch[chan].apron_bv == boundval;
    if (known && g->ch[chan].apron_valid) return GVX_OK;  // the apron already holds these copies (the splat's)
    gvx_status rc;
    if (known && g->ch[chan].apron_partial_from >= 0 && g->nbr_valid)
        rc = gvx_apron_run_partial(g, chan, boundval, g->ch[chan].apron_partial_from);  // new bricks + neighbours
    else
        rc = gvx_apron_run(g, chan, boundval);
    if (rc) return rc;
    g->ch[chan].apron_valid = true;
    g->ch[chan].apron_partial_from = -1;
    g->ch[chan].apron_bv = boundval;
    return GVX_OK;
}

gvx_status gvx_update_apron(gvx_grid* g, int chan, float boundval)
{
    GVX_GUARD(g);
    return update_apron_one(g, chan, boundval);
}

gvx_status gvx_update_apron_faces(gvx_grid* g, int chan)
{
    GVX_GUARD(g);
    return gvx_apron_faces_run(g, chan);
}

gvx_status gvx_update_neighbors(gvx_grid* g)
{
    GVX_GUARD(g);
    if (g->root_level < 0 || !g->nbr_valid) {
        gvx_set_error("UpdateNeighbors: no topology");
        return GVX_ERR_STATE;
    }
    return GVX_OK;  // the neighbour table is built with every topology
}

gvx_status gvx_update_apron_all(gvx_grid* g)
{
    GVX_GUARD(g);
    for (int c = 0; c < GVX_MAXCH; c++) {
        if (!g->ch[c].used) continue;
        gvx_status rc = update_apron_one(g, c, 0.0f);
        if (rc) return rc;
    }
    return GVX_OK;
}

// test hook: a sort pass whose first tile never reports (bounded look-back, error status, usable context)
gvx_status gvx_test_sort_withheld_tile(gvx_grid* g, const uint32_t* keys_in, const uint32_t* vals_in,
                                       uint32_t* keys_out, uint32_t* vals_out, uint32_t n)
{
    GVX_GUARD(g);
    if (!keys_in || !vals_in || !keys_out || !vals_out) {
        gvx_set_error("test_sort_withheld_tile: null buffer");
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(gvx_ensure(g->d_err, 64));
    GVX_CK(cudaMemsetAsync(g->d_err.p, 0, 4, g->stream));
    gvx_status rc = gvx_sort_pass_withheld_tile(keys_in, vals_in, keys_out, vals_out, n, g->sort, g->stream,
                                                g->d_err.as<uint32_t>(), &g->launches);
    if (rc) return rc;
    rc = gvx_check_device_error(g, "test_sort_withheld_tile");
    GVX_CK(cudaMemsetAsync(g->d_err.p, 0, 4, g->stream));  // the grid goes on with a clean error word
    return rc;
}

gvx_status gvx_radix_sort(gvx_grid* g, const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                          uint32_t* vals_out, uint32_t n, int bits)
{
    GVX_GUARD(g);
    if (n > 0 && (!keys_in || !vals_in || !keys_out || !vals_out)) {
        gvx_set_error("RadixSortByByte: null buffer");
        return GVX_ERR_INVALID_ARG;
    }
    if (bits < 1 || bits > 32) {
        gvx_set_error("RadixSortByByte: bits must be 1..32, got %d", bits);
        return GVX_ERR_INVALID_ARG;
    }
    if (n == 0) return GVX_OK;
    for (int k = 0; k < 2; k++) {
        GVX_CK(gvx_ensure(g->api_keys[k], (size_t)n * 4));
        GVX_CK(gvx_ensure(g->api_vals[k], (size_t)n * 4));
    }
    GVX_CK(gvx_ensure(g->d_err, 64));
    GVX_CK(cudaMemsetAsync(g->d_err.p, 0, 4, g->stream));
    GVX_CK(cudaMemcpyAsync(g->api_keys[0].p, keys_in, (size_t)n * 4, cudaMemcpyDeviceToDevice, g->stream));
    GVX_CK(cudaMemcpyAsync(g->api_vals[0].p, vals_in, (size_t)n * 4, cudaMemcpyDeviceToDevice, g->stream));
    uint32_t* kk[2] = {g->api_keys[0].as<uint32_t>(), g->api_keys[1].as<uint32_t>()};
    uint32_t* vv[2] = {g->api_vals[0].as<uint32_t>(), g->api_vals[1].as<uint32_t>()};
    int res = 0;
    gvx_status rc = gvx_sort_pairs(kk, vv, n, bits, g->sort, false, g->stream, g->d_err.as<uint32_t>(), &res,
                                   &g->launches);
    if (rc) return rc;
    GVX_CK(cudaMemcpyAsync(keys_out, kk[res], (size_t)n * 4, cudaMemcpyDeviceToDevice, g->stream));
    GVX_CK(cudaMemcpyAsync(vals_out, vv[res], (size_t)n * 4, cudaMemcpyDeviceToDevice, g->stream));
    return GVX_OK;
}

static int top_lev_of(const gvx_grid* g)
{
    int tlev = 1;
    for (int n = g->levels - 1; n >= 0; n--)
        if (g->count[n] == 1) tlev = n;
    return tlev;
}

gvx_status gvx_get_info(gvx_grid* g, gvx_info* out)
{
    GVX_GUARD(g);
    if (!out) {
        gvx_set_error("get_info: null output");
        return GVX_ERR_INVALID_ARG;
    }
    gvx_status rc = gvx_topo_read_bounds(g);
    if (rc) return rc;
    memset(out, 0, sizeof(*out));
    out->levels = g->levels;
    for (int l = 0; l < GVX_MAXLEV; l++) {
        out->logdim[l] = g->logdim[l];
        out->node_count[l] = g->count[l];
    }
    out->brick_res = g->brick;
    out->apron = g->apron;
    out->root_level = g->root_level;
    out->top_lev = g->root_level >= 0 ? top_lev_of(g) : -1;
    out->used_leaves = g->used_leaves;
    for (int a = 0; a < 3; a++) {
        out->atlas_subdim[a] = g->sub[a];
        out->atlas_res[a] = g->sub[a] * g->P;
        out->root_pos[a] = g->root_pos[a];
        out->bbox_min[a] = g->bbox_min[a];
        out->bbox_max[a] = g->bbox_max[a];
        out->obj_min[a] = g->obj_min[a];
        out->obj_max[a] = g->obj_max[a];
        out->vox_res[a] = g->obj_max[a] - g->obj_min[a];
        out->vox_res_max[a] = g->vox_res_max[a];
    }
    int nch = 0;
    for (int c = 0; c < GVX_MAXCH; c++) nch += g->ch[c].used;
    out->channels = nch;
    out->last_rebuild = g->last_rebuild;
    out->planned_builds = g->planned_builds;
    return GVX_OK;
}

gvx_status gvx_read_nodes(gvx_grid* g, int level, void* out, int64_t cap_nodes)
{
    GVX_GUARD(g);
    if (level < 0 || level >= g->levels || !out || cap_nodes < g->count[level]) {
        gvx_set_error("read_nodes: level %d, capacity %lld < %lld", level, (long long)cap_nodes,
                      (long long)(level >= 0 && level < GVX_MAXLEV ? g->count[level] : 0));
        return GVX_ERR_INVALID_ARG;
    }
    if (g->count[level])
        GVX_CK(cudaMemcpyAsync(out, g->nodes[level].p, (size_t)g->count[level] * sizeof(GvxNode),
                               cudaMemcpyDeviceToHost, g->stream));
    GVX_CK(cudaStreamSynchronize(g->stream));
    return GVX_OK;
}

gvx_status gvx_read_childlist(gvx_grid* g, int level, uint64_t* out, int64_t cap)
{
    GVX_GUARD(g);
    if (level <= 0 || level >= g->levels || !out) {
        gvx_set_error("read_childlist: level %d", level);
        return GVX_ERR_INVALID_ARG;
    }
    const int64_t n = g->count[level] * (int64_t)g->res[level] * g->res[level] * g->res[level];
    if (cap < n) {
        gvx_set_error("read_childlist: capacity %lld < %lld", (long long)cap, (long long)n);
        return GVX_ERR_INVALID_ARG;
    }
    if (n)
        GVX_CK(cudaMemcpyAsync(out, g->clist[level].p, (size_t)n * 8, cudaMemcpyDeviceToHost, g->stream));
    GVX_CK(cudaStreamSynchronize(g->stream));
    return GVX_OK;
}

gvx_status gvx_read_atlas_map(gvx_grid* g, int32_t* out4, int64_t cap_slots)
{
    GVX_GUARD(g);
    const int64_t slots = (int64_t)g->sub[0] * g->sub[1] * g->sub[2];
    if (!g->atlas_valid || !out4 || cap_slots < slots) {
        gvx_set_error("read_atlas_map: no atlas or capacity %lld < %lld", (long long)cap_slots, (long long)slots);
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(cudaMemcpyAsync(out4, g->amap.p, (size_t)slots * 16, cudaMemcpyDeviceToHost, g->stream));
    GVX_CK(cudaStreamSynchronize(g->stream));
    return GVX_OK;
}

gvx_status gvx_channel_bytes(gvx_grid* g, int chan, int64_t* bytes)
{
    GVX_GUARD(g);
    if (chan < 0 || chan >= GVX_MAXCH || !g->ch[chan].used || !bytes) {
        gvx_set_error("channel_bytes: channel %d", chan);
        return GVX_ERR_INVALID_ARG;
    }
    *bytes = g->ch[chan].slots * g->P * g->P * g->P * g->ch[chan].elem_bytes;
    return GVX_OK;
}

gvx_status gvx_read_channel(gvx_grid* g, int chan, void* out, int64_t cap)
{
    int64_t bytes = 0;
    gvx_status rc = gvx_channel_bytes(g, chan, &bytes);
    if (rc) return rc;
    if (!out || cap < bytes) {
        gvx_set_error("read_channel: capacity %lld < %lld", (long long)cap, (long long)bytes);
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(cudaMemcpyAsync(out, g->ch[chan].data.p, (size_t)bytes, cudaMemcpyDeviceToHost, g->stream));
    GVX_CK(cudaStreamSynchronize(g->stream));
    return GVX_OK;
}

gvx_status gvx_read_channel_dense(gvx_grid* g, int chan, void* out, int64_t cap)
{
    int64_t bytes = 0;
    gvx_status rc = gvx_channel_bytes(g, chan, &bytes);
    if (rc) return rc;
    if (!out || cap < bytes) {
        gvx_set_error("read_channel_dense: capacity %lld < %lld", (long long)cap, (long long)bytes);
        return GVX_ERR_INVALID_ARG;
    }
    std::vector<unsigned char> tmp((size_t)bytes);
    GVX_CK(cudaMemcpyAsync(tmp.data(), g->ch[chan].data.p, (size_t)bytes, cudaMemcpyDeviceToHost, g->stream));
    GVX_CK(cudaStreamSynchronize(g->stream));
    const int P = g->P, eb = g->ch[chan].elem_bytes;
    const int64_t W = (int64_t)g->sub[0] * P, H = (int64_t)g->sub[1] * P;
    unsigned char* o = (unsigned char*)out;
    for (int64_t s = 0; s < g->ch[chan].slots; s++) {
        const int64_t bx = s % g->sub[0], by = (s / g->sub[0]) % g->sub[1], bz = s / ((int64_t)g->sub[0] * g->sub[1]);
        for (int z = 0; z < P; z++)
            for (int y = 0; y < P; y++) {
                const int64_t src = (((s * P + z) * P + y) * P) * eb;
                const int64_t dst = (((bz * P + z) * H + (by * P + y)) * W + bx * P) * eb;
                memcpy(o + dst, tmp.data() + src, (size_t)P * eb);
            }
    }
    return GVX_OK;
}

gvx_status gvx_channel_type(gvx_grid* g, int chan, int* type)
{
    GVX_GUARD(g);
    if (chan < 0 || chan >= GVX_MAXCH || !type) {
        gvx_set_error("channel_type: channel %d", chan);
        return GVX_ERR_INVALID_ARG;
    }
    *type = g->ch[chan].used ? g->ch[chan].type : -1;
    return GVX_OK;
}

gvx_status gvx_channel_device_ptr(gvx_grid* g, int chan, void** dev_ptr, int64_t* bytes)
{
    gvx_status rc = gvx_channel_bytes(g, chan, bytes);
    if (rc) return rc;
    if (!dev_ptr) {
        gvx_set_error("channel_device_ptr: null output");
        return GVX_ERR_INVALID_ARG;
    }
    *dev_ptr = g->ch[chan].data.p;
    apron_invalidate(g->ch[chan]);  // the caller may write the voxels: UpdateApron runs again
    return GVX_OK;
}

gvx_status gvx_retrieve_brick(gvx_grid* g, int chan, const int corner[3], void* out, int64_t cap)
{
    int64_t bytes = 0;
    gvx_status rc = gvx_channel_bytes(g, chan, &bytes);
    if (rc) return rc;
    const int P = g->P, b = g->brick, eb = g->ch[chan].elem_bytes;
    if (!corner || !out || cap < (int64_t)b * b * b * eb) {
        gvx_set_error("retrieve_brick: output too small");
        return GVX_ERR_INVALID_ARG;
    }
    const int bx = corner[0] / P, by = corner[1] / P, bz = corner[2] / P;
    const int ox = corner[0] - bx * P, oy = corner[1] - by * P, oz = corner[2] - bz * P;
    if (bx < 0 || by < 0 || bz < 0 || bx >= g->sub[0] || by >= g->sub[1] || bz >= g->sub[2] || ox + b > P ||
        oy + b > P || oz + b > P) {
        gvx_set_error("retrieve_brick: corner (%d,%d,%d) is not inside one atlas brick", corner[0], corner[1],
                      corner[2]);
        return GVX_ERR_INVALID_ARG;
    }
    const int64_t s = ((int64_t)bz * g->sub[1] + by) * g->sub[0] + bx;
    std::vector<unsigned char> tmp((size_t)P * P * P * eb);
    GVX_CK(cudaMemcpyAsync(tmp.data(), g->ch[chan].data.as<unsigned char>() + s * P * P * P * eb, tmp.size(),
                           cudaMemcpyDeviceToHost, g->stream));
    GVX_CK(cudaStreamSynchronize(g->stream));
    // kernelRetrieveTexXYZ (cuda_gvdb_copydata.cu:74-79) writes buf[(x*ry + y)*rx + z]
    unsigned char* o = (unsigned char*)out;
    for (int x = 0; x < b; x++)
        for (int y = 0; y < b; y++)
            for (int z = 0; z < b; z++)
                memcpy(o + (((int64_t)x * b + y) * b + z) * eb,
                       tmp.data() + ((((int64_t)(oz + z)) * P + (oy + y)) * P + (ox + x)) * eb, (size_t)eb);
    return GVX_OK;
}

gvx_status gvx_kernel_launches(gvx_grid* g, int64_t* count)
{
    if (!g || !count) {
        gvx_set_error("kernel_launches: null argument");
        return GVX_ERR_INVALID_ARG;
    }
    *count = g->launches;
    return GVX_OK;
}

gvx_status gvx_device_alloc(int device, size_t bytes, void** out)
{
    if (!out) {
        gvx_set_error("device_alloc: null output");
        return GVX_ERR_INVALID_ARG;
    }
    *out = nullptr;
    GVX_CK(cudaSetDevice(device));
    GVX_CK(cudaMalloc(out, bytes ? bytes : 16));
    return GVX_OK;
}

gvx_status gvx_device_free(int device, void* ptr)
{
    if (!ptr) return GVX_OK;
    GVX_CK(cudaSetDevice(device));
    GVX_CK(cudaFree(ptr));
    return GVX_OK;
}

gvx_status gvx_memcpy(int device, void* dst, const void* src, size_t bytes, int kind)
{
    if ((!dst || !src) && bytes) {
        gvx_set_error("memcpy: null pointer");
        return GVX_ERR_INVALID_ARG;
    }
    const cudaMemcpyKind k = kind == GVX_COPY_H2D   ? cudaMemcpyHostToDevice
                             : kind == GVX_COPY_D2H ? cudaMemcpyDeviceToHost
                             : kind == GVX_COPY_D2D ? cudaMemcpyDeviceToDevice
                                                    : cudaMemcpyDefault;
    if (kind < 0 || kind > 2) {
        gvx_set_error("memcpy: unknown kind %d", kind);
        return GVX_ERR_INVALID_ARG;
    }
    if (!bytes) return GVX_OK;
    GVX_CK(cudaSetDevice(device));
    GVX_CK(cudaMemcpy(dst, src, bytes, k));
    return GVX_OK;
}

}  // extern "C"
