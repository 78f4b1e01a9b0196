// gvx_grid.cuh -- the grid handle behind gvx_grid* and the host entry points
// of the topology, splat and apron stages.
#pragma once

#include "gvx_internal.cuh"

struct GvxChannel {
    bool used = false;
    int type = 0;
    int ncomp = 1;       // components per voxel
    int elem_bytes = 4;  // bytes per voxel
    DevBuf data;         // slots * P^3 * elem_bytes, brick-major
    int64_t slots = 0;
    bool apron_valid = false;  // apron voxels hold the neighbours' interior values / boundval
    float apron_bv = 0.f;      // the boundary value they were filled with
    // >= 0: the apron holds those copies except in the bricks of slots >= apron_partial_from
    // (added by an appending topology build) and their neighbours
    int64_t apron_partial_from = -1;
};

// the channel's apron no longer holds the neighbours' values anywhere it is known to
inline void apron_invalidate(GvxChannel& ch)
{
    ch.apron_valid = false;
    ch.apron_partial_from = -1;
}

struct GvxPoints {
    int n = 0;
    const char* pos = nullptr;
    int pos_off = 0, pos_stride = 12;
    const char* vel = nullptr;
    int vel_off = 0, vel_stride = 12;
    const char* clr = nullptr;
    int clr_off = 0, clr_stride = 4;
    const float* weight = nullptr;
    const float* radius = nullptr;
};

// How a key maps to a leaf pool index: a set bit in `a` -> rank in a (+ remap),
// else a set bit in `b` -> b_offset + rank in b, else -1.
struct LeafLookup {
    KeySpace ks;
    BitRank a;
    BitRank b;
    uint32_t b_offset;
    const int* remap;  // optional rank -> pool index
    const uint32_t* b_offset_p;  // optional: b_offset read from device memory (planned builds)
    uint32_t cap;                // optional (0: none): pool indices >= cap are not returned
};

__device__ inline int ll_find(const LeafLookup& L, int cx, int cy, int cz)
{
    if (cx < 0 || cy < 0 || cz < 0 || cx >= (1 << L.ks.bits[0]) || cy >= (1 << L.ks.bits[1]) ||
        cz >= (1 << L.ks.bits[2]))
        return -1;
    const uint32_t key = ks_pack(L.ks, cx, cy, cz, 0);
    uint32_t r;
    if (br_test(L.a, key)) {
        r = br_rank(L.a, key);
        if (L.remap) return L.remap[r];
    } else if (L.b.bits && br_test(L.b, key)) {
        r = (L.b_offset_p ? *L.b_offset_p : L.b_offset) + br_rank(L.b, key);
    } else {
        return -1;
    }
    return (L.cap && r >= L.cap) ? -1 : (int)r;
}

struct gvx_grid {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // host uploads of the point attributes run on a side stream, overlapping the topology
    // build; the point permute, the only device reader of them, waits for ev_attr_ready
    cudaStream_t aux_stream = nullptr;
    cudaEvent_t ev_set_free[2] = {nullptr, nullptr};  // the work queued before a set was last replaced
    cudaEvent_t ev_pos_ready = nullptr, ev_attr_ready = nullptr;
    bool pos_pending = false, attr_pending = false;

    // configuration (Configure)
    bool configured = false;
    int levels = 0;
    int logdim[GVX_MAXLEV] = {};
    int res[GVX_MAXLEV] = {};
    int range[GVX_MAXLEV] = {};
    int tshift[GVX_MAXLEV] = {};  // log2(range[l] / res[0]): level-l node size in leaves
    int brick = 0, apron = 1, P = 0;
    bool apron_set = false;
    int defsub[3] = {16, 16, 1};

    // topology state
    int root_level = -1;
    int root_pos[3] = {0, 0, 0};
    bool rebuild_topo = true;  // mRebuildTopo
    int curr_depth = -1;       // mCurrDepth
    int last_rebuild = 0;
    int64_t count[GVX_MAXLEV] = {};
    int64_t used_leaves = 0;
    DevBuf nodes[GVX_MAXLEV];
    DevBuf clist[GVX_MAXLEV];
    float bbox_min[3] = {0, 0, 0}, bbox_max[3] = {0, 0, 0};
    float obj_min[3] = {0, 0, 0}, obj_max[3] = {0, 0, 0};
    float vox_res_max[3] = {0, 0, 0};  // mVoxResMax (sticky since Configure)
    bool bounds_pending = false;
    bool vox_res_max_reset = true;     // the next ComputeBounds zeroes mVoxResMax first

    // lookup of leaves by key for the current topology
    LeafLookup lookup{};
    bool lookup_valid = false;
    DevBuf bm_a, bm_a_prefix, bm_b, bm_b_prefix;  // active-leaf bitmap of UpdateAtlas
    DevBuf lk_bits, lk_prefix, remap;             // active-leaf bitmap + rank -> pool index after an incremental build

    // per-leaf data
    DevBuf leaf_key;     // compact level-0 key per leaf (pool order)
    DevBuf leaf_range;   // int2 [start, end) in the sorted point order
    DevBuf leaf_oct;     // 8 ints per leaf: first sorted index of each octant of the leaf's points
    int key_shift = 0;       // the sort keys are leaf key << key_shift | octant (key_shift 3) or the leaf key (0)
    bool oct_valid = false;  // the sorted points are in octant order inside every leaf, leaf_oct filled
    uint32_t oct_leaves = 0;
    DevCount oct_count{};  // leaves to partition, read on the device (a planned build); else oct_leaves
    DevBuf leaf_slot;    // atlas slot per leaf, -1 if inactive
    DevBuf slot_leaf;    // leaf per atlas slot (active slots only)
    DevBuf nbr;          // 27 leaf indices per leaf
    bool nbr_valid = false;

    // atlas
    int sub[3] = {0, 0, 0};
    bool have_atlas = false;
    bool atlas_valid = false;  // mValue/atlas map reflect the topology
    int64_t atlas_used = 0;
    GvxChannel ch[GVX_MAXCH];
    DevBuf amap;       // 4 ints per slot
    DevBuf apron_tab;  // apron voxel table of the apron kernel, for bricks of side apron_tab_P
    int apron_tab_P = 0;
    int64_t atlas_prefix = -1;  // UpdateAtlas gave leaf i slot i for every leaf < atlas_prefix (all active)
    bool pools_appended = false;  // the last topology build kept the pools' nodes and only appended
    DevBuf apron_mark;            // per slot: 1 = its apron needs the copies (partial UpdateApron)
    int64_t apron_mark_from = -1; // the marks are those of slots >= apron_mark_from ...
    uint64_t apron_mark_gen = 0;  // ... for the atlas of this generation
    uint64_t atlas_gen = 0;       // bumped by every UpdateAtlas
    DevBuf atlas_tmp;  // second atlas of the unpacked (Jacobi) smoothing

    // points
    GvxPoints pts;
    // storage of gvx_commit_points_host: two sets, filled in turn, so that a commit's copies
    // overlap the work still reading the other set
    DevBuf own_pos[2], own_vel[2], own_w[2], own_r[2];
    int own_set = 0;
    bool own_set_used[2] = {false, false};
    DevBuf own_stage;                       // strided host records as copied, before packing

    // grouping of points by leaf (sorted order)
    DevBuf keys[2], vals[2];
    int sorted_buf = 0;
    uint32_t n_sorted = 0;
    float sort_trans[3] = {0, 0, 0};  // translation of the positions the sorted keys were made from
    bool group_valid = false;
    float group_trans[3] = {0, 0, 0};
    const void* group_pos = nullptr;
    int group_n = -1;
    DevBuf spos, svel;  // sorted float4 (x,y,z,weight) and (vx,vy,vz,radius)
    bool perm_valid = false;  // spos/svel match the grouping and the bound attributes
    bool perm_has_svel = false;
    const void* perm_vel = nullptr;
    const void* perm_w = nullptr;
    const void* perm_r = nullptr;
    SortScratch sort;

    // scratch of the topology build
    DevBuf d0_bits, d0_prefix, x0_bits, x0_prefix, masks, upper, lists, tmp_scan, d_counts;
    DevBuf inc0, inc_remap;  // incremental build: linked + new level-0 bitmaps, linked rank -> pool index
    DevBuf d_err, d_bbox;
    DevBuf d_rmax;  // float bits of the largest per-point radius of the last point permute
    DevBuf d_next;  // work-unit counter of the splat launch (+ the count of touched slots)
    DevBuf touched; // slots an accumulating splat visits
    void* h_pin = nullptr;  // pinned staging of the topology's small readbacks
    struct gvx_topo_staged* staged = nullptr;  // a staged RebuildTopology between its stages (batches)
    struct gvx_topo_plan* plan = nullptr;      // fixed key space and capacities of planned builds
    int64_t planned_builds = 0;                // single-grid full builds that ran under the plan
    DevBuf host_stage;  // pinned staging of small readbacks

    // subcell lists of InsertPointsSubcell: entries sorted by subcell index
    // (atlas slot * (b/s)^3 + local subcell), point order within a subcell
    DevBuf sc_cnt, sc_off;          // per point: entry count, then its offset
    DevBuf sc_keys[2], sc_vals[2];  // entries: subcell index, point index
    DevBuf sc_pts;                  // float4 per entry: translated position, colour bits in .w
    DevBuf sc_beg, sc_end;          // per subcell: [beg, end) in the entry arrays
    DevBuf sc_q, sc_qclr;           // FP16 lists: uint2 (x | y << 16, z) per entry, colour per entry
    float sc_qmin[3] = {0, 0, 0}, sc_qrange[3] = {0, 0, 0};  // mPosMin / mPosRange they were stored against
    bool sc_fp16 = false;           // the lists are InsertPointsSubcell_FP16's
    bool colavg_seen = false;       // an avgColor ScatterDensity ran (the reference's AUX_COLAVG exists)
    int sc_size = 0;
    uint32_t sc_len = 0, sc_nsub = 0;
    bool sc_has_clr = false;
    bool sc_valid = false;  // the lists match the current topology and atlas

    // scratch of gvx_radix_sort (kept apart from the topology's grouping)
    DevBuf api_keys[2], api_vals[2];

    int64_t launches = 0;

    // host copy of the pools for ActivateSpace / RebuildTopologyCPU (gvx_cputopo.cu)
    struct GvxHostTree* htree = nullptr;
    uint64_t topo_gen = 0;  // advances whenever the device tree changes
};

// topology (gvx_topology.cu)
gvx_status gvx_topo_rebuild(gvx_grid* g, int n, float radius, const float orig[3], int mode, int min_depth);
gvx_status gvx_topo_update_atlas(gvx_grid* g);
// host-side topology (gvx_cputopo.cu): FinishTopology's commit, release
gvx_status gvx_host_tree_commit(gvx_grid* g);
void gvx_host_tree_free(gvx_grid* g);
// a tree given as host node pools / child lists (levels 0..root_level; clists[0] unused)
gvx_status gvx_topo_import(gvx_grid* g, int root_level, const int64_t* counts, const GvxNode* const* nodes,
                           const uint64_t* const* clists);
gvx_status gvx_topo_group_points(gvx_grid* g, int n, const float trans[3]);
// sorted point attributes written by the octant pass of InsertPoints (spos null: none)
struct GvxSortedAttr {
    const char* vel;
    int vel_off, vel_stride;
    const float* weight;
    const float* radius;
    float4* spos;          // (x, y, z, weight) of the translated positions
    float4* svel;          // (vx, vy, vz, radius), or null
    unsigned int* rmax;    // float bits of the largest radius, or null
};
gvx_status gvx_topo_octants(gvx_grid* g, const GvxSortedAttr* attr);
gvx_status gvx_wait_attributes(gvx_grid* g);
gvx_status gvx_wait_positions(gvx_grid* g);
gvx_status gvx_topo_compute_bounds(gvx_grid* g);
// RebuildTopology in three stages (for batches of grids; see gvx_topology.cu): between two
// stages of one grid the host may queue other grids' work, so that one synchronisation per
// stage serves the whole batch
gvx_status gvx_topo_stage1(gvx_grid* g, int n, float radius, int mode, int min_depth);
gvx_status gvx_topo_stage2(gvx_grid* g);
gvx_status gvx_topo_stage3(gvx_grid* g);
void gvx_topo_staged_free(gvx_grid* g);
gvx_status gvx_topo_read_bounds(gvx_grid* g);
// Planned full builds (see gvx_topology.cu): a plan made from the grid's last full build; a
// planned build queues RebuildTopology (full) -- with frame, UpdateAtlas and InsertPoints' octant
// pass writing `attr` too -- with no host wait and no allocation (capturable); plan_finish, after
// the stream has passed it, checks that the plan held and sets the host state (*held false: the
// build is void, the grid is to be built again without the plan)
gvx_status gvx_topo_plan_make(gvx_grid* g);
bool gvx_topo_plan_ready(const gvx_grid* g);
gvx_status gvx_topo_plan_enqueue(gvx_grid* g, const GvxSortedAttr* attr, bool frame);
gvx_status gvx_topo_plan_record_error(gvx_grid* g, cudaStream_t st);
void gvx_topo_plan_replayed(gvx_grid* g);  // its captured build was launched again
gvx_status gvx_topo_plan_finish(gvx_grid* g, bool* held, bool frame);
void gvx_topo_plan_free(gvx_grid* g);
uint64_t gvx_topo_plan_id(const gvx_grid* g);  // changes whenever the plan is made again
// device count of the atlas slots a planned build assigns (clamped to *cap by the reader)
const uint32_t* gvx_topo_plan_slots(const gvx_grid* g, uint32_t* cap);
// InsertPoints: grouping + sorted attribute arrays
gvx_status gvx_prepare_points(gvx_grid* g, int n, const float trans[3], bool need_svel);
gvx_status gvx_check_device_error(gvx_grid* g, const char* stage);

// splats (gvx_splat.cu) and gathers (gvx_gather.cu)
gvx_status gvx_splat_run(gvx_grid* g, int mode, int n, float radius, const float trans[3], int chan_d,
                         int chan_v, int accum);
gvx_status gvx_scatter_ref(gvx_grid* g, int n, float radius, const float trans[3], int expand, int avg_color);
gvx_status gvx_gather_run(gvx_grid* g, int levelset, int subcell, float radius, int sc_len, int chan, int chan_clr,
                          int accum);

// apron (gvx_apron.cu)
gvx_status gvx_apron_run(gvx_grid* g, int chan, float boundval);
// UpdateApron of the bricks of slots >= from and of their neighbours only (the other aprons
// already hold the copies)
gvx_status gvx_apron_run_partial(gvx_grid* g, int chan, float boundval, int64_t from);
gvx_status gvx_apron_faces_run(gvx_grid* g, int chan);

// channel storage (gvx_api.cu)
gvx_status gvx_grow_atlas(gvx_grid* g, int64_t need_slots);
