/*
 * gvx_oracle.h -- CPU oracle for the GVDB point -> sparse-volume path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (dunyazad/gvdb-voxels, GVDB Voxels 1.1.1) used as the checker for
 * the CUDA implementation.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py may load it.  The product library
 * (libgvx) never links, loads or calls anything in this directory.
 *
 * Topology and atlas bookkeeping are integer work and are restated step by
 * step from the reference (keys per point per level, sort, unique, pool
 * allocation loop, root descent link / delink), in the same FP32 arithmetic
 * the reference uses for the float->index conversions, so the node pools it
 * produces are the reference's bit for bit.  Splat values are accumulated in
 * FP64.
 *
 * Where the reference reads outside an allocation or races (see
 * ORC_ERR_DEGENERATE) the oracle stops and reports it instead of guessing.
 */
#ifndef GVX_ORACLE_H
#define GVX_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ORC_OK = 0,
    ORC_ERR_ARG = 1,
    ORC_ERR_DEPTH = 2,       /* point extents smaller than one brick or deeper than the tree */
    ORC_ERR_DEGENERATE = 3,  /* the reference reads out of range / races on this input */
    ORC_ERR_STATE = 4,       /* call order (e.g. splat before topology) */
    ORC_ERR_NOMEM = 5
};

/* topology modes */
enum {
    ORC_TOPO_AUTO = 0,       /* VolumeGVDB::RebuildTopology state machine (VG.cpp:1181-1218) */
    ORC_TOPO_FULL = 1,       /* RequestFullRebuild(true) + RebuildTopology */
    ORC_TOPO_ACCUMULATE = 2  /* VolumeGVDB::AccumulateTopology (VG.cpp:1158-1178) */
};

/* splat modes */
enum {
    ORC_SPLAT_TRILINEAR = 0,   /* new: cloud-in-cell, integer sample positions */
    ORC_SPLAT_CUBIC = 1,       /* new: Monaghan M4 cubic spline, support R = 2h */
    ORC_SPLAT_REF_SCATTER = 2, /* gvdbScatterPointDensity (PT.cuh:525-573), race-free sum */
    ORC_SPLAT_GATHER_DENSITY = 3,  /* gvdbGatherDensity (PT.cuh:696-733) */
    ORC_SPLAT_GATHER_LEVELSET = 4  /* gvdbGatherLevelSet (PT.cuh:736-773) */
};

/* channel types, same numbering as gvdb_types.h:70-78 */
enum { ORC_T_UCHAR = 0, ORC_T_UCHAR4 = 2, ORC_T_FLOAT = 3, ORC_T_FLOAT3 = 4, ORC_T_FLOAT4 = 5 };

/* 64-byte node record, same layout as VDBNode (cuda_gvdb_nodes.cuh:24-35) */
typedef struct orc_node {
    uint8_t lev, flags, prio, pad;
    int32_t pos[3];
    int32_t value[3];
    float vrange[3];
    uint64_t parent;
    uint64_t childlist;
    uint64_t mask;
} orc_node;

typedef struct orc_grid orc_grid;

orc_grid* orc_create(int levels, const int* logdim, int apron, int cx, int cy, int cz);
void orc_destroy(orc_grid* g);

/* channels: values are held as FP64, 4 components per voxel for FLOAT3/FLOAT4 */
int orc_add_channel(orc_grid* g, int chan, int type);
int orc_clear_channel(orc_grid* g, int chan);

/* positions: n points, xyz floats at pos + i*stride_floats */
int orc_rebuild_topology(orc_grid* g, int n, const float* pos, int stride_floats,
                         float radius, const float orig[3], int mode, int min_depth);
int orc_update_atlas(orc_grid* g);
/* the atlas layout without channel storage (UpdateAtlas then assigns slots) */
int orc_atlas_layout_only(orc_grid* g);

/* queries */
int orc_root_level(const orc_grid* g);   /* level of the root node, -1 if none */
int orc_top_lev(const orc_grid* g);      /* VDBInfo.top_lev as PrepareVDB computes it */
int orc_num_nodes(const orc_grid* g, int level);
int orc_num_used_leaves(const orc_grid* g);
int orc_last_mode(const orc_grid* g);    /* 1 = the last rebuild was full, 2 = incremental, 0 = no-op */
int orc_get_nodes(const orc_grid* g, int level, orc_node* out, int cap);
int orc_get_childlist(const orc_grid* g, int level, uint64_t* out, int64_t cap);
int orc_atlas_subdim(const orc_grid* g, int out[3]);
/* atlas map: per atlas brick slot (x fastest): pos[3], leaf id */
int orc_get_atlas_map(const orc_grid* g, int32_t* out4, int cap);

/* splat / gather.  pos,vel: xyz floats at stride_floats; weight, radius may be NULL
 * (weight 1, radius = `radius`).  For REF_SCATTER `expand` selects the 6-neighbour
 * stencil; for the gathers `subcell` is the subcell size and `radius_ins` the
 * insertion radius of InsertPointsSubcell; `accum` keeps the previous values. */
int orc_splat(orc_grid* g, int mode, int n, const float* pos, int pos_stride,
              const float* weight, const float* radius_pp, const float* vel, int vel_stride,
              float radius, const float trans[3], int chan_density, int chan_vel,
              int accum, int expand, int subcell, float radius_ins);

/* TRILINEAR / CUBIC splat values of a sample of leaves (level-0 pool
 * indices) without atlas channels, for checks at sizes whose FP64 atlas
 * would not fit: ADDED to dens_out[k][P][P][P] and vel_out[k][P][P][P][3]
 * (either may be NULL); zero_unowned sets the sampled apron voxels that no
 * active leaf owns to 0 afterwards (a non-accumulating splat). */
int orc_splat_sample(orc_grid* g, int mode, int n, const float* pos, int pos_stride, const float* weight,
                     const float* radius_pp, const float* vel, int vel_stride, float radius, const float trans[3],
                     const int* leaves, int nleaves, int zero_unowned, double* dens_out, double* vel_out);

/* InsertPointsSubcell + GatherDensity / GatherLevelSet with the optional
 * colour average (PT.cuh:696-773): clr holds one uchar4 per point (or NULL),
 * chan_clr a T_UCHAR4 channel (or -1).  *sc_len receives the number of
 * (point, subcell) entries (pSCPntsLength).  The colour is stored as
 * uchar(c * 255) saturated to [0, 255] (the reference's conversion of values
 * outside that range is undefined). */
int orc_gather(orc_grid* g, int levelset, int n, const float* pos, int pos_stride, const uint8_t* clr,
               float radius, float radius_ins, const float trans[3], int subcell, int chan, int chan_clr,
               int accum, int64_t* sc_len);
/* ScatterDensity (VG.cpp:5624-5660) with the point colours of clr (4 bytes per
 * point, may be NULL): density into channel 0, colours into channel 1
 * (avg_color) or 3 */
int orc_scatter_density(orc_grid* g, int n, const float* pos, int pos_stride, const uint8_t* clr, float radius,
                        const float trans[3], int expand, int avg_color);
/* InsertPointsSubcell_FP16 + GatherLevelSet_FP16 (VG.cpp:5094-5190, 5375-5401) */
int orc_gather_fp16(orc_grid* g, int n, const float* pos, int pos_stride, const uint8_t* clr, float radius,
                    float radius_ins, const float trans[3], int subcell, int chan, int chan_clr, int64_t* sc_len);
/* the reference's host tree (ActivateSpace, VG.cpp:2707-3027) kept across calls */
void* orc_cpu_tree_new(int levels, const int* logdim);
void orc_cpu_tree_free(void* h);
int orc_cpu_tree_activate(void* h, int n, const float* pos, int stride, const float orig[3]);
int orc_cpu_tree_count(void* h, int lev);
int64_t orc_cpu_tree_root(void* h);
int orc_cpu_tree_nodes(void* h, int lev, orc_node* out, int cap);
int orc_cpu_tree_childlist(void* h, int lev, uint64_t* out, int64_t cap);
/* UpdateNeighbors + UpdateApronFaces (VG.cpp:2527-2556, 4461-4496): face aprons of float channels */
int orc_update_apron_faces(orc_grid* g, int chan);
/* ConvertAndTransform (VG.cpp:5668-5682) on host arrays */
int orc_convert_and_transform(int n, const void* src, int src_bits, float* dst, const float wmin[3],
                              const float wdelta[3], const float trans[3], const float scal[3]);
/* ComputeBounds (VG.cpp:1792-1816): out = mVoxMin[3], mVoxMax[3], mVoxRes[3], mVoxResMax[3] */
int orc_compute_bounds(orc_grid* g, float out[12]);
/* mPosMin / mPosMax of the last GetBoundingBox */
void orc_pos_bounds(orc_grid* g, float out[6]);

int orc_update_apron(orc_grid* g, int chan, double boundval);

/* Compute(effect, chan, iterations, (p1,p2,p3), bUpdateApron, skipOverAprons,
 * boundval) (VG.cpp:4534-4558) for the operators below, numbered as the
 * reference's FUNC_* ids (VG.h:201-204) */
enum { ORC_FUNC_FILL_F = 110, ORC_FUNC_FILL_C = 111, ORC_FUNC_FILL_C4 = 112, ORC_FUNC_SMOOTH = 113 };
int orc_compute(orc_grid* g, int effect, int chan, int iterations, const float params[3], int update_apron,
                int skip_over_aprons, double boundval);

/* readback of a channel in the native brick-major layout:
 * slot s, padded local (lx,ly,lz), component c ->
 *   out[((s*P + lz)*P + ly)*P + lx)*ncomp + c],  P = brick + 2*apron */
int64_t orc_channel_size(const orc_grid* g, int chan);   /* number of doubles */
int orc_read_channel(const orc_grid* g, int chan, double* out, int64_t cap);
int orc_write_channel(orc_grid* g, int chan, const double* in, int64_t count);

/* host CPU topology (VG.cpp:2766-2855): ActivateSpace for every point, root
 * grows through Reparent.  Returns the number of leaves, or -1. */
int orc_activate_space_cpu(int levels, const int* logdim, int n, const float* pos,
                           int stride_floats, const float orig[3], int32_t* leaf_pos_out,
                           int cap, int* root_level_out);

/* dense (single-threaded) timing helper for the CPU baseline */
double orc_now_seconds(void);

#ifdef __cplusplus
}
#endif
#endif
