/*
 * gvx.h -- C ABI of the GB300 point -> sparse-volume engine (libgvx.so).
 *
 * Drop-in boundary for the GVDB point path.  Each entry point replaces one
 * VolumeGVDB method of the reference (dunyazad/gvdb-voxels, GVDB Voxels
 * 1.1.1); the citation beside each declaration is the method it stands in for
 * (file:line relative to the reference project):
 *   VG.h   = source/gvdb_library/src/gvdb_volume_gvdb.h
 *   VG.cpp = source/gvdb_library/src/gvdb_volume_gvdb.cpp
 *
 * Conventions
 *  - Every call returns gvx_status (0 = GVX_OK).  Nothing ever calls exit();
 *    gvx_last_error() returns a thread-local description of the last failure.
 *  - Point buffers are BORROWED device pointers (as SetDataGPU/SetPoints alias
 *    caller memory, VG.cpp:4872-4908); the library never frees them.
 *  - All device work is ordered on the grid's stream (gvx_set_stream); calls
 *    that return counts to the host synchronise that stream.
 *  - Channel data lives in HBM in brick-major order: atlas slot s (the atlas
 *    brick index (z*sy + y)*sx + x of the reference) holds P^3 voxels,
 *    P = brick + 2*apron, x fastest.  Node mValue and the atlas map keep the
 *    reference's atlas voxel coordinates, so gvx_read_channel_dense returns the
 *    reference's 3D-array layout byte for byte.
 */
#ifndef GVX_H
#define GVX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gvx_grid gvx_grid;
typedef int gvx_status;

#define GVX_OK 0
#define GVX_ERR_INVALID_ARG 1
#define GVX_ERR_NOT_CONFIGURED 2
#define GVX_ERR_CAPACITY 3
#define GVX_ERR_DEVICE 4
#define GVX_ERR_TIMEOUT 5
#define GVX_ERR_UNSUPPORTED 6
#define GVX_ERR_DEPTH 7
#define GVX_ERR_STATE 8
#define GVX_ERR_IO 9

/* channel types: gvdb_types.h:70-78 */
#define GVX_T_UCHAR 0
#define GVX_T_UCHAR4 2
#define GVX_T_FLOAT 3
#define GVX_T_FLOAT3 4
#define GVX_T_FLOAT4 5

/* topology modes */
#define GVX_TOPO_AUTO 0       /* RebuildTopology state machine, VG.cpp:1181-1218 */
#define GVX_TOPO_FULL 1       /* RequestFullRebuild(true) then RebuildTopology, VG.h:432 */
#define GVX_TOPO_ACCUMULATE 2 /* AccumulateTopology, VG.cpp:1158-1178 */

/* splat modes of gvx_splat */
#define GVX_SPLAT_TRILINEAR 0 /* cloud-in-cell into the 8 voxels around a point (no reference counterpart) */
#define GVX_SPLAT_CUBIC 1     /* Monaghan M4 cubic spline, support R = 2h (no reference counterpart) */

#define GVX_NODE_BYTES 64 /* Node, gvdb_node.h:27-40 */
#define GVX_MAX_LEVELS 10 /* tree levels a grid can have */

typedef struct gvx_info {
    int levels;
    int logdim[10];
    int brick_res;         /* voxels per brick side, res[0] */
    int apron;
    int root_level;        /* -1 before the first topology */
    int top_lev;           /* VDBInfo.top_lev */
    int64_t node_count[10];/* getNumTotalNodes(level) */
    int64_t used_leaves;   /* getNumUsedNodes(0) */
    int atlas_subdim[3];   /* bricks per atlas axis */
    int atlas_res[3];      /* voxels per atlas axis */
    int channels;
    int last_rebuild;      /* 1 full, 2 incremental, 0 no change */
    int root_pos[3];
    float bbox_min[3];     /* getBoundMin(), posMin after GetBoundingBox */
    float bbox_max[3];
    float obj_min[3];      /* ComputeBounds (VG.cpp:1792-1816) of the last FinishTopology: */
    float obj_max[3];      /*   mObjMin/mObjMax (= mVoxMin/mVoxMax), seeded by pool node 0 */
    float vox_res[3];      /* mVoxRes = obj_max - obj_min */
    float vox_res_max[3];  /* mVoxResMax: largest mVoxRes since Configure */
    int64_t planned_builds;/* full RebuildTopology calls that ran under the plan of the previous
                              full build (one host wait), since the grid was created */
} gvx_info;

const char* gvx_last_error(void);
const char* gvx_version(void);

/* lifecycle: SetCudaDevice + Initialize (VG.h:325-326) */
gvx_status gvx_create(int device, gvx_grid** out);
gvx_status gvx_destroy(gvx_grid* g);
/* explicit stream for every launch (the reference launches on the NULL stream) */
gvx_status gvx_set_stream(gvx_grid* g, void* cuda_stream);
gvx_status gvx_sync(gvx_grid* g);

/* Configure(int levs, int* r, int* ncnt) (VG.h:388, VG.cpp:2380-2434);
 * logdim[0] is the leaf (brick) level.  init_counts may be NULL. */
gvx_status gvx_configure(gvx_grid* g, int levels, const int* logdim, const int* init_counts);
/* SetChannelDefault (VG.h:390) */
gvx_status gvx_set_channel_default(gvx_grid* g, int cx, int cy, int cz);
/* AddChannel (VG.h:392, VG.cpp:2437-2453); apron 0 or 1 */
gvx_status gvx_add_channel(gvx_grid* g, int chan, int type, int apron);
/* ClearChannel / FillChannel (VG.h:393-395) */
gvx_status gvx_clear_channel(gvx_grid* g, int chan);
gvx_status gvx_fill_channel(gvx_grid* g, int chan, const float value[4]);

/* SetPoints (VG.h:541, VG.cpp:4900-4908) + SetDataGPU (VG.cpp:4872-4880):
 * borrowed device pointers, byte offset and byte stride per point.
 * vel and clr may be NULL; clr holds 4 bytes (uchar4) per point.  All
 * pointers, offsets and strides 4-byte aligned. */
gvx_status gvx_set_points(gvx_grid* g, int n, const void* pos, int pos_offset, int pos_stride,
                          const void* vel, int vel_offset, int vel_stride,
                          const void* clr, int clr_offset, int clr_stride);
/* per-point FP32 weight and splat radius for gvx_splat (no reference counterpart;
 * NULL = weight 1 / the call's radius) */
gvx_status gvx_set_point_attribs(gvx_grid* g, const float* weight, const float* radius);
/* CommitData of host points (VG.cpp:532-538): copies n host points (and optional
 * velocities, weights, radii) into library-owned device buffers and binds them
 * as by gvx_set_points.  Strides are in bytes.  The copies are asynchronous:
 * the host arrays may be reused once the grid's stream has passed the next call
 * that takes points (gvx_rebuild_topology, gvx_insert_points, a splat), or after
 * gvx_sync.  (The copies run on a side stream into one of two buffer sets, filled
 * in turn, after the work queued before the previous commit: a commit issued
 * while the previous frame still runs overlaps it.  Those calls, and
 * gvx_insert_points_subcell for the positions, make the grid's stream wait for
 * the copies.) */
gvx_status gvx_commit_points_host(gvx_grid* g, int n, const void* pos, int pos_stride,
                                  const void* vel, int vel_stride, const float* weight,
                                  const float* radius);

/* RebuildTopology (VG.h:429, VG.cpp:1181-1218) with mode GVX_TOPO_AUTO/FULL,
 * AccumulateTopology (VG.h:431) with GVX_TOPO_ACCUMULATE (min_depth = iDepth).
 * A GVX_TOPO_FULL build with the point count and radius of the grid's previous full
 * build (and no origin) runs under that build's plan: queued whole, one host wait
 * instead of two, the same result (checked; rebuilt without the plan when the points
 * left its key space or root or outgrew its pools' capacities, 25% over the counts
 * it was made from).  gvx_info.planned_builds counts these. */
gvx_status gvx_rebuild_topology(gvx_grid* g, int n, float radius, const float orig[3], int mode,
                                int min_depth);
/* RequestFullRebuild (VG.h:432) */
gvx_status gvx_request_full_rebuild(gvx_grid* g, int on);
/* FinishTopology (VG.h:405, VG.cpp:1579-1593): commits the space activated
 * by gvx_activate_space / gvx_rebuild_topology_cpu to the device, then the
 * bounds of the active leaves */
gvx_status gvx_finish_topology(gvx_grid* g);
/* FinishTopology(pCommitPool, pComputeBounds): ComputeBounds only when
 * compute_bounds != 0; the host-activated space is committed either way
 * (the device pools are the tree) */
gvx_status gvx_finish_topology_ex(gvx_grid* g, int commit_pool, int compute_bounds);
/* Clear (VG.h:327, VG.cpp:2487-2503): empty tree, next rebuild full */
gvx_status gvx_clear(gvx_grid* g);
/* ActivateSpace(Vector3DF) (VG.h:398, VG.cpp:2768-2855) and
 * RebuildTopologyCPU (VG.h:430, VG.cpp:1220-1227): the reference's host-side
 * topology, one point at a time on the CPU (positions truncated to integers),
 * on a host copy of the tree that FinishTopology commits: nodes are created in
 * the reference's order (the leaf covering the point and its ancestors;
 * Reparent grows the root upward), with mFlags 1.  node_id receives the leaf's
 * id when it existed already, ID_UNDEFL (0xFFFFFFFF) when it is new.  A tree
 * that needs more levels than configured makes FinishTopology fail with
 * GVX_ERR_DEPTH.  host_pos: n float3, host memory. */
gvx_status gvx_activate_space(gvx_grid* g, const float pos[3], uint64_t* node_id);
gvx_status gvx_rebuild_topology_cpu(gvx_grid* g, int n, const float orig[3], const float* host_pos);
/* UpdateAtlas (VG.h:406, VG.cpp:2630-2704) */
gvx_status gvx_update_atlas(gvx_grid* g);

/* InsertPoints (VG.h:542, VG.cpp:5219-5267): brick of every point, points
 * grouped by brick for the splats.  If pnode_out is not NULL it receives the
 * leaf pool index of every point (0xFFFFFFFF if none), host memory. */
gvx_status gvx_insert_points(gvx_grid* g, int n, const float trans[3], int32_t* pnode_out);
/* ScatterDensity (VG.h:555, VG.cpp:5624-5660, kernels PT.cuh:525-573, 610-642):
 * (1 - d^2/r^2)^3 at the point's voxel and, with expand, its 6 face
 * neighbours, summed into channel 0 of the point's own brick (apron included),
 * without the reference's racy read-modify-write.  With point colours bound
 * (gvx_set_points clr), each point also colours the interior voxel it lies in:
 * avg_color != 0 -> channel 1 = (integer mean of r, g, b, 255) over the
 * voxel's points; avg_color == 0 -> channel 3 = one point's colour (the
 * highest index; the reference's writers race) -- unless an avg_color call
 * ever ran on this grid, after which, as in the reference, no colour is
 * written.  The colour channel must be a 4-byte channel. */
gvx_status gvx_scatter_density(gvx_grid* g, int n, float radius, float amp, const float trans[3],
                               int expand, int avg_color);
/* InsertPointsSubcell (VG.h:551, VG.cpp:4971-5092): every point joins each
 * subcell (size `subcell`, dividing the brick size) of an active brick that
 * its box [(int(p-r)/s)s, (int(p+1+r)/s)s] touches.  sc_len receives the
 * number of (point, subcell) entries, as pSCPntsLength.  Needs UpdateAtlas
 * after the topology build.  Points with z == NOHIT (1e10) are skipped. */
gvx_status gvx_insert_points_subcell(gvx_grid* g, int subcell, int n, float radius,
                                     const float trans[3], int* sc_len);
/* GatherDensity / GatherLevelSet (VG.h:556-557, VG.cpp:5318-5373): every
 * interior voxel v of every active brick takes max(R - |p - v|) (density,
 * start 0) or min(|p - v| - R) (level set, start 3) over the points listed in
 * its subcell by the last InsertPointsSubcell (same subcell size), starting
 * from the old value with accum.  chan is a T_FLOAT channel; chan_clr a
 * T_UCHAR4 channel or -1: it receives the mean colour of the listed points
 * when SetPoints bound colours.  GatherDensity does nothing when sc_len is 0,
 * as in the reference; n and trans are unused, as in the reference. */
gvx_status gvx_gather_density(gvx_grid* g, int subcell, int n, float radius, const float trans[3],
                              int sc_len, int chan_density, int chan_clr, int accum);
gvx_status gvx_gather_levelset(gvx_grid* g, int subcell, int n, float radius, const float trans[3],
                               int sc_len, int chan_levelset, int chan_clr, int accum);
/* InsertPointsSubcell_FP16 (VG.h:552, VG.cpp:5094-5190): the subcell lists of
 * gvx_insert_points_subcell, each entry's position kept as 16-bit fractions
 * (w - mPosMin) / mPosRange * 65535 of the last topology build's bounding box
 * (gvx_info bbox_min / bbox_max), half the bytes per entry.  The point
 * velocities the reference also quantises are read by no kernel and are not
 * stored. */
gvx_status gvx_insert_points_subcell_fp16(gvx_grid* g, int subcell, int n, float radius,
                                          const float trans[3], int* sc_len);
/* GatherLevelSet_FP16 (VG.h:558, VG.cpp:5375-5401, kernel PT.cuh:775-813):
 * every interior voxel v of every active brick = min(3, min over the listed
 * points of |p - v| - R), p read back as q / 65535 * range + min; no
 * accumulation.  When the lists hold colours and chan_clr >= 0, chan_clr (any
 * 4-byte channel, possibly chan_levelset) then receives the inverse-distance
 * colour sum of the reference: sum of colour / |p - v|, each component * 255
 * truncated and added at byte offsets (carries included).  n, trans and
 * sc_len are accepted as the reference's arguments; the lists hold the rest. */
gvx_status gvx_gather_levelset_fp16(gvx_grid* g, int subcell, int n, float radius, const float trans[3],
                                    int sc_len, int chan_levelset, int chan_clr);
/* SaveVBX / LoadVBX (VG.h:374-375, VG.cpp:1626-1768 / 507-686): the VBX
 * file (GVDB_FILESPEC.txt, version 1.11 written) with the field order those
 * functions use: header, one grid of topology type 2 (node pools and child
 * lists of every level) and atlas layout 0 (each channel's dense atlas, slice
 * by slice; FLOAT3 voxels 12 bytes on file).  Channels must be numbered
 * 0..n-1.  LoadVBX configures the grid from the file (levels, dimensions,
 * apron, atlas brick counts), takes the pools as they are, adds the channels,
 * runs UpdateAtlas and uploads the atlas; it reads every grid of the file in
 * turn, leaving the last, and the next RebuildTopology is a full one.
 * force_major / force_minor > 0 override the file's version, as the
 * reference's arguments do.  GVX_ERR_IO when the file cannot be opened,
 * written or parsed. */
gvx_status gvx_save_vbx(gvx_grid* g, const char* path);
gvx_status gvx_load_vbx(gvx_grid* g, const char* path, int force_major, int force_minor);

/* ConvertAndTransform (VG.h:559, VG.cpp:5668-5682, kernel PT.cuh:120-142):
 * device points src (three uint16 per point when src_bits is 2, three floats
 * when 4, densely packed) -> device float3 dst = (wmin + p * wdelta) * scal +
 * trans, each multiply-add one FMA.  dst is always float3, whatever dst_bits
 * says (as the reference writes it). */
gvx_status gvx_convert_and_transform(gvx_grid* g, const void* src, int src_bits, void* dst, int dst_bits, int n,
                                     const float wmin[3], const float wdelta[3], const float trans[3],
                                     const float scal[3]);
/* TRILINEAR / CUBIC splat of weight (and velocity*weight into a FLOAT3/FLOAT4
 * channel) of the points that lie in active bricks; chan_vel may be -1.
 * Every voxel of each active brick, apron included, receives the sum of the
 * contributions at its index-space position, so the apron comes out as the
 * exact copy UpdateApron(chan, 0) would make (a following UpdateApron with
 * boundary value 0 has nothing left to do).  Without accum the bricks start
 * from 0 and apron voxels that no brick owns are set to 0; with accum the
 * contributions are added to the previous values.  The sum of every voxel is
 * formed in the points' sorted order: results are deterministic. */
gvx_status gvx_splat(gvx_grid* g, int mode, int n, float radius, const float trans[3],
                     int chan_density, int chan_vel, int accum);
/* Adjoint of gvx_splat's density (no counterpart in the reference).  dL_drho
 * holds dL/drho in the density channel's brick-major layout (device memory;
 * only interior voxels are read, an apron voxel being a copy).  Writes, in the
 * points' original order and to device memory, dL/dp (3 floats per point),
 * dL/dw and, when grad_r is not NULL, dL/dR per point (the CUBIC radius;
 * the bound per-point radii if any).  Points outside the active bricks get 0.
 * Uses the grouping of the forward splat, re-sorting if the points changed. */
gvx_status gvx_splat_backward(gvx_grid* g, int mode, int n, float radius, const float trans[3],
                              const float* dL_drho, float* grad_pos, float* grad_w, float* grad_r);
/* gvx_splat_backward with flags: GVX_BWD_RECOMPUTE recomputes the points' sorted-key
 * permutation from the positions (re-key, re-sort, octant partition) instead of
 * reusing the forward's stored grouping; the gradients are identical. */
#define GVX_BWD_RECOMPUTE 1
gvx_status gvx_splat_backward_ex(gvx_grid* g, int mode, int n, float radius, const float trans[3],
                                 const float* dL_drho, float* grad_pos, float* grad_w, float* grad_r, int flags);
/* UpdateApron(chan, boundval) / UpdateApron() (VG.h:407-408, VG.cpp:4411-4457) */
gvx_status gvx_update_apron(gvx_grid* g, int chan, float boundval);
gvx_status gvx_update_apron_all(gvx_grid* g);
/* UpdateApronFaces (VG.h:409, VG.cpp:4461-4496, kernel OP.cuh:27-63): float
 * channels only; per brick and face neighbour (-x, -y, -z), the apron voxels
 * across the shared face take each other's interior layer.  Edges, corners
 * and faces without a neighbour keep their values. */
gvx_status gvx_update_apron_faces(gvx_grid* g, int chan);
/* UpdateNeighbors (VG.h:448, VG.cpp:2527-2556): the face-neighbour table of
 * UpdateApronFaces.  Every topology build makes the 26-neighbour table here,
 * so this only checks that a topology exists. */
gvx_status gvx_update_neighbors(gvx_grid* g);

/* Compute(effect, channel, num_iterations, parameters, bUpdateApron,
 * skipOverAprons, boundval) (VG.h:355, VG.cpp:4532-4558) for the operators
 * the point path uses (FUNC_* ids VG.h:201-204, bodies OP.cuh:352-400),
 * params = (p1, p2, p3):
 *   GVX_FUNC_FILL_F   float  = p1 (p3 < 0: sum over the axes of sin(12 X / (30 pi)))
 *   GVX_FUNC_FILL_C   uchar  = p1 truncated, saturating at 0 and 255
 *   GVX_FUNC_FILL_C4  uchar4 = CLR2INT(p1, p2, p3, 1): the components * 255 ORed
 *   GVX_FUNC_SMOOTH   float  = (p1 c + sum of the 6 face neighbours) / (p1 + 6) + p2
 * As in the reference, each operator's own indexing picks its voxels and
 * skip_over_aprons only sizes the launch: the fills write the atlas voxels
 * whose coordinates all lie in [1, hi) with hi = the atlas resolution, or
 * min(8 ceil(bricks * brick / 8) + 1, atlas resolution) when skip_over_aprons;
 * FUNC_SMOOTH writes every brick interior, from neighbours read before any
 * write (in the brick's apron; with apron 0, atlas neighbours, 0 outside the
 * atlas).  update_apron != 0 runs UpdateApron(chan, boundval) after every
 * iteration.  An operator the channel's type has no body for ->
 * GVX_ERR_UNSUPPORTED. */
#define GVX_FUNC_FILL_F 110
#define GVX_FUNC_FILL_C 111
#define GVX_FUNC_FILL_C4 112
#define GVX_FUNC_SMOOTH 113
gvx_status gvx_compute(gvx_grid* g, int effect, int chan, int iterations, const float params[3], int update_apron,
                       int skip_over_aprons, float boundval);

/* RadixSortByByte (VG.h:423, VG.cpp:904-928): stable ascending sort of n
 * (key, value) pairs by the low `bits` (1..32) bits of 32-bit keys -- the
 * onesweep radix sort the topology uses for brick keys.  Device pointers; the
 * inputs are not modified; the grid owns the scratch memory (allocated on
 * first use, kept for later calls).  Stream-ordered on the grid's stream. */
gvx_status gvx_radix_sort(gvx_grid* g, const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                          uint32_t* vals_out, uint32_t n, int bits);

/* gvx_radix_sort without any device allocation -- no counterpart in the
 * reference.  For callers that must not allocate device memory (a host that
 * hands the library a fixed memory budget, a plugin whose host owns all
 * device allocations): same result as gvx_radix_sort, but the scratch lives in
 * a static __device__ array inside libgvx, so the call allocates nothing.
 * At most GVX_NOALLOC_SORT_MAX_KEYS pairs (larger n -> GVX_ERR_CAPACITY); the
 * array (about 2.4 MB) stays resident on every GPU that loads the library;
 * calls share it, so calls that overlap on the GPU race -- order them on one
 * stream.  Sorting in place is allowed (keys_out == keys_in, vals_out ==
 * vals_in); keys_out and vals_out must not overlap (GVX_ERR_INVALID_ARG).
 * Runs on the current device and the given stream (NULL = legacy default
 * stream); its first call on a device (and the first after the device's
 * context was replaced, e.g. by cudaDeviceReset) looks up the array's address,
 * so make that first call before any stream capture.  The call returns before
 * the sort runs, so it cannot report a device-side failure itself: a bounded
 * look-back wait that gave up sets a sticky flag in the array, which
 * gvx_radix_sort_noalloc_status reads. */
#define GVX_NOALLOC_SORT_MAX_KEYS (1u << 18)
gvx_status gvx_radix_sort_noalloc(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                                  uint32_t* vals_out, uint32_t n, int bits, void* stream);
/* Waits for `stream`, then reads and clears the sticky device flag of
 * gvx_radix_sort_noalloc on the current device: GVX_ERR_TIMEOUT when a call
 * since the last query had a look-back wait give up (that call's output is
 * wrong), else GVX_OK.  Allocates nothing. */
gvx_status gvx_radix_sort_noalloc_status(void* stream);

/* queries: getNumTotalNodes/getNumUsedNodes (VG.h:637-643), getBoundMin/Max */
gvx_status gvx_get_info(gvx_grid* g, gvx_info* out);
/* node pool of one level as 64-byte Node records (host memory) */
gvx_status gvx_read_nodes(gvx_grid* g, int level, void* out, int64_t cap_nodes);
/* child lists of one level (>0): res^3 uint64 Elem references per node */
gvx_status gvx_read_childlist(gvx_grid* g, int level, uint64_t* out, int64_t cap_entries);
/* atlas map: per atlas slot {pos.x, pos.y, pos.z, leaf id} */
gvx_status gvx_read_atlas_map(gvx_grid* g, int32_t* out4, int64_t cap_slots);
/* channel bytes: brick-major native layout, and the reference's dense layout */
gvx_status gvx_channel_bytes(gvx_grid* g, int chan, int64_t* bytes);
gvx_status gvx_read_channel(gvx_grid* g, int chan, void* out, int64_t cap_bytes);
gvx_status gvx_read_channel_dense(gvx_grid* g, int chan, void* out, int64_t cap_bytes);
/* type of channel chan (GVX_T_*), -1 when the channel does not exist
 * (mPool->getAtlas(chan).type, gvdb_allocator.h) */
gvx_status gvx_channel_type(gvx_grid* g, int chan, int* type);
/* device pointer of a channel (for in-HBM consumers and producers).  The
 * pointer stays the same until the atlas is reallocated (UpdateAtlas growing
 * it, or a channel re-added); the caller may write through it, so the next
 * UpdateApron of the channel always runs. */
gvx_status gvx_channel_device_ptr(gvx_grid* g, int chan, void** dev_ptr, int64_t* bytes);
/* AtlasRetrieveBrickXYZ (VG.h:412): one brick's interior (res0^3 values of the
 * channel's element size) at the brick whose interior corner is the atlas
 * voxel `corner`, into host memory with z fastest, out[(x*b + y)*b + z], the
 * order of kernelRetrieveTexXYZ (cuda_gvdb_copydata.cu:74-79) */
gvx_status gvx_retrieve_brick(gvx_grid* g, int chan, const int corner[3], void* out, int64_t cap_bytes);

/* number of kernels the library has launched on this grid (instrumentation) */
gvx_status gvx_kernel_launches(gvx_grid* g, int64_t* count);

/* device memory for hosts without a CUDA runtime of their own: the backing of
 * VolumeGVDB::AllocData / FreeData / CommitData / RetrieveData
 * (VG.h:532-535, VG.cpp:4820-4885).  gvx_memcpy is synchronous; kind is
 * GVX_COPY_H2D, GVX_COPY_D2H or GVX_COPY_D2D. */
#define GVX_COPY_H2D 0
#define GVX_COPY_D2H 1
#define GVX_COPY_D2D 2
gvx_status gvx_device_alloc(int device, size_t bytes, void** out);
gvx_status gvx_device_free(int device, void* ptr);
gvx_status gvx_memcpy(int device, void* dst, const void* src, size_t bytes, int kind);

/* ---- batched multi-grid splat (no counterpart in the reference, where each
 * VolumeGVDB splats on its own).  A batch splats many grids -- one per point
 * cloud, all configured with the same brick shape and channel kinds, each
 * with its topology, atlas and InsertPoints grouping done -- in ONE persistent
 * launch.  With GVX_BATCH_GRAPH the launch is captured in a CUDA graph and
 * replayed while no grid's buffers move (a change re-captures it); with
 * GVX_BATCH_TUNE the first call of a (GPU, brick shape, kind) times a few slab
 * heights and CTAs per SM on the live batch and caches the fastest for the
 * process.  Results are those of gvx_splat on each grid, bit for bit. */
typedef struct gvx_batch gvx_batch;
#define GVX_BATCH_GRAPH 1
#define GVX_BATCH_TUNE 2
gvx_status gvx_batch_create(int device, gvx_batch** out);
gvx_status gvx_batch_destroy(gvx_batch* b);
gvx_status gvx_batch_set_stream(gvx_batch* b, void* stream);
gvx_status gvx_batch_set_grids(gvx_batch* b, gvx_grid* const* grids, int count);
gvx_status gvx_batch_splat(gvx_batch* b, int mode, float radius, int chan_density, int chan_vel, int accum,
                           int flags);
gvx_status gvx_batch_get_tuning(gvx_batch* b, int* slab_layers, int* blocks_per_sm, float* ms);
/* Topology of every grid of the batch (no reference counterpart): per grid, what
 * gvx_rebuild_topology(radius, no origin, mode), gvx_update_atlas and
 * gvx_insert_points over its bound points do, with the same results.
 * threads == 0: staged from the calling thread -- every grid's GetBoundingBox is
 * queued, then every grid's build up to its node counts, then every grid's pools,
 * UpdateAtlas and InsertPoints -- so the host waits on each grid twice, where the
 * stream has had the other grids' launches to get there, and the grids' streams
 * overlap on the GPU.  threads > 0: the per-grid calls themselves from that many
 * host threads.  Grids that share a stream build one after another.  The first
 * failing grid's status is returned, its index in gvx_last_error(). */
gvx_status gvx_batch_topology(gvx_batch* b, float radius, int mode, int threads);
/* A whole frame of a batch (no reference counterpart; it replaces, per point cloud,
 * the loop RebuildTopology gvdb_volume_gvdb.cpp:1181-1218 -> UpdateAtlas
 * :2650-2690 -> InsertPoints :5219-5267 -> the splat with its aprons): every
 * grid's full rebuild over its bound points (topo_radius, no origin), UpdateAtlas,
 * InsertPoints, then gvx_batch_splat(mode, radius, chan_density, chan_vel, no
 * accumulation).  Results are those of the per-grid calls, bit for bit.
 * The first frame (and any frame after set_grids, a new topo_radius or rebound
 * points) runs gvx_batch_topology staged and gvx_batch_splat, and makes every
 * grid a PLAN from its build: the compact key space widened by an eighth of its
 * extent and a leaf per side, the depth and root, and each pool's capacity (count + 25% +
 * 64).  Later frames build under the plans: no host wait and no allocation
 * inside the frame, counts read by the kernels from device memory.  With
 * GVX_BATCH_GRAPH, from the second planned frame on, all grids' builds (each on
 * its grid's stream, forked from the batch stream) and the splat run as ONE
 * captured CUDA graph, replayed while no libgvx buffer has moved.  The call
 * waits for the frame (one host synchronisation) and checks every plan: a grid
 * whose points left the plan's root or key space, or outgrew a capacity, is built
 * and splatted again without it and planned anew (gvx_batch_frame_path reports
 * how many).  GVX_BATCH_TUNE as for gvx_batch_splat, on the first frame. */
gvx_status gvx_batch_frame(gvx_batch* b, float topo_radius, int mode, float radius, int chan_density, int chan_vel,
                           int flags);
/* How the last gvx_batch_frame ran: *path 0 = unplanned (staged topology, plans
 * made), 1 = planned without a graph, 2 = the captured graph replayed;
 * *rebuilt = the grids built again without a plan. */
gvx_status gvx_batch_frame_path(gvx_batch* b, int* path, int* rebuilt);

/* Test hook (no reference counterpart): one pass of the radix sort over n > 4096
 * keys with its first tile withheld, so the decoupled look-back of the second
 * tile waits for a flag that nothing sets.  The wait gives up after about two
 * seconds and the call returns GVX_ERR_TIMEOUT; the outputs are undefined, and
 * the grid and the CUDA context stay usable. */
gvx_status gvx_test_sort_withheld_tile(gvx_grid* g, const uint32_t* keys_in, const uint32_t* vals_in,
                                       uint32_t* keys_out, uint32_t* vals_out, uint32_t n);
/* The same test on gvx_radix_sort_noalloc's static scratch (4096 < n <=
 * GVX_NOALLOC_SORT_MAX_KEYS, separate input and output buffers): the call
 * returns GVX_OK at once, and gvx_radix_sort_noalloc_status then reports
 * GVX_ERR_TIMEOUT. */
gvx_status gvx_test_sort_noalloc_withheld_tile(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                                               uint32_t* vals_out, uint32_t n, void* stream);
gvx_status gvx_batch_kernel_launches(gvx_batch* b, int64_t* count);

#ifdef __cplusplus
}
#endif
#endif
