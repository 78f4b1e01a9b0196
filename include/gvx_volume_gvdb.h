/*
 * gvx_volume_gvdb.h -- nvdb::VolumeGVDB for the point -> sparse-volume path,
 * implemented over the libgvx C ABI (gvx.h).
 *
 * The class keeps the reference's names, argument order and argument meaning
 * (gvdb_volume_gvdb.h, VG.h below) for the methods of its point path, so that
 * an application of the reference that builds volumes from points compiles
 * against this header and links libgvx_volume + libgvx instead.  The types it
 * needs (Vector3DF/I, Vector4DF, DataPtr, Node) are declared here with the
 * reference's field names and layouts (Node: 64 bytes, gvdb_node.h:27-40).
 *
 * Differences a caller can notice:
 *   - errors throw nvdb::GvxError (status code + text) where the reference
 *     prints and exits;
 *   - node pools are read back on demand: a Node* from getNode / getNodeAtLevel
 *     points into a host copy that is refreshed after the next topology or
 *     atlas change, and writing through it changes nothing on the device;
 *   - SetCudaDevice ignores a CUcontext (the library uses the device's primary
 *     context).
 * Methods with no reference counterpart are grouped at the end.
 */
#ifndef GVX_VOLUME_GVDB_H
#define GVX_VOLUME_GVDB_H

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "gvx.h"

/* channel types, filter and border modes, as gvdb_types.h:70-85 */
#ifndef T_UCHAR
#define T_UCHAR 0
#define T_UCHAR3 1
#define T_UCHAR4 2
#define T_FLOAT 3
#define T_FLOAT3 4
#define T_FLOAT4 5
#endif
#ifndef F_LINEAR
#define F_LINEAR 0
#define F_POINT 1
#define F_BORDER 0
#define F_CLAMP 1
#define F_WRAP 2
#endif
#ifndef ID_UNDEFL
#define ID_UNDEFL 0xFFFFFFFF
#define ID_UNDEF64 0xFFFFFFFFFFFFFFFFull
#endif
/* Compute operators, as gvdb_volume_gvdb.h:201-204 */
#ifndef FUNC_FILL_F
#define FUNC_FILL_F GVX_FUNC_FILL_F
#define FUNC_FILL_C GVX_FUNC_FILL_C
#define FUNC_FILL_C4 GVX_FUNC_FILL_C4
#define FUNC_SMOOTH GVX_FUNC_SMOOTH
#endif
/* auxiliary buffer ids of getAux, as gvdb_volume_gvdb.h:219-258 */
#ifndef AUX_PNTPOS
#define AUX_PNTPOS 0
#define AUX_PNTCLR 1
#define AUX_PNODE 2
#define AUX_PNTVEL 44
#endif

namespace nvdb {

typedef unsigned char uchar;
typedef int64_t slong;
typedef uint64_t uint64;
typedef uint32_t uint32;
typedef unsigned int uint;
typedef unsigned long long CUdeviceptr;  // the driver API's device pointer type

struct Vector3DF {
    float x, y, z;
    Vector3DF() : x(0), y(0), z(0) {}
    Vector3DF(float a, float b, float c) : x(a), y(b), z(c) {}
    void Set(float a, float b, float c) { x = a; y = b; z = c; }
};

struct Vector3DI {
    int x, y, z;
    Vector3DI() : x(0), y(0), z(0) {}
    Vector3DI(int a, int b, int c) : x(a), y(b), z(c) {}
    void Set(int a, int b, int c) { x = a; y = b; z = c; }
};

struct Vector4DF {
    float x, y, z, w;
    Vector4DF() : x(0), y(0), z(0), w(0) {}
    Vector4DF(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
};

/* the reference's DataPtr fields a point path uses (gvdb_allocator.h:35-55):
 * element counts, stride, subdim.x = byte offset of the xyz inside an
 * element, host and device pointers.  own_cpu / own_gpu record what
 * AllocData allocated (FreeData releases only that). */
struct DataPtr {
    uint64 max = 0, lastEle = 0, usedNum = 0, size = 0, stride = 0;
    Vector3DI subdim;
    char* cpu = nullptr;
    CUdeviceptr gpu = 0;
    bool own_cpu = false, own_gpu = false;
};

struct alignas(16) Node {
    uchar mLev, mFlags, mPriority, pad;
    Vector3DI mPos;    // index-space position
    Vector3DI mValue;  // atlas voxel of the interior corner (leaves)
    Vector3DF mVRange;
    uint64 mParent;
    uint64 mChildList;
    uint64 mMask;
};
static_assert(sizeof(Node) == 64, "Node is 64 bytes");
static_assert(sizeof(Vector3DF) == 12, "point arrays are packed float3");

class GvxError : public std::runtime_error {
public:
    GvxError(int status, const std::string& what) : std::runtime_error(what), status(status) {}
    int status;
};

class VolumeGVDB {
public:
    VolumeGVDB();
    ~VolumeGVDB();
    VolumeGVDB(const VolumeGVDB&) = delete;
    VolumeGVDB& operator=(const VolumeGVDB&) = delete;

    // ---- setup (VG.h:325-327)
    void SetCudaDevice(int devid, void* ctx = nullptr);
    void Initialize();
    void Clear();

    // ---- topology (VG.h:387-432)
    void Configure(int r4, int r3, int r2, int r1, int r0);
    void Configure(int levs, int* r, int* ncnt, bool use_masks = false);
    void SetChannelDefault(int cx, int cy, int cz);
    void SetApron(int n);
    void AddChannel(uchar chan, int dt, int apron, int filter = F_LINEAR, int border = F_CLAMP,
                    Vector3DI axiscnt = Vector3DI(0, 0, 0));
    void FillChannel(uchar chan, Vector4DF val);
    void ClearChannel(uchar chan);
    void FinishTopology(bool pCommitPool = true, bool pComputeBounds = true);
    void UpdateAtlas();
    void UpdateApron();
    void UpdateApron(uchar chan, float boundval = 0.0f, bool changeCtx = true);
    void UpdateApronFaces(uchar chan);
    void UpdateNeighbors();
    void AtlasRetrieveBrickXYZ(uchar channel, Vector3DI minimumCorner, DataPtr& dest);
    void RebuildTopology(int pNumPnts, float pRadius, Vector3DF pOrig);
    void RebuildTopologyCPU(int pNumPnts, Vector3DF pOrig, Vector3DF* pPos);
    slong ActivateSpace(Vector3DF pos);
    void AccumulateTopology(int pNumPnts, float pRadius, Vector3DF pOrig, int iDepth = 1);
    void RequestFullRebuild(bool tf);
    int GetLevels() { return levels_; }

    // ---- data (VG.h:532-542)
    void AllocData(DataPtr& ptr, int cnt, int stride, bool bCPU = true);
    void FreeData(DataPtr& ptr);
    void RetrieveData(DataPtr ptr);
    void CommitData(DataPtr ptr);
    void CommitData(DataPtr& ptr, int cnt, char* cptr, int offs, int stride);
    void SetDataCPU(DataPtr& dat, int cnt, char* cptr, int offs, int stride);
    void SetDataGPU(DataPtr& dat, int cnt, CUdeviceptr gptr, int offs, int stride);
    char* getDataCPU(DataPtr ptr, int n, int stride) { return ptr.cpu + (size_t)n * stride; }
    void SetPoints(DataPtr& pntpos, DataPtr& pntvel, DataPtr& clrpos);
    void InsertPoints(int num_pnts, Vector3DF trans, bool bPrefix = false);
    void InsertPointsSubcell(int subcell_size, int num_pnts, float pRadius, Vector3DF trans, int& pSCPntsLength);
    void ScatterDensity(int num_pnts, float radius, float amp, Vector3DF trans, bool expand = true,
                        bool avgColor = false);
    void GatherDensity(int subcell_size, int num_pnts, float radius, Vector3DF trans, int& pSCPntsLength,
                       int chanDensity, int chanClr, bool bAccum = false);
    void GatherLevelSet(int subcell_size, int num_pnts, float radius, Vector3DF trans, int& pSCPntsLength,
                        int chanLevelset, int chanClr, bool bAccum = false);
    void InsertPointsSubcell_FP16(int subcell_size, int num_pnts, float radius, Vector3DF trans,
                                  int& pSCPntsLength);
    void GatherLevelSet_FP16(int subcell_size, int num_pnts, float radius, Vector3DF trans, int& pSCPntsLength,
                             int chanLevelSet, int chanClr);
    void ConvertAndTransform(DataPtr& psrc, char psrcbits, DataPtr& pdest, char pdestbits, int num_pnts,
                             Vector3DF wMin, Vector3DF wDelta, Vector3DF trans, Vector3DF scal);
    DataPtr& getAux(int id);

    // ---- files (VG.h:374-375): VBX 1.11
    bool LoadVBX(const std::string fname, int force_maj = 0, int force_min = 0);
    void SaveVBX(const std::string fname);

    // ---- compute (VG.h:355): FUNC_FILL_F/C/C4 and FUNC_SMOOTH
    void Compute(int effect, uchar channel, int num_iterations, Vector3DF parameters, bool bUpdateApron,
                 bool skipOverAprons, float boundval = 0.0f);

    // ---- queries (VG.h:453, 637-643)
    uint64 getNumNodes(int lev) { return getNumTotalNodes(lev); }
    uint64 getNumUsedNodes(int lev);
    uint64 getNumTotalNodes(int lev);
    Node* getNodeAtLevel(int n, int lev);
    Node* getNode(int grp, int lev, slong ndx);
    Node* getNode(slong nodeid);
    // bounds of the last ComputeBounds (VG.cpp:1792-1816, run by FinishTopology):
    // getWorldMin/Max (VG.cpp:5804-5810) and VolumeBase's getVolMin/Max return mObjMin/mObjMax;
    // getVoxRes/getVoxResMax stand in for the public members mVoxRes/mVoxResMax
    Vector3DF getWorldMin();
    Vector3DF getWorldMax();
    Vector3DF getVolMin() { return getWorldMin(); }
    Vector3DF getVolMax() { return getWorldMax(); }
    Vector3DF getVoxRes();
    Vector3DF getVoxResMax();

    // ---- tree shape (VG.h:592-621) and host-side tree queries (VG.h:449-470) on the pools and
    //      child lists read back on demand: getChildNode/isOn (VG.cpp:2787-2796, 3079-3092),
    //      getChildRefAtBit/getChildAtBit (3052-3076), getPosInNode (2858-2875),
    //      getNodeAtPoint/isActive/getValue (4650-4755)
    int getRes(int lev) { return (lev >= 0 && lev < levels_) ? (1 << logdim_[lev]) : 0; }
    Vector3DI getRes3DI(int lev)
    {
        const int r = getRes(lev);
        return Vector3DI(r, r, r);
    }
    Vector3DI getRange(int lev);
    Vector3DF getCover(int lev)
    {
        const Vector3DI r = getRange(lev);
        return Vector3DF((float)r.x, (float)r.y, (float)r.z);
    }
    int getBitPos(int lv, Vector3DI pos)
    {
        const int res = getRes(lv);
        return (pos.z * res + pos.y) * res + pos.x;
    }
    bool isLeaf(slong nodeid) { return (((uint64)nodeid >> 8) & 0xFF) == 0; }
    uint64 getChildNode(slong nodeid, uint b);
    uint64 getChildRefAtBit(Node* curr, uint b);
    Node* getChildAtBit(Node* curr, uint b);
    bool isOn(slong nodeid, uint32 b);
    bool getPosInNode(slong curr_id, Vector3DI pos, uint32& bit);
    uint64 getNodeAtPoint(uint64 nodeid, Vector3DF pos);
    bool isActive(Vector3DI wpos);
    bool isActive(Vector3DI wpos, slong nodeid);
    // `atlas`: channel 0 in the reference's dense atlas layout (gvx_read_channel_dense)
    float getValue(slong nodeid, Vector3DF pos, float* atlas);
    // no reference counterpart (the reference keeps mRoot protected): Elem id of the root node
    uint64 getRootNodeID();

    // ---- no reference counterpart
    // TRILINEAR / CUBIC splat of weight (and velocity) into channels (gvx_splat)
    void Splat(int mode, int num_pnts, float radius, Vector3DF trans, int chanDensity, int chanVel,
               bool bAccum = false);
    // its adjoint (gvx_splat_backward); all buffers device memory
    void SplatBackward(int mode, int num_pnts, float radius, Vector3DF trans, CUdeviceptr dL_drho,
                       CUdeviceptr grad_pos, CUdeviceptr grad_w, CUdeviceptr grad_r);
    // per-point weight and radius (device arrays of num_pnts floats, or 0)
    void SetPointAttribs(CUdeviceptr weight, CUdeviceptr radius);
    gvx_grid* getHandle() { return g_; }

private:
    void check(gvx_status st) const;
    void need_grid();
    void topology_changed() { gen_++; }
    Node* mirror(int lev, uint64 ndx);
    const uint64* child_list(uint64 listid);  // the res^3 entries of a child list (group 1)

    gvx_grid* g_ = nullptr;
    int dev_ = 0;
    int levels_ = 0;
    int apron_ = 1;
    bool apron_set_ = false;
    uint64 gen_ = 1;
    std::vector<std::vector<Node>> mirror_;
    std::vector<uint64> mirror_gen_;
    std::vector<std::vector<uint64>> clmirror_;
    std::vector<uint64> clmirror_gen_;
    int logdim_[GVX_MAX_LEVELS] = {};
    DataPtr pos_, vel_, clr_, pnode_;
    int last_insert_n_ = 0;
    int chan_type_[32];  // the type each AddChannel gave, -1 for none
    float last_trans_[3] = {0, 0, 0};
    uint64 pnode_gen_ = 0;
};

}  // namespace nvdb

#endif
