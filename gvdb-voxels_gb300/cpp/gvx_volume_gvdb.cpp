// gvx_volume_gvdb.cpp -- nvdb::VolumeGVDB (point -> sparse-volume path) over
// the libgvx C ABI.  Each method cites the reference method it stands in for
// (gvdb_volume_gvdb.cpp = VG.cpp).
#include "gvx_volume_gvdb.h"

#include <cstdio>
#include <cstring>

namespace nvdb {

VolumeGVDB::VolumeGVDB()
{
    for (int& t : chan_type_) t = -1;
}

VolumeGVDB::~VolumeGVDB()
{
    FreeData(pnode_);
    if (g_) gvx_destroy(g_);
}

void VolumeGVDB::check(gvx_status st) const
{
    if (st != GVX_OK) throw GvxError((int)st, std::string("gvx: ") + gvx_last_error());
}

void VolumeGVDB::need_grid()
{
    if (!g_) check(gvx_create(dev_, &g_));
}

// SetCudaDevice (VG.cpp:186-260): the device of every later allocation
void VolumeGVDB::SetCudaDevice(int devid, void* ctx)
{
    (void)ctx;
    if (g_ && devid != dev_) {
        gvx_destroy(g_);
        g_ = nullptr;
    }
    dev_ = devid;
}

// Initialize (VG.cpp:262-300)
void VolumeGVDB::Initialize() { need_grid(); }

// Clear (VG.cpp:2487-2503): the next RebuildTopology starts from an empty tree
// Clear (VG.cpp:2487-2503): empty tree, next rebuild full
void VolumeGVDB::Clear()
{
    need_grid();
    check(gvx_clear(g_));
    topology_changed();
}

// Configure(q4..q0) (VG.cpp:2364-2377): level 0 takes the last argument
void VolumeGVDB::Configure(int r4, int r3, int r2, int r1, int r0)
{
    int r[5] = {r0, r1, r2, r3, r4};
    Configure(5, r, nullptr);
}

// Configure(levs, r, ncnt) (VG.cpp:2380-2434); pools grow as needed, so ncnt
// (the initial pool sizes) and bitmasks change nothing here
void VolumeGVDB::Configure(int levs, int* r, int* ncnt, bool use_masks)
{
    (void)use_masks;
    need_grid();
    check(gvx_configure(g_, levs, r, ncnt));
    levels_ = levs;
    mirror_.assign(levs, std::vector<Node>());
    mirror_gen_.assign(levs, 0);
    clmirror_.assign(levs, std::vector<uint64>());
    clmirror_gen_.assign(levs, 0);
    gvx_info inf;
    check(gvx_get_info(g_, &inf));
    for (int l = 0; l < levs && l < GVX_MAX_LEVELS; l++) logdim_[l] = inf.logdim[l];
    topology_changed();
}

void VolumeGVDB::SetChannelDefault(int cx, int cy, int cz)
{
    need_grid();
    check(gvx_set_channel_default(g_, cx, cy, cz));
}

void VolumeGVDB::SetApron(int n)
{
    apron_ = n;
    apron_set_ = true;
}

// AddChannel (VG.cpp:2436-2454); filter and border modes belong to texture
// sampling, which the point path does not use
void VolumeGVDB::AddChannel(uchar chan, int dt, int apron, int filter, int border, Vector3DI axiscnt)
{
    (void)filter;
    (void)border;
    need_grid();
    if (axiscnt.x > 0 && axiscnt.y > 0 && axiscnt.z > 0)
        check(gvx_set_channel_default(g_, axiscnt.x, axiscnt.y, axiscnt.z));
    check(gvx_add_channel(g_, chan, dt, apron));
    if (chan < 32) chan_type_[chan] = dt;
    apron_ = apron;
}

// FillChannel (VG.cpp:2456-2471): all zero clears the channel; otherwise the
// FILL operator of the channel's type over the unpacked atlas (no effect on
// float3/float4 channels)
void VolumeGVDB::FillChannel(uchar chan, Vector4DF val)
{
    need_grid();
    if (val.x == 0 && val.y == 0 && val.z == 0 && val.w == 0) {
        ClearChannel(chan);
        return;
    }
    const int t = chan < 32 ? chan_type_[chan] : -1;
    const Vector3DF p(val.x, val.y, val.z);
    if (t == T_FLOAT) Compute(FUNC_FILL_F, chan, 1, p, false, false);
    else if (t == T_UCHAR) Compute(FUNC_FILL_C, chan, 1, p, false, false);
    else if (t == T_UCHAR4) Compute(FUNC_FILL_C4, chan, 1, p, false, false);
}

// LoadVBX (VG.cpp:507-686): false when the file cannot be opened, as the
// reference returns; a malformed file throws
bool VolumeGVDB::LoadVBX(const std::string fname, int force_maj, int force_min)
{
    need_grid();
    FILE* probe = fopen(fname.c_str(), "rb");
    if (!probe) return false;
    fclose(probe);
    check(gvx_load_vbx(g_, fname.c_str(), force_maj, force_min));
    gvx_info inf;
    check(gvx_get_info(g_, &inf));
    levels_ = inf.levels;
    apron_ = inf.apron;
    mirror_.assign(levels_, std::vector<Node>());
    mirror_gen_.assign(levels_, 0);
    clmirror_.assign(levels_, std::vector<uint64>());
    clmirror_gen_.assign(levels_, 0);
    for (int l = 0; l < levels_ && l < GVX_MAX_LEVELS; l++) logdim_[l] = inf.logdim[l];
    for (int c = 0; c < 32; c++) check(gvx_channel_type(g_, c, &chan_type_[c]));
    topology_changed();
    return true;
}

// SaveVBX (VG.cpp:1626-1768)
void VolumeGVDB::SaveVBX(const std::string fname)
{
    need_grid();
    check(gvx_save_vbx(g_, fname.c_str()));
}

// Compute (VG.cpp:4534-4558)
void VolumeGVDB::Compute(int effect, uchar channel, int num_iterations, Vector3DF parameters, bool bUpdateApron,
                         bool skipOverAprons, float boundval)
{
    need_grid();
    const float p[3] = {parameters.x, parameters.y, parameters.z};
    check(gvx_compute(g_, effect, channel, num_iterations, p, bUpdateApron ? 1 : 0, skipOverAprons ? 1 : 0,
                      boundval));
}

// ClearChannel (VG.cpp:1596-1603)
void VolumeGVDB::ClearChannel(uchar chan)
{
    need_grid();
    check(gvx_clear_channel(g_, chan));
}

// FinishTopology (VG.cpp:1579-1593): space activated on the host is committed
// to the device (whatever pCommitPool says: the device pools are the tree);
// ComputeBounds when pComputeBounds
void VolumeGVDB::FinishTopology(bool pCommitPool, bool pComputeBounds)
{
    need_grid();
    check(gvx_finish_topology_ex(g_, pCommitPool ? 1 : 0, pComputeBounds ? 1 : 0));
    topology_changed();
}

// ActivateSpace(Vector3DF) (VG.cpp:2768-2776): the leaf's id when it existed, else ID_UNDEFL
slong VolumeGVDB::ActivateSpace(Vector3DF pos)
{
    need_grid();
    const float p[3] = {pos.x, pos.y, pos.z};
    uint64_t id = ID_UNDEFL;
    check(gvx_activate_space(g_, p, &id));
    return (slong)id;
}

// RebuildTopologyCPU (VG.cpp:1220-1227): ActivateSpace of every point + pOrig
void VolumeGVDB::RebuildTopologyCPU(int pNumPnts, Vector3DF pOrig, Vector3DF* pPos)
{
    need_grid();
    const float o[3] = {pOrig.x, pOrig.y, pOrig.z};
    check(gvx_rebuild_topology_cpu(g_, pNumPnts, o, (const float*)pPos));
}

// UpdateAtlas (VG.cpp:2630-2704): leaves get their atlas slots (mValue)
void VolumeGVDB::UpdateAtlas()
{
    need_grid();
    check(gvx_update_atlas(g_));
    topology_changed();
}

// UpdateApron() (VG.cpp:4411-4416)
void VolumeGVDB::UpdateApron()
{
    need_grid();
    check(gvx_update_apron_all(g_));
}

// UpdateApronFaces (VG.cpp:4461-4496): face aprons between face neighbours, float channels
void VolumeGVDB::UpdateApronFaces(uchar chan)
{
    need_grid();
    check(gvx_update_apron_faces(g_, chan));
}

// UpdateNeighbors (VG.cpp:2527-2556): the neighbour table comes with every topology
void VolumeGVDB::UpdateNeighbors()
{
    need_grid();
    check(gvx_update_neighbors(g_));
}

// UpdateApron(chan, boundval) (VG.cpp:4418-4457)
void VolumeGVDB::UpdateApron(uchar chan, float boundval, bool changeCtx)
{
    (void)changeCtx;
    need_grid();
    check(gvx_update_apron(g_, chan, boundval));
}

// AtlasRetrieveBrickXYZ (VG.h:412): one brick's interior into dest.cpu, and
// into dest.gpu when the caller gave one
void VolumeGVDB::AtlasRetrieveBrickXYZ(uchar channel, Vector3DI minimumCorner, DataPtr& dest)
{
    need_grid();
    int64_t bytes = 0;
    check(gvx_channel_bytes(g_, channel, &bytes));
    gvx_info inf;
    check(gvx_get_info(g_, &inf));
    const int64_t b = inf.brick_res;
    const int64_t elem = bytes / ((int64_t)inf.atlas_res[0] * inf.atlas_res[1] * inf.atlas_res[2]);
    const int64_t need = b * b * b * elem;
    std::vector<char> tmp;
    char* out = dest.cpu;
    if (!out) {
        tmp.resize((size_t)need);
        out = tmp.data();
    }
    const int corner[3] = {minimumCorner.x, minimumCorner.y, minimumCorner.z};
    check(gvx_retrieve_brick(g_, channel, corner, out, need));
    if (dest.gpu) check(gvx_memcpy(dev_, (void*)dest.gpu, out, (size_t)need, GVX_COPY_H2D));
}

// RebuildTopology (VG.cpp:1181-1218), with its full / incremental state machine
void VolumeGVDB::RebuildTopology(int pNumPnts, float pRadius, Vector3DF pOrig)
{
    need_grid();
    const float o[3] = {pOrig.x, pOrig.y, pOrig.z};
    check(gvx_rebuild_topology(g_, pNumPnts, pRadius, o, GVX_TOPO_AUTO, 1));
    topology_changed();
}

// AccumulateTopology (VG.cpp:1158-1178)
void VolumeGVDB::AccumulateTopology(int pNumPnts, float pRadius, Vector3DF pOrig, int iDepth)
{
    need_grid();
    const float o[3] = {pOrig.x, pOrig.y, pOrig.z};
    check(gvx_rebuild_topology(g_, pNumPnts, pRadius, o, GVX_TOPO_ACCUMULATE, iDepth));
    topology_changed();
}

// RequestFullRebuild (VG.h:432)
void VolumeGVDB::RequestFullRebuild(bool tf)
{
    need_grid();
    check(gvx_request_full_rebuild(g_, tf ? 1 : 0));
}

// AllocData (VG.cpp:4820-4826): (re)allocates when missing, too small or of another stride
void VolumeGVDB::AllocData(DataPtr& ptr, int cnt, int stride, bool bCPU)
{
    if (!((ptr.cpu == nullptr && bCPU) || ptr.gpu == 0 || (uint64)cnt > ptr.max || (uint64)stride != ptr.stride))
        return;
    FreeData(ptr);
    const size_t bytes = (size_t)cnt * (size_t)stride;
    if (bCPU) {
        ptr.cpu = new char[bytes ? bytes : 1];
        ptr.own_cpu = true;
    }
    void* d = nullptr;
    check(gvx_device_alloc(dev_, bytes, &d));
    ptr.gpu = (CUdeviceptr)d;
    ptr.own_gpu = true;
    ptr.max = ptr.lastEle = ptr.usedNum = (uint64)cnt;
    ptr.stride = (uint64)stride;
    ptr.size = bytes;
    ptr.subdim.Set(0, stride, 0);
}

// FreeData (VG.cpp:4827-4832): releases what AllocData allocated
void VolumeGVDB::FreeData(DataPtr& ptr)
{
    if (ptr.own_cpu) delete[] ptr.cpu;
    if (ptr.own_gpu && ptr.gpu) gvx_device_free(dev_, (void*)ptr.gpu);
    ptr = DataPtr();
}

static size_t data_bytes(const DataPtr& p)
{
    return p.size ? (size_t)p.size : (size_t)(p.lastEle * p.stride);
}

// RetrieveData (VG.cpp:4879-4884): device -> host
void VolumeGVDB::RetrieveData(DataPtr ptr)
{
    if (!ptr.cpu || !ptr.gpu) throw GvxError(GVX_ERR_INVALID_ARG, "RetrieveData: buffer not allocated on both sides");
    check(gvx_memcpy(dev_, ptr.cpu, (const void*)ptr.gpu, data_bytes(ptr), GVX_COPY_D2H));
}

// CommitData (VG.cpp:4833-4840): host -> device
void VolumeGVDB::CommitData(DataPtr ptr)
{
    if (!ptr.cpu || !ptr.gpu) throw GvxError(GVX_ERR_INVALID_ARG, "CommitData: buffer not allocated on both sides");
    check(gvx_memcpy(dev_, (void*)ptr.gpu, ptr.cpu, data_bytes(ptr), GVX_COPY_H2D));
}

// CommitData(ptr, cnt, cpubuf, offs, stride) (VG.cpp:4841-4861)
void VolumeGVDB::CommitData(DataPtr& dat, int cnt, char* cptr, int offs, int stride)
{
    dat.cpu = cptr;
    dat.own_cpu = false;
    dat.usedNum = dat.lastEle = dat.max = (uint64)cnt;
    dat.stride = (uint64)stride;
    dat.size = (uint64)cnt * (uint64)stride;
    dat.subdim.Set(offs, stride, 0);
    if (dat.gpu == 0) throw GvxError(GVX_ERR_INVALID_ARG, "CommitData: buffer not allocated on the GPU (AllocData)");
    CommitData(dat);
}

// SetDataCPU (VG.cpp:4862-4870)
void VolumeGVDB::SetDataCPU(DataPtr& dat, int cnt, char* cptr, int offs, int stride)
{
    dat.usedNum = dat.lastEle = dat.max = (uint64)cnt;
    dat.cpu = cptr;
    dat.own_cpu = false;
    dat.stride = (uint64)stride;
    dat.size = (uint64)cnt * (uint64)stride;
    dat.subdim.Set(offs, stride, 0);
}

// SetDataGPU (VG.cpp:4871-4879): a borrowed device buffer
void VolumeGVDB::SetDataGPU(DataPtr& dat, int cnt, CUdeviceptr gptr, int offs, int stride)
{
    dat.usedNum = dat.lastEle = dat.max = (uint64)cnt;
    dat.gpu = gptr;
    dat.own_gpu = false;
    dat.stride = (uint64)stride;
    dat.size = (uint64)cnt * (uint64)stride;
    dat.subdim.Set(offs, stride, 0);
}

// SetPoints (VG.cpp:4900-4908): binds (does not copy) the point buffers; the
// xyz of point i is at gpu + i * stride + subdim.x
void VolumeGVDB::SetPoints(DataPtr& pntpos, DataPtr& pntvel, DataPtr& clrpos)
{
    need_grid();
    pos_ = pntpos;
    vel_ = pntvel;
    clr_ = clrpos;
    pos_.own_cpu = pos_.own_gpu = vel_.own_cpu = vel_.own_gpu = clr_.own_cpu = clr_.own_gpu = false;
    check(gvx_set_points(g_, (int)pntpos.lastEle, (const void*)pntpos.gpu, pntpos.subdim.x, (int)pntpos.stride,
                         pntvel.gpu ? (const void*)pntvel.gpu : nullptr, pntvel.subdim.x, (int)pntvel.stride,
                         clrpos.gpu ? (const void*)clrpos.gpu : nullptr, clrpos.subdim.x, (int)clrpos.stride));
    pnode_gen_ = 0;
}

// InsertPoints (VG.cpp:5219-5267): groups the points by brick for the splats
void VolumeGVDB::InsertPoints(int num_pnts, Vector3DF trans, bool bPrefix)
{
    (void)bPrefix;
    need_grid();
    const float t[3] = {trans.x, trans.y, trans.z};
    check(gvx_insert_points(g_, num_pnts, t, nullptr));
    last_insert_n_ = num_pnts;
    memcpy(last_trans_, t, sizeof(t));
    pnode_gen_ = 0;
}

// InsertPointsSubcell (VG.cpp:4971-5092)
void VolumeGVDB::InsertPointsSubcell(int subcell_size, int num_pnts, float pRadius, Vector3DF trans,
                                     int& pSCPntsLength)
{
    need_grid();
    const float t[3] = {trans.x, trans.y, trans.z};
    check(gvx_insert_points_subcell(g_, subcell_size, num_pnts, pRadius, t, &pSCPntsLength));
}

// ScatterDensity (VG.cpp:5624-5660)
void VolumeGVDB::ScatterDensity(int num_pnts, float radius, float amp, Vector3DF trans, bool expand, bool avgColor)
{
    need_grid();
    const float t[3] = {trans.x, trans.y, trans.z};
    check(gvx_scatter_density(g_, num_pnts, radius, amp, t, expand ? 1 : 0, avgColor ? 1 : 0));
}

// GatherDensity (VG.cpp:5318-5344)
void VolumeGVDB::GatherDensity(int subcell_size, int num_pnts, float radius, Vector3DF trans, int& pSCPntsLength,
                               int chanDensity, int chanClr, bool bAccum)
{
    need_grid();
    const float t[3] = {trans.x, trans.y, trans.z};
    check(gvx_gather_density(g_, subcell_size, num_pnts, radius, t, pSCPntsLength, chanDensity, chanClr,
                             bAccum ? 1 : 0));
}

// GatherLevelSet (VG.cpp:5348-5373)
void VolumeGVDB::GatherLevelSet(int subcell_size, int num_pnts, float radius, Vector3DF trans, int& pSCPntsLength,
                                int chanLevelset, int chanClr, bool bAccum)
{
    need_grid();
    const float t[3] = {trans.x, trans.y, trans.z};
    check(gvx_gather_levelset(g_, subcell_size, num_pnts, radius, t, pSCPntsLength, chanLevelset, chanClr,
                              bAccum ? 1 : 0));
}

// InsertPointsSubcell_FP16 (VG.cpp:5094-5190)
void VolumeGVDB::InsertPointsSubcell_FP16(int subcell_size, int num_pnts, float pRadius, Vector3DF trans,
                                          int& pSCPntsLength)
{
    need_grid();
    const float t[3] = {trans.x, trans.y, trans.z};
    check(gvx_insert_points_subcell_fp16(g_, subcell_size, num_pnts, pRadius, t, &pSCPntsLength));
}

// GatherLevelSet_FP16 (VG.cpp:5375-5401)
void VolumeGVDB::GatherLevelSet_FP16(int subcell_size, int num_pnts, float radius, Vector3DF trans,
                                     int& pSCPntsLength, int chanLevelSet, int chanClr)
{
    need_grid();
    const float t[3] = {trans.x, trans.y, trans.z};
    check(gvx_gather_levelset_fp16(g_, subcell_size, num_pnts, radius, t, pSCPntsLength, chanLevelSet, chanClr));
}

// ConvertAndTransform (VG.cpp:5668-5682) on the DataPtrs' device buffers
void VolumeGVDB::ConvertAndTransform(DataPtr& psrc, char psrcbits, DataPtr& pdest, char pdestbits, int num_pnts,
                                     Vector3DF wMin, Vector3DF wDelta, Vector3DF trans, Vector3DF scal)
{
    need_grid();
    const float mn[3] = {wMin.x, wMin.y, wMin.z}, dl[3] = {wDelta.x, wDelta.y, wDelta.z};
    const float tr[3] = {trans.x, trans.y, trans.z}, sc[3] = {scal.x, scal.y, scal.z};
    check(gvx_convert_and_transform(g_, (const void*)psrc.gpu, psrcbits, (void*)pdest.gpu, pdestbits, num_pnts, mn,
                                    dl, tr, sc));
}

// getAux (VG.h:625) for the point buffers and AUX_PNODE, the leaf of every
// point after InsertPoints (ID_UNDEFL when none), on the host and the device
DataPtr& VolumeGVDB::getAux(int id)
{
    switch (id) {
    case AUX_PNTPOS: return pos_;
    case AUX_PNTVEL: return vel_;
    case AUX_PNTCLR: return clr_;
    case AUX_PNODE:
        if (pnode_gen_ != gen_ && last_insert_n_ > 0) {
            AllocData(pnode_, last_insert_n_, sizeof(int), true);
            check(gvx_insert_points(g_, last_insert_n_, last_trans_, (int32_t*)pnode_.cpu));
            CommitData(pnode_);
            pnode_gen_ = gen_;
        }
        return pnode_;
    }
    throw GvxError(GVX_ERR_UNSUPPORTED, "getAux: buffer " + std::to_string(id) + " is not kept by this library");
}

uint64 VolumeGVDB::getNumUsedNodes(int lev)
{
    need_grid();
    gvx_info inf;
    check(gvx_get_info(g_, &inf));
    if (lev < 0 || lev >= GVX_MAX_LEVELS) return 0;
    return lev == 0 ? (uint64)inf.used_leaves : (uint64)inf.node_count[lev];
}

uint64 VolumeGVDB::getNumTotalNodes(int lev)
{
    need_grid();
    gvx_info inf;
    check(gvx_get_info(g_, &inf));
    if (lev < 0 || lev >= GVX_MAX_LEVELS) return 0;
    return (uint64)inf.node_count[lev];
}

Node* VolumeGVDB::mirror(int lev, uint64 ndx)
{
    if (lev < 0 || lev >= (int)mirror_.size()) return nullptr;
    if (mirror_gen_[lev] != gen_) {
        const uint64 cnt = getNumTotalNodes(lev);
        mirror_[lev].resize((size_t)cnt);
        if (cnt) check(gvx_read_nodes(g_, lev, mirror_[lev].data(), (int64_t)cnt));
        mirror_gen_[lev] = gen_;
    }
    return ndx < mirror_[lev].size() ? &mirror_[lev][ndx] : nullptr;
}

// getNodeAtLevel (VG.h:643)
Node* VolumeGVDB::getNodeAtLevel(int n, int lev) { return n < 0 ? nullptr : mirror(lev, (uint64)n); }

// getNode(grp, lev, ndx) (VG.h:451): node pools are group 0
Node* VolumeGVDB::getNode(int grp, int lev, slong ndx)
{
    return (grp != 0 || ndx < 0) ? nullptr : mirror(lev, (uint64)ndx);
}

// getNode(Elem id) (VG.h:453), id = grp | lev << 8 | ndx << 16
Node* VolumeGVDB::getNode(slong nodeid)
{
    const uint64 id = (uint64)nodeid;
    return getNode((int)(id & 0xFF), (int)((id >> 8) & 0xFF), (slong)(id >> 16));
}

// ---- host-side tree queries, on the pools and child lists read back on demand

// child list `listid` = Elem(1, lev, ndx): entries [ndx * res^3, (ndx + 1) * res^3) of level lev's lists
const uint64* VolumeGVDB::child_list(uint64 listid)
{
    if (listid == ID_UNDEFL || listid == ID_UNDEF64 || (listid & 0xFF) != 1) return nullptr;
    const int lev = (int)((listid >> 8) & 0xFF);
    if (lev < 1 || lev >= (int)clmirror_.size()) return nullptr;
    const uint64 vc = (uint64)getRes(lev) * getRes(lev) * getRes(lev);
    if (clmirror_gen_[lev] != gen_) {
        const uint64 cnt = getNumTotalNodes(lev) * vc;
        clmirror_[lev].resize((size_t)cnt);
        if (cnt) check(gvx_read_childlist(g_, lev, clmirror_[lev].data(), (int64_t)cnt));
        clmirror_gen_[lev] = gen_;
    }
    const uint64 at = (listid >> 16) * vc;
    return at + vc <= clmirror_[lev].size() ? clmirror_[lev].data() + at : nullptr;
}

// getRange (VG.h:614-619): index-space extent of a level-lev node
Vector3DI VolumeGVDB::getRange(int lev)
{
    int r = getRes(0);
    for (int l = 1; l <= lev; l++) r *= getRes(l);
    return Vector3DI(r, r, r);
}

uint64 VolumeGVDB::getRootNodeID()
{
    need_grid();
    gvx_info inf;
    check(gvx_get_info(g_, &inf));
    if (inf.root_level < 0) return ID_UNDEF64;
    return (uint64)inf.root_level << 8;  // Elem(0, root level, 0)
}

// getChildNode (VG.cpp:3079-3092), bitmasks off: entry b of the node's child list
uint64 VolumeGVDB::getChildNode(slong nodeid, uint b)
{
    Node* curr = getNode(nodeid);
    return curr ? getChildRefAtBit(curr, b) : ID_UNDEF64;
}

// getChildRefAtBit (VG.cpp:3066-3076)
uint64 VolumeGVDB::getChildRefAtBit(Node* curr, uint b)
{
    const uint64* cl = curr ? child_list(curr->mChildList) : nullptr;
    if (!cl || b >= (uint)(getRes(curr->mLev) * getRes(curr->mLev) * getRes(curr->mLev))) return ID_UNDEF64;
    return cl[b];
}

// getChildAtBit (VG.cpp:3052-3064)
Node* VolumeGVDB::getChildAtBit(Node* curr, uint b)
{
    const uint64 ch = getChildRefAtBit(curr, b);
    return ch == ID_UNDEF64 ? nullptr : getNode((slong)ch);
}

// isOn (VG.cpp:2787-2796), bitmasks off
bool VolumeGVDB::isOn(slong nodeid, uint32 b) { return getChildNode(nodeid, b) != ID_UNDEF64; }

// getPosInNode (VG.cpp:2858-2875): integer position inside the node, and its child bit
bool VolumeGVDB::getPosInNode(slong curr_id, Vector3DI pos, uint32& bit)
{
    bit = 0;
    Node* curr = getNode(curr_id);
    if (!curr) return false;
    const int res = getRes(curr->mLev);
    const Vector3DI range = getRange(curr->mLev);
    int p[3] = {pos.x - curr->mPos.x, pos.y - curr->mPos.y, pos.z - curr->mPos.z};
    const int rg[3] = {range.x, range.y, range.z};
    for (int a = 0; a < 3; a++)
        if (p[a] < 0 || p[a] >= rg[a]) return false;
    for (int a = 0; a < 3; a++) p[a] = p[a] * res / rg[a];
    bit = (uint32)getBitPos(curr->mLev, Vector3DI(p[0], p[1], p[2]));
    return true;
}

// getNodeAtPoint (VG.cpp:4650-4684): the leaf holding an index-space position, by descent
uint64 VolumeGVDB::getNodeAtPoint(uint64 nodeid, Vector3DF pos)
{
    Node* curr = getNode((slong)nodeid);
    if (!curr) return ID_UNDEFL;
    const Vector3DI range = getRange(curr->mLev);
    float p[3] = {pos.x - (float)curr->mPos.x, pos.y - (float)curr->mPos.y, pos.z - (float)curr->mPos.z};
    const float rg[3] = {(float)range.x, (float)range.y, (float)range.z};
    if (!(p[0] >= 0 && p[1] >= 0 && p[2] >= 0 && p[0] < rg[0] && p[1] < rg[1] && p[2] < rg[2])) return ID_UNDEFL;
    const float res = (float)getRes(curr->mLev);
    for (int a = 0; a < 3; a++) p[a] = p[a] * res / rg[a];
    if (isLeaf((slong)nodeid)) return nodeid;
    const uint32 i = (uint32)getBitPos(curr->mLev, Vector3DI((int)p[0], (int)p[1], (int)p[2]));
    if (!isOn((slong)nodeid, i)) return ID_UNDEFL;
    return getNodeAtPoint(getChildNode((slong)nodeid, i), pos);
}

// isActive (VG.cpp:4688-4711): is the integer position inside a leaf of the tree
bool VolumeGVDB::isActive(Vector3DI wpos)
{
    const uint64 root = getRootNodeID();
    return root != ID_UNDEF64 && isActive(wpos, (slong)root);
}

bool VolumeGVDB::isActive(Vector3DI pos, slong nodeid)
{
    uint32 b = 0;
    if (!getPosInNode(nodeid, pos, b)) return false;
    if (isLeaf(nodeid)) return true;
    if (!isOn(nodeid, b)) return false;
    return isActive(pos, (slong)getChildNode(nodeid, b));
}

// getValue (VG.cpp:4713-4755): descend to the leaf, then read the atlas voxel at the leaf's
// mValue plus the position's offset inside it, from a dense atlas of channel 0
float VolumeGVDB::getValue(slong nodeid, Vector3DF pos, float* atlas)
{
    Node* curr = getNode(nodeid);
    if (!curr || !atlas) return 0.0f;
    const Vector3DI range = getRange(curr->mLev);
    float p[3] = {pos.x - (float)curr->mPos.x, pos.y - (float)curr->mPos.y, pos.z - (float)curr->mPos.z};
    const float rg[3] = {(float)range.x, (float)range.y, (float)range.z};
    if (!(p[0] >= 0 && p[1] >= 0 && p[2] >= 0 && p[0] < rg[0] && p[1] < rg[1] && p[2] < rg[2])) return 0.0f;
    const float res = (float)getRes(curr->mLev);
    for (int a = 0; a < 3; a++) p[a] = p[a] * res / rg[a];
    if (isLeaf(nodeid)) {
        gvx_info inf;
        check(gvx_get_info(g_, &inf));
        const float x = p[0] + (float)curr->mValue.x, y = p[1] + (float)curr->mValue.y, z = p[2] + (float)curr->mValue.z;
        return atlas[((size_t)(int)z * inf.atlas_res[1] + (size_t)(int)y) * inf.atlas_res[0] + (size_t)(int)x];
    }
    const uint32 i = (uint32)getBitPos(curr->mLev, Vector3DI((int)p[0], (int)p[1], (int)p[2]));
    if (!isOn(nodeid, i)) return 0.0f;
    return getValue((slong)getChildNode(nodeid, i), pos, atlas);
}

Vector3DF VolumeGVDB::getWorldMin()
{
    need_grid();
    gvx_info inf;
    check(gvx_get_info(g_, &inf));
    return Vector3DF(inf.obj_min[0], inf.obj_min[1], inf.obj_min[2]);
}

Vector3DF VolumeGVDB::getWorldMax()
{
    need_grid();
    gvx_info inf;
    check(gvx_get_info(g_, &inf));
    return Vector3DF(inf.obj_max[0], inf.obj_max[1], inf.obj_max[2]);
}

Vector3DF VolumeGVDB::getVoxRes()
{
    need_grid();
    gvx_info inf;
    check(gvx_get_info(g_, &inf));
    return Vector3DF(inf.vox_res[0], inf.vox_res[1], inf.vox_res[2]);
}

Vector3DF VolumeGVDB::getVoxResMax()
{
    need_grid();
    gvx_info inf;
    check(gvx_get_info(g_, &inf));
    return Vector3DF(inf.vox_res_max[0], inf.vox_res_max[1], inf.vox_res_max[2]);
}

void VolumeGVDB::Splat(int mode, int num_pnts, float radius, Vector3DF trans, int chanDensity, int chanVel,
                       bool bAccum)
{
    need_grid();
    const float t[3] = {trans.x, trans.y, trans.z};
    check(gvx_splat(g_, mode, num_pnts, radius, t, chanDensity, chanVel, bAccum ? 1 : 0));
}

void VolumeGVDB::SplatBackward(int mode, int num_pnts, float radius, Vector3DF trans, CUdeviceptr dL_drho,
                               CUdeviceptr grad_pos, CUdeviceptr grad_w, CUdeviceptr grad_r)
{
    need_grid();
    const float t[3] = {trans.x, trans.y, trans.z};
    check(gvx_splat_backward(g_, mode, num_pnts, radius, t, (const float*)dL_drho, (float*)grad_pos,
                             (float*)grad_w, (float*)grad_r));
}

void VolumeGVDB::SetPointAttribs(CUdeviceptr weight, CUdeviceptr radius)
{
    need_grid();
    check(gvx_set_point_attribs(g_, (const float*)weight, (const float*)radius));
}

}  // namespace nvdb
