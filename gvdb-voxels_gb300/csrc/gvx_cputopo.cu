// gvx_cputopo.cu -- the reference's host-side topology: ActivateSpace
// (VG.cpp:2768-2855) and RebuildTopologyCPU (VG.cpp:1220-1227), used by
// callers that build or extend a tree point by point on the CPU
// (gFluidSurface's CPU path, main_fluid_surface.cpp:335-345).
//
// The grid keeps a host copy of its pools.  It is taken from the device when
// the device tree changed since the last copy, grows point by point exactly
// as the reference's host pools do (node creation order, Reparent growing the
// root upward, child lists), and goes back to the device at FinishTopology
// (VG.cpp:1579-1593 commits the pools) through the same import a VBX load uses.
#include <string.h>

#include <vector>

#include "gvx_grid.cuh"

namespace {

constexpr uint64_t kUndefL = 0xFFFFFFFFull;  // ID_UNDEFL
constexpr uint64_t kUndef64 = ~0ull;         // ID_UNDEF64
constexpr int kRefMaxLev = 10;               // MAXLEV of the reference

inline uint64_t elem_id(int grp, int lev, uint64_t ndx) { return (uint64_t)grp | ((uint64_t)lev << 8) | (ndx << 16); }
inline int elem_lev(uint64_t id) { return (int)((id >> 8) & 0xFF); }
inline uint64_t elem_ndx(uint64_t id) { return id >> 16; }

}  // namespace

struct GvxHostTree {
    int levels = 0, res[GVX_MAXLEV] = {}, range[GVX_MAXLEV] = {};
    std::vector<GvxNode> nodes[GVX_MAXLEV];
    std::vector<uint64_t> clist[GVX_MAXLEV];  // res^3 child ids per node, levels >= 1
    uint64_t root = kUndefL;                  // mRoot
    uint64_t gen = ~0ull;                     // device topology generation this copy matches
    bool dirty = false;                       // changes not yet on the device
    bool failed = false;

    size_t vox(int l) const { return (size_t)res[l] * res[l] * res[l]; }
    GvxNode& node(uint64_t id) { return nodes[elem_lev(id)][elem_ndx(id)]; }
    // a node id that names a node of the pools (pools read from the device or a file may hold others)
    bool valid(uint64_t id) const
    {
        return (id & 0xFF) == 0 && elem_lev(id) < levels && elem_ndx(id) < nodes[elem_lev(id)].size();
    }

    // AllocateNode + SetupNode (VG.cpp:2506-2525): marker true, no parent, no child list, no atlas brick
    uint64_t alloc(int lev, const int p[3])
    {
        if (lev < 0 || lev >= levels) return kUndefL;
        GvxNode n;
        memset(&n, 0, sizeof(n));
        n.lev = (uint8_t)lev;
        n.flags = 1;
        for (int a = 0; a < 3; a++) {
            n.pos[a] = p[a];
            n.value[a] = -1;
        }
        n.parent = kUndefL;
        n.childlist = kUndefL;
        nodes[lev].push_back(n);
        if (lev > 0) clist[lev].resize(nodes[lev].size() * vox(lev), kUndef64);
        return elem_id(0, lev, nodes[lev].size() - 1);
    }
    // GetCoveringNode (VG.cpp:2915-2931)
    void covering(int lev, const int pos[3], int out[3]) const
    {
        for (int a = 0; a < 3; a++) {
            if (lev == kRefMaxLev - 1) {
                out[a] = 0;
                continue;
            }
            int np = pos[a] / range[lev] * range[lev];
            if (pos[a] < np) np -= range[lev];
            out[a] = np;
        }
    }
    // getPosInNode (VG.cpp:2858-2875)
    bool pos_in_node(uint64_t id, const int pos[3], int& bit)
    {
        const GvxNode& c = node(id);
        const int l = c.lev;
        int p[3];
        for (int a = 0; a < 3; a++) {
            p[a] = pos[a] - c.pos[a];
            if (p[a] < 0 || p[a] >= range[l]) {
                bit = 0;
                return false;
            }
        }
        for (int a = 0; a < 3; a++) p[a] = p[a] * res[l] / range[l];
        bit = (p[2] * res[l] + p[1]) * res[l] + p[0];
        return true;
    }
    // getChildNode / isOn without bitmasks: the child list entry
    uint64_t child(uint64_t id, int bit)
    {
        const GvxNode& c = node(id);
        if (c.childlist == kUndefL || c.childlist == kUndef64) return kUndef64;
        const int l = elem_lev(c.childlist);
        const size_t at = elem_ndx(c.childlist) * vox(l) + (size_t)bit;
        return l < levels && at < clist[l].size() ? clist[l][at] : kUndef64;
    }
    // InsertChild (VG.cpp:2980-3027, no bitmasks).  A node's child list is allocated at its first child,
    // which a descent gives it right after its creation: list index and node index coincide.
    uint64_t insert_child(uint64_t id, uint64_t cid, int bit)
    {
        node(cid).parent = id;
        GvxNode& c = node(id);
        if (c.childlist == kUndefL || c.childlist == kUndef64) c.childlist = elem_id(1, c.lev, elem_ndx(id));
        clist[c.lev][elem_ndx(id) * vox(c.lev) + bit] = cid;
        return cid;
    }
    // AddChildNode (VG.cpp:2707-2723)
    uint64_t add_child(uint64_t id, int bit)
    {
        const int plev = node(id).lev, r = range[plev - 1], rs = res[plev];
        const int p[3] = {(bit % rs) * r + node(id).pos[0], ((bit / rs) % rs) * r + node(id).pos[1],
                          (bit / (rs * rs)) * r + node(id).pos[2]};
        const uint64_t c = alloc(plev - 1, p);
        if (c == kUndefL) return kUndefL;
        return insert_child(id, c, bit);
    }
    // Reparent (VG.cpp:2726-2763): a new root covering the old root and pos
    uint64_t reparent(int lev, uint64_t prev, const int pos[3], bool& bnew)
    {
        const int pp[3] = {node(prev).pos[0], node(prev).pos[1], node(prev).pos[2]};
        int p1[3], p2[3];
        bool cover = false;
        while (!cover && lev < kRefMaxLev) {
            lev++;
            if (lev >= levels) return kUndefL;  // past the configured levels
            covering(lev, pos, p1);
            covering(lev, pp, p2);
            cover = p1[0] == p2[0] && p1[1] == p2[1] && p1[2] == p2[2];
        }
        if (lev >= kRefMaxLev) return kUndefL;
        const uint64_t nr = alloc(lev, p1);
        if (nr == kUndefL) return kUndefL;
        bool bn = false;
        activate(nr, pp, bn, prev);
        const uint64_t leaf = activate(nr, pos, bnew, kUndefL);
        root = nr;
        if (leaf == kUndefL) return kUndefL;
        return node(leaf).parent;
    }
    // ActivateSpace (VG.cpp:2805-2855), stop level 0, iterative
    uint64_t activate(uint64_t id, const int pos[3], bool& bnew, uint64_t stopnode)
    {
        for (;;) {
            if (root == kUndefL && id == root) {
                int p[3];
                covering(0, pos, p);
                root = alloc(0, p);
                if (root == kUndefL) return kUndefL;
                id = root;
            }
            if (!valid(id)) return kUndefL;
            int bit;
            if (pos_in_node(id, pos, bit)) {
                const int lev = node(id).lev;
                if (stopnode != kUndefL) {
                    const GvxNode& sn = node(stopnode);
                    if (pos[0] == sn.pos[0] && pos[1] == sn.pos[1] && pos[2] == sn.pos[2] &&
                        child(id, bit) == kUndef64 && lev == sn.lev + 1)
                        return insert_child(id, stopnode, bit);
                }
                if (lev == 0) return id;
                uint64_t c = child(id, bit);
                if (c == kUndef64) {
                    c = add_child(id, bit);
                    if (c == kUndefL) return kUndefL;
                    if (lev == 1) bnew = true;
                }
                if (!valid(c)) return kUndefL;
                if (elem_lev(c) == 0) return c;
                id = c;
            } else {
                uint64_t parent = node(id).parent;
                if (parent == kUndefL || parent == kUndef64) {
                    parent = reparent(node(id).lev, id, pos, bnew);
                    if (parent == kUndefL) return kUndefL;
                }
                id = parent;
            }
        }
    }
};

// the host copy, taken from the device tree when that changed
static gvx_status host_tree(gvx_grid* g, GvxHostTree** out)
{
    if (!g->configured) {
        gvx_set_error("ActivateSpace: Configure was not called");
        return GVX_ERR_NOT_CONFIGURED;
    }
    if (!g->htree) g->htree = new GvxHostTree();
    GvxHostTree* t = g->htree;
    if (t->gen != g->topo_gen || t->levels != g->levels) {
        *t = GvxHostTree();
        t->levels = g->levels;
        for (int l = 0; l < g->levels; l++) {
            t->res[l] = g->res[l];
            t->range[l] = g->range[l];
        }
        if (g->root_level >= 0) {
            for (int l = 0; l <= g->root_level; l++) {
                t->nodes[l].resize((size_t)g->count[l]);
                if (g->count[l])
                    GVX_CK(cudaMemcpyAsync(t->nodes[l].data(), g->nodes[l].p, (size_t)g->count[l] * sizeof(GvxNode),
                                           cudaMemcpyDeviceToHost, g->stream));
                if (l > 0) {
                    t->clist[l].resize((size_t)g->count[l] * t->vox(l));
                    if (g->count[l])
                        GVX_CK(cudaMemcpyAsync(t->clist[l].data(), g->clist[l].p,
                                               t->clist[l].size() * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                                               g->stream));
                }
            }
            GVX_CK(cudaStreamSynchronize(g->stream));
            t->root = elem_id(0, g->root_level, 0);
        }
        t->gen = g->topo_gen;
    }
    *out = t;
    return GVX_OK;
}

void gvx_host_tree_free(gvx_grid* g)
{
    delete g->htree;
    g->htree = nullptr;
}

// FinishTopology's commit: the host pools to the device
gvx_status gvx_host_tree_commit(gvx_grid* g)
{
    GvxHostTree* t = g->htree;
    if (!t || !t->dirty) return GVX_OK;
    if (t->failed) {
        gvx_set_error("FinishTopology: an ActivateSpace failed (tree beyond the configured levels)");
        return GVX_ERR_DEPTH;
    }
    const int R = t->root == kUndefL ? -1 : elem_lev(t->root);
    if (R < 1) {
        gvx_set_error("FinishTopology: the activated space fits one brick (root level %d); a tree needs level 1", R);
        return GVX_ERR_DEPTH;
    }
    for (int l = 0; l <= R; l++)
        for (const GvxNode& n : t->nodes[l])
            if (n.pos[0] < 0 || n.pos[1] < 0 || n.pos[2] < 0) {
                gvx_set_error("FinishTopology: activated space at a negative coordinate (%d, %d, %d)", n.pos[0],
                              n.pos[1], n.pos[2]);
                return GVX_ERR_UNSUPPORTED;
            }
    if (elem_ndx(t->root) != 0) {
        // the root moves to index 0 of its level: the tree's references to it follow
        gvx_set_error("FinishTopology: root at index %llu of its level", (unsigned long long)elem_ndx(t->root));
        return GVX_ERR_UNSUPPORTED;
    }
    int64_t counts[GVX_MAXLEV];
    const GvxNode* np[GVX_MAXLEV];
    const uint64_t* cp[GVX_MAXLEV];
    for (int l = 0; l < GVX_MAXLEV; l++) {
        counts[l] = l < t->levels ? (int64_t)t->nodes[l].size() : 0;
        np[l] = l < t->levels ? t->nodes[l].data() : nullptr;
        cp[l] = l > 0 && l < t->levels ? t->clist[l].data() : nullptr;
    }
    const bool rebuild = g->rebuild_topo;  // the host path leaves mRebuildTopo as it was
    gvx_status rc = gvx_topo_import(g, R, counts, np, cp);
    if (rc) return rc;
    g->rebuild_topo = rebuild;
    t->dirty = false;
    t->gen = g->topo_gen;  // the import advanced the generation; the host copy is that tree
    return GVX_OK;
}

extern "C" gvx_status gvx_activate_space(gvx_grid* g, const float pos[3], uint64_t* node_id)
{
    if (!g || !pos) {
        gvx_set_error("ActivateSpace: null argument");
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(cudaSetDevice(g->device));
    GvxHostTree* t = nullptr;
    gvx_status rc = host_tree(g, &t);
    if (rc) return rc;
    const int p[3] = {(int)pos[0], (int)pos[1], (int)pos[2]};  // Vector3DF -> Vector3DI truncation
    bool bnew = false;
    const uint64_t id = t->activate(t->root, p, bnew, kUndefL);
    t->dirty = true;
    if (id == kUndefL) t->failed = true;
    // ActivateSpace(Vector3DF) (VG.cpp:2768-2776): an existing leaf's id, else ID_UNDEFL
    if (node_id) *node_id = (id == kUndefL || bnew) ? kUndefL : id;
    return GVX_OK;
}

extern "C" gvx_status gvx_rebuild_topology_cpu(gvx_grid* g, int n, const float orig[3], const float* host_pos)
{
    if (!g || n < 0 || (n > 0 && !host_pos)) {
        gvx_set_error("RebuildTopologyCPU: %d points, null buffer", n);
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(cudaSetDevice(g->device));
    GvxHostTree* t = nullptr;
    gvx_status rc = host_tree(g, &t);
    if (rc) return rc;
    const float o[3] = {orig ? orig[0] : 0.f, orig ? orig[1] : 0.f, orig ? orig[2] : 0.f};
    for (int i = 0; i < n; i++) {
        const int p[3] = {(int)(host_pos[3 * (size_t)i] + o[0]), (int)(host_pos[3 * (size_t)i + 1] + o[1]),
                          (int)(host_pos[3 * (size_t)i + 2] + o[2])};
        bool bnew = false;
        if (t->activate(t->root, p, bnew, kUndefL) == kUndefL) t->failed = true;
    }
    t->dirty = true;
    return GVX_OK;
}
