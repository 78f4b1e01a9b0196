/*
 * gvx_oracle.c -- CPU oracle for the GVDB point -> sparse-volume path.
 *
 * TEST INFRASTRUCTURE ONLY (see gvx_oracle.h).  Each function names the
 * reference lines it restates; paths are relative to the reference project:
 *   VG.cpp = source/gvdb_library/src/gvdb_volume_gvdb.cpp
 *   AL.cpp = source/gvdb_library/src/gvdb_allocator.cpp
 *   PT.cuh = source/gvdb_library/kernels/cuda_gvdb_particles.cuh
 *   ND.cuh = source/gvdb_library/kernels/cuda_gvdb_nodes.cuh
 *   OP.cuh = source/gvdb_library/kernels/cuda_gvdb_operators.cuh
 *
 * Parity pin: the reference ships no tests, golden vectors or fixtures for
 * this path, and its host library does not build without OpenGL/X11, so this
 * restatement is pinned by hand-worked known answers in tests/ (parity of the
 * oracle itself against the reference is otherwise unpinned).
 */
#include "gvx_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define MAXLEV 10
#define ID_UNDEFL 0xFFFFFFFFull          /* gvdb_types.h:55, as a 64-bit value */
#define ID_UNDEF64 0xFFFFFFFFFFFFFFFFull /* gvdb_types.h:56 */
#define NOHIT 1.0e10f                    /* gvdb_types.h:53 */
#define MAXCH 32

typedef struct pool {
    orc_node* nodes;
    int cnt, cap;
    uint64_t* clist; /* cnt * res^3 entries (levels > 0) */
    int used;
} pool;

struct orc_grid {
    int levels;
    int logdim[MAXLEV];
    int res[MAXLEV];
    int range[MAXLEV];
    int apron, brick, P;
    int defsub[3];
    pool pools[MAXLEV];
    int root_level;
    int rebuild_topo; /* mRebuildTopo */
    int curr_depth;   /* mCurrDepth */
    int last_mode;
    float pos_min[3], pos_max[3]; /* mPosMin / mPosMax of the last GetBoundingBox */
    float vox_res_max[3];         /* mVoxResMax: zeroed by Configure (VG.cpp:2428), grown by ComputeBounds */
    int colavg_seen;              /* AUX_COLAVG exists: an avgColor ScatterDensity ran */
    int degenerate;
    /* atlas (shared subdim, as UpdateAtlas resizes every channel together) */
    int sub[3];
    int have_atlas;
    int atlas_last;
    int32_t* amap;  /* 4 ints per slot */
    int amap_slots;
    int chtype[MAXCH];
    int ncomp[MAXCH];
    double* ch[MAXCH];
    int64_t chslots[MAXCH];
};

double orc_now_seconds(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* ------------------------------------------------------------------ */
/* configuration: VG.cpp:2380-2434 (Configure), VG.h:592-621 (getRes/getRange) */

orc_grid* orc_create(int levels, const int* logdim, int apron, int cx, int cy, int cz)
{
    if (levels < 2 || levels > MAXLEV || apron < 0 || apron > 1) return NULL;
    orc_grid* g = (orc_grid*)calloc(1, sizeof(orc_grid));
    if (!g) return NULL;
    g->levels = levels;
    int r = 1;
    for (int l = 0; l < levels; l++) {
        g->logdim[l] = logdim[l] == 0 ? 1 : logdim[l];
        g->res[l] = 1 << g->logdim[l];
        r = (l == 0) ? g->res[0] : r * g->res[l];
        g->range[l] = r;
    }
    g->apron = apron;
    g->brick = g->res[0];
    g->P = g->brick + 2 * apron;
    g->defsub[0] = cx > 0 ? cx : 16;
    g->defsub[1] = cy > 0 ? cy : 16;
    g->defsub[2] = cz > 0 ? cz : 1;
    g->root_level = -1;
    g->rebuild_topo = 1;
    g->curr_depth = -1;
    return g;
}

void orc_destroy(orc_grid* g)
{
    if (!g) return;
    for (int l = 0; l < MAXLEV; l++) {
        free(g->pools[l].nodes);
        free(g->pools[l].clist);
    }
    for (int c = 0; c < MAXCH; c++) free(g->ch[c]);
    free(g->amap);
    free(g);
}

static int64_t voxcnt(const orc_grid* g, int l) { return (int64_t)g->res[l] * g->res[l] * g->res[l]; }

/* Allocator::PoolAlloc (AL.cpp:158-188) + SetupNode (VG.cpp:2512-2524) */
static int pool_alloc(orc_grid* g, int lev, const int pos[3])
{
    pool* p = &g->pools[lev];
    if (p->cnt >= p->cap) {
        int nc = p->cap ? p->cap * 2 : 64;
        orc_node* nn = (orc_node*)realloc(p->nodes, (size_t)nc * sizeof(orc_node));
        if (!nn) return -1;
        p->nodes = nn;
        if (lev > 0) {
            uint64_t* cl = (uint64_t*)realloc(p->clist, (size_t)nc * voxcnt(g, lev) * sizeof(uint64_t));
            if (!cl) return -1;
            p->clist = cl;
        }
        p->cap = nc;
    }
    int i = p->cnt++;
    p->used++;
    orc_node* n = &p->nodes[i];
    memset(n, 0, sizeof(*n));
    n->lev = (uint8_t)lev;
    n->pos[0] = pos[0]; n->pos[1] = pos[1]; n->pos[2] = pos[2];
    n->childlist = ID_UNDEFL;
    n->parent = ID_UNDEFL;
    n->value[0] = n->value[1] = n->value[2] = -1;
    n->flags = 1;
    if (lev > 0) {
        /* child list allocated in lockstep: Elem(1, lev, i), filled with 0xFF (VG.cpp:1322-1328) */
        n->childlist = 1ull | ((uint64_t)lev << 8) | ((uint64_t)i << 16);
        memset(p->clist + (int64_t)i * voxcnt(g, lev), 0xFF, (size_t)voxcnt(g, lev) * sizeof(uint64_t));
    }
    return i;
}

/* Clear (VG.cpp:2487-2503): pools emptied, not freed */
static void clear_tree(orc_grid* g)
{
    for (int l = 0; l < MAXLEV; l++) { g->pools[l].cnt = 0; g->pools[l].used = 0; }
    g->root_level = -1;
    g->atlas_last = 0;
    g->rebuild_topo = 1;
}

/* PrepareVDBPartially (VG.cpp:3996-4020): top_lev = lowest level with exactly one node */
static int top_lev_of(const orc_grid* g)
{
    int tlev = 1;
    for (int n = g->levels - 1; n >= 0; n--)
        if (g->pools[n].cnt == 1) tlev = n;
    return tlev;
}

/* getChild (ND.cuh:115-124), returning the int the reference returns */
static int get_child(orc_grid* g, const orc_node* nd, int b)
{
    uint64_t listid = nd->childlist;
    if (listid == ID_UNDEFL) return -1;
    int clev = (int)((listid >> 8) & 0xFF);
    int64_t cndx = (int64_t)(listid >> 16);
    if (clev <= 0 || clev >= g->levels || cndx >= g->pools[clev].cnt || b < 0 || b >= voxcnt(g, clev)) {
        g->degenerate = 1;
        return -1;
    }
    uint64_t v = g->pools[clev].clist[cndx * voxcnt(g, clev) + b];
    return (int)(int64_t)(v >> 16);
}

static orc_node* node_at(orc_grid* g, int lev, int64_t i)
{
    if (lev < 0 || lev >= g->levels || i < 0 || i >= g->pools[lev].cnt) { g->degenerate = 1; return NULL; }
    return &g->pools[lev].nodes[i];
}

/* node 0 at VDBInfo.top_lev, where every reference descent starts.  When a
 * level below the root holds exactly one node, top_lev is not the root's level
 * and the reference descends from the wrong node (VG.cpp:3957-3968); the
 * oracle reports that input as degenerate. */
static orc_node* root_node(orc_grid* g)
{
    int tl = top_lev_of(g);
    if (tl != g->root_level) g->degenerate = 1;
    return node_at(g, tl, 0);
}

/* bit position of a child inside a node, with the out-of-range check the
 * reference omits (it then reads outside the child list) */
static int child_bit(orc_grid* g, int l, const int32_t* ppos, const int* pos)
{
    int res = g->res[l], rng = g->range[l];
    int p[3];
    for (int a = 0; a < 3; a++) {
        p[a] = ((pos[a] - ppos[a]) * res) / rng;   /* int trunc as in ND.cuh:317-321 */
        if (p[a] < 0 || p[a] >= res || pos[a] - ppos[a] < 0) { g->degenerate = 1; return -1; }
    }
    return (p[2] * res + p[1]) * res + p[0];
}

/* getParent (ND.cuh:350-397).  Returns the node index at stopLev or -1. */
static int64_t get_parent(orc_grid* g, int stopLev, const int32_t* pos)
{
    orc_node* nd = root_node(g);
    if (!nd) return -1;
    if (!nd->flags) return 0;
    int l = nd->lev;
    if (l == stopLev) return 0;
    while (l > stopLev) {
        int p3[3] = {pos[0], pos[1], pos[2]};
        int b = child_bit(g, l, nd->pos, p3);
        if (b < 0) return -1;
        l--;
        int c = get_child(g, nd, b);
        if (c == -1) {
            /* the reference compares a sign-extended 64-bit -1 with the 32-bit
             * ID_UNDEFL here and goes on with a pointer before the pool */
            g->degenerate = 1;
            return -1;
        }
        if (l == stopLev) return c;
        nd = node_at(g, l, c);
        if (!nd) return -1;
    }
    return -1;
}

/* getPosParent (ND.cuh:303-348) */
static int64_t get_pos_parent(orc_grid* g, const int* pos, int stopLev)
{
    orc_node* nd = root_node(g);
    if (!nd) return -1;
    int l = nd->lev;
    if (l == 0) return 0;
    while (l > 0) {
        int b = child_bit(g, l, nd->pos, pos);
        if (b < 0) return -1;
        int c = get_child(g, nd, b);
        l--;
        if (c == -1) return -1;
        if (l == stopLev) return c;
        nd = node_at(g, l, c);
        if (!nd) return -1;
    }
    return -1;
}

/* getPosLeafParent (ND.cuh:255-288) */
static int64_t get_pos_leaf_parent(orc_grid* g, const int* pos)
{
    orc_node* nd = root_node(g);
    if (!nd) return -1;
    int l = nd->lev;
    if (l == 0) return 0;
    for (;;) {
        int b = child_bit(g, l, nd->pos, pos);
        if (b < 0) return -1;
        int c = get_child(g, nd, b);
        if (c == -1) return -1;
        l--;
        if (l == 0) return c;
        nd = node_at(g, l, c);
        if (!nd) return -1;
    }
}

/* getNode descent in float (ND.cuh:199-253): leaf at an index-space point */
static int64_t get_node_at_point(orc_grid* g, const float* pos)
{
    orc_node* node = root_node(g);
    if (!node) return -1;
    int lev = node->lev;
    int64_t id = 0;
    float vmin[3] = {(float)node->pos[0], (float)node->pos[1], (float)node->pos[2]};
    while (lev > 0 && node) {
        float nr = (float)g->range[lev];
        for (int a = 0; a < 3; a++)
            if (pos[a] < vmin[a] || pos[a] >= vmin[a] + nr) return -1;
        float vdel = (float)g->range[lev] / (float)g->res[lev];
        int p[3];
        for (int a = 0; a < 3; a++) p[a] = (int)((pos[a] - vmin[a]) / vdel);
        int b = (((p[2] << g->logdim[lev]) + p[1]) << g->logdim[lev]) + p[0];
        lev--;
        int c = get_child(g, node, b);
        if (c == -1) return -1;
        id = c;
        node = node_at(g, lev, c);
        if (!node) return -1;
        vmin[0] = (float)node->pos[0]; vmin[1] = (float)node->pos[1]; vmin[2] = (float)node->pos[2];
    }
    return id;
}

/* gvdbLinkBricks (ND.cuh:470-505) over every level, top-down (VG.cpp:1395-1401) */
static void link_levels(orc_grid* g, int depth)
{
    for (int lev = depth - 1; lev >= 0; lev--) {
        pool* p = &g->pools[lev];
        for (int i = 0; i < p->cnt; i++) {
            orc_node* node = &p->nodes[i];
            if (!node->flags) continue;
            int64_t pid = get_parent(g, lev + 1, node->pos);
            if (pid < 0) { g->degenerate = 1; continue; }
            orc_node* pn = node_at(g, lev + 1, pid);
            if (!pn) continue;
            int pos3[3] = {node->pos[0], node->pos[1], node->pos[2]};
            int b = child_bit(g, lev + 1, pn->pos, pos3);
            if (b < 0) continue;
            node->parent = ((uint64_t)pid << 16) | ((uint64_t)(lev + 1) << 8);
            uint64_t cndx = pn->childlist >> 16;
            if ((int64_t)cndx >= g->pools[lev + 1].cnt) continue;
            uint64_t* slot = &g->pools[lev + 1].clist[cndx * voxcnt(g, lev + 1) + b];
            uint64_t v = ((uint64_t)i << 16) | ((uint64_t)lev << 8);
            if (*slot != ID_UNDEF64 && *slot != v) g->degenerate = 1; /* two nodes race for one slot */
            *slot = v;
        }
    }
}

/* ------------------------------------------------------------------ */
/* keys: gvdbCalcBrickId (PT.cuh:352-382) + GetCoveringNode (PT.cuh:88-100) */

static int cover_f(float p, int range)
{
    int np = (int)(ceilf(p / (float)range) * (float)range);
    if (p < (float)np) np -= range;
    return np;
}

static uint64_t make_key(int lev, int x, int y, int z)
{
    return ((uint64_t)(uint16_t)z) | ((uint64_t)(uint16_t)y << 16) | ((uint64_t)(uint16_t)x << 32) |
           ((uint64_t)(uint16_t)lev << 48);
}

static int cmp_u64(const void* a, const void* b)
{
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* FindUniqueBrick (VG.cpp:843-873, PT.cuh:336-350, 934-943): sorted unique
 * keys and per-level counts (lev 255 excluded from the counts) */
static int64_t sort_unique(uint64_t* keys, int64_t n, int* levcnt, int depth)
{
    for (int l = 0; l < depth; l++) levcnt[l] = 0;
    if (n == 0) return 0;
    qsort(keys, (size_t)n, sizeof(uint64_t), cmp_u64);
    int64_t u = 0;
    for (int64_t i = 0; i < n; i++) {
        if (i == 0 || keys[i] != keys[i - 1]) {
            keys[u++] = keys[i];
            int lev = (int)((keys[i] >> 48) & 0xFF);
            if (lev != 255 && lev < depth) levcnt[lev]++;
        }
    }
    return u;
}

/* host allocation loop (VG.cpp:1308-1331 / 966-988 / 1088-1111) */
static int alloc_from_keys(orc_grid* g, const uint64_t* uk, const int* levcnt, int depth)
{
    int64_t pre = 0;
    for (int lev = 0; lev < depth; lev++) {
        int rng = g->range[lev];
        for (int64_t n = pre; n < pre + levcnt[lev]; n++) {
            int pos[3] = {(int)((uk[n] >> 32) & 0xFFFF) * rng, (int)((uk[n] >> 16) & 0xFFFF) * rng,
                          (int)(uk[n] & 0xFFFF) * rng};
            if (pool_alloc(g, lev, pos) < 0) return ORC_ERR_NOMEM;
        }
        pre += levcnt[lev];
    }
    return ORC_OK;
}

/* GetBoundingBox (VG.cpp:5404-5467) + DetermineDepth (VG.cpp:821-837) */
static int bbox_depth(orc_grid* g, int n, const float* pos, int stride, const float* orig, int* rootpos)
{
    float mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
    for (int i = 0; i < n; i++) {
        for (int a = 0; a < 3; a++) {
            float w = pos[(int64_t)i * stride + a] + orig[a];
            if (i == 0 || w < mn[a]) mn[a] = w;
            if (i == 0 || w > mx[a]) mx[a] = w;
        }
    }
    int pmin[3], pmax[3];
    for (int a = 0; a < 3; a++) {
        float lo = mn[a] - 1.0f, hi = mx[a] + 2.0f;
        lo = 0 > lo ? 0 : lo;
        hi = 0 > hi ? 0 : hi;
        g->pos_min[a] = lo;
        g->pos_max[a] = hi;
        pmin[a] = (int)lo;
        pmax[a] = (int)hi;
    }
    for (int lev = 0; lev < MAXLEV; lev++) {
        if (lev >= g->levels) return -1;
        int rng = g->range[lev];
        int same = 1;
        int cm[3];
        for (int a = 0; a < 3; a++) {
            cm[a] = pmin[a] / rng * rng;
            if (cm[a] != pmax[a] / rng * rng) same = 0;
        }
        if (same) {
            rootpos[0] = cm[0]; rootpos[1] = cm[1]; rootpos[2] = cm[2];
            return lev;
        }
    }
    return -1;
}

/* ActivateBricksGPU (VG.cpp:1229-1413) */
static int activate_bricks(orc_grid* g, int n, const float* pos, int stride, const float* orig, int depth,
                           const int* rootpos)
{
    int rootidx = pool_alloc(g, depth, rootpos);
    if (rootidx < 0) return ORC_ERR_NOMEM;
    g->root_level = depth;

    int64_t nk = (int64_t)n * depth;
    uint64_t* keys = (uint64_t*)malloc((size_t)(nk > 0 ? nk : 1) * sizeof(uint64_t));
    if (!keys) return ORC_ERR_NOMEM;
    for (int i = 0; i < n; i++) {
        float w[3];
        for (int a = 0; a < 3; a++) w[a] = pos[(int64_t)i * stride + a] + orig[a];
        for (int lev = 0; lev < depth; lev++) {
            if (w[0] < 0 || w[1] < 0 || w[2] < 0) {
                keys[(int64_t)i * depth + lev] = make_key(255, 0, 0, 0);
            } else {
                int rng = g->range[lev];
                keys[(int64_t)i * depth + lev] =
                    make_key(lev, cover_f(w[0], rng) / rng, cover_f(w[1], rng) / rng, cover_f(w[2], rng) / rng);
            }
        }
    }
    int levcnt[MAXLEV];
    sort_unique(keys, nk, levcnt, depth);
    int rc = alloc_from_keys(g, keys, levcnt, depth);
    free(keys);
    if (rc) return rc;
    link_levels(g, depth);
    return ORC_OK;
}

/* box of a point for the extra / incremental passes (PT.cuh:433-434, 481-482) */
static void point_box(const float* w, float radius, int full, int* bmin, int* bmax)
{
    for (int a = 0; a < 3; a++) {
        bmin[a] = (int)((float)(int)w[a] - radius);
        bmax[a] = (int)((float)(int)w[a] + (full ? 2.0f * radius : radius));
    }
}

/* ActivateExtraBricksGPU (VG.cpp:931-1016) + gvdbCalcExtraBrickId (PT.cuh:467-512) */
static int activate_extra(orc_grid* g, int n, const float* pos, int stride, const float* orig, float radius,
                          int depth)
{
    int64_t cap = 1024, cnt = 0;
    uint64_t* keys = (uint64_t*)malloc((size_t)cap * sizeof(uint64_t));
    if (!keys) return ORC_ERR_NOMEM;
    for (int i = 0; i < n; i++) {
        float w[3];
        for (int a = 0; a < 3; a++) w[a] = pos[(int64_t)i * stride + a] + orig[a];
        if (w[0] < 0 || w[1] < 0 || w[2] < 0) continue;
        int bmin[3], bmax[3];
        point_box(w, radius, 1, bmin, bmax);
        for (int lev = 0; lev < depth; lev++) {
            int r = g->range[lev];
            int nd[3];
            for (nd[0] = bmin[0] / r * r; nd[0] <= bmax[0] / r * r; nd[0] += r)
                for (nd[1] = bmin[1] / r * r; nd[1] <= bmax[1] / r * r; nd[1] += r)
                    for (nd[2] = bmin[2] / r * r; nd[2] <= bmax[2] / r * r; nd[2] += r) {
                        if (nd[0] < 0 || nd[1] < 0 || nd[2] < 0) { g->degenerate = 1; continue; }
                        int64_t pid = get_pos_parent(g, nd, lev);
                        if (pid == -1) {
                            if (cnt >= cap) {
                                cap *= 2;
                                uint64_t* k2 = (uint64_t*)realloc(keys, (size_t)cap * sizeof(uint64_t));
                                if (!k2) { free(keys); return ORC_ERR_NOMEM; }
                                keys = k2;
                            }
                            keys[cnt++] = make_key(lev, nd[0] / r, nd[1] / r, nd[2] / r);
                        }
                    }
        }
    }
    int levcnt[MAXLEV];
    sort_unique(keys, cnt, levcnt, depth);
    int rc = alloc_from_keys(g, keys, levcnt, depth);
    free(keys);
    if (rc) return rc;
    link_levels(g, depth);
    return ORC_OK;
}

/* gvdbDelinkLeafBricks / gvdbDelinkBricks (ND.cuh:401-467), VG.cpp:1131-1140 */
static void delink(orc_grid* g, int depth)
{
    pool* p0 = &g->pools[0];
    for (int i = 0; i < p0->cnt; i++) {
        orc_node* node = &p0->nodes[i];
        if (node->flags) continue;
        if (node->parent == ID_UNDEF64) continue;
        int64_t pid = get_parent(g, 1, node->pos);
        orc_node* pn = node_at(g, 1, pid);
        if (!pn) continue;
        int pos3[3] = {node->pos[0], node->pos[1], node->pos[2]};
        int b = child_bit(g, 1, pn->pos, pos3);
        if (b < 0) continue;
        node->parent = ID_UNDEF64;
        g->pools[1].clist[(int64_t)(pn->childlist >> 16) * voxcnt(g, 1) + b] = ID_UNDEF64;
    }
    for (int lev = 1; lev < depth; lev++) {
        pool* p = &g->pools[lev];
        int64_t vc = voxcnt(g, lev);
        for (int i = 0; i < p->cnt; i++) {
            orc_node* node = &p->nodes[i];
            if (node->parent == ID_UNDEF64) { node->flags = 0; continue; }
            int any = 0;
            for (int64_t ci = 0; ci < vc; ci++)
                if (p->clist[(int64_t)i * vc + ci] != ID_UNDEF64) { any = 1; break; }
            if (any) { node->flags = 1; continue; }
            node->flags = 0;
            int64_t pid = get_parent(g, lev + 1, node->pos);
            orc_node* pn = node_at(g, lev + 1, pid);
            if (!pn) continue;
            int pos3[3] = {node->pos[0], node->pos[1], node->pos[2]};
            int b = child_bit(g, lev + 1, pn->pos, pos3);
            if (b < 0) continue;
            node->parent = ID_UNDEF64;
            g->pools[lev + 1].clist[(int64_t)(pn->childlist >> 16) * voxcnt(g, lev + 1) + b] = ID_UNDEF64;
        }
    }
}

/* ActivateIncreBricksGPU (VG.cpp:1020-1156) + gvdbCalcIncreExtraBrickId (PT.cuh:420-465) */
static int activate_incremental(orc_grid* g, int n, const float* pos, int stride, const float* orig,
                                float radius, int depth, int accum)
{
    pool* p0 = &g->pools[0];
    if (p0->cnt == 0) return ORC_OK;
    int total = p0->cnt;
    int* marker = (int*)calloc((size_t)total, sizeof(int));
    if (!marker) return ORC_ERR_NOMEM;
    if (accum)
        for (int i = 0; i < total; i++) marker[i] = p0->nodes[i].flags;

    int64_t cap = 1024, cnt = 0;
    uint64_t* keys = (uint64_t*)malloc((size_t)cap * sizeof(uint64_t));
    if (!keys) { free(marker); return ORC_ERR_NOMEM; }
    for (int i = 0; i < n; i++) {
        float w[3];
        for (int a = 0; a < 3; a++) w[a] = pos[(int64_t)i * stride + a] + orig[a];
        if (w[0] < 0 || w[1] < 0 || w[2] < 0) continue;
        int bmin[3], bmax[3];
        point_box(w, radius, 0, bmin, bmax);
        for (int lev = 0; lev < depth; lev++) {
            int r = g->range[lev];
            int nd[3];
            for (nd[0] = bmin[0] / r * r; nd[0] <= bmax[0] / r * r; nd[0] += r)
                for (nd[1] = bmin[1] / r * r; nd[1] <= bmax[1] / r * r; nd[1] += r)
                    for (nd[2] = bmin[2] / r * r; nd[2] <= bmax[2] / r * r; nd[2] += r) {
                        if (nd[0] < 0 || nd[1] < 0 || nd[2] < 0) { g->degenerate = 1; continue; }
                        int64_t pid = get_pos_parent(g, nd, lev);
                        if (pid == -1) {
                            if (cnt >= cap) {
                                cap *= 2;
                                uint64_t* k2 = (uint64_t*)realloc(keys, (size_t)cap * sizeof(uint64_t));
                                if (!k2) { free(keys); free(marker); return ORC_ERR_NOMEM; }
                                keys = k2;
                            }
                            keys[cnt++] = make_key(lev, nd[0] / r, nd[1] / r, nd[2] / r);
                        } else if (lev == 0) {
                            if (pid >= 0 && pid < total) marker[pid] = 1;
                        }
                    }
        }
    }
    if (cnt == 0) {  /* VG.cpp:1066: no new node, markers are not applied */
        free(keys);
        free(marker);
        g->last_mode = 0;
        return ORC_OK;
    }
    int levcnt[MAXLEV];
    sort_unique(keys, cnt, levcnt, depth);
    for (int i = 0; i < total; i++) p0->nodes[i].flags = (uint8_t)marker[i];
    free(marker);
    int rc = alloc_from_keys(g, keys, levcnt, depth);
    free(keys);
    if (rc) return rc;
    link_levels(g, depth);
    delink(g, depth);
    int used = p0->cnt;
    for (int i = 0; i < p0->cnt; i++)
        if (!p0->nodes[i].flags) used--;
    p0->used = used;
    g->last_mode = 2;
    return ORC_OK;
}

/* RebuildTopology (VG.cpp:1181-1218) / AccumulateTopology (VG.cpp:1158-1178) */
int orc_rebuild_topology(orc_grid* g, int n, const float* pos, int stride, float radius, const float orig[3],
                         int mode, int min_depth)
{
    if (!g || n < 0 || (n > 0 && !pos) || stride < 3) return ORC_ERR_ARG;
    float o[3] = {orig ? orig[0] : 0.f, orig ? orig[1] : 0.f, orig ? orig[2] : 0.f};
    g->degenerate = 0;
    int rootpos[3];
    int depth = bbox_depth(g, n, pos, stride, o, rootpos);
    if (mode == ORC_TOPO_ACCUMULATE && !g->rebuild_topo) {
        /* AccumulateTopology raises the depth to iDepth and never checks a depth change */
        int d = depth;
        if (d >= 0 && d < min_depth) d = min_depth;
        if (d <= 0 || d >= g->levels) return ORC_ERR_DEPTH;
        int rc = activate_incremental(g, n, pos, stride, o, radius, d, 1);
        return rc ? rc : (g->degenerate ? ORC_ERR_DEGENERATE : ORC_OK);
    }
    if (depth <= 0 || depth >= g->levels) return ORC_ERR_DEPTH;
    if (mode == ORC_TOPO_FULL) g->rebuild_topo = 1;
    if (g->rebuild_topo) {
        clear_tree(g);
    } else if (depth != g->curr_depth) {
        clear_tree(g);
        g->curr_depth = depth;
    }
    int rc;
    if (g->rebuild_topo) {
        rc = activate_bricks(g, n, pos, stride, o, depth, rootpos);
        if (!rc && radius >= 1) rc = activate_extra(g, n, pos, stride, o, radius, depth);
        g->rebuild_topo = 0;
        g->last_mode = 1;
    } else {
        rc = activate_incremental(g, n, pos, stride, o, radius, depth, 0);
    }
    if (rc) return rc;
    return g->degenerate ? ORC_ERR_DEGENERATE : ORC_OK;
}

/* ------------------------------------------------------------------ */
/* atlas: UpdateAtlas (VG.cpp:2630-2704), AtlasAlloc/getAtlasPos (AL.cpp:692-715),
 * AtlasResize (AL.cpp:622-650), ClearMapping/AssignMapping (VG.cpp:2559-2588) */

static int resize_channels(orc_grid* g, const int* nsub)
{
    int64_t slots = (int64_t)nsub[0] * nsub[1] * nsub[2];
    int64_t vox = (int64_t)g->P * g->P * g->P;
    for (int c = 0; c < MAXCH; c++) {
        if (!g->chtype[c] && !g->ch[c]) continue;
        if (!g->ch[c] && g->chslots[c] == 0 && g->ncomp[c] == 0) continue;
        double* nd = (double*)calloc((size_t)(slots * vox * g->ncomp[c]), sizeof(double));
        if (!nd) return ORC_ERR_NOMEM;
        if (g->ch[c]) {
            int64_t keep = g->chslots[c] < slots ? g->chslots[c] : slots;
            memcpy(nd, g->ch[c], (size_t)(keep * vox * g->ncomp[c]) * sizeof(double));
            free(g->ch[c]);
        }
        g->ch[c] = nd;
        g->chslots[c] = slots;
    }
    g->sub[0] = nsub[0]; g->sub[1] = nsub[1]; g->sub[2] = nsub[2];
    return ORC_OK;
}

int orc_add_channel(orc_grid* g, int chan, int type)
{
    if (!g || chan < 0 || chan >= MAXCH) return ORC_ERR_ARG;
    int nc;
    switch (type) {
    case ORC_T_FLOAT: case ORC_T_UCHAR: nc = 1; break;
    case ORC_T_FLOAT3: case ORC_T_FLOAT4: case ORC_T_UCHAR4: nc = 4; break;
    default: return ORC_ERR_ARG;
    }
    if (!g->have_atlas) {
        g->sub[0] = g->defsub[0]; g->sub[1] = g->defsub[1]; g->sub[2] = g->defsub[2];
        g->have_atlas = 1;
    }
    g->chtype[chan] = type == 0 ? 100 : type;   /* nonzero marker even for T_UCHAR */
    g->ncomp[chan] = nc;
    int64_t slots = (int64_t)g->sub[0] * g->sub[1] * g->sub[2];
    int64_t vox = (int64_t)g->P * g->P * g->P;
    free(g->ch[chan]);
    g->ch[chan] = (double*)calloc((size_t)(slots * vox * nc), sizeof(double));
    if (!g->ch[chan]) return ORC_ERR_NOMEM;
    g->chslots[chan] = slots;
    return ORC_OK;
}

/* the atlas layout (slot assignment, atlas map, mValue) without any channel
 * storage, for topology and sampled-splat checks at sizes whose FP64 atlas
 * would not fit; the subdivision starts as AddChannel's would */
int orc_atlas_layout_only(orc_grid* g)
{
    if (!g) return ORC_ERR_ARG;
    if (!g->have_atlas) {
        g->sub[0] = g->defsub[0]; g->sub[1] = g->defsub[1]; g->sub[2] = g->defsub[2];
        g->have_atlas = 1;
    }
    return ORC_OK;
}

int orc_clear_channel(orc_grid* g, int chan)
{
    if (!g || chan < 0 || chan >= MAXCH || !g->ch[chan]) return ORC_ERR_ARG;
    memset(g->ch[chan], 0, (size_t)(g->chslots[chan] * g->P * g->P * g->P * g->ncomp[chan]) * sizeof(double));
    return ORC_OK;
}

int orc_update_atlas(orc_grid* g)
{
    if (!g || !g->have_atlas) return ORC_ERR_STATE;
    pool* p0 = &g->pools[0];
    int used = p0->used;
    int amax = g->sub[0] * g->sub[1] * g->sub[2];
    g->atlas_last = 0;
    if (used > amax) {
        int nsub[3] = {g->sub[0], g->sub[1], (int)ceil(used / (float)(g->sub[0] * g->sub[1]))};
        int rc = resize_channels(g, nsub);
        if (rc) return rc;
    }
    int P = g->P, a = g->apron;
    for (int i = 0; i < p0->cnt; i++) {
        orc_node* nd = &p0->nodes[i];
        if (!nd->flags) continue;
        int id = g->atlas_last++;
        int a2 = g->sub[0] * g->sub[1];
        int z = id / a2, rem = id - z * a2;
        int y = rem / g->sub[0], x = rem - y * g->sub[0];
        nd->value[0] = x * P + a; nd->value[1] = y * P + a; nd->value[2] = z * P + a;
    }
    int slots = g->sub[0] * g->sub[1] * g->sub[2];
    free(g->amap);
    g->amap = (int32_t*)malloc((size_t)slots * 4 * sizeof(int32_t));
    if (!g->amap) return ORC_ERR_NOMEM;
    g->amap_slots = slots;
    for (int s = 0; s < slots; s++) {
        g->amap[4 * s + 0] = g->amap[4 * s + 1] = g->amap[4 * s + 2] = (int32_t)0xFFFFFFFF;
        g->amap[4 * s + 3] = (int32_t)0xFFFFFFFF;
    }
    for (int i = 0; i < p0->cnt; i++) {
        orc_node* nd = &p0->nodes[i];
        if (!nd->flags) continue;
        int bx = nd->value[0] / P, by = nd->value[1] / P, bz = nd->value[2] / P;
        int id = (bz * g->sub[1] + by) * g->sub[0] + bx;
        g->amap[4 * id + 0] = nd->pos[0]; g->amap[4 * id + 1] = nd->pos[1]; g->amap[4 * id + 2] = nd->pos[2];
        g->amap[4 * id + 3] = i;
    }
    return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* queries */
int orc_root_level(const orc_grid* g) { return g ? g->root_level : -1; }
int orc_top_lev(const orc_grid* g) { return g ? top_lev_of(g) : -1; }
int orc_num_nodes(const orc_grid* g, int l) { return (g && l >= 0 && l < g->levels) ? g->pools[l].cnt : -1; }
int orc_num_used_leaves(const orc_grid* g) { return g ? g->pools[0].used : -1; }
int orc_last_mode(const orc_grid* g) { return g ? g->last_mode : -1; }
int orc_get_nodes(const orc_grid* g, int l, orc_node* out, int cap)
{
    if (!g || l < 0 || l >= g->levels || cap < g->pools[l].cnt) return ORC_ERR_ARG;
    if (g->pools[l].cnt) memcpy(out, g->pools[l].nodes, (size_t)g->pools[l].cnt * sizeof(orc_node));
    return ORC_OK;
}
int orc_get_childlist(const orc_grid* g, int l, uint64_t* out, int64_t cap)
{
    if (!g || l <= 0 || l >= g->levels) return ORC_ERR_ARG;
    int64_t n = (int64_t)g->pools[l].cnt * voxcnt(g, l);
    if (cap < n) return ORC_ERR_ARG;
    if (n) memcpy(out, g->pools[l].clist, (size_t)n * sizeof(uint64_t));
    return ORC_OK;
}
int orc_atlas_subdim(const orc_grid* g, int out[3])
{
    if (!g) return ORC_ERR_ARG;
    out[0] = g->sub[0]; out[1] = g->sub[1]; out[2] = g->sub[2];
    return ORC_OK;
}
int orc_get_atlas_map(const orc_grid* g, int32_t* out4, int cap)
{
    if (!g || !g->amap || cap < g->amap_slots) return ORC_ERR_ARG;
    memcpy(out4, g->amap, (size_t)g->amap_slots * 4 * sizeof(int32_t));
    return ORC_OK;
}
int64_t orc_channel_size(const orc_grid* g, int chan)
{
    if (!g || chan < 0 || chan >= MAXCH || !g->ch[chan]) return -1;
    return g->chslots[chan] * g->P * g->P * g->P * g->ncomp[chan];
}
int orc_read_channel(const orc_grid* g, int chan, double* out, int64_t cap)
{
    int64_t n = orc_channel_size(g, chan);
    if (n < 0 || cap < n) return ORC_ERR_ARG;
    memcpy(out, g->ch[chan], (size_t)n * sizeof(double));
    return ORC_OK;
}
int orc_write_channel(orc_grid* g, int chan, const double* in, int64_t count)
{
    int64_t n = orc_channel_size(g, chan);
    if (n < 0 || count != n) return ORC_ERR_ARG;
    memcpy(g->ch[chan], in, (size_t)n * sizeof(double));
    return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* splats */

/* voxel in an atlas slot: brick-major padded layout */
static double* vox_ptr(orc_grid* g, int chan, const int32_t* value, int lx, int ly, int lz)
{
    /* value = atlas voxel of the interior corner (mValue); padded local = interior local + apron */
    int P = g->P;
    int bx = value[0] / P, by = value[1] / P, bz = value[2] / P;
    int64_t slot = ((int64_t)bz * g->sub[1] + by) * g->sub[0] + bx;
    int ox = lx + g->apron, oy = ly + g->apron, oz = lz + g->apron;
    int64_t loc = ((slot * P + oz) * P + oy) * P + ox;
    return g->ch[chan] + loc * g->ncomp[chan];
}

/* Monaghan & Lattanzio (1985) M4 cubic spline, 3D normalisation 1/(pi h^3) */
static double m4(double q)
{
    if (q < 1.0) return 1.0 - 1.5 * q * q + 0.75 * q * q * q;
    if (q < 2.0) { double t = 2.0 - q; return 0.25 * t * t * t; }
    return 0.0;
}

/* leaf index of every integer voxel: active leaf containing it, -1 if none.
 * Uses the pool directly (a voxel belongs to the active leaf whose box holds it). */
typedef struct { int64_t key; int idx; } kv;
static int cmp_kv(const void* a, const void* b)
{
    int64_t x = ((const kv*)a)->key, y = ((const kv*)b)->key;
    return x < y ? -1 : (x > y ? 1 : 0);
}
static int64_t leaf_key(int bx, int by, int bz) { return ((int64_t)bx << 42) | ((int64_t)by << 21) | (int64_t)bz; }
static int find_leaf(const kv* tab, int n, int64_t key)
{
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        if (tab[mid].key == key) return tab[mid].idx;
        if (tab[mid].key < key) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}
static kv* active_leaf_table(orc_grid* g, int* nout)
{
    pool* p0 = &g->pools[0];
    kv* t = (kv*)malloc((size_t)(p0->cnt + 1) * sizeof(kv));
    int m = 0;
    int b = g->brick;
    for (int i = 0; i < p0->cnt; i++) {
        if (!p0->nodes[i].flags || p0->nodes[i].value[0] < 0) continue;
        t[m].key = leaf_key(p0->nodes[i].pos[0] / b, p0->nodes[i].pos[1] / b, p0->nodes[i].pos[2] / b);
        t[m].idx = i;
        m++;
    }
    qsort(t, (size_t)m, sizeof(kv), cmp_kv);
    *nout = m;
    return t;
}

/* adds a contribution at world voxel v to every active brick whose padded box
 * holds v: the owner's interior voxel and the apron copies in its neighbours */
static void add_contrib(orc_grid* g, const kv* tab, int nt, int chan_d, int chan_v, int vx, int vy, int vz,
                        double wgt, const double* u)
{
    if (vx < 0 || vy < 0 || vz < 0) return;
    int b = g->brick, a = g->apron;
    int c0[3] = {vx / b, vy / b, vz / b};
    for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
                int k[3] = {c0[0] + dx, c0[1] + dy, c0[2] + dz};
                if (k[0] < 0 || k[1] < 0 || k[2] < 0) continue;
                int lx = vx - k[0] * b, ly = vy - k[1] * b, lz = vz - k[2] * b;
                if (lx < -a || ly < -a || lz < -a || lx >= b + a || ly >= b + a || lz >= b + a) continue;
                int li = find_leaf(tab, nt, leaf_key(k[0], k[1], k[2]));
                if (li < 0) continue;
                orc_node* nd = &g->pools[0].nodes[li];
                if (chan_d >= 0) *vox_ptr(g, chan_d, nd->value, lx, ly, lz) += wgt;
                if (chan_v >= 0 && u) {
                    double* v = vox_ptr(g, chan_v, nd->value, lx, ly, lz);
                    v[0] += wgt * u[0]; v[1] += wgt * u[1]; v[2] += wgt * u[2];
                }
            }
}

/* apron voxels whose world position lies in no active brick -> value */
static void apron_unowned(orc_grid* g, const kv* tab, int nt, int chan, double value)
{
    if (chan < 0 || g->apron == 0) return;
    pool* p0 = &g->pools[0];
    int b = g->brick;
    for (int i = 0; i < p0->cnt; i++) {
        orc_node* nd = &p0->nodes[i];
        if (!nd->flags || nd->value[0] < 0) continue;
        for (int z = -1; z <= b; z++)
            for (int y = -1; y <= b; y++)
                for (int x = -1; x <= b; x++) {
                    if (x >= 0 && x < b && y >= 0 && y < b && z >= 0 && z < b) continue;
                    int w[3] = {nd->pos[0] + x, nd->pos[1] + y, nd->pos[2] + z};
                    int li = -1;
                    if (w[0] >= 0 && w[1] >= 0 && w[2] >= 0)
                        li = find_leaf(tab, nt, leaf_key(w[0] / b, w[1] / b, w[2] / b));
                    if (li >= 0) continue;
                    double* v = vox_ptr(g, chan, nd->value, x, y, z);
                    for (int c = 0; c < g->ncomp[chan]; c++) v[c] = value;
                }
    }
}

/* zero every voxel (interior and apron) of the active bricks */
static void zero_active(orc_grid* g, int chan)
{
    if (chan < 0) return;
    pool* p0 = &g->pools[0];
    int P = g->P;
    for (int i = 0; i < p0->cnt; i++) {
        orc_node* nd = &p0->nodes[i];
        if (!nd->flags || nd->value[0] < 0) continue;
        for (int z = -g->apron; z < g->brick + g->apron; z++)
            for (int y = -g->apron; y < g->brick + g->apron; y++)
                for (int x = -g->apron; x < g->brick + g->apron; x++) {
                    double* v = vox_ptr(g, chan, nd->value, x, y, z);
                    for (int c = 0; c < g->ncomp[chan]; c++) v[c] = 0.0;
                }
    }
    (void)P;
}

static int splat_new(orc_grid* g, int mode, int n, const float* pos, int ps, const float* weight,
                     const float* rad_pp, const float* vel, int vs, float radius, const float* tr, int chan_d,
                     int chan_v, int accum)
{
    int nt;
    kv* tab = active_leaf_table(g, &nt);
    if (!accum) { zero_active(g, chan_d); zero_active(g, chan_v); }
    for (int i = 0; i < n; i++) {
        float wf[3];
        for (int a = 0; a < 3; a++) wf[a] = pos[(int64_t)i * ps + a] + tr[a];
        if (wf[0] < 0 || wf[1] < 0 || wf[2] < 0) continue;
        /* only points inside an active brick are splatted */
        if (find_leaf(tab, nt, leaf_key((int)floorf(wf[0]) / g->brick, (int)floorf(wf[1]) / g->brick,
                                        (int)floorf(wf[2]) / g->brick)) < 0)
            continue;
        double p[3] = {wf[0], wf[1], wf[2]};
        double w = weight ? (double)weight[i] : 1.0;
        double u[3] = {0, 0, 0};
        if (vel) { u[0] = vel[(int64_t)i * vs]; u[1] = vel[(int64_t)i * vs + 1]; u[2] = vel[(int64_t)i * vs + 2]; }
        if (mode == ORC_SPLAT_TRILINEAR) {
            int i0[3];
            double f[3];
            for (int a = 0; a < 3; a++) { i0[a] = (int)floor(p[a]); f[a] = p[a] - i0[a]; }
            for (int dz = 0; dz < 2; dz++)
                for (int dy = 0; dy < 2; dy++)
                    for (int dx = 0; dx < 2; dx++) {
                        double wt = (dx ? f[0] : 1 - f[0]) * (dy ? f[1] : 1 - f[1]) * (dz ? f[2] : 1 - f[2]);
                        add_contrib(g, tab, nt, chan_d, chan_v, i0[0] + dx, i0[1] + dy, i0[2] + dz, w * wt,
                                    vel ? u : NULL);
                    }
        } else {
            double R = rad_pp ? (double)rad_pp[i] : (double)radius;
            double h = 0.5 * R;
            double norm = 1.0 / (3.14159265358979323846 * h * h * h);
            int lo[3], hi[3];
            for (int a = 0; a < 3; a++) { lo[a] = (int)floor(p[a] - R); hi[a] = (int)ceil(p[a] + R); }
            for (int z = lo[2]; z <= hi[2]; z++)
                for (int y = lo[1]; y <= hi[1]; y++)
                    for (int x = lo[0]; x <= hi[0]; x++) {
                        double dx = x - p[0], dy = y - p[1], dz = z - p[2];
                        double q = sqrt(dx * dx + dy * dy + dz * dz) / h;
                        if (q >= 2.0) continue;
                        add_contrib(g, tab, nt, chan_d, chan_v, x, y, z, w * norm * m4(q), vel ? u : NULL);
                    }
        }
    }
    if (!accum) { apron_unowned(g, tab, nt, chan_d, 0.0); apron_unowned(g, tab, nt, chan_v, 0.0); }
    free(tab);
    return ORC_OK;
}

static int floor_div(int v, int b) { return v >= 0 ? v / b : -((-v + b - 1) / b); }

/* The trilinear / cubic splat of splat_new restricted to a sample of leaves,
 * without atlas channels (a 4M-point frame's FP64 atlas would take tens of
 * GB): the same per-point weights and the same rule for which bricks receive
 * a contribution (every active leaf whose padded box holds the voxel), so a
 * sampled leaf's padded P^3 voxels get exactly what splat_new writes there.
 * Values are ADDED to dens_out[((k*P + lz)*P + ly)*P + lx] and to
 * vel_out[(...)*3 + c] (k = index in `leaves`; either output may be NULL);
 * the caller zeroes them for a fresh splat and keeps them to accumulate.  A
 * listed pool index that is not an active leaf with an atlas slot takes
 * nothing.  zero_unowned: afterwards the sampled apron voxels whose world
 * position lies in no active leaf are set to 0, as a non-accumulating splat
 * leaves them (apron_unowned). */
int orc_splat_sample(orc_grid* g, int mode, int n, const float* pos, int ps, const float* weight,
                     const float* rad_pp, const float* vel, int vs, float radius, const float trans[3],
                     const int* leaves, int nleaves, int zero_unowned, double* dens_out, double* vel_out)
{
    if (!g || n < 0 || (n > 0 && !pos) || ps < 3 || nleaves < 0 || (nleaves > 0 && !leaves)) return ORC_ERR_ARG;
    if (mode != ORC_SPLAT_TRILINEAR && mode != ORC_SPLAT_CUBIC) return ORC_ERR_ARG;
    if (g->root_level < 0) return ORC_ERR_STATE;
    const float tr[3] = {trans ? trans[0] : 0.f, trans ? trans[1] : 0.f, trans ? trans[2] : 0.f};
    const int b = g->brick, a = g->apron, P = g->P;
    const int64_t P3 = (int64_t)P * P * P;
    pool* p0 = &g->pools[0];
    /* dense map brick coordinate -> sample index over the sampled bricks' box */
    int kmin[3] = {1 << 30, 1 << 30, 1 << 30}, kmax[3] = {-1, -1, -1};
    int valid = 0;
    for (int k = 0; k < nleaves; k++) {
        const int li = leaves[k];
        if (li < 0 || li >= p0->cnt || !p0->nodes[li].flags || p0->nodes[li].value[0] < 0) continue;
        for (int c = 0; c < 3; c++) {
            const int kc = p0->nodes[li].pos[c] / b;
            if (kc < kmin[c]) kmin[c] = kc;
            if (kc > kmax[c]) kmax[c] = kc;
        }
        valid++;
    }
    if (!valid) return ORC_OK;
    const int64_t ext[3] = {kmax[0] - kmin[0] + 1, kmax[1] - kmin[1] + 1, kmax[2] - kmin[2] + 1};
    const int64_t cells = ext[0] * ext[1] * ext[2];
    if (cells > ((int64_t)1 << 27)) return ORC_ERR_NOMEM;
    int* dmap = (int*)malloc((size_t)cells * sizeof(int));
    if (!dmap) return ORC_ERR_NOMEM;
    for (int64_t c = 0; c < cells; c++) dmap[c] = -1;
    for (int k = 0; k < nleaves; k++) {
        const int li = leaves[k];
        if (li < 0 || li >= p0->cnt || !p0->nodes[li].flags || p0->nodes[li].value[0] < 0) continue;
        const int64_t c = ((int64_t)(p0->nodes[li].pos[2] / b - kmin[2]) * ext[1] +
                           (p0->nodes[li].pos[1] / b - kmin[1])) * ext[0] + (p0->nodes[li].pos[0] / b - kmin[0]);
        dmap[c] = k;
    }
#define SAMPLE_AT(kx, ky, kz)                                                                              \
    (((kx) < kmin[0] || (ky) < kmin[1] || (kz) < kmin[2] || (kx) > kmax[0] || (ky) > kmax[1] ||          \
      (kz) > kmax[2])                                                                                      \
         ? -1                                                                                              \
         : dmap[((int64_t)((kz) - kmin[2]) * ext[1] + ((ky) - kmin[1])) * ext[0] + ((kx) - kmin[0])])
    int nt;
    kv* tab = active_leaf_table(g, &nt);
    for (int i = 0; i < n; i++) {
        float wf[3];
        for (int c = 0; c < 3; c++) wf[c] = pos[(int64_t)i * ps + c] + tr[c];
        if (wf[0] < 0 || wf[1] < 0 || wf[2] < 0) continue;
        if (find_leaf(tab, nt, leaf_key((int)floorf(wf[0]) / b, (int)floorf(wf[1]) / b, (int)floorf(wf[2]) / b)) < 0)
            continue;
        double p[3] = {wf[0], wf[1], wf[2]};
        const double R = rad_pp ? (double)rad_pp[i] : (double)radius;
        int lo[3], hi[3];
        for (int c = 0; c < 3; c++) {
            if (mode == ORC_SPLAT_TRILINEAR) { lo[c] = (int)floor(p[c]); hi[c] = lo[c] + 1; }
            else { lo[c] = (int)floor(p[c] - R); hi[c] = (int)ceil(p[c] + R); }
        }
        /* does the footprint reach a sampled brick at all? */
        int hit = 0;
        const int h0[3] = {floor_div(lo[0] - a, b), floor_div(lo[1] - a, b), floor_div(lo[2] - a, b)};
        const int h1[3] = {floor_div(hi[0] + a, b), floor_div(hi[1] + a, b), floor_div(hi[2] + a, b)};
        for (int kz = h0[2]; kz <= h1[2] && !hit; kz++)
            for (int ky = h0[1]; ky <= h1[1] && !hit; ky++)
                for (int kx = h0[0]; kx <= h1[0] && !hit; kx++)
                    if (SAMPLE_AT(kx, ky, kz) >= 0) hit = 1;
        if (!hit) continue;
        const double w = weight ? (double)weight[i] : 1.0;
        double u[3] = {0, 0, 0};
        if (vel) { u[0] = vel[(int64_t)i * vs]; u[1] = vel[(int64_t)i * vs + 1]; u[2] = vel[(int64_t)i * vs + 2]; }
        double f[3];
        for (int c = 0; c < 3; c++) f[c] = p[c] - floor(p[c]);
        const double h = 0.5 * R;
        const double norm = 1.0 / (3.14159265358979323846 * h * h * h);
        for (int z = lo[2]; z <= hi[2]; z++)
            for (int y = lo[1]; y <= hi[1]; y++)
                for (int x = lo[0]; x <= hi[0]; x++) {
                    double wt;
                    if (mode == ORC_SPLAT_TRILINEAR) {
                        const int dx = x - lo[0], dy = y - lo[1], dz = z - lo[2];
                        wt = w * ((dx ? f[0] : 1 - f[0]) * (dy ? f[1] : 1 - f[1]) * (dz ? f[2] : 1 - f[2]));
                    } else {
                        const double ddx = x - p[0], ddy = y - p[1], ddz = z - p[2];
                        const double q = sqrt(ddx * ddx + ddy * ddy + ddz * ddz) / h;
                        if (q >= 2.0) continue;
                        wt = w * norm * m4(q);
                    }
                    if (x < 0 || y < 0 || z < 0) continue;
                    for (int kz = floor_div(z - a, b); kz <= floor_div(z + a, b); kz++)
                        for (int ky = floor_div(y - a, b); ky <= floor_div(y + a, b); ky++)
                            for (int kx = floor_div(x - a, b); kx <= floor_div(x + a, b); kx++) {
                                if (kx < 0 || ky < 0 || kz < 0) continue;
                                const int sk = SAMPLE_AT(kx, ky, kz);
                                if (sk < 0) continue;
                                const int lx = x - kx * b + a, ly = y - ky * b + a, lz = z - kz * b + a;
                                const int64_t vi = (int64_t)sk * P3 + ((int64_t)lz * P + ly) * P + lx;
                                if (dens_out) dens_out[vi] += wt;
                                if (vel_out && vel) {
                                    vel_out[vi * 3] += wt * u[0];
                                    vel_out[vi * 3 + 1] += wt * u[1];
                                    vel_out[vi * 3 + 2] += wt * u[2];
                                }
                            }
                }
    }
    if (zero_unowned && a > 0) {
        for (int k = 0; k < nleaves; k++) {
            const int li = leaves[k];
            if (li < 0 || li >= p0->cnt || !p0->nodes[li].flags || p0->nodes[li].value[0] < 0) continue;
            const orc_node* nd = &p0->nodes[li];
            for (int z = -a; z < b + a; z++)
                for (int y = -a; y < b + a; y++)
                    for (int x = -a; x < b + a; x++) {
                        if (x >= 0 && x < b && y >= 0 && y < b && z >= 0 && z < b) continue;
                        const int wv[3] = {nd->pos[0] + x, nd->pos[1] + y, nd->pos[2] + z};
                        int li2 = -1;
                        if (wv[0] >= 0 && wv[1] >= 0 && wv[2] >= 0)
                            li2 = find_leaf(tab, nt, leaf_key(wv[0] / b, wv[1] / b, wv[2] / b));
                        if (li2 >= 0) continue;
                        const int64_t vi = (int64_t)k * P3 + ((int64_t)(z + a) * P + (y + a)) * P + (x + a);
                        if (dens_out) dens_out[vi] = 0.0;
                        if (vel_out) vel_out[vi * 3] = vel_out[vi * 3 + 1] = vel_out[vi * 3 + 2] = 0.0;
                    }
        }
    }
#undef SAMPLE_AT
    free(tab);
    free(dmap);
    return ORC_OK;
}

/* InsertPoints (VG.cpp:5219-5267, PT.cuh:19-36) + ScatterDensity (VG.cpp:5624-5660,
 * PT.cuh:516-573), summed without the race of the surface read-modify-write */
static int splat_ref_scatter(orc_grid* g, int n, const float* pos, int ps, float radius, const float* tr,
                             int expand)
{
    int chan = 0; /* the reference kernel writes volOut[0] */
    if (!g->ch[chan]) return ORC_ERR_STATE;
    int res0 = g->res[0];
    for (int i = 0; i < n; i++) {
        const float* raw = pos + (int64_t)i * ps;
        if (raw[2] == NOHIT) continue;
        float w[3] = {raw[0] + tr[0], raw[1] + tr[1], raw[2] + tr[2]};
        int64_t nid = get_node_at_point(g, w);
        if (nid < 0) continue;
        orc_node* nd = &g->pools[0].nodes[nid];
        float p[3], pi[3];
        for (int a = 0; a < 3; a++) { p[a] = w[a] - (float)nd->pos[a]; pi[a] = (float)(int)p[a]; }
        if (pi[0] < 0 || pi[1] < 0 || pi[2] < 0 || pi[0] >= res0 || pi[1] >= res0 || pi[2] >= res0) continue;
        if (nd->value[0] < 0) continue;
        static const int offs[7][3] = {{0, 0, 0}, {-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
        int cnt = expand ? 7 : 1;
        for (int k = 0; k < cnt; k++) {
            double bx = (double)pi[0] + offs[k][0] - p[0];
            double by = (double)pi[1] + offs[k][1] - p[1];
            double bz = (double)pi[2] + offs[k][2] - p[2];
            double c = (bx * bx + by * by + bz * bz) / ((double)radius * (double)radius);
            double v = 1.0 + c * (-3.0 + c * (3.0 - c));
            int lx = (int)pi[0] + offs[k][0], ly = (int)pi[1] + offs[k][1], lz = (int)pi[2] + offs[k][2];
            if (lx < -g->apron || ly < -g->apron || lz < -g->apron || lx >= res0 + g->apron ||
                ly >= res0 + g->apron || lz >= res0 + g->apron)
                continue;
            *vox_ptr(g, chan, nd->value, lx, ly, lz) += v;
        }
    }
    return ORC_OK;
}

/* the colour half of gvdbScatterPointDensity (PT.cuh:555-571) and
 * gvdbScatterPointAvgCol (PT.cuh:610-642), from VolumeGVDB::ScatterDensity
 * (VG.cpp:5624-5660).  A point colours the interior voxel it lies in:
 *  - avg_color: the voxel of channel 1 = (sum r / count, sum g / count,
 *    sum b / count, 255), integer sums and division, over the voxel's points;
 *  - otherwise, unless an avg_color scatter ever ran on this grid (its colour
 *    buffer then exists and takes the sums, which nothing reads): channel 3
 *    gets one point's colour as given; the reference's writers race, the
 *    restatement takes the point of highest index. */
typedef struct { int64_t vox; int pt; } vox_pt;
static int cmp_vox_pt(const void* a, const void* b)
{
    const vox_pt *x = (const vox_pt*)a, *y = (const vox_pt*)b;
    if (x->vox != y->vox) return x->vox < y->vox ? -1 : 1;
    return x->pt < y->pt ? -1 : (x->pt > y->pt);
}

static int scatter_colour(orc_grid* g, int n, const float* pos, int ps, const uint8_t* clr, const float* tr,
                          int avg_color)
{
    const int chan = avg_color ? 1 : 3;
    if (avg_color) g->colavg_seen = 1;
    else if (g->colavg_seen) return ORC_OK;
    if (!g->ch[chan] || g->ncomp[chan] != 4) return ORC_ERR_ARG;
    int res0 = g->res[0];
    vox_pt* list = (vox_pt*)malloc((size_t)(n + 1) * sizeof(vox_pt));
    int64_t m = 0;
    for (int i = 0; i < n; i++) {
        const float* raw = pos + (int64_t)i * ps;
        if (raw[2] == NOHIT) continue;
        float w[3] = {raw[0] + tr[0], raw[1] + tr[1], raw[2] + tr[2]};
        int64_t nid = get_node_at_point(g, w);
        if (nid < 0) continue;
        orc_node* nd = &g->pools[0].nodes[nid];
        int pi[3];
        for (int a = 0; a < 3; a++) pi[a] = (int)(w[a] - (float)nd->pos[a]);
        if (pi[0] < 0 || pi[1] < 0 || pi[2] < 0 || pi[0] >= res0 || pi[1] >= res0 || pi[2] >= res0) continue;
        if (nd->value[0] < 0) continue;
        list[m].vox = vox_ptr(g, chan, nd->value, pi[0], pi[1], pi[2]) - g->ch[chan];
        list[m].pt = i;
        m++;
    }
    qsort(list, (size_t)m, sizeof(vox_pt), cmp_vox_pt);
    for (int64_t k = 0; k < m;) {
        int64_t e = k;
        uint32_t cnt = 0, sum[3] = {0, 0, 0};
        while (e < m && list[e].vox == list[k].vox) {
            for (int c = 0; c < 3; c++) sum[c] += clr[(int64_t)list[e].pt * 4 + c];
            cnt++;
            e++;
        }
        double* out = g->ch[chan] + list[k].vox;
        if (avg_color) {
            for (int c = 0; c < 3; c++) out[c] = (double)(uint8_t)(sum[c] / cnt);
            out[3] = 255.0;
        } else {
            const uint8_t* src = clr + (int64_t)list[e - 1].pt * 4;
            for (int c = 0; c < 4; c++) out[c] = (double)src[c];
        }
        k = e;
    }
    free(list);
    return ORC_OK;
}

int orc_scatter_density(orc_grid* g, int n, const float* pos, int pos_stride, const uint8_t* clr, float radius,
                        const float trans[3], int expand, int avg_color)
{
    if (!g || n < 0 || (n > 0 && !pos) || pos_stride < 3) return ORC_ERR_ARG;
    if (g->root_level < 0) return ORC_ERR_STATE;
    float tr[3] = {trans ? trans[0] : 0.f, trans ? trans[1] : 0.f, trans ? trans[2] : 0.f};
    g->degenerate = 0;
    int rc = splat_ref_scatter(g, n, pos, pos_stride, radius, tr, expand);
    if (rc || !clr) return rc;
    return scatter_colour(g, n, pos, pos_stride, clr, tr, avg_color);
}

/* float -> uint16 / uint32 as the GPU converts (truncation, saturating, NaN -> 0) */
static uint32_t f2u16_sat(float v)
{
    if (!(v > 0.0f)) return 0u;
    if (v >= 65535.0f) return 65535u;
    return (uint32_t)v;
}
static uint32_t f2u32_sat(float v)
{
    if (!(v > 0.0f)) return 0u;
    if (v >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)v;
}

/* the FP16 variant's point storage (gvdbInsertSubcell_fp16, PT.cuh:204-207):
 * (w - mPosMin) / mPosRange * 65535 per axis, truncated to 16 bits, and its
 * read-back in gvdbGatherLevelSet_fp16 (PT.cuh:797-799): q / 65535 * range + min,
 * every step a rounded float operation */
static void quantize_pos(const orc_grid* g, const float w[3], uint32_t q[3])
{
    for (int a = 0; a < 3; a++) {
        float range = g->pos_max[a] - g->pos_min[a];
        float t = (w[a] - g->pos_min[a]) / range;
        q[a] = f2u16_sat(t * 65535.0f);
    }
}
static void dequantize_pos(const orc_grid* g, const uint32_t q[3], float p[3])
{
    for (int a = 0; a < 3; a++) {
        float range = g->pos_max[a] - g->pos_min[a];
        float t = (float)q[a] / 65535.0f;
        t = t * range;
        p[a] = t + g->pos_min[a];
    }
}

/* InsertPointsSubcell (VG.cpp:4971-5092; PT.cuh:109-118, 218-315, 677-694) and
 * GatherDensity / GatherLevelSet (VG.cpp:5318-5373; PT.cuh:696-773) */
static int splat_gather(orc_grid* g, int levelset, int n, const float* pos, int ps, const uint8_t* clr,
                        float radius, float rins, const float* tr, int sc, int chan, int chan_clr, int accum,
                        int64_t* sc_len, int fp16)
{
    pool* p0 = &g->pools[0];
    if (!g->ch[chan]) return ORC_ERR_STATE;
    if (!fp16 && chan_clr >= 0 && (chan_clr >= MAXCH || !g->ch[chan_clr] || g->ncomp[chan_clr] != 4)) return ORC_ERR_ARG;
    if (fp16 && chan_clr >= 0 && (chan_clr >= MAXCH || !g->ch[chan_clr])) return ORC_ERR_ARG;
    if (!clr) chan_clr = -1; /* no point colours: the colour channel is not written */
    int b = g->brick;
    if (sc <= 0 || b % sc) return ORC_ERR_ARG;
    int scdim = b / sc, spb = scdim * scdim * scdim;
    int total = p0->cnt;
    int* mapping = (int*)malloc((size_t)(total + 1) * sizeof(int));
    int nflag = 0;
    for (int i = 0; i < total; i++) {
        mapping[i] = nflag;
        if (p0->nodes[i].parent != ID_UNDEF64) nflag++;
    }
    int64_t nsc = (int64_t)spb * p0->used;
    if (nflag != p0->used) { g->degenerate = 1; free(mapping); return ORC_ERR_DEGENERATE; }
    /* subcell point lists */
    int64_t* cnt = (int64_t*)calloc((size_t)(nsc + 1), sizeof(int64_t));
    int64_t lcap = 1024, lcnt = 0;
    int64_t* lsc = (int64_t*)malloc((size_t)lcap * sizeof(int64_t));
    int* lpt = (int*)malloc((size_t)lcap * sizeof(int));
    for (int i = 0; i < n; i++) {
        const float* raw = pos + (int64_t)i * ps;
        if (raw[2] == NOHIT) continue;
        float w[3] = {raw[0] + tr[0], raw[1] + tr[1], raw[2] + tr[2]};
        if (w[0] < 0 || w[1] < 0 || w[2] < 0) continue;
        int mn[3], mx[3];
        for (int a = 0; a < 3; a++) {
            mn[a] = ((int)(w[a] - rins) / sc) * sc;
            mx[a] = ((int)(w[a] + 1 + rins) / sc) * sc;
        }
        int s[3];
        for (s[0] = mn[0]; s[0] <= mx[0]; s[0] += sc)
            for (s[1] = mn[1]; s[1] <= mx[1]; s[1] += sc)
                for (s[2] = mn[2]; s[2] <= mx[2]; s[2] += sc) {
                    if (s[0] < 0 || s[1] < 0 || s[2] < 0) { g->degenerate = 1; continue; }
                    int64_t pid = get_pos_leaf_parent(g, s);
                    if (pid < 0) continue;
                    orc_node* nd = &p0->nodes[pid];
                    int pin[3] = {(s[0] - nd->pos[0]) / sc, (s[1] - nd->pos[1]) / sc, (s[2] - nd->pos[2]) / sc};
                    int loc = (pin[2] * scdim + pin[1]) * scdim + pin[0];
                    int64_t idx = (int64_t)mapping[pid] * spb + loc;
                    if (idx < 0 || idx >= nsc) { g->degenerate = 1; continue; }
                    if (lcnt >= lcap) {
                        lcap *= 2;
                        lsc = (int64_t*)realloc(lsc, (size_t)lcap * sizeof(int64_t));
                        lpt = (int*)realloc(lpt, (size_t)lcap * sizeof(int));
                    }
                    lsc[lcnt] = idx;
                    lpt[lcnt] = i;
                    lcnt++;
                    cnt[idx]++;
                }
    }
    int64_t* off = (int64_t*)calloc((size_t)(nsc + 1), sizeof(int64_t));
    for (int64_t k = 0; k < nsc; k++) off[k + 1] = off[k] + cnt[k];
    int* list = (int*)malloc((size_t)(lcnt + 1) * sizeof(int));
    int64_t* fill = (int64_t*)calloc((size_t)(nsc + 1), sizeof(int64_t));
    for (int64_t k = 0; k < lcnt; k++) list[off[lsc[k]] + fill[lsc[k]]++] = lpt[k];
    if (sc_len) *sc_len = lcnt;
    const int skip = !levelset && lcnt == 0; /* GatherDensity returns when pSCPntsLength is 0 (VG.cpp:5321) */
    /* gather per subcell voxel */
    for (int i = 0; i < total && !skip; i++) {
        orc_node* nd = &p0->nodes[i];
        if (nd->parent == ID_UNDEF64) continue;
        if (nd->value[0] < 0) continue;
        for (int s = 0; s < spb; s++) {
            int64_t idx = (int64_t)mapping[i] * spb + s;
            int so[3] = {(s % scdim) * sc, ((s / scdim) % scdim) * sc, ((s / scdim / scdim) % scdim) * sc};
            for (int tz = 0; tz < sc; tz++)
                for (int ty = 0; ty < sc; ty++)
                    for (int tx = 0; tx < sc; tx++) {
                        int lx = so[0] + tx, ly = so[1] + ty, lz = so[2] + tz;
                        double vpos[3] = {(double)(nd->pos[0] + lx), (double)(nd->pos[1] + ly),
                                          (double)(nd->pos[2] + lz)};
                        double* out = vox_ptr(g, chan, nd->value, lx, ly, lz);
                        if (fp16) {
                            /* gvdbGatherLevelSet_fp16 (PT.cuh:775-813) in its own float arithmetic:
                             * dist from 3, min(|p - v| - R); the colour sum of INT2CLR(c) / |p - v|
                             * from 0 (the reference leaves it uninitialised), written as CLR2INT of
                             * particles.cuh (components * 255 added with carries) */
                            float vf[3] = {(float)(nd->pos[0] + lx), (float)(nd->pos[1] + ly),
                                           (float)(nd->pos[2] + lz)};
                            float dist = 3.0f, c4[4] = {0.f, 0.f, 0.f, 0.f};
                            for (int64_t j = off[idx]; j < off[idx + 1]; j++) {
                                const float* raw = pos + (int64_t)list[j] * ps;
                                float w[3] = {raw[0] + tr[0], raw[1] + tr[1], raw[2] + tr[2]}, pq[3];
                                uint32_t q[3];
                                quantize_pos(g, w, q);
                                dequantize_pos(g, q, pq);
                                float dx = pq[0] - vf[0], dy = pq[1] - vf[1], dz = pq[2] - vf[2];
                                float s2 = dx * dx;
                                s2 = s2 + dy * dy;
                                s2 = s2 + dz * dz;
                                float c = sqrtf(s2);
                                float t = c - radius;
                                dist = t < dist ? t : dist;
                                if (chan_clr >= 0)
                                    for (int k = 0; k < 4; k++) {
                                        float comp = (float)clr[(int64_t)list[j] * 4 + k] / 255.0f;
                                        c4[k] = c4[k] + comp / c;
                                    }
                            }
                            *out = (double)dist;
                            if (chan_clr >= 0) {
                                uint32_t u = 0;
                                for (int k = 0; k < 4; k++) u += f2u32_sat(c4[k] * 255.0f) << (8 * k);
                                double* co = vox_ptr(g, chan_clr, nd->value, lx, ly, lz);
                                if (g->ncomp[chan_clr] == 4)
                                    for (int k = 0; k < 4; k++) co[k] = (double)((u >> (8 * k)) & 255u);
                                else {
                                    float bits;
                                    memcpy(&bits, &u, 4);
                                    co[0] = (double)bits;
                                }
                            }
                            continue;
                        }
                        double val = accum ? *out : (levelset ? 3.0 : 0.0);
                        for (int64_t j = off[idx]; j < off[idx + 1]; j++) {
                            const float* raw = pos + (int64_t)list[j] * ps;
                            double d[3];
                            for (int a = 0; a < 3; a++) d[a] = (double)(raw[a] + tr[a]) - vpos[a];
                            double c = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                            if (levelset) { double t = c - radius; if (t < val) val = t; }
                            else { double t = radius - c; if (t > val) val = t; }
                        }
                        *out = val;
                        if (chan_clr < 0) continue;
                        /* colour: mean of the listed points' colours and, with accum, the old one */
                        double* co = vox_ptr(g, chan_clr, nd->value, lx, ly, lz);
                        double c4[4] = {0.0, 0.0, 0.0, 1.0};
                        if (accum)
                            for (int k = 0; k < 4; k++) c4[k] = co[k] / 255.0;
                        for (int64_t j = off[idx]; j < off[idx + 1]; j++)
                            for (int k = 0; k < 4; k++) c4[k] += clr[(int64_t)list[j] * 4 + k] / 255.0;
                        double den = (double)(off[idx + 1] - off[idx]) + (accum ? 1.0 : 0.0);
                        for (int k = 0; k < 4; k++) {
                            double v = c4[k] / den * 255.0;
                            v = v != v ? 0.0 : (v < 0.0 ? 0.0 : (v > 255.0 ? 255.0 : v));
                            co[k] = floor(v);
                        }
                    }
        }
    }
    free(mapping); free(cnt); free(lsc); free(lpt); free(off); free(list); free(fill);
    (void)nsc;
    return g->degenerate ? ORC_ERR_DEGENERATE : ORC_OK;
}

int orc_splat(orc_grid* g, int mode, int n, const float* pos, int pos_stride, const float* weight,
              const float* radius_pp, const float* vel, int vel_stride, float radius, const float trans[3],
              int chan_density, int chan_vel, int accum, int expand, int subcell, float radius_ins)
{
    if (!g || n < 0 || (n > 0 && !pos) || pos_stride < 3) return ORC_ERR_ARG;
    if (g->root_level < 0) return ORC_ERR_STATE;
    float tr[3] = {trans ? trans[0] : 0.f, trans ? trans[1] : 0.f, trans ? trans[2] : 0.f};
    g->degenerate = 0;
    if (chan_density >= 0 && (chan_density >= MAXCH || !g->ch[chan_density])) return ORC_ERR_ARG;
    if (chan_vel >= 0 && (chan_vel >= MAXCH || !g->ch[chan_vel] || g->ncomp[chan_vel] != 4)) return ORC_ERR_ARG;
    switch (mode) {
    case ORC_SPLAT_TRILINEAR:
    case ORC_SPLAT_CUBIC:
        return splat_new(g, mode, n, pos, pos_stride, weight, radius_pp, vel, vel_stride, radius, tr,
                         chan_density, chan_vel, accum);
    case ORC_SPLAT_REF_SCATTER:
        return splat_ref_scatter(g, n, pos, pos_stride, radius, tr, expand);
    case ORC_SPLAT_GATHER_DENSITY:
    case ORC_SPLAT_GATHER_LEVELSET:
        return splat_gather(g, mode == ORC_SPLAT_GATHER_LEVELSET, n, pos, pos_stride, NULL, radius, radius_ins, tr,
                            subcell, chan_density, -1, accum, NULL, 0);
    }
    return ORC_ERR_ARG;
}

int orc_gather(orc_grid* g, int levelset, int n, const float* pos, int pos_stride, const uint8_t* clr,
               float radius, float radius_ins, const float trans[3], int subcell, int chan, int chan_clr,
               int accum, int64_t* sc_len)
{
    if (!g || n < 0 || (n > 0 && !pos) || pos_stride < 3) return ORC_ERR_ARG;
    if (g->root_level < 0) return ORC_ERR_STATE;
    if (chan < 0 || chan >= MAXCH || !g->ch[chan]) return ORC_ERR_ARG;
    float tr[3] = {trans ? trans[0] : 0.f, trans ? trans[1] : 0.f, trans ? trans[2] : 0.f};
    g->degenerate = 0;
    return splat_gather(g, levelset, n, pos, pos_stride, clr, radius, radius_ins, tr, subcell, chan, chan_clr,
                        accum, sc_len, 0);
}

/* ConvertAndTransform (VG.cpp:5668-5682, gvdbConvAndTransform PT.cuh:120-142):
 * (wmin + p * wdelta) * scal + trans per axis, each multiply-add one fused
 * (single-rounding) operation, p from three uint16 (src_bits 2) or floats (4) */
int orc_convert_and_transform(int n, const void* src, int src_bits, float* dst, const float wmin[3],
                              const float wdelta[3], const float trans[3], const float scal[3])
{
    if (n < 0 || (src_bits != 2 && src_bits != 4)) return ORC_ERR_ARG;
    for (int i = 0; i < n; i++) {
        for (int a = 0; a < 3; a++) {
            float p = src_bits == 2 ? (float)((const uint16_t*)src)[(int64_t)i * 3 + a]
                                    : ((const float*)src)[(int64_t)i * 3 + a];
            dst[(int64_t)i * 3 + a] = fmaf(fmaf(p, wdelta[a], wmin[a]), scal[a], trans[a]);
        }
    }
    return ORC_OK;
}

/* ComputeBounds (VG.cpp:1792-1816), run by FinishTopology (VG.cpp:1584):
 * mVoxMin and mVoxMax both start at the position of level-0 pool node 0,
 * whatever its flags (a delinked node still seeds them); then every active
 * leaf lowers the minimum to its position and raises the maximum to its
 * position + range.  mObjMin/Max = mVoxMin/Max, mVoxRes = max - min, and
 * mVoxResMax keeps the largest mVoxRes per axis since Configure.  The
 * reference reads pool node 0 of an empty pool (undefined); here an empty
 * pool gives zeros.  out: min[3], max[3], res[3], res_max[3]. */
int orc_compute_bounds(orc_grid* g, float out[12])
{
    float mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
    const pool* p0 = &g->pools[0];
    if (p0->cnt > 0) {
        const int range = g->range[0];
        for (int a = 0; a < 3; a++) mn[a] = mx[a] = (float)p0->nodes[0].pos[a];
        for (int n = 0; n < p0->cnt; n++) {
            const orc_node* c = &p0->nodes[n];
            if (!c->flags) continue;
            for (int a = 0; a < 3; a++) {
                if (c->pos[a] < mn[a]) mn[a] = (float)c->pos[a];
                if (c->pos[a] + range > mx[a]) mx[a] = (float)(c->pos[a] + range);
            }
        }
    }
    for (int a = 0; a < 3; a++) {
        const float res = mx[a] - mn[a];
        if (res > g->vox_res_max[a]) g->vox_res_max[a] = res;
        out[a] = mn[a];
        out[3 + a] = mx[a];
        out[6 + a] = res;
        out[9 + a] = g->vox_res_max[a];
    }
    return ORC_OK;
}

void orc_pos_bounds(orc_grid* g, float out[6])
{
    for (int a = 0; a < 3; a++) {
        out[a] = g->pos_min[a];
        out[3 + a] = g->pos_max[a];
    }
}

/* InsertPointsSubcell_FP16 (VG.cpp:5094-5190) + GatherLevelSet_FP16
 * (VG.cpp:5375-5401): the same subcell lists, positions stored as 16-bit
 * fractions of the last GetBoundingBox's box; chan_clr may be any 4-byte channel */
int orc_gather_fp16(orc_grid* g, int n, const float* pos, int pos_stride, const uint8_t* clr, float radius,
                    float radius_ins, const float trans[3], int subcell, int chan, int chan_clr, int64_t* sc_len)
{
    if (!g || n < 0 || (n > 0 && !pos) || pos_stride < 3) return ORC_ERR_ARG;
    if (g->root_level < 0) return ORC_ERR_STATE;
    if (chan < 0 || chan >= MAXCH || !g->ch[chan] || g->ncomp[chan] != 1) return ORC_ERR_ARG;
    float tr[3] = {trans ? trans[0] : 0.f, trans ? trans[1] : 0.f, trans ? trans[2] : 0.f};
    g->degenerate = 0;
    return splat_gather(g, 1, n, pos, pos_stride, clr, radius, radius_ins, tr, subcell, chan, chan_clr, 0, sc_len,
                        1);
}

/* ------------------------------------------------------------------ */
/* UpdateApron (VG.cpp:4418-4457) -> UpdateApron<T> (OP.cuh:73-126),
 * getAtlasToWorld (ND.cuh:145-153), getNodeAtPoint (ND.cuh:243-253) */
int orc_update_apron(orc_grid* g, int chan, double boundval)
{
    if (!g || chan < 0 || chan >= MAXCH || !g->ch[chan]) return ORC_ERR_ARG;
    g->degenerate = 0;
    if (g->apron == 0) return ORC_OK;
    pool* p0 = &g->pools[0];
    int P = g->P, b = g->brick, nc = g->ncomp[chan];
    for (int i = 0; i < p0->cnt; i++) {
        orc_node* nd = &p0->nodes[i];
        if (!nd->flags || nd->value[0] < 0) continue;
        for (int z = 0; z < P; z++)
            for (int y = 0; y < P; y++)
                for (int x = 0; x < P; x++) {
                    if (x > 0 && x < P - 1 && y > 0 && y < P - 1 && z > 0 && z < P - 1) continue;
                    int lx = x - 1, ly = y - 1, lz = z - 1;
                    float wpos[3] = {(float)(nd->pos[0] + lx) + 0.5f, (float)(nd->pos[1] + ly) + 0.5f,
                                     (float)(nd->pos[2] + lz) + 0.5f};
                    double* dst = vox_ptr(g, chan, nd->value, lx, ly, lz);
                    int64_t src = get_node_at_point(g, wpos);
                    if (src < 0) {
                        for (int c = 0; c < nc; c++) dst[c] = boundval;
                    } else {
                        orc_node* sn = &p0->nodes[src];
                        int sx = (int)(wpos[0] - (float)sn->pos[0]);
                        int sy = (int)(wpos[1] - (float)sn->pos[1]);
                        int sz = (int)(wpos[2] - (float)sn->pos[2]);
                        if (sx < 0 || sy < 0 || sz < 0 || sx >= b || sy >= b || sz >= b || sn->value[0] < 0) {
                            g->degenerate = 1;
                            continue;
                        }
                        double* s = vox_ptr(g, chan, sn->value, sx, sy, sz);
                        for (int c = 0; c < nc; c++) dst[c] = s[c];
                    }
                }
    }
    return g->degenerate ? ORC_ERR_DEGENERATE : ORC_OK;
}

/* UpdateNeighbors (VG.cpp:2527-2556) + UpdateApronFaces (VG.cpp:4461-4496,
 * gvdbUpdateApronFacesF OP.cuh:27-63): per leaf, its -x, -y, -z face
 * neighbours (the leaf covering the centre minus one brick), and for each
 * the b^2 voxel pairs across the shared face: the neighbour's +side apron
 * takes the leaf's first layer, the leaf's -side apron the neighbour's last
 * layer.  Edges, corners and faces without a neighbour are not written.
 * Float channels only, as the reference's kernel. */
int orc_update_apron_faces(orc_grid* g, int chan)
{
    if (!g || chan < 0 || chan >= MAXCH || !g->ch[chan] || g->ncomp[chan] != 1) return ORC_ERR_ARG;
    if (g->apron == 0) return ORC_OK;
    pool* p0 = &g->pools[0];
    const int b = g->brick;
    for (int i = 0; i < p0->cnt; i++) {
        orc_node* nd = &p0->nodes[i];
        if (!nd->flags || nd->value[0] < 0) continue;
        for (int side = 0; side < 3; side++) {
            float ct[3] = {(float)nd->pos[0] + 0.5f * b, (float)nd->pos[1] + 0.5f * b, (float)nd->pos[2] + 0.5f * b};
            ct[side] -= (float)b;
            int64_t nid = get_node_at_point(g, ct);
            if (nid < 0) continue;
            orc_node* nb = &p0->nodes[nid];
            if (nb->value[0] < 0) continue;
            for (int u = 0; u < b; u++)
                for (int v = 0; v < b; v++) {
                    int self[3], other[3];
                    if (side == 0) { self[0] = 0; self[1] = u; self[2] = v; }
                    else if (side == 1) { self[0] = u; self[1] = 0; self[2] = v; }
                    else { self[0] = u; self[1] = v; self[2] = 0; }
                    for (int a = 0; a < 3; a++) other[a] = self[a];
                    other[side] = b - 1;
                    double v1 = *vox_ptr(g, chan, nd->value, self[0], self[1], self[2]);
                    double v2 = *vox_ptr(g, chan, nb->value, other[0], other[1], other[2]);
                    int na[3] = {other[0], other[1], other[2]}, sa[3] = {self[0], self[1], self[2]};
                    na[side] = b;   /* the neighbour's apron across the face */
                    sa[side] = -1;  /* the leaf's apron across the face */
                    *vox_ptr(g, chan, nb->value, na[0], na[1], na[2]) = v1;
                    *vox_ptr(g, chan, nd->value, sa[0], sa[1], sa[2]) = v2;
                }
        }
    }
    return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* atlas voxel (X, Y, Z) of a channel, brick-major storage */
static double* atlas_voxel(orc_grid* g, int chan, int X, int Y, int Z)
{
    int P = g->P;
    int64_t slot = ((int64_t)(Z / P) * g->sub[1] + Y / P) * g->sub[0] + X / P;
    int64_t loc = ((slot * P + Z % P) * P + Y % P) * P + X % P;
    return g->ch[chan] + loc * g->ncomp[chan];
}

/* float -> uint32 as the GPU converts (truncation, saturating at 0 and 2^32-1) */
static uint32_t f2u_sat(float v)
{
    if (!(v > 0.0f)) return 0u;
    if (v >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)v;
}

/* Compute (VG.cpp:4532-4558): a launch of 8^3-thread blocks over
 * T = skipOverAprons ? getAtlasPackres : getAtlasRes threads per axis
 * (gvdb_allocator.cpp:953-961), rounded up to whole blocks, per iteration,
 * UpdateApron(channel, boundval) after each when bUpdateApron.
 * The operator's own index macro picks its voxels (OP.cuh:189-223):
 *  - the fills (GVDB_VOXUNPACKED, OP.cuh:352-380) write atlas voxel
 *    blockIdx*8 + threadIdx + 1: every voxel with all coordinates in
 *    [1, min(8*ceil(T/8) + 1, atlasRes)).
 *  - FUNC_SMOOTH (GVDB_VOXPACKED, OP.cuh:383-400) writes every brick interior
 *    voxel (packed voxel p -> p + (p / b) * 2a + a; threads past the atlas
 *    return, so both thread counts give the same voxels), from the six face
 *    neighbours in the atlas read before any write (LoadSharedMemory,
 *    OP.cuh:151-181).  With an apron those lie in the brick's own apron; with
 *    none they can lie in another brick or outside the atlas, where this
 *    restatement reads 0 (the reference's surface read there is out of range). */
int orc_compute(orc_grid* g, int effect, int chan, int iterations, const float params[3], int update_apron,
                int skip_over_aprons, double boundval)
{
    if (!g || chan < 0 || chan >= MAXCH || !g->ch[chan] || !params) return ORC_ERR_ARG;
    const int P = g->P, a = g->apron, b = g->P - 2 * g->apron, nc = g->ncomp[chan];
    const int res[3] = {g->sub[0] * P, g->sub[1] * P, g->sub[2] * P};
    int hi[3];
    for (int k = 0; k < 3; k++) {
        int T = skip_over_aprons ? g->sub[k] * b : res[k];
        int cover = (T + 7) / 8 * 8 + 1;
        hi[k] = cover < res[k] ? cover : res[k];
    }
    const int64_t total = (int64_t)res[0] * res[1] * res[2] * nc;
    const float p1 = params[0], p2 = params[1], p3 = params[2];
    if (effect == ORC_FUNC_FILL_F || effect == ORC_FUNC_SMOOTH) { if (nc != 1) return ORC_ERR_ARG; }
    else if (effect == ORC_FUNC_FILL_C4) { if (nc != 4) return ORC_ERR_ARG; }
    else if (effect != ORC_FUNC_FILL_C) return ORC_ERR_ARG;
    for (int it = 0; it < iterations; it++) {
        double* old = (double*)malloc((size_t)total * sizeof(double));
        if (!old) return ORC_ERR_NOMEM;
        memcpy(old, g->ch[chan], (size_t)total * sizeof(double));
        for (int Z = 0; Z < res[2]; Z++)
            for (int Y = 0; Y < res[1]; Y++)
                for (int X = 0; X < res[0]; X++) {
                    int inside;
                    if (effect == ORC_FUNC_SMOOTH) {
                        int lx = X % P, ly = Y % P, lz = Z % P;
                        inside = lx >= a && ly >= a && lz >= a && lx < P - a && ly < P - a && lz < P - a;
                    } else {
                        inside = X >= 1 && Y >= 1 && Z >= 1 && X < hi[0] && Y < hi[1] && Z < hi[2];
                    }
                    if (!inside) continue;
                    double* out = atlas_voxel(g, chan, X, Y, Z);
                    switch (effect) {
                    case ORC_FUNC_FILL_F:
                        if (p3 < 0)
                            out[0] = (double)(sinf((float)((double)(X * 12) / (3.141592 * 30.0))) +
                                              sinf((float)((double)(Y * 12) / (3.141592 * 30.0))) +
                                              sinf((float)((double)(Z * 12) / (3.141592 * 30.0))));
                        else
                            out[0] = p1;
                        break;
                    case ORC_FUNC_FILL_C: /* static_cast<uchar>(p1) on the GPU: truncated, saturating at 0 and 255 */
                        out[0] = (double)(f2u_sat(p1) > 255u ? 255u : f2u_sat(p1));
                        break;
                    case ORC_FUNC_FILL_C4: { /* CLR2INT (OP.cuh:20): components * 255 ORed, unmasked */
                        uint32_t c = (255u << 24) | (f2u_sat(p3 * 255.0f) << 16) | (f2u_sat(p2 * 255.0f) << 8) |
                                     f2u_sat(p1 * 255.0f);
                        for (int k = 0; k < 4; k++) out[k] = (double)((c >> (8 * k)) & 255u);
                        break;
                    }
                    default: { /* ORC_FUNC_SMOOTH */
                        const int64_t base = out - g->ch[chan];
                        double v = p1 * old[base];
                        static const int d[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
                        for (int k = 0; k < 6; k++) {
                            int nx = X + d[k][0], ny = Y + d[k][1], nz = Z + d[k][2];
                            if (nx < 0 || ny < 0 || nz < 0 || nx >= res[0] || ny >= res[1] || nz >= res[2]) continue;
                            v += old[atlas_voxel(g, chan, nx, ny, nz) - g->ch[chan]];
                        }
                        out[0] = v / ((double)p1 + 6.0) + p2;
                        break;
                    }
                    }
                }
        free(old);
        if (update_apron) {
            int rc = orc_update_apron(g, chan, boundval);
            if (rc) return rc;
        }
    }
    return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* host CPU topology: ActivateSpace (VG.cpp:2766-2855), Reparent (VG.cpp:2726-2763),
 * AddChildNode (VG.cpp:2707-2723), InsertChild (VG.cpp:2980-3027),
 * getPosInNode (VG.cpp:2858-2875), GetCoveringNode host (VG.cpp:2915-2931) */

typedef struct cpu_tree {
    int levels, logdim[MAXLEV], res[MAXLEV], range[MAXLEV];
    orc_node* nodes[MAXLEV];
    int cnt[MAXLEV], cap[MAXLEV];
    uint64_t* clist[MAXLEV];
    int64_t root; /* Elem id */
} cpu_tree;

static uint64_t elem(int grp, int lev, int64_t ndx) { return (uint64_t)grp | ((uint64_t)lev << 8) | ((uint64_t)ndx << 16); }
static int elev(uint64_t id) { return (int)((id >> 8) & 0xFF); }
static int64_t endx(uint64_t id) { return (int64_t)(id >> 16); }

static orc_node* cnode(cpu_tree* t, uint64_t id) { return &t->nodes[elev(id)][endx(id)]; }

static int64_t cpu_vc(cpu_tree* t, int l) { return (int64_t)t->res[l] * t->res[l] * t->res[l]; }

static int64_t cpu_alloc(cpu_tree* t, int lev, const int* pos)
{
    if (lev >= t->levels) return -1;
    if (t->cnt[lev] >= t->cap[lev]) {
        int nc = t->cap[lev] ? 2 * t->cap[lev] : 64;
        t->nodes[lev] = (orc_node*)realloc(t->nodes[lev], (size_t)nc * sizeof(orc_node));
        if (lev > 0) t->clist[lev] = (uint64_t*)realloc(t->clist[lev], (size_t)nc * cpu_vc(t, lev) * sizeof(uint64_t));
        t->cap[lev] = nc;
    }
    int64_t i = t->cnt[lev]++;
    orc_node* n = &t->nodes[lev][i];
    memset(n, 0, sizeof(*n));
    n->lev = (uint8_t)lev;
    n->pos[0] = pos[0]; n->pos[1] = pos[1]; n->pos[2] = pos[2];
    n->childlist = ID_UNDEFL;
    n->parent = ID_UNDEFL;
    n->value[0] = n->value[1] = n->value[2] = -1;
    n->flags = 1;
    return (int64_t)elem(0, lev, i);
}

static void cpu_cover(cpu_tree* t, int lev, const int* pos, int* out)
{
    if (lev == MAXLEV - 1) { out[0] = out[1] = out[2] = 0; return; }
    int r = t->range[lev];
    for (int a = 0; a < 3; a++) {
        int np = pos[a] / r * r;
        if (pos[a] < np) np -= r;
        out[a] = np;
    }
}

static int cpu_pos_in_node(cpu_tree* t, uint64_t id, const int* pos, int* bit)
{
    orc_node* c = cnode(t, id);
    int l = c->lev, res = t->res[l], r = t->range[l];
    int p[3];
    for (int a = 0; a < 3; a++) {
        p[a] = pos[a] - c->pos[a];
        if (p[a] < 0 || p[a] >= r) { *bit = 0; return 0; }
    }
    for (int a = 0; a < 3; a++) p[a] = p[a] * res / r;
    *bit = (p[2] * res + p[1]) * res + p[0];
    return 1;
}

static uint64_t cpu_child(cpu_tree* t, uint64_t id, int b)
{
    orc_node* c = cnode(t, id);
    if (c->childlist == ID_UNDEFL) return ID_UNDEF64;
    return t->clist[elev(c->childlist)][endx(c->childlist) * cpu_vc(t, elev(c->childlist)) + b];
}

static uint64_t cpu_insert_child(cpu_tree* t, uint64_t nid, uint64_t cid, int b)
{
    orc_node* cur = cnode(t, nid);
    cnode(t, cid)->parent = nid;
    if (cur->childlist == ID_UNDEFL) {
        int l = cur->lev;
        /* child list pool in lockstep with an own counter per level */
        int64_t ci = endx(nid);
        cur->childlist = elem(1, l, ci);
        memset(t->clist[l] + ci * cpu_vc(t, l), 0xFF, (size_t)cpu_vc(t, l) * sizeof(uint64_t));
        cur = cnode(t, nid);
    }
    t->clist[elev(cur->childlist)][endx(cur->childlist) * cpu_vc(t, elev(cur->childlist)) + b] = cid;
    return cid;
}

static int64_t cpu_activate(cpu_tree* t, uint64_t nid, const int* pos, int* bnew, int64_t stopnode, int stoplev);

static int64_t cpu_reparent(cpu_tree* t, int lev, uint64_t prev, const int* pos, int* bnew)
{
    int prevpos[3] = {cnode(t, prev)->pos[0], cnode(t, prev)->pos[1], cnode(t, prev)->pos[2]};
    int p1[3], p2[3], cover = 0;
    while (!cover && lev < MAXLEV) {
        lev++;
        if (lev >= t->levels) return -1;
        cpu_cover(t, lev, pos, p1);
        cpu_cover(t, lev, prevpos, p2);
        cover = p1[0] == p2[0] && p1[1] == p2[1] && p1[2] == p2[2];
    }
    if (lev >= MAXLEV) return -1;
    int64_t nr = cpu_alloc(t, lev, p1);
    if (nr < 0) return -1;
    int bn = 0;
    cpu_activate(t, (uint64_t)nr, prevpos, &bn, (int64_t)prev, 0);
    int64_t leaf = cpu_activate(t, (uint64_t)nr, pos, bnew, -1, 0);
    t->root = nr;
    if (leaf < 0) return -1;
    return (int64_t)cnode(t, (uint64_t)leaf)->parent;
}

static int64_t cpu_activate(cpu_tree* t, uint64_t nid, const int* pos, int* bnew, int64_t stopnode, int stoplev)
{
    for (;;) {
        if (t->root < 0 && (int64_t)nid == t->root) {
            int p[3];
            cpu_cover(t, stoplev, pos, p);
            t->root = cpu_alloc(t, stoplev, p);
            nid = (uint64_t)t->root;
        }
        orc_node* cur = cnode(t, nid);
        int b;
        if (cpu_pos_in_node(t, nid, pos, &b)) {
            if (stopnode >= 0) {
                orc_node* sn = cnode(t, (uint64_t)stopnode);
                if (pos[0] == sn->pos[0] && pos[1] == sn->pos[1] && pos[2] == sn->pos[2] &&
                    cpu_child(t, nid, b) == ID_UNDEF64 && cur->lev == sn->lev + 1)
                    return (int64_t)cpu_insert_child(t, nid, (uint64_t)stopnode, b);
            }
            if (cur->lev == stoplev) return (int64_t)nid;
            uint64_t child;
            if (cpu_child(t, nid, b) == ID_UNDEF64) {
                int plev = cur->lev;
                int r = t->range[plev - 1], res = t->res[plev];
                int cp[3] = {(b % res) * r + cur->pos[0], ((b / res) % res) * r + cur->pos[1],
                             (b / (res * res)) * r + cur->pos[2]};
                int64_t c = cpu_alloc(t, plev - 1, cp);
                if (c < 0) return -1;
                child = cpu_insert_child(t, nid, (uint64_t)c, b);
                if (plev == 1) *bnew = 1;
            } else {
                child = cpu_child(t, nid, b);
            }
            if (elev(child) == 0) return (int64_t)child;
            nid = child;
        } else {
            uint64_t parent = cur->parent;
            if (parent == ID_UNDEFL) {
                int64_t pr = cpu_reparent(t, cur->lev, nid, pos, bnew);
                if (pr < 0) return -1;
                parent = (uint64_t)pr;
            }
            nid = parent;
        }
    }
}

/* the host tree kept across calls, its pools read back whole (the reference's
 * host pools after ActivateSpace calls: nodes, child lists, root) */
void* orc_cpu_tree_new(int levels, const int* logdim)
{
    if (levels < 2 || levels > MAXLEV) return NULL;
    cpu_tree* t = (cpu_tree*)calloc(1, sizeof(cpu_tree));
    t->levels = levels;
    int r = 1;
    for (int l = 0; l < levels; l++) {
        t->logdim[l] = logdim[l];
        t->res[l] = 1 << logdim[l];
        r = l == 0 ? t->res[0] : r * t->res[l];
        t->range[l] = r;
    }
    t->root = -1;
    return t;
}

void orc_cpu_tree_free(void* h)
{
    cpu_tree* t = (cpu_tree*)h;
    if (!t) return;
    for (int l = 0; l < MAXLEV; l++) { free(t->nodes[l]); free(t->clist[l]); }
    free(t);
}

/* ActivateSpace of each point + orig (RebuildTopologyCPU, VG.cpp:1220-1227) */
int orc_cpu_tree_activate(void* h, int n, const float* pos, int stride, const float orig[3])
{
    cpu_tree* t = (cpu_tree*)h;
    for (int i = 0; i < n; i++) {
        int p[3];
        for (int a = 0; a < 3; a++) p[a] = (int)(pos[(int64_t)i * stride + a] + (orig ? orig[a] : 0.f));
        int bnew = 0;
        if (cpu_activate(t, (uint64_t)t->root, p, &bnew, -1, 0) < 0) return ORC_ERR_DEPTH;
    }
    return ORC_OK;
}

int orc_cpu_tree_count(void* h, int lev) { return ((cpu_tree*)h)->cnt[lev]; }
int64_t orc_cpu_tree_root(void* h) { return ((cpu_tree*)h)->root; }

int orc_cpu_tree_nodes(void* h, int lev, orc_node* out, int cap)
{
    cpu_tree* t = (cpu_tree*)h;
    if (cap < t->cnt[lev]) return ORC_ERR_ARG;
    memcpy(out, t->nodes[lev], (size_t)t->cnt[lev] * sizeof(orc_node));
    return ORC_OK;
}

int orc_cpu_tree_childlist(void* h, int lev, uint64_t* out, int64_t cap)
{
    cpu_tree* t = (cpu_tree*)h;
    int64_t n = (int64_t)t->cnt[lev] * cpu_vc(t, lev);
    if (lev < 1 || cap < n) return ORC_ERR_ARG;
    memcpy(out, t->clist[lev], (size_t)n * sizeof(uint64_t));
    return ORC_OK;
}

int orc_activate_space_cpu(int levels, const int* logdim, int n, const float* pos, int stride,
                           const float orig[3], int32_t* leaf_pos_out, int cap, int* root_level_out)
{
    cpu_tree t;
    memset(&t, 0, sizeof(t));
    t.levels = levels;
    int r = 1;
    for (int l = 0; l < levels; l++) {
        t.logdim[l] = logdim[l];
        t.res[l] = 1 << logdim[l];
        r = l == 0 ? t.res[0] : r * t.res[l];
        t.range[l] = r;
    }
    t.root = -1;
    int ok = 1;
    for (int i = 0; i < n && ok; i++) {
        int p[3];
        for (int a = 0; a < 3; a++) p[a] = (int)(pos[(int64_t)i * stride + a] + (orig ? orig[a] : 0.f));
        int bnew = 0;
        if (cpu_activate(&t, (uint64_t)t.root, p, &bnew, -1, 0) < 0) ok = 0;
    }
    int nl = t.cnt[0];
    if (ok && leaf_pos_out && cap >= nl)
        for (int i = 0; i < nl; i++) {
            leaf_pos_out[3 * i + 0] = t.nodes[0][i].pos[0];
            leaf_pos_out[3 * i + 1] = t.nodes[0][i].pos[1];
            leaf_pos_out[3 * i + 2] = t.nodes[0][i].pos[2];
        }
    if (root_level_out) *root_level_out = t.root >= 0 ? elev((uint64_t)t.root) : -1;
    for (int l = 0; l < MAXLEV; l++) { free(t.nodes[l]); free(t.clist[l]); }
    return ok ? nl : -1;
}
