// gvx_vbx.cu -- VBX files: SaveVBX (VG.cpp:1626-1768) and LoadVBX
// (VG.cpp:507-686), in the field order those functions use (the field list
// of GVDB_FILESPEC.txt lacks the channel count and the child-list count that
// both write and read):
//
//   u8 major, u8 minor                      (1.11 here)
//   [1.11+] f32x3 pretrans, angles, scale, translation
//   i32 num_grids                           [2.0+: u8 bitmasks]
//   u64 grid_offset[num_grids]
//   per grid:
//     char name[256]; u8 dtype ('f'); u8 components; u8 compression
//     f32x3 voxel size; i32 leaf count; i32x3 brick dims; i32 apron
//     i32 channels; u64 atlas bytes (channel 0); u8 topology type (2)
//     i32 topology reuse; u8 layout (0 = atlas); i32x3 atlas bricks; i32x3 atlas res
//     i32 levels; u64 root id
//     per level: i32 log2 dim, i32 res, i32x3 range, i32 count0, i32 width0, i32 count1, i32 width1
//     pool 0 of every level (count0 rows of width0: the 64-byte Node, then a bitmask when width0 > 64)
//     pool 1 of every level (count1 rows of width1: res^3 child ids; level 0 has none)
//     per channel: i32 type, i32 voxel bytes, then the atlas as res.z slices of res.x * res.y voxels
//
// The grid is written with the transform of an untransformed grid (the
// renderer's transform is outside this library) and a zero name; FLOAT3
// channels are 12 bytes a voxel on file (16 in HBM).  Loading reads every grid
// in turn, as the reference does, leaving the last.
#include <stdio.h>
#include <string.h>

#include <vector>

#include "gvx_grid.cuh"

namespace {

constexpr unsigned char kMajor = 1, kMinor = 11;  // MAJOR_VERSION / MINOR_VERSION, VG.cpp:31-32

struct File {
    FILE* f = nullptr;
    bool ok = true;
    // bytes from the current position to the end (sizes read from a file are checked against it
    // before anything is allocated)
    int64_t left()
    {
        const long here = ftell(f);
        if (here < 0 || fseek(f, 0, SEEK_END) != 0) return -1;
        const long end = ftell(f);
        if (fseek(f, here, SEEK_SET) != 0) return -1;
        return (int64_t)end - (int64_t)here;
    }
    ~File()
    {
        if (f) fclose(f);
    }
    void put(const void* p, size_t n)
    {
        if (ok && n && fwrite(p, 1, n, f) != n) ok = false;
    }
    void get(void* p, size_t n)
    {
        if (ok && n && fread(p, 1, n, f) != n) ok = false;
    }
    template <class T> void put(const T& v) { put(&v, sizeof(T)); }
    template <class T> void get(T& v) { get(&v, sizeof(T)); }
};

int file_voxel_bytes(int type)
{
    switch (type) {
    case GVX_T_UCHAR: return 1;
    case GVX_T_UCHAR4: return 4;
    case GVX_T_FLOAT: return 4;
    case GVX_T_FLOAT3: return 12;
    case GVX_T_FLOAT4: return 16;
    }
    return 0;
}

}  // namespace

extern "C" gvx_status gvx_save_vbx(gvx_grid* g, const char* path)
{
    if (!g || !path) {
        gvx_set_error("SaveVBX: null grid or path");
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(cudaSetDevice(g->device));
    if (g->root_level < 0 || !g->atlas_valid) {
        gvx_set_error("SaveVBX: the grid has no topology and atlas (RebuildTopology + UpdateAtlas)");
        return GVX_ERR_STATE;
    }
    int nchan = 0;
    while (nchan < GVX_MAXCH && g->ch[nchan].used) nchan++;
    for (int c = nchan; c < GVX_MAXCH; c++)
        if (g->ch[c].used) {
            gvx_set_error("SaveVBX: channels must be numbered 0..n-1 (channel %d follows a gap)", c);
            return GVX_ERR_UNSUPPORTED;
        }
    if (nchan == 0) {
        gvx_set_error("SaveVBX: no channel");
        return GVX_ERR_STATE;
    }
    File fp;
    fp.f = fopen(path, "wb");
    if (!fp.f) {
        gvx_set_error("SaveVBX: cannot open %s for writing", path);
        return GVX_ERR_IO;
    }
    const int levels = g->levels, P = g->P;
    const int res3[3] = {g->sub[0] * P, g->sub[1] * P, g->sub[2] * P};
    fp.put(kMajor);
    fp.put(kMinor);
    const float pretrans[3] = {0, 0, 0}, angs[3] = {0, 0, 0}, scale[3] = {1, 1, 1}, trans[3] = {0, 0, 0};
    fp.put(pretrans, 12);
    fp.put(angs, 12);
    fp.put(scale, 12);
    fp.put(trans, 12);
    const int num_grids = 1;
    fp.put(num_grids);
    const long table = ftell(fp.f);
    uint64_t grid_off = 0;
    fp.put(grid_off);
    grid_off = (uint64_t)ftell(fp.f);
    // ---- grid header
    char name[256];
    memset(name, 0, sizeof(name));
    fp.put(name, sizeof(name));
    const unsigned char dtype = 'f', comps = 1, compress = 0, topotype = 2, layout = 0;
    fp.put(dtype);
    fp.put(comps);
    fp.put(compress);
    const float vsize[3] = {1, 1, 1};
    fp.put(vsize, 12);
    const int leafcnt = (int)g->count[0];
    fp.put(leafcnt);
    const int leafdim[3] = {g->brick, g->brick, g->brick};
    fp.put(leafdim, 12);
    const int apron = g->apron;
    fp.put(apron);
    fp.put(nchan);
    const uint64_t atlas_sz = (uint64_t)res3[0] * res3[1] * res3[2] * file_voxel_bytes(g->ch[0].type);
    fp.put(atlas_sz);
    fp.put(topotype);
    const int reuse = 0;
    fp.put(reuse);
    fp.put(layout);
    fp.put(g->sub, 12);
    fp.put(res3, 12);
    // ---- topology
    fp.put(levels);
    const uint64_t root = (uint64_t)g->root_level << 8;  // Elem(group 0, root level, index 0)
    fp.put(root);
    for (int l = 0; l < levels; l++) {
        const int range3[3] = {g->range[l], g->range[l], g->range[l]};
        const int cnt0 = (int)g->count[l], w0 = GVX_NODE_BYTES;
        const int cnt1 = l > 0 ? cnt0 : 0, w1 = l > 0 ? (int)(sizeof(uint64_t) * g->res[l] * g->res[l] * g->res[l]) : 0;
        fp.put(g->logdim[l]);
        fp.put(g->res[l]);
        fp.put(range3, 12);
        fp.put(cnt0);
        fp.put(w0);
        fp.put(cnt1);
        fp.put(w1);
    }
    std::vector<unsigned char> buf;
    for (int l = 0; l < levels; l++) {
        const size_t bytes = (size_t)g->count[l] * GVX_NODE_BYTES;
        buf.resize(bytes);
        if (bytes) GVX_CK(cudaMemcpyAsync(buf.data(), g->nodes[l].p, bytes, cudaMemcpyDeviceToHost, g->stream));
        GVX_CK(cudaStreamSynchronize(g->stream));
        fp.put(buf.data(), bytes);
    }
    for (int l = 1; l < levels; l++) {
        const size_t bytes = (size_t)g->count[l] * g->res[l] * g->res[l] * g->res[l] * sizeof(uint64_t);
        buf.resize(bytes);
        if (bytes) GVX_CK(cudaMemcpyAsync(buf.data(), g->clist[l].p, bytes, cudaMemcpyDeviceToHost, g->stream));
        GVX_CK(cudaStreamSynchronize(g->stream));
        fp.put(buf.data(), bytes);
    }
    // ---- atlas: per channel, the dense atlas slice by slice
    for (int c = 0; c < nchan; c++) {
        int64_t bytes = 0;
        gvx_status rc = gvx_channel_bytes(g, c, &bytes);
        if (rc) return rc;
        std::vector<unsigned char> dense((size_t)bytes);
        rc = gvx_read_channel_dense(g, c, dense.data(), bytes);
        if (rc) return rc;
        const int type = g->ch[c].type, fb = file_voxel_bytes(type), eb = g->ch[c].elem_bytes;
        fp.put(type);
        fp.put(fb);
        if (fb == eb) {
            fp.put(dense.data(), dense.size());
        } else {  // FLOAT3: the xyz of each float4
            const size_t nv = dense.size() / (size_t)eb;
            std::vector<unsigned char> packed(nv * (size_t)fb);
            for (size_t v = 0; v < nv; v++) memcpy(&packed[v * fb], &dense[v * eb], (size_t)fb);
            fp.put(packed.data(), packed.size());
        }
    }
    if (fp.ok) {
        fseek(fp.f, table, SEEK_SET);
        fp.put(grid_off);
    }
    if (!fp.ok || fflush(fp.f) != 0) {
        gvx_set_error("SaveVBX: write to %s failed", path);
        return GVX_ERR_IO;
    }
    return GVX_OK;
}

extern "C" gvx_status gvx_load_vbx(gvx_grid* g, const char* path, int force_major, int force_minor)
{
    if (!g || !path) {
        gvx_set_error("LoadVBX: null grid or path");
        return GVX_ERR_INVALID_ARG;
    }
    GVX_CK(cudaSetDevice(g->device));
    File fp;
    fp.f = fopen(path, "rb");
    if (!fp.f) {
        gvx_set_error("LoadVBX: unable to open %s", path);
        return GVX_ERR_IO;
    }
    unsigned char major = 0, minor = 0;
    fp.get(major);
    fp.get(minor);
    if (force_major > 0 || force_minor > 0) {
        major = (unsigned char)force_major;
        minor = (unsigned char)force_minor;
    }
    if ((major == 1 && minor >= 11) || major > 1) {
        float xf[12];
        fp.get(xf, sizeof(xf));  // the renderer's grid transform: not kept by this library
    }
    int num_grids = 0;
    fp.get(num_grids);
    unsigned char read_masks = 0;
    if (major >= 2)
        fp.get(read_masks);
    else if (major == 1 && minor == 0)
        read_masks = 1;
    (void)read_masks;  // a node row's first 64 bytes are the Node; a bitmask after it is not kept
    if (!fp.ok || num_grids < 0 || num_grids > (1 << 20)) {
        gvx_set_error("LoadVBX: %s: bad header", path);
        return GVX_ERR_IO;
    }
    std::vector<uint64_t> offs((size_t)num_grids);
    for (auto& o : offs) fp.get(o);
    for (int gi = 0; gi < num_grids; gi++) {
        char name[256];
        unsigned char dtype = 0, comps = 0, compress = 0, topotype = 0, layout = 0;
        float vsize[3];
        int leafcnt = 0, leafdim[3], apron = 0, nchan = 0, reuse = 0, axiscnt[3], axisres[3], levels = 0;
        uint64_t atlas_sz = 0, root = 0;
        fp.get(name, sizeof(name));
        fp.get(dtype);
        fp.get(comps);
        fp.get(compress);
        fp.get(vsize, 12);
        fp.get(leafcnt);
        fp.get(leafdim, 12);
        fp.get(apron);
        fp.get(nchan);
        fp.get(atlas_sz);
        fp.get(topotype);
        fp.get(reuse);
        fp.get(layout);
        fp.get(axiscnt, 12);
        fp.get(axisres, 12);
        fp.get(levels);
        fp.get(root);
        if (!fp.ok || levels < 2 || levels > GVX_MAX_LEVELS || nchan < 0 || nchan > GVX_MAXCH) {
            gvx_set_error("LoadVBX: %s: bad grid header", path);
            return GVX_ERR_IO;
        }
        if (topotype != 2 || layout != 0 || compress != 0) {
            gvx_set_error("LoadVBX: %s: topology type %d, layout %d, compression %d (only 2, 0, 0 are read)", path,
                          topotype, layout, compress);
            return GVX_ERR_UNSUPPORTED;
        }
        int ld[GVX_MAX_LEVELS], res[GVX_MAX_LEVELS], cnt0[GVX_MAX_LEVELS], w0[GVX_MAX_LEVELS], cnt1[GVX_MAX_LEVELS],
            w1[GVX_MAX_LEVELS];
        for (int l = 0; l < levels; l++) {
            int range3[3];
            fp.get(ld[l]);
            fp.get(res[l]);
            fp.get(range3, 12);
            fp.get(cnt0[l]);
            fp.get(w0[l]);
            fp.get(cnt1[l]);
            fp.get(w1[l]);
            if (!fp.ok || cnt0[l] < 0 || cnt1[l] < 0 || w0[l] < GVX_NODE_BYTES || ld[l] < 1 || ld[l] > 10 ||
                (l > 0 && (cnt1[l] < cnt0[l] || w1[l] < (int)(8u << (3 * ld[l]))))) {
                gvx_set_error("LoadVBX: %s: level %d of the topology table is not a GVDB tree", path, l);
                return GVX_ERR_IO;
            }
        }
        {
            int64_t need = 0;
            for (int l = 0; l < levels; l++) need += (int64_t)cnt0[l] * w0[l] + (int64_t)cnt1[l] * w1[l];
            if (need > fp.left()) {
                gvx_set_error("LoadVBX: %s: the topology tables need %lld bytes, the file holds fewer", path,
                              (long long)need);
                return GVX_ERR_IO;
            }
        }
        // Configure (VG.cpp:598): the file's levels and dimensions
        gvx_status rc = gvx_configure(g, levels, ld, nullptr);
        if (rc) return rc;
        if (g->brick != leafdim[0] || (apron != 0 && apron != 1)) {
            gvx_set_error("LoadVBX: %s: brick %d / apron %d do not match the tree", path, leafdim[0], apron);
            return GVX_ERR_IO;
        }
        // pools: node rows (first 64 bytes), then child lists
        std::vector<std::vector<GvxNode>> nodes((size_t)levels);
        std::vector<std::vector<uint64_t>> clists((size_t)levels);
        std::vector<unsigned char> row;
        for (int l = 0; l < levels; l++) {
            nodes[l].resize((size_t)cnt0[l]);
            row.resize((size_t)w0[l]);
            for (int i = 0; i < cnt0[l]; i++) {
                fp.get(row.data(), row.size());
                memcpy(&nodes[l][i], row.data(), GVX_NODE_BYTES);
            }
        }
        for (int l = 0; l < levels; l++) {
            if (l == 0) {
                std::vector<unsigned char> skip((size_t)cnt1[0] * (size_t)w1[0]);
                fp.get(skip.data(), skip.size());
                continue;
            }
            const size_t vc = (size_t)1 << (3 * ld[l]);
            clists[l].resize((size_t)cnt0[l] * vc);
            row.resize((size_t)w1[l]);
            for (int i = 0; i < cnt1[l]; i++) {
                fp.get(row.data(), row.size());
                if (i < cnt0[l]) memcpy(&clists[l][(size_t)i * vc], row.data(), vc * sizeof(uint64_t));
            }
        }
        if (!fp.ok) {
            gvx_set_error("LoadVBX: %s: truncated topology", path);
            return GVX_ERR_IO;
        }
        const int rlev = (int)((root >> 8) & 0xFF);
        int64_t counts[GVX_MAX_LEVELS];
        std::vector<const GvxNode*> np((size_t)levels);
        std::vector<const uint64_t*> cp((size_t)levels, nullptr);
        for (int l = 0; l < levels; l++) {
            counts[l] = cnt0[l];
            np[l] = nodes[l].data();
            if (l > 0) cp[l] = clists[l].data();
        }
        if ((root >> 16) != 0 || rlev >= levels) {
            gvx_set_error("LoadVBX: %s: root id 0x%llx is not node 0 of a level", path, (unsigned long long)root);
            return GVX_ERR_IO;
        }
        rc = gvx_topo_import(g, rlev, counts, np.data(), cp.data());
        if (rc) return rc;
        rc = gvx_topo_compute_bounds(g);  // FinishTopology (VG.cpp:621)
        if (rc) return rc;
        // atlas: channels with the file's atlas shape (x, y brick counts), then the data
        for (int c = 0; c < GVX_MAXCH; c++) g->ch[c].used = false;  // DestroyChannels (VG.cpp:624)
        g->have_atlas = false;
        rc = gvx_set_channel_default(g, axiscnt[0], axiscnt[1], std::max(axiscnt[2], 1));
        if (rc) return rc;
        std::vector<int> types((size_t)nchan), strides((size_t)nchan);
        std::vector<std::vector<unsigned char>> dense((size_t)nchan);
        for (int c = 0; c < nchan; c++) {
            fp.get(types[c]);
            fp.get(strides[c]);
            if (!fp.ok || file_voxel_bytes(types[c]) == 0 || strides[c] != file_voxel_bytes(types[c])) {
                gvx_set_error("LoadVBX: %s: channel %d of type %d, %d bytes a voxel", path, c, types[c], strides[c]);
                return GVX_ERR_UNSUPPORTED;
            }
            if (axisres[0] <= 0 || axisres[1] <= 0 || axisres[2] <= 0 ||
                (int64_t)axisres[0] * axisres[1] * axisres[2] * strides[c] > fp.left()) {
                gvx_set_error("LoadVBX: %s: atlas %d x %d x %d of channel %d exceeds the file", path, axisres[0],
                              axisres[1], axisres[2], c);
                return GVX_ERR_IO;
            }
            dense[c].resize((size_t)axisres[0] * axisres[1] * axisres[2] * (size_t)strides[c]);
            fp.get(dense[c].data(), dense[c].size());
            if (!fp.ok) {
                gvx_set_error("LoadVBX: %s: truncated atlas of channel %d", path, c);
                return GVX_ERR_IO;
            }
            rc = gvx_add_channel(g, c, types[c], apron);
            if (rc) return rc;
        }
        rc = gvx_update_atlas(g);  // UpdateAtlas (VG.cpp:679)
        if (rc) return rc;
        // the file's dense atlas into the brick-major channels (voxels past the file's atlas stay 0)
        const int P = g->P;
        for (int c = 0; c < nchan; c++) {
            const int fb = strides[c], eb = g->ch[c].elem_bytes;
            std::vector<unsigned char> bm((size_t)g->ch[c].slots * P * P * P * eb, 0);
            for (int64_t s = 0; s < g->ch[c].slots; s++) {
                const int64_t bx = s % g->sub[0], by = (s / g->sub[0]) % g->sub[1], bz = s / ((int64_t)g->sub[0] * g->sub[1]);
                for (int z = 0; z < P; z++)
                    for (int y = 0; y < P; y++)
                        for (int x = 0; x < P; x++) {
                            const int64_t X = bx * P + x, Y = by * P + y, Z = bz * P + z;
                            if (X >= axisres[0] || Y >= axisres[1] || Z >= axisres[2]) continue;
                            const size_t src = (size_t)((Z * axisres[1] + Y) * axisres[0] + X) * fb;
                            const size_t dst = (size_t)(((s * P + z) * P + y) * P + x) * eb;
                            memcpy(&bm[dst], &dense[c][src], (size_t)fb);
                        }
            }
            GVX_CK(cudaMemcpyAsync(g->ch[c].data.p, bm.data(), bm.size(), cudaMemcpyHostToDevice, g->stream));
            GVX_CK(cudaStreamSynchronize(g->stream));
            apron_invalidate(g->ch[c]);
        }
    }
    return GVX_OK;
}
