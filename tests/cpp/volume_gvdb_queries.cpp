// volume_gvdb_queries.cpp -- test program for the host-side tree queries of the
// nvdb::VolumeGVDB drop-in: an application builds a volume from points
// (RebuildTopology, UpdateAtlas, InsertPoints, ScatterDensity, UpdateApron),
// reads channel 0 back as the reference's dense atlas, then asks the tree,
// point by point, for the leaf at a position (getNodeAtPoint from the root),
// whether an integer position is active (isActive) and the value there
// (getValue on the dense atlas).
//
//   volume_gvdb_queries <in.bin> <out.bin>
// in:  int32 n, int32 q, float radius, n x float3 points, q x float3 queries
// out: int32 levels; uint64 level-0 node count + those 64-byte nodes; int32 atlas res[3];
//      uint64 root id; per query: uint64 leaf id, int32 active, float value;
//      then int32 slots + slots x int32[4] atlas map + slots x P^3 floats of channel 0
#include <cstdio>
#include <cstring>
#include <vector>

#include "gvx_volume_gvdb.h"

using namespace nvdb;

int main(int argc, char** argv)
{
    if (argc != 3) {
        fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
        return 2;
    }
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 2;
    int n = 0, q = 0;
    float radius = 0.f;
    if (fread(&n, 4, 1, f) != 1 || fread(&q, 4, 1, f) != 1 || fread(&radius, 4, 1, f) != 1) return 2;
    std::vector<Vector3DF> pts((size_t)n), qs((size_t)q);
    if (fread(pts.data(), sizeof(Vector3DF), (size_t)n, f) != (size_t)n) return 2;
    if (fread(qs.data(), sizeof(Vector3DF), (size_t)q, f) != (size_t)q) return 2;
    fclose(f);

    try {
        VolumeGVDB gvdb;
        gvdb.SetCudaDevice(0);
        gvdb.Initialize();
        gvdb.Configure(5, 3, 3, 3, 3);
        gvdb.SetChannelDefault(16, 16, 1);
        gvdb.AddChannel(0, T_FLOAT, 1);

        DataPtr pos, vel, clr;
        gvdb.AllocData(pos, n, sizeof(Vector3DF), true);
        memcpy(pos.cpu, pts.data(), pts.size() * sizeof(Vector3DF));
        gvdb.CommitData(pos);
        gvdb.SetPoints(pos, vel, clr);
        gvdb.RebuildTopology(n, radius, Vector3DF(0, 0, 0));
        gvdb.FinishTopology(false, true);
        gvdb.UpdateAtlas();
        gvdb.ClearChannel(0);
        gvdb.InsertPoints(n, Vector3DF(0, 0, 0), false);
        gvdb.ScatterDensity(n, radius, 1.0f, Vector3DF(0, 0, 0), true, false);
        gvdb.UpdateApron(0, 0.0f);

        gvx_grid* h = gvdb.getHandle();
        gvx_info inf;
        if (gvx_get_info(h, &inf) != GVX_OK) return 3;
        if (inf.channels < 1) return 3;
        int64_t bytes = 0;
        if (gvx_channel_bytes(h, 0, &bytes) != GVX_OK) return 3;
        std::vector<float> atlas((size_t)bytes / 4);  // every atlas slot, as the dense array holds them
        if (gvx_read_channel_dense(h, 0, atlas.data(), bytes) != GVX_OK) return 3;

        FILE* o = fopen(argv[2], "wb");
        if (!o) return 2;
        const int levels = gvdb.GetLevels();
        fwrite(&levels, 4, 1, o);
        const uint64 cnt = gvdb.getNumTotalNodes(0);
        fwrite(&cnt, 8, 1, o);
        for (uint64 i = 0; i < cnt; i++) fwrite(gvdb.getNodeAtLevel((int)i, 0), sizeof(Node), 1, o);
        fwrite(inf.atlas_res, 4, 3, o);
        const uint64 root = gvdb.getRootNodeID();
        fwrite(&root, 8, 1, o);
        for (int i = 0; i < q; i++) {
            const Vector3DF p = qs[(size_t)i];
            const uint64 leaf = gvdb.getNodeAtPoint(root, p);
            const int active = gvdb.isActive(Vector3DI((int)p.x, (int)p.y, (int)p.z)) ? 1 : 0;
            const float val = gvdb.getValue((slong)root, p, atlas.data());
            fwrite(&leaf, 8, 1, o);
            fwrite(&active, 4, 1, o);
            fwrite(&val, 4, 1, o);
        }
        const int slots = (int)inf.used_leaves;
        fwrite(&slots, 4, 1, o);
        const int64_t all_slots = (int64_t)inf.atlas_subdim[0] * inf.atlas_subdim[1] * inf.atlas_subdim[2];
        std::vector<int32_t> amap((size_t)all_slots * 4);
        if (gvx_read_atlas_map(h, amap.data(), all_slots) != GVX_OK) return 3;
        fwrite(amap.data(), 4, (size_t)slots * 4, o);
        std::vector<char> ch((size_t)bytes);
        if (gvx_read_channel(h, 0, ch.data(), bytes) != GVX_OK) return 3;
        const int P = inf.brick_res + 2 * inf.apron;
        fwrite(ch.data(), 4, (size_t)slots * P * P * P, o);
        fclose(o);
    } catch (const GvxError& e) {
        fprintf(stderr, "GvxError: %s\n", e.what());
        return 1;
    }
    return 0;
}
