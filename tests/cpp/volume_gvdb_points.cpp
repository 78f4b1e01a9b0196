// volume_gvdb_points.cpp -- test program for the nvdb::VolumeGVDB drop-in:
// the call sequence of an application of the reference that builds a volume
// from points (configure, channel, AllocData/CommitData/SetPoints,
// RebuildTopology, FinishTopology, UpdateAtlas, InsertPoints, ScatterDensity or
// the cubic Splat, UpdateApron, Compute(FUNC_SMOOTH)), dumping the node pools, the leaf of every
// point and every active brick's values for the test to compare.
//
//   volume_gvdb_points <in.bin> <out.bin>
// in:  int32 n, int32 mode (0 ScatterDensity, 1 cubic Splat, 2 ScatterDensity then two
//      FUNC_SMOOTH iterations as gSprayDeposit runs them, 3 gPointCloud's FP16 level set:
//      topology at 2 radius, InsertPointsSubcell_FP16 + GatherLevelSet_FP16, UpdateApron(0, 3),
//      two FUNC_SMOOTH iterations), float radius, n x float3
// out: int32 levels; per level uint64 count + count 64-byte nodes; uint64 used;
//      n int32 leaf ids (AUX_PNODE); per active leaf in pool order, brick^3 floats
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
    int n = 0, mode = 0;
    float radius = 0.f;
    if (fread(&n, 4, 1, f) != 1 || fread(&mode, 4, 1, f) != 1 || fread(&radius, 4, 1, f) != 1) return 2;
    std::vector<Vector3DF> pts((size_t)n);
    if (fread(pts.data(), sizeof(Vector3DF), (size_t)n, f) != (size_t)n) return 2;
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

        gvdb.RequestFullRebuild(true);
        gvdb.RebuildTopology(n, mode == 3 ? 2.0f * radius : radius, Vector3DF(0, 0, 0));
        gvdb.FinishTopology(false, true);
        gvdb.UpdateAtlas();
        gvdb.ClearChannel(0);
        gvdb.InsertPoints(n, Vector3DF(0, 0, 0), false);
        if (mode == 3) {
            int sc_len = 0;
            gvdb.InsertPointsSubcell_FP16(4, n, radius, Vector3DF(0, 0, 0), sc_len);
            gvdb.GatherLevelSet_FP16(4, n, radius, Vector3DF(0, 0, 0), sc_len, 0, 0);
            gvdb.UpdateApron(0, 3.0f);
            gvdb.Compute(FUNC_SMOOTH, 0, 2, Vector3DF(1, 0, 0), true, true, 3.0f);
        } else if (mode == 0 || mode == 2) {
            gvdb.ScatterDensity(n, radius, 1.0f, Vector3DF(0, 0, 0), true, false);
            gvdb.UpdateApron(0, 0.0f);
            if (mode == 2) gvdb.Compute(FUNC_SMOOTH, 0, 2, Vector3DF(4, 0, 0), true, true);
        } else {
            gvdb.Splat(GVX_SPLAT_CUBIC, n, radius, Vector3DF(0, 0, 0), 0, -1);
        }

        FILE* o = fopen(argv[2], "wb");
        if (!o) return 2;
        const int levels = gvdb.GetLevels();
        fwrite(&levels, 4, 1, o);
        for (int l = 0; l < levels; l++) {
            const uint64 cnt = gvdb.getNumTotalNodes(l);
            fwrite(&cnt, 8, 1, o);
            for (uint64 i = 0; i < cnt; i++) fwrite(gvdb.getNodeAtLevel((int)i, l), sizeof(Node), 1, o);
        }
        const uint64 used = gvdb.getNumUsedNodes(0);
        fwrite(&used, 8, 1, o);
        DataPtr& pnode = gvdb.getAux(AUX_PNODE);
        fwrite(pnode.cpu, 4, (size_t)n, o);
        const int b = 8;
        std::vector<float> brick((size_t)b * b * b);
        DataPtr dest;
        gvdb.SetDataCPU(dest, b * b * b, (char*)brick.data(), 0, sizeof(float));
        for (uint64 i = 0; i < gvdb.getNumTotalNodes(0); i++) {
            Node* nd = gvdb.getNodeAtLevel((int)i, 0);
            if (!nd->mFlags) continue;
            gvdb.AtlasRetrieveBrickXYZ(0, nd->mValue, dest);
            fwrite(brick.data(), 4, brick.size(), o);
        }
        fclose(o);
        gvdb.FreeData(pos);
    } catch (const GvxError& e) {
        fprintf(stderr, "GvxError %d: %s\n", e.status, e.what());
        return 1;
    }
    return 0;
}
