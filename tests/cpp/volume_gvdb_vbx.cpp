// volume_gvdb_vbx.cpp -- test program for SaveVBX / LoadVBX of the
// nvdb::VolumeGVDB drop-in: a volume built from points is saved, loaded into a
// second VolumeGVDB, and compared node by node and brick by brick; LoadVBX of
// a missing file returns false.
//
//   volume_gvdb_vbx <in.bin> <file.vbx>
// in: int32 n, n x float3.  Exit status 0 when everything matches.
#include <cstdio>
#include <cstring>
#include <vector>

#include "gvx_volume_gvdb.h"

using namespace nvdb;

int main(int argc, char** argv)
{
    if (argc != 3) return 2;
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 2;
    int n = 0;
    if (fread(&n, 4, 1, f) != 1) return 2;
    std::vector<Vector3DF> pts((size_t)n);
    if (fread(pts.data(), sizeof(Vector3DF), (size_t)n, f) != (size_t)n) return 2;
    fclose(f);
    try {
        VolumeGVDB a;
        a.SetCudaDevice(0);
        a.Initialize();
        a.Configure(5, 3, 3, 3, 3);
        a.SetChannelDefault(16, 16, 1);
        a.AddChannel(0, T_FLOAT, 1);
        DataPtr pos, vel, clr;
        a.AllocData(pos, n, sizeof(Vector3DF), true);
        memcpy(pos.cpu, pts.data(), pts.size() * sizeof(Vector3DF));
        a.CommitData(pos);
        a.SetPoints(pos, vel, clr);
        a.RebuildTopology(n, 1.0f, Vector3DF(0, 0, 0));
        a.FinishTopology(false, true);
        a.UpdateAtlas();
        a.ClearChannel(0);
        a.InsertPoints(n, Vector3DF(0, 0, 0), false);
        a.ScatterDensity(n, 1.5f, 1.0f, Vector3DF(0, 0, 0), true, false);
        a.UpdateApron(0, 0.0f);
        a.SaveVBX(argv[2]);

        VolumeGVDB b;
        b.SetCudaDevice(0);
        b.Initialize();
        if (b.LoadVBX(std::string(argv[2]) + ".missing")) {
            fprintf(stderr, "LoadVBX of a missing file returned true\n");
            return 1;
        }
        if (!b.LoadVBX(argv[2])) {
            fprintf(stderr, "LoadVBX failed\n");
            return 1;
        }
        if (a.GetLevels() != b.GetLevels()) return 1;
        for (int l = 0; l < a.GetLevels(); l++) {
            if (a.getNumTotalNodes(l) != b.getNumTotalNodes(l)) {
                fprintf(stderr, "level %d: %llu vs %llu nodes\n", l, (unsigned long long)a.getNumTotalNodes(l),
                        (unsigned long long)b.getNumTotalNodes(l));
                return 1;
            }
            for (uint64 i = 0; i < a.getNumTotalNodes(l); i++)
                if (memcmp(a.getNodeAtLevel((int)i, l), b.getNodeAtLevel((int)i, l), sizeof(Node)) != 0) {
                    fprintf(stderr, "level %d node %llu differs\n", l, (unsigned long long)i);
                    return 1;
                }
        }
        const int bres = 8;
        std::vector<float> ba((size_t)bres * bres * bres), bb(ba.size());
        DataPtr da, db;
        a.SetDataCPU(da, bres * bres * bres, (char*)ba.data(), 0, sizeof(float));
        b.SetDataCPU(db, bres * bres * bres, (char*)bb.data(), 0, sizeof(float));
        int bricks = 0;
        for (uint64 i = 0; i < a.getNumTotalNodes(0); i++) {
            Node* nd = a.getNodeAtLevel((int)i, 0);
            if (!nd->mFlags) continue;
            a.AtlasRetrieveBrickXYZ(0, nd->mValue, da);
            b.AtlasRetrieveBrickXYZ(0, nd->mValue, db);
            if (memcmp(ba.data(), bb.data(), ba.size() * sizeof(float)) != 0) {
                fprintf(stderr, "brick %llu differs\n", (unsigned long long)i);
                return 1;
            }
            bricks++;
        }
        printf("%d bricks identical\n", bricks);
        a.FreeData(pos);
    } catch (const GvxError& e) {
        fprintf(stderr, "GvxError %d: %s\n", e.status, e.what());
        return 1;
    }
    return 0;
}
