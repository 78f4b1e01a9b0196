"""GPU parity of the surface-fusion workload (depth frames of an analytic
scene, AccumulateTopology + accumulating trilinear splats of a density and a
confidence-weighted channel) against the oracle, frame by frame: pools bit
for bit, channels within the density tolerance."""
import numpy as np
import pytest

from parity_util import DENSITY_TOL, compare_topology, rel_error

pytestmark = pytest.mark.gpu

LOGDIM = (3, 3, 3, 3, 5)


@pytest.mark.parametrize("apron", [False, True])
def test_fusion_frames_match_oracle(gvx_mod, orc, apron):
    """apron=True: UpdateApron(c, 0) after every frame on both sides, whole bricks compared.
    Under AccumulateTopology the bricks keep their slots, so libgvx updates only the aprons of
    the new bricks and of their neighbours; the oracle updates every apron."""
    import workloads

    # a quarter-resolution camera, the scene at half scale in 1024^3 (it spans several level-2
    # nodes, so no level below the root holds a single node: the reference's top_lev quirk)
    frames = list(workloads.depth_fusion(frames=4, seed=5, width=160, height=120, f=131.25, scale=0.5,
                                         extent=1024.0))
    g = gvx_mod.Grid(0)
    g.configure(LOGDIM)
    g.add_channel(0, gvx_mod.T_FLOAT, 1)
    g.add_channel(1, gvx_mod.T_FLOAT, 1)
    o = orc.Oracle(LOGDIM)
    o.add_channel(0, orc.T_FLOAT)
    o.add_channel(1, orc.T_FLOAT)
    for k, (pos, conf) in enumerate(frames):
        n = len(pos)
        g.commit_points_host(pos)
        g.rebuild_topology(n, 1.0, mode=gvx_mod.TOPO_ACCUMULATE)
        g.update_atlas()
        g.insert_points(n)
        g.splat(gvx_mod.SPLAT_TRILINEAR, n, 1.0, chan_density=0, accum=True)
        g.commit_points_host(pos, weight=conf)
        g.splat(gvx_mod.SPLAT_TRILINEAR, n, 1.0, chan_density=1, accum=True)
        assert o.rebuild_topology(pos, 1.0, mode=orc.TOPO_ACCUMULATE) == orc.OK
        o.update_atlas()
        o.splat(orc.SPLAT_TRILINEAR, pos, 1.0, chan_density=0, accum=True)
        o.splat(orc.SPLAT_TRILINEAR, pos, 1.0, weight=conf, chan_density=1, accum=True)
        if apron:
            for c in (0, 1):
                g.update_apron(c, 0.0)
                o.update_apron(c, 0.0)
        compare_topology(g, o)
        assert g.info()["last_rebuild"] == o.last_mode(), "frame %d" % k
        used = o.used_leaves()
        for c in (0, 1):
            assert rel_error(g.read_channel(c)[:used], o.read_channel(c)[:used]) <= DENSITY_TOL, (k, c)
    assert o.last_mode() == 2
