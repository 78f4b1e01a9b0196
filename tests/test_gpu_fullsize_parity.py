"""GPU parity at the full sizes of the measured workloads, against the FP64
oracle and (for topology) the reference's own kernels.

- SPH slab (4M points, 1024^3, cubic R = 2, density + float3 velocity):
  advected frames under a full rebuild every frame and under the reference's
  default RebuildTopology state machine (two full builds, then incremental).
  Node pools, child lists and the atlas map are compared bit for bit with the
  oracle and with the reference's kernels; density and velocity on 2,000
  sampled active bricks (seeded) with the oracle's FP64 sums.
- Surface fusion (30 depth frames of 640x480 in 2048^3, AccumulateTopology
  r = 1, accumulating trilinear density and confidence channels, UpdateApron
  after every frame): pools every frame; the interior voxels of 2,000 sampled
  bricks after frames 10, 20 and 30.
- Batched clouds (64 clouds, seed 7): the three smallest, built and splatted
  through the batched path, against the oracle (pools, whole channel).
- Differentiable splat (1M points in 512^3, w ~ U(0,1), R ~ U(1,3)): the
  adjoint against FP64 central differences (h = 1e-3) on 1,000 points drawn
  with seed 2, and the forward on the bricks those points touch.

The oracle restates the splat over sampled bricks (orc_splat_sample): a whole
FP64 atlas of the 4M frame would take about 13 GB.  Each test prints its
error statistics ("ERRSTAT ...", shown with pytest -s)."""
import json

import numpy as np
import pytest

from parity_util import DENSITY_TOL, compare_topology, leaf_slots, rel_error, rel_error_significant

pytestmark = pytest.mark.gpu

LOGDIM = (3, 3, 3, 3, 5)
P = 10
SAMPLE = 2000
VEL_TOL = 1e-5      # |v - v_ref| <= VEL_TOL * max|v_ref|
GRAD_TOL = 1e-4     # per family: max |g - g_fd| <= GRAD_TOL * max |g_fd|
NODE_FIELDS = ("lev", "flags", "pos", "value", "parent", "childlist")


def errstat(config, **kw):
    print("ERRSTAT " + json.dumps(dict(config=config, **kw), sort_keys=True))


def ref_harness():
    try:
        import ref_harness as rh
    except ImportError:
        return None
    return rh if rh.available() else None


def same_pools_ref(r, o):
    """pools and child lists of the reference's kernels against the oracle's.
    The harness grid has no channel (a 4M-point FP32 atlas of its own is not
    needed), so UpdateAtlas is not run on it and mValue is not compared here;
    the atlas assignment is compared between libgvx and the oracle."""
    assert r.root_level() == o.root_level()
    for lev in range(o.root_level() + 1):
        na, nb = r.nodes(lev), o.nodes(lev)
        assert len(na) == len(nb), "level %d: %d vs %d nodes" % (lev, len(na), len(nb))
        for f in NODE_FIELDS:
            if f == "value" and lev == 0:
                continue
            assert np.array_equal(na[f], nb[f]), "level %d field %s" % (lev, f)
        if lev > 0:
            assert np.array_equal(r.childlist(lev), o.childlist(lev)), "level %d child lists" % lev
    assert r.used_leaves() == o.used_leaves()


def sample_leaves(o, count, seed):
    nodes = o.nodes(0)
    act = np.nonzero(nodes["flags"] == 1)[0]
    rng = np.random.default_rng(seed)
    pick = np.sort(rng.choice(act, size=min(count, len(act)), replace=False)).astype(np.int32)
    return pick, leaf_slots(nodes, o.atlas_subdim(), P)[pick]


# ---------------------------------------------------------------- SPH slab


def sph_grid(gvx):
    g = gvx.Grid(0)
    g.configure(LOGDIM)
    g.add_channel(0, gvx.T_FLOAT, 1)
    g.add_channel(1, gvx.T_FLOAT3, 1)
    return g


def sph_frame(gvx, g, pos, vel, mode):
    n = len(pos)
    g.commit_points_host(pos, vel=vel)
    g.rebuild_topology(n, 2.0, mode=mode)
    g.update_atlas()
    g.insert_points(n)
    g.splat(gvx.SPLAT_CUBIC, n, 2.0, chan_density=0, chan_vel=1)
    g.update_apron(0, 0.0)
    g.update_apron(1, 0.0)
    g.sync()


def check_sph_values(g, o, orc, pos, vel, label, seed):
    pick, slots = sample_leaves(o, SAMPLE, seed)
    d_ref, v_ref = o.splat_sample(orc.SPLAT_CUBIC, pos, pick, 2.0, vel=vel)
    d = g.read_slots(0, slots)
    v = g.read_slots(1, slots)[..., :3]
    e_d = rel_error(d, d_ref)
    e_v = float(np.abs(v - v_ref).max() / np.abs(v_ref).max())
    errstat(label, bricks=len(pick), density_rel=e_d, density_rel_significant=rel_error_significant(d, d_ref),
            velocity_rel_to_max=e_v)
    assert e_d <= DENSITY_TOL, e_d
    assert e_v <= VEL_TOL, e_v


def sph_frames(count):
    import workloads

    pos, vel = workloads.sph_slab()
    frames = [pos]
    for _ in range(count - 1):
        frames.append(workloads.advect(frames[-1], vel))
    return frames, vel


@pytest.mark.parametrize("semantics", ["full", "auto"])
def test_sph_4m_frames_match_oracle_and_reference_kernels(gvx_mod, orc, semantics):
    frames, vel = sph_frames(3 if semantics == "full" else 4)
    mode_g = gvx_mod.TOPO_FULL if semantics == "full" else gvx_mod.TOPO_AUTO
    mode_o = orc.TOPO_FULL if semantics == "full" else orc.TOPO_AUTO
    rh = ref_harness()
    r = rh.RefGrid(LOGDIM) if rh else None
    g = sph_grid(gvx_mod)
    o = orc.Oracle(LOGDIM)
    o.atlas_layout_only()
    modes = []
    for k, pos in enumerate(frames):
        sph_frame(gvx_mod, g, pos, vel, mode_g)
        assert o.rebuild_topology(pos, 2.0, mode=mode_o) == orc.OK
        o.update_atlas()
        modes.append(o.last_mode())
        compare_topology(g, o)
        assert g.info()["last_rebuild"] == o.last_mode(), k
        assert np.array_equal(g.read_atlas_map(), o.atlas_map()), k
        if r is not None:
            r.set_points(pos)
            assert r.rebuild(2.0, mode=mode_o) == 0, k
            assert r.last_mode() == o.last_mode()
            same_pools_ref(r, o)
        if k == 0 or k == len(frames) - 1:
            check_sph_values(g, o, orc, pos, vel, "sph4m_%s_frame%d" % (semantics, k), seed=100 + k)
    errstat("sph4m_%s_topology" % semantics, frames=len(frames), modes=modes, leaves=int(o.num_nodes(0)),
            reference_kernels=r is not None, bit_exact=True)
    if semantics == "auto":
        assert modes[:2] == [1, 1] and all(m in (0, 2) for m in modes[2:])
    g.close()
    if r is not None:
        r.close()


# ---------------------------------------------------------------- surface fusion


def test_fusion_30_frames_full_size(gvx_mod, orc):
    import workloads

    frames = list(workloads.depth_fusion(frames=30, seed=3))
    # the bricks to sample come from the final tree (pools only grow under accumulation)
    o = orc.Oracle(LOGDIM)
    o.atlas_layout_only()
    for pos, _ in frames:
        assert o.rebuild_topology(pos, 1.0, mode=orc.TOPO_ACCUMULATE) == orc.OK
    o.update_atlas()
    pick, _ = sample_leaves(o, SAMPLE, 7)

    g = gvx_mod.Grid(0)
    g.configure(LOGDIM)
    g.add_channel(0, gvx_mod.T_FLOAT, 1)
    g.add_channel(1, gvx_mod.T_FLOAT, 1)
    o = orc.Oracle(LOGDIM)
    o.atlas_layout_only()
    dens = np.zeros((len(pick), P, P, P))
    conf_ch = np.zeros((len(pick), P, P, P))
    worst = [0.0, 0.0]
    for k, (pos, conf) in enumerate(frames):
        n = len(pos)
        g.commit_points_host(pos)
        g.rebuild_topology(n, 1.0, mode=gvx_mod.TOPO_ACCUMULATE)
        g.update_atlas()
        g.insert_points(n)
        g.splat(gvx_mod.SPLAT_TRILINEAR, n, 1.0, chan_density=0, accum=True)
        g.commit_points_host(pos, weight=conf)
        g.splat(gvx_mod.SPLAT_TRILINEAR, n, 1.0, chan_density=1, accum=True)
        g.update_apron(0, 0.0)
        g.update_apron(1, 0.0)
        assert o.rebuild_topology(pos, 1.0, mode=orc.TOPO_ACCUMULATE) == orc.OK
        o.update_atlas()
        compare_topology(g, o)
        assert g.info()["last_rebuild"] == o.last_mode(), k
        o.splat_sample(orc.SPLAT_TRILINEAR, pos, pick, 1.0, zero_unowned=False, dens=dens)
        o.splat_sample(orc.SPLAT_TRILINEAR, pos, pick, 1.0, weight=conf, zero_unowned=False, dens=conf_ch)
        if k in (9, 19, 29):
            # interior voxels: the UpdateApron run after every frame overwrites the aprons with the
            # neighbours' interiors (its copies are pinned bit for bit elsewhere), and the next
            # accumulating splat adds onto those
            live = pick < o.num_nodes(0)
            slots = leaf_slots(o.nodes(0), o.atlas_subdim(), P)[pick[live]]
            for c, ref in ((0, dens), (1, conf_ch)):
                e = rel_error(g.read_slots(c, slots)[:, 1:-1, 1:-1, 1:-1], ref[live][:, 1:-1, 1:-1, 1:-1])
                worst[c] = max(worst[c], e)
                assert e <= DENSITY_TOL, (k, c, e)
    errstat("fusion_640x480_2048_30frames", bricks=len(pick), leaves=int(o.num_nodes(0)),
            density_rel=worst[0], confidence_rel=worst[1], topology_bit_exact=True)
    g.close()


# ---------------------------------------------------------------- batched clouds


def test_batched_smallest_clouds_match_oracle(gvx_mod, orc):
    import workloads

    clouds = workloads.batched_clouds()
    small = np.argsort([len(p) for p, _ in clouds])[:3]
    grids = []
    for i in small:
        p, w = clouds[i]
        g = gvx_mod.Grid(0)
        g.configure(LOGDIM)
        g.add_channel(0, gvx_mod.T_FLOAT, 1)
        g.commit_points_host(p, weight=w)
        grids.append(g)
    b = gvx_mod.Batch(0)
    b.set_grids(grids)
    b.topology(1.0, threads=0)
    b.splat(gvx_mod.SPLAT_TRILINEAR, 1.0, chan_density=0, graph=True)
    for g in grids:
        g.update_apron(0, 0.0)
        g.sync()
    worst = 0.0
    for g, i in zip(grids, small):
        p, w = clouds[i]
        o = orc.Oracle(LOGDIM)
        o.add_channel(0, orc.T_FLOAT)
        assert o.rebuild_topology(p, 1.0) == orc.OK
        o.update_atlas()
        o.splat(orc.SPLAT_TRILINEAR, p, 1.0, weight=w)
        compare_topology(g, o)
        used = o.used_leaves()
        e = rel_error(g.read_channel(0)[:used], o.read_channel(0)[:used])
        worst = max(worst, e)
        assert e <= DENSITY_TOL, (int(i), e)
    errstat("batched_3_smallest", points=[int(len(clouds[i][0])) for i in small], density_rel=worst,
            topology_bit_exact=True)
    b.close()
    for g in grids:
        g.close()


# ---------------------------------------------------------------- differentiable splat


def m4(q):
    t = np.clip(2.0 - q, 0.0, None)
    return np.where(q < 1.0, 1.0 - 1.5 * q * q + 0.75 * q ** 3, 0.25 * t ** 3)


def point_contrib(p, w, R, vox):
    """FP64 cubic contribution of one point to voxels `vox` (zero beyond R)"""
    d = np.sqrt(((vox - p) ** 2).sum(-1))
    h = 0.5 * R
    return w * m4(d / h) / (np.pi * h ** 3)


def test_differentiable_1m_gradients_against_finite_differences(gvx_mod, orc):
    import torch
    import workloads

    pos, w, R = workloads.differentiable()
    n = len(pos)
    rng = np.random.default_rng(1)
    tgt = np.clip(pos + rng.normal(0, 0.5, pos.shape), 8.0, 504.0).astype(np.float32)
    both = np.vstack([pos, tgt])
    g = gvx_mod.Grid(0)
    g.configure(LOGDIM)
    g.add_channel(0, gvx_mod.T_FLOAT, 1)
    g.commit_points_host(both)
    g.rebuild_topology(len(both), 3.0, mode=gvx_mod.TOPO_FULL)
    g.update_atlas()
    g.commit_points_host(tgt, weight=w, radius=R)
    g.splat(gvx_mod.SPLAT_CUBIC, n, 1.0, chan_density=0)
    rho_t = g.read_channel(0)
    g.commit_points_host(pos, weight=w, radius=R)
    g.splat(gvx_mod.SPLAT_CUBIC, n, 1.0, chan_density=0)
    rho = g.read_channel(0)
    G = np.zeros_like(rho)
    G[:, 1:-1, 1:-1, 1:-1] = rho[:, 1:-1, 1:-1, 1:-1] - rho_t[:, 1:-1, 1:-1, 1:-1]
    del rho_t
    Gd = torch.from_numpy(G).cuda()
    del G
    gp = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    gw = torch.zeros(n, dtype=torch.float32, device="cuda")
    gr = torch.zeros(n, dtype=torch.float32, device="cuda")
    g.splat_backward(gvx_mod.SPLAT_CUBIC, n, 1.0, Gd, gp, gw, gr)
    g.sync()
    gp, gw, gr = gp.cpu().numpy(), gw.cpu().numpy(), gr.cpu().numpy()

    # the oracle's tree of the same points, and FP64 rho, rho* on the bricks the sample touches
    o = orc.Oracle(LOGDIM)
    o.atlas_layout_only()
    assert o.rebuild_topology(both, 3.0, mode=orc.TOPO_FULL) == orc.OK
    o.update_atlas()
    compare_topology(g, o)
    nodes = o.nodes(0)
    act = np.nonzero(nodes["flags"] == 1)[0]
    bpos = nodes["pos"][act].astype(np.int64) // 8
    bkey = (bpos[:, 0] << 42) | (bpos[:, 1] << 21) | bpos[:, 2]
    korder = np.argsort(bkey)
    bkey, bleaf = bkey[korder], act[korder]

    sample = np.sort(np.random.default_rng(2).choice(n, 1000, replace=False))
    off = np.stack(np.meshgrid(*(np.arange(-3, 4),) * 3, indexing="ij"), -1).reshape(-1, 3)
    supports = []
    for i in sample:
        v = np.floor(pos[i]).astype(np.int64) + off
        v = v[((v - pos[i].astype(np.float64)) ** 2).sum(-1) < float(R[i]) ** 2 * 1.01]
        bk = v >> 3
        key = (bk[:, 0] << 42) | (bk[:, 1] << 21) | bk[:, 2]
        j = np.minimum(np.searchsorted(bkey, key), len(bkey) - 1)
        ok = bkey[j] == key
        supports.append((v[ok], bleaf[j[ok]]))
    leaves = np.unique(np.concatenate([s[1] for s in supports])).astype(np.int32)
    rho64, _ = o.splat_sample(orc.SPLAT_CUBIC, pos, leaves, 1.0, weight=w, radius_pp=R)
    rhot64, _ = o.splat_sample(orc.SPLAT_CUBIC, tgt, leaves, 1.0, weight=w, radius_pp=R)
    lslot = {int(l): k for k, l in enumerate(leaves)}
    # the GPU forward on those bricks
    slots = leaf_slots(nodes, o.atlas_subdim(), P)[leaves]
    e_fwd = rel_error(rho[slots], rho64)

    h = 1e-3
    fd = np.zeros((len(sample), 5))
    for k, (i, (vox, lv)) in enumerate(zip(sample, supports)):
        ks = np.array([lslot[int(x)] for x in lv])
        loc = (vox & 7) + 1
        r_all = rho64[ks, loc[:, 2], loc[:, 1], loc[:, 0]] - rhot64[ks, loc[:, 2], loc[:, 1], loc[:, 0]]
        p0, w0, R0 = pos[i].astype(np.float64), float(w[i]), float(R[i])
        vx = vox.astype(np.float64)
        base = r_all - point_contrib(p0, w0, R0, vx)

        def dl(p_, w_, R_):
            rr = base + point_contrib(p_, w_, R_, vx)
            return 0.5 * (rr * rr).sum()

        for a in range(3):
            e = np.zeros(3)
            e[a] = h
            fd[k, a] = (dl(p0 + e, w0, R0) - dl(p0 - e, w0, R0)) / (2 * h)
        fd[k, 3] = (dl(p0, w0 + h, R0) - dl(p0, w0 - h, R0)) / (2 * h)
        fd[k, 4] = (dl(p0, w0, R0 + h) - dl(p0, w0, R0 - h)) / (2 * h)
    errs = {}
    for name, got, ref in (("dpos", gp[sample], fd[:, :3]), ("dw", gw[sample], fd[:, 3]),
                           ("dR", gr[sample], fd[:, 4])):
        errs[name] = float(np.abs(got - ref).max() / np.abs(ref).max())
    errstat("differentiable_1m", sampled_points=len(sample), forward_bricks=len(leaves), forward_density_rel=e_fwd,
            **{"grad_%s_rel_to_max" % k: v for k, v in errs.items()})
    assert e_fwd <= DENSITY_TOL, e_fwd
    for name, e in errs.items():
        assert e <= GRAD_TOL, (name, e)
    g.close()
