"""GPU parity of Compute (FUNC_SMOOTH, FUNC_FILL_F/C/C4) against the oracle on
the same channel contents: smoothing within FP32 rounding (a float sum and
division against an FP64 restatement), fills and UpdateApronFaces bit for
bit, over the whole atlas (aprons and unused slots included)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LOGDIM = (3, 3, 3, 3, 5)
# float sums of 7 terms against FP64: |a - b| <= SMOOTH_TOL * max(1, max|b|)
SMOOTH_TOL = 2e-6


def build(gvx, orc, apron=1, channels=((0, 3),), n=20000, seed=21):
    rng = np.random.default_rng(seed)
    pos = (rng.random((n, 3)) * np.array([120.0, 90.0, 150.0]) + 2.0).astype(np.float32)
    g = gvx.Grid(0)
    g.configure(LOGDIM)
    o = orc.Oracle(LOGDIM, apron=apron)
    for c, t in channels:
        g.add_channel(c, t, apron)
        o.add_channel(c, t)
    g.commit_points_host(pos)
    g.rebuild_topology(n, 1.0, mode=gvx.TOPO_FULL)
    g.update_atlas()
    assert o.rebuild_topology(pos, 1.0) == orc.OK
    o.update_atlas()
    assert tuple(g.info()["atlas_subdim"]) == o.atlas_subdim()
    assert g.info()["used_leaves"] == o.used_leaves()
    return g, o


def seeded(g, chan, seed):
    """the same eighths in [-8, 8) (exact in FP32) written to the GPU channel; returned for the oracle"""
    shape = g.read_channel(chan).shape
    return (np.random.default_rng(seed).integers(-64, 64, shape) / 8.0).astype(np.float32)


def close(got, ref, tol=SMOOTH_TOL):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.abs(got - ref).max()) <= tol * max(1.0, float(np.abs(ref).max()))


@pytest.mark.parametrize("params,iters,boundval", [((4.0, 0.0, 0.0), 3, 3.0), ((1.0, -0.05, 0.0), 2, 0.0)])
def test_smooth_matches_oracle(gvx_mod, orc, params, iters, boundval):
    g, o = build(gvx_mod, orc)
    data = seeded(g, 0, 5)
    g.write_channel(0, data)
    o.write_channel(0, data)
    g.update_apron(0, boundval)
    o.update_apron(0, boundval)
    g.compute(gvx_mod.FUNC_SMOOTH, 0, iters, params, update_apron=True, skip_over_aprons=True, boundval=boundval)
    o.compute(orc.FUNC_SMOOTH, 0, iters, params, update_apron=True, skip_over_aprons=True, boundval=boundval)
    a = g.read_channel(0)
    assert close(a, o.read_channel(0))
    # gvdbOpSmooth indexes packed whatever skipOverAprons: the unpacked launch writes the same voxels
    g.write_channel(0, data)
    g.update_apron(0, boundval)
    g.compute(gvx_mod.FUNC_SMOOTH, 0, iters, params, update_apron=True, skip_over_aprons=False, boundval=boundval)
    assert np.array_equal(g.read_channel(0), a)


def test_smooth_without_apron(gvx_mod, orc):
    g, o = build(gvx_mod, orc, apron=0)
    data = seeded(g, 0, 6)
    g.write_channel(0, data)
    o.write_channel(0, data)
    ptr = g.channel_device_ptr(0)[0]
    g.compute(gvx_mod.FUNC_SMOOTH, 0, 2, (4.0, 0.0, 0.0), update_apron=False, skip_over_aprons=True)
    o.compute(orc.FUNC_SMOOTH, 0, 2, (4.0, 0.0, 0.0), update_apron=False, skip_over_aprons=True)
    assert close(g.read_channel(0), o.read_channel(0))
    assert g.channel_device_ptr(0)[0] == ptr  # the channel stays where it was


def test_smooth_after_splat(gvx_mod, orc):
    """the gPointCloud sequence: splat, then Compute(FUNC_SMOOTH, 0, n, (p1, p2, 0), true, true, 3)"""
    rng = np.random.default_rng(9)
    pos = (rng.random((30000, 3)) * np.array([100.0, 80.0, 60.0]) + 4.0).astype(np.float32)
    g = gvx_mod.Grid(0)
    g.configure(LOGDIM)
    g.add_channel(0, gvx_mod.T_FLOAT, 1)
    o = orc.Oracle(LOGDIM)
    o.add_channel(0, orc.T_FLOAT)
    g.commit_points_host(pos)
    g.rebuild_topology(len(pos), 1.0, mode=gvx_mod.TOPO_FULL)
    g.update_atlas()
    g.insert_points(len(pos))
    g.splat(gvx_mod.SPLAT_TRILINEAR, len(pos), 1.0, chan_density=0)
    assert o.rebuild_topology(pos, 1.0) == orc.OK
    o.update_atlas()
    o.splat(orc.SPLAT_TRILINEAR, pos, 1.0, chan_density=0)
    g.compute(gvx_mod.FUNC_SMOOTH, 0, 4, (2.0, 0.01, 0.0), update_apron=True, skip_over_aprons=True, boundval=3.0)
    o.compute(orc.FUNC_SMOOTH, 0, 4, (2.0, 0.01, 0.0), update_apron=True, skip_over_aprons=True, boundval=3.0)
    # the splat's own FP32 tolerance carries through the averaging
    assert close(g.read_channel(0), o.read_channel(0), tol=1e-5)


@pytest.mark.parametrize("skip", [False, True])
def test_fills_match_oracle(gvx_mod, orc, skip):
    g, o = build(gvx_mod, orc, channels=((0, 3), (1, 2), (2, 0)))
    for c in (0, 1, 2):
        g.clear_channel(c)
    g.compute(gvx_mod.FUNC_FILL_F, 0, 1, (2.5, 0.0, 0.0), update_apron=False, skip_over_aprons=skip)
    o.compute(orc.FUNC_FILL_F, 0, 1, (2.5, 0.0, 0.0), update_apron=False, skip_over_aprons=skip)
    assert np.array_equal(g.read_channel(0).astype(np.float64), o.read_channel(0))
    g.compute(gvx_mod.FUNC_FILL_C4, 1, 1, (0.5, 1.0, 2.0), update_apron=False, skip_over_aprons=skip)
    o.compute(orc.FUNC_FILL_C4, 1, 1, (0.5, 1.0, 2.0), update_apron=False, skip_over_aprons=skip)
    assert np.array_equal(g.read_channel(1).astype(np.float64), o.read_channel(1))
    for p1 in (7.9, 300.0, -3.0):
        g.compute(gvx_mod.FUNC_FILL_C, 2, 1, (p1, 0.0, 0.0), update_apron=False, skip_over_aprons=skip)
        o.compute(orc.FUNC_FILL_C, 2, 1, (p1, 0.0, 0.0), update_apron=False, skip_over_aprons=skip)
        assert np.array_equal(g.read_channel(2).astype(np.float64), o.read_channel(2))


def test_fill_pattern(gvx_mod, orc):
    g, o = build(gvx_mod, orc)
    g.clear_channel(0)
    g.compute(gvx_mod.FUNC_FILL_F, 0, 1, (0.0, 0.0, -1.0), update_apron=True, skip_over_aprons=False)
    o.compute(orc.FUNC_FILL_F, 0, 1, (0.0, 0.0, -1.0), update_apron=True, skip_over_aprons=False)
    # sinf on the device and on the host: a few units in the last place of values up to 3
    assert close(g.read_channel(0), o.read_channel(0), tol=1e-6)


def test_unsupported_operator(gvx_mod, orc):
    g, _ = build(gvx_mod, orc, channels=((0, 3), (1, 2)))
    with pytest.raises(gvx_mod.GvxError):
        g.compute(gvx_mod.FUNC_SMOOTH, 1, 1, (4.0, 0.0, 0.0), update_apron=False, skip_over_aprons=True)
    with pytest.raises(gvx_mod.GvxError):
        g.compute(gvx_mod.FUNC_FILL_C4, 0, 1, (1.0, 1.0, 1.0), update_apron=False, skip_over_aprons=True)


def test_update_apron_faces_matches_oracle(gvx_mod, orc):
    """UpdateApronFaces: face aprons exchanged between face neighbours; edges, corners and faces
    without a neighbour keep their values (bit for bit against the oracle)"""
    g, o = build(gvx_mod, orc)
    data = seeded(g, 0, 9)
    g.write_channel(0, data)
    o.write_channel(0, data)
    g.update_neighbors()
    g.update_apron_faces(0)
    o.update_apron_faces(0)
    a, b = g.read_channel(0), o.read_channel(0)
    assert np.array_equal(a.astype(np.float64), b)
    changed = a != data
    assert changed.any()
    # only apron voxels of faces change: no interior voxel, no edge or corner
    P = a.shape[1]
    on = np.zeros((P, P, P), int)
    for ax in range(3):
        sl = [slice(None)] * 3
        for end in (0, P - 1):
            sl[ax] = end
            on[tuple(sl)] += 1
    assert not changed[:, on != 1].any()
