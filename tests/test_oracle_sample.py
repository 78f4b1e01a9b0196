"""CPU tests: the oracle's sampled-leaf splat (used by the full-size GPU
parity tests, where a whole FP64 atlas would not fit) gives exactly the
values of its whole-atlas splat on the sampled leaves."""
import numpy as np
import pytest

from parity_util import leaf_slots


def _cloud(n, seed, box=(60.0, 44.0, 70.0)):
    rng = np.random.default_rng(seed)
    pos = (rng.random((n, 3)) * np.asarray(box) + rng.normal(0, 0.3, (n, 3)) + 0.4).astype(np.float32)
    return pos, rng


@pytest.mark.parametrize("mode_name", ["TRILINEAR", "CUBIC"])
def test_sample_equals_whole_atlas(orc, mode_name):
    mode = getattr(orc, "SPLAT_" + mode_name)
    pos, rng = _cloud(6000, 11)
    vel = rng.normal(0, 1, pos.shape).astype(np.float32)
    w = rng.uniform(0.5, 1.5, len(pos)).astype(np.float32)
    rad = rng.uniform(1.0, 3.0, len(pos)).astype(np.float32) if mode_name == "CUBIC" else None
    o = orc.Oracle()
    o.add_channel(0, orc.T_FLOAT)
    o.add_channel(1, orc.T_FLOAT3)
    assert o.rebuild_topology(pos, 3.0) == orc.OK
    o.update_atlas()
    o.splat(mode, pos, 2.0, weight=w, radius_pp=rad, vel=vel, chan_density=0, chan_vel=1)
    dens_all, vel_all = o.read_channel(0), o.read_channel(1)
    nodes = o.nodes(0)
    slots = leaf_slots(nodes, o.atlas_subdim(), 10)
    active = np.nonzero(nodes["flags"] == 1)[0]
    pick = rng.choice(active, size=min(40, len(active)), replace=False)
    d, v = o.splat_sample(mode, pos, pick, 2.0, weight=w, radius_pp=rad, vel=vel)
    assert np.array_equal(d, dens_all[slots[pick]])
    assert np.array_equal(v, vel_all[slots[pick]][..., :3])
    assert np.abs(d).max() > 0


def test_sample_accumulates_and_skips_inactive(orc):
    pos, rng = _cloud(3000, 12)
    o = orc.Oracle()
    o.add_channel(0, orc.T_FLOAT)
    assert o.rebuild_topology(pos, 1.0) == orc.OK
    o.update_atlas()
    leaves = np.array([0, 1, 2, 10 ** 6], np.int32)  # the last is beyond the pool: takes nothing
    d1, _ = o.splat_sample(orc.SPLAT_TRILINEAR, pos, leaves, zero_unowned=False)
    d2, _ = o.splat_sample(orc.SPLAT_TRILINEAR, pos, leaves, zero_unowned=False, dens=d1.copy())
    assert np.allclose(d2, 2 * d1, rtol=1e-12, atol=0)
    assert not d1[3].any()
