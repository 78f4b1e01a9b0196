"""GPU tests of gvx_splat_backward, the adjoint of the density splat.

The reference gradient is torch.autograd of an FP64 restatement of the
forward over (point, voxel) pairs, on the voxels of the bricks the GPU
activated; the restatement itself is checked against central differences
(h = 1e-3, FP64).  Workload: points U[lo, hi)^3, w ~ U(0, 1), per-point
radius R ~ U(1, 3), target rho* = splat of p + N(0, 0.5) with the same w and
R, L = 1/2 |rho - rho*|^2.  Tolerance: per gradient family (dL/dp, dL/dw,
dL/dR), max |g - g_ref| <= 1e-4 * max |g_ref|."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-4
LOGDIM = (3, 3, 3, 3, 5)


def m4(q):
    import torch

    inner = 1.0 - 1.5 * q * q + 0.75 * q * q * q
    t = torch.clamp(2.0 - q, min=0.0)
    return torch.where(q < 1.0, inner, 0.25 * t * t * t)


def pairs(pos, R, slot_of_brick, mode):
    """(point, voxel) pairs of the forward's support on active bricks, and the
    voxel numbers (slot * 512 + interior local index)"""
    p = pos.astype(np.float64)
    fl = np.floor(p).astype(np.int64)
    rng = np.arange(-3, 4) if mode == "cubic" else np.arange(0, 2)
    off = np.stack(np.meshgrid(rng, rng, rng, indexing="ij"), -1).reshape(-1, 3)
    v = fl[:, None, :] + off[None, :, :]  # (n, k, 3)
    pi = np.broadcast_to(np.arange(len(p))[:, None], v.shape[:2])
    d2 = ((v - p[:, None, :]) ** 2).sum(-1)
    keep = (v >= 0).all(-1)
    if mode == "cubic":
        keep &= d2 < (R.astype(np.float64) ** 2)[:, None]
    bk = v >> 3
    key = (bk[..., 0] << 42) | (bk[..., 1] << 21) | bk[..., 2]
    slot = np.full(key.shape, -1, np.int64)
    ks, ss = slot_of_brick
    j = np.searchsorted(ks, key)
    jc = np.minimum(j, len(ks) - 1)
    hit = ks[jc] == key
    slot[hit] = ss[jc[hit]]
    keep &= slot >= 0
    loc = v & 7
    vid = slot * 512 + (loc[..., 2] * 8 + loc[..., 1]) * 8 + loc[..., 0]
    return pi[keep], v[keep], vid[keep]


def restated_rho(pos, w, R, pi, vox, vid, nvox, mode):
    """FP64 torch restatement of the forward: rho over the interior voxels"""
    import torch

    dv = torch.as_tensor(vox, dtype=torch.float64) - pos[pi]
    if mode == "cubic":
        d = torch.sqrt((dv * dv).sum(-1))
        h = 0.5 * R[pi]
        val = w[pi] * m4(d / h) / (np.pi * h ** 3)
    else:
        wgt = 1.0 - torch.abs(dv)  # CIC: 1 - |v - p| per axis on the 2 nearest voxels
        val = w[pi] * wgt[:, 0] * wgt[:, 1] * wgt[:, 2]
    return torch.zeros(nvox, dtype=torch.float64).index_add(0, torch.as_tensor(vid), val)


def make_case(gvx, n, seed, lo, hi, mode):
    import torch

    rng = np.random.default_rng(seed)
    pos = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    w = rng.uniform(0, 1, n).astype(np.float32)
    R = rng.uniform(1, 3, n).astype(np.float32) if mode == "cubic" else np.full(n, 1.0, np.float32)
    tgt = np.clip(pos + rng.normal(0, 0.5, pos.shape), lo, hi).astype(np.float32)
    g = gvx.Grid(0)
    g.configure(LOGDIM)
    g.add_channel(0, gvx.T_FLOAT, 1)
    both = np.vstack([pos, tgt])
    g.commit_points_host(both)
    g.rebuild_topology(len(both), 3.0, mode=gvx.TOPO_FULL)
    g.update_atlas()
    m = gvx.SPLAT_CUBIC if mode == "cubic" else gvx.SPLAT_TRILINEAR
    g.commit_points_host(tgt, weight=w, radius=R if mode == "cubic" else None)
    g.splat(m, n, 1.0, chan_density=0)
    rho_t = g.read_channel(0).copy()
    g.commit_points_host(pos, weight=w, radius=R if mode == "cubic" else None)
    g.splat(m, n, 1.0, chan_density=0)
    rho = g.read_channel(0).copy()
    G = np.zeros_like(rho)
    G[:, 1:-1, 1:-1, 1:-1] = rho[:, 1:-1, 1:-1, 1:-1] - rho_t[:, 1:-1, 1:-1, 1:-1]
    Gd = torch.from_numpy(G).cuda()
    gp = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    gw = torch.zeros(n, dtype=torch.float32, device="cuda")
    gr = torch.zeros(n, dtype=torch.float32, device="cuda")
    g.splat_backward(m, n, 1.0, Gd, gp, gw, gr)
    g.sync()
    used = g.info()["used_leaves"]
    amap = g.read_atlas_map()[:used]
    bk = amap[:, :3].astype(np.int64) >> 3
    keys = (bk[:, 0] << 42) | (bk[:, 1] << 21) | bk[:, 2]
    order = np.argsort(keys)
    slot_of_brick = (keys[order], np.arange(used, dtype=np.int64)[order])
    return dict(g=g, pos=pos, w=w, R=R, tgt=tgt, used=used, slot_of_brick=slot_of_brick, mode=mode,
                gpu=(gp.cpu().numpy(), gw.cpu().numpy(), gr.cpu().numpy()), G=G, rho_t=rho_t)


def reference_grads(c):
    import torch

    n, mode = len(c["pos"]), c["mode"]
    nvox = c["used"] * 512
    pi, vox, vid = pairs(c["pos"], c["R"], c["slot_of_brick"], mode)
    ti, tvox, tvid = pairs(c["tgt"], c["R"], c["slot_of_brick"], mode)
    pos = torch.tensor(c["pos"], dtype=torch.float64, requires_grad=True)
    w = torch.tensor(c["w"], dtype=torch.float64, requires_grad=True)
    R = torch.tensor(c["R"], dtype=torch.float64, requires_grad=True)
    with torch.no_grad():
        rho_t = restated_rho(torch.tensor(c["tgt"], dtype=torch.float64), w, R, ti, tvox, tvid, nvox, mode)
    rho = restated_rho(pos, w, R, pi, vox, vid, nvox, mode)
    L = 0.5 * ((rho - rho_t) ** 2).sum()
    L.backward()
    gR = R.grad.numpy() if R.grad is not None else np.zeros(n)  # trilinear has no radius
    return pos.grad.numpy(), w.grad.numpy(), gR, (pi, vox, vid, rho.detach(), rho_t)


def close(got, ref):
    return float(np.abs(got - ref).max()) <= GRAD_TOL * float(np.abs(ref).max())


@pytest.mark.parametrize("mode", ["cubic", "trilinear"])
def test_backward_matches_fp64_autograd(gvx_mod, mode):
    c = make_case(gvx_mod, 20_000, 3, 8.0, 120.0, mode)
    gp, gw, gr, _ = reference_grads(c)
    assert close(c["gpu"][0], gp), float(np.abs(c["gpu"][0] - gp).max() / np.abs(gp).max())
    assert close(c["gpu"][1], gw)
    if mode == "cubic":
        assert close(c["gpu"][2], gr)


def point_contrib(p, w, R, vox):
    """FP64 contribution of one cubic point to the voxels `vox`"""
    d = np.sqrt(((vox - p) ** 2).sum(-1))
    h = 0.5 * R
    q = d / h
    t = np.clip(2.0 - q, 0.0, None)
    m = np.where(q < 1.0, 1.0 - 1.5 * q * q + 0.75 * q ** 3, 0.25 * t ** 3)
    return w * m / (np.pi * h ** 3)


def test_backward_against_finite_differences(gvx_mod):
    # central differences h = 1e-3 in FP64 for each of p.xyz, w, R of every one of
    # the 1,000 points: a perturbation only changes the point's own support, so the
    # loss difference is summed over those voxels
    c = make_case(gvx_mod, 1_000, 2, 8.0, 40.0, "cubic")
    gp, gw, gr, (pi, vox, vid, rho, rho_t) = reference_grads(c)
    rho, rho_t = rho.numpy(), rho_t.numpy()
    h = 1e-3
    pos = c["pos"].astype(np.float64)
    w = c["w"].astype(np.float64)
    R = c["R"].astype(np.float64)
    order = np.argsort(pi, kind="stable")
    bounds = np.searchsorted(pi[order], np.arange(len(pos) + 1))
    fd = np.zeros((len(pos), 5))
    for i in range(len(pos)):
        rows = order[bounds[i]:bounds[i + 1]]
        vx, vi = vox[rows].astype(np.float64), vid[rows]
        base = rho[vi] - rho_t[vi] - point_contrib(pos[i], w[i], R[i], vx)

        def dl(p_, w_, R_):
            r = base + point_contrib(p_, w_, R_, vx)
            return 0.5 * (r * r).sum()

        for k in range(3):
            e = np.zeros(3)
            e[k] = h
            fd[i, k] = (dl(pos[i] + e, w[i], R[i]) - dl(pos[i] - e, w[i], R[i])) / (2 * h)
        fd[i, 3] = (dl(pos[i], w[i] + h, R[i]) - dl(pos[i], w[i] - h, R[i])) / (2 * h)
        fd[i, 4] = (dl(pos[i], w[i], R[i] + h) - dl(pos[i], w[i], R[i] - h)) / (2 * h)
    # the FP64 restatement agrees with its own central differences
    assert close(gp, fd[:, :3]) and close(gw, fd[:, 3]) and close(gr, fd[:, 4])
    # and the GPU adjoint with both
    assert close(c["gpu"][0], fd[:, :3])
    assert close(c["gpu"][1], fd[:, 3])
    assert close(c["gpu"][2], fd[:, 4])


def test_backward_is_deterministic(gvx_mod):
    import torch

    c = make_case(gvx_mod, 30_000, 7, 8.0, 150.0, "cubic")
    g, n = c["g"], len(c["pos"])
    Gd = torch.from_numpy(c["G"]).cuda()
    gp = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    gw = torch.zeros(n, dtype=torch.float32, device="cuda")
    gr = torch.zeros(n, dtype=torch.float32, device="cuda")
    g.splat_backward(gvx_mod.SPLAT_CUBIC, n, 1.0, Gd, gp, gw, gr)
    g.sync()
    assert np.array_equal(gp.cpu().numpy(), c["gpu"][0])
    assert np.array_equal(gw.cpu().numpy(), c["gpu"][1])
    assert np.array_equal(gr.cpu().numpy(), c["gpu"][2])


def test_backward_with_recomputed_permutation(gvx_mod):
    """GVX_BWD_RECOMPUTE: the permutation re-keyed and re-sorted from the positions gives the
    gradients of the stored grouping bit for bit, and the forward after it is unchanged"""
    import torch

    c = make_case(gvx_mod, 30_000, 9, 8.0, 150.0, "cubic")
    g, n = c["g"], len(c["pos"])
    Gd = torch.from_numpy(c["G"]).cuda()
    gp = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    gw = torch.zeros(n, dtype=torch.float32, device="cuda")
    gr = torch.zeros(n, dtype=torch.float32, device="cuda")
    launches = g.kernel_launches()
    g.splat_backward(gvx_mod.SPLAT_CUBIC, n, 1.0, Gd, gp, gw, gr, recompute=True)
    g.sync()
    assert g.kernel_launches() - launches > 2  # keys, sort passes, octant partition, then the adjoint
    assert np.array_equal(gp.cpu().numpy(), c["gpu"][0])
    assert np.array_equal(gw.cpu().numpy(), c["gpu"][1])
    assert np.array_equal(gr.cpu().numpy(), c["gpu"][2])
    rho = g.read_channel(0).copy()
    g.splat(gvx_mod.SPLAT_CUBIC, n, 1.0, chan_density=0)
    assert np.array_equal(g.read_channel(0), rho)


def test_autograd_function_wrapper(gvx_mod):
    """the adjoint behind a torch.autograd.Function (test harness only): the
    splat of (pos, w, R) as a differentiable op, L = 1/2 |rho - rho*|^2 over
    the interior voxels, gradients of all three inputs against the FP64
    restatement's autograd (and identical to a direct gvx_splat_backward)"""
    import torch

    c = make_case(gvx_mod, 20_000, 4, 8.0, 120.0, "cubic")
    g, n = c["g"], len(c["pos"])

    class Splat(torch.autograd.Function):
        @staticmethod
        def forward(ctx, pos, w, R):
            g.set_points(n, pos.detach())
            g.set_point_attribs(weight=w.detach(), radius=R.detach())
            g.splat(gvx_mod.SPLAT_CUBIC, n, 1.0, chan_density=0)
            g.sync()
            return torch.from_numpy(g.read_channel(0).copy()).cuda()

        @staticmethod
        def backward(ctx, grad_out):
            gp = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
            gw = torch.zeros(n, dtype=torch.float32, device="cuda")
            gr = torch.zeros(n, dtype=torch.float32, device="cuda")
            g.splat_backward(gvx_mod.SPLAT_CUBIC, n, 1.0, grad_out.contiguous(), gp, gw, gr)
            g.sync()
            return gp, gw, gr

    pos = torch.from_numpy(c["pos"]).cuda().requires_grad_(True)
    w = torch.from_numpy(c["w"]).cuda().requires_grad_(True)
    R = torch.from_numpy(c["R"]).cuda().requires_grad_(True)
    rho = Splat.apply(pos, w, R)
    rho_t = torch.from_numpy(c["rho_t"]).cuda()
    P = rho.shape[1]
    mask = torch.zeros((P, P, P), device="cuda")
    mask[1:-1, 1:-1, 1:-1] = 1.0
    L = 0.5 * (((rho - rho_t) * mask) ** 2).sum()
    L.backward()
    got = (pos.grad.cpu().numpy(), w.grad.cpu().numpy(), R.grad.cpu().numpy())
    for a, b in zip(got, c["gpu"]):
        assert np.array_equal(a, b)
    gp, gw, gr, _ = reference_grads(c)
    assert close(got[0], gp), float(np.abs(got[0] - gp).max() / np.abs(gp).max())
    assert close(got[1], gw)
    assert close(got[2], gr)
