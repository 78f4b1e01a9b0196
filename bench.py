"""Benchmark of the point -> sparse-volume path (topology + splat + apron).

One step = one frame of the SPH slab workload: 4M points in a 1024^3 index
space, advected by dt * u (30 precomputed frames, cycled), FULL topology
rebuild with dilation radius 2, cubic-spline splat (R = 2) of density and
float3 velocity into 8^3 bricks with a 1-voxel apron, then UpdateApron of both
channels.  Metric: Mpoints/s = points / step time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the same path (the reference's
host library does not build without OpenGL/X11) on the host cores, on
bounded sub-box samples of the same workload.
"""
import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "gvdb-voxels_gb300")
ORACLE = os.path.join(ROOT, "oracle")
sys.path.insert(0, PKG)

METRIC = "Mpoints/s (topology+splat+apron, 4M pts)"
UNIT = "Mpoints/s"
N_POINTS = 4_000_000
FRAMES = 30
DT = 0.5
RADIUS = 2.0
LOGDIM = (3, 3, 3, 3, 5)
BOX = (512.0, 256.0, 1024.0)
L2_FLUSH_BYTES = 256 << 20


def config_dict(points=N_POINTS):
    return {"workload": "sph_slab: %d points in x<512,y<256,z<1024 of a 1024^3 space, N(0,0.3) jitter, "
                        "velocity N(0,1), %d frames of Euler advection dt=%.1f cycled; FULL topology rebuild "
                        "(radius %.0f) + cubic-spline splat R=%.0f of density (float) and velocity (float3) "
                        "+ UpdateApron of both channels" % (points, FRAMES, DT, RADIUS, RADIUS),
            "points": points, "frames": FRAMES, "bricks": "8^3 (+1 apron)", "levels": list(LOGDIM),
            "radius": RADIUS, "rebuild": "full", "l2": "flushed by a 256 MB write before every timed step"}


# --------------------------------------------------------------------------
# CPU side: the oracle (restatement of the reference path) on sub-box samples

def _cpu_sample(args):
    """one sub-box of the slab at the workload's point density, through the
    oracle: topology + atlas + cubic splat (density, velocity) + apron x2"""
    frac, seed = args
    import numpy as np
    sys.path.insert(0, ORACLE)
    import oracle as O

    sub = (BOX[0] * frac[0], BOX[1] * frac[1], BOX[2] * frac[2])
    n = int(round(N_POINTS * frac[0] * frac[1] * frac[2]))
    rng = np.random.default_rng(seed)
    pos = (rng.random((n, 3)) * np.asarray(sub) + 2.0 + rng.normal(0, 0.3, (n, 3))).astype(np.float32)
    vel = rng.normal(0, 1, (n, 3)).astype(np.float32)
    t0 = time.perf_counter()
    o = O.Oracle(LOGDIM)
    o.add_channel(0, O.T_FLOAT)
    o.add_channel(1, O.T_FLOAT3)
    o.rebuild_topology(pos, RADIUS, allow_degenerate=True)
    o.update_atlas()
    o.splat(O.SPLAT_CUBIC, pos, RADIUS, vel=vel, chan_density=0, chan_vel=1)
    o.update_apron(0, 0.0)
    o.update_apron(1, 0.0)
    dt = time.perf_counter() - t0
    o.close()
    return n, dt


SAMPLE_FRAC = (0.25, 0.25, 0.125)  # 1/128 of the slab: 31,250 points at the same density


def cpu_pool(workers):
    ctx = mp.get_context("spawn")
    return ctx.Pool(workers)


def cpu_baseline(pool=None, samples=24):
    """single-core port: `samples` sub-boxes one after the other"""
    tot_n, tot_t = 0, 0.0
    for s in range(samples):
        n, dt = pool.apply(_cpu_sample, ((SAMPLE_FRAC, 100 + s),)) if pool else _cpu_sample((SAMPLE_FRAC, 100 + s))
        tot_n += n
        tot_t += dt
    return {"value": tot_n / tot_t / 1e6, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "%d sub-boxes of 1/128 of the slab (%d points in all, same density), oracle topology + "
                      "cubic splat (density+velocity) + apron, single thread" % (samples, tot_n)}


# --------------------------------------------------------------------------
# clocks during the timed region

class ClockSampler:
    REASONS = {0x1: "gpu_idle", 0x2: "applications_clocks_setting", 0x4: "sw_power_cap", 0x8: "hw_slowdown",
               0x10: "sync_boost", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown", 0x100: "display_clock_setting"}

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        """start sampling every 50 ms and wait (up to 10 s) for the first sample, so that the
        sampler is live when the timed region begins"""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.active",
                 "--format=csv,noheader,nounits", "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
            return
        t_end = time.perf_counter() + 10.0
        while not self.lines and time.perf_counter() < t_end and self.proc.poll() is None:
            time.sleep(0.01)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def stop(self, t0=None, t1=None):
        """the samples taken from 0.1 s before the timed region [t0, t1] to 0.1 s after it (the
        region of a short run is shorter than the sampling period: the samples that bracket it),
        after waiting (up to 2 s) for one taken after t1"""
        if not self.proc:
            return None
        if t1 is not None:
            t_end = time.perf_counter() + 2.0
            while time.perf_counter() < t_end and self.proc.poll() is None and \
                    not any(t > t1 for t, _ in self.lines):
                time.sleep(0.01)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        lines = list(self.lines)
        if t0 is not None and t1 is not None:
            window = [(t, ln) for t, ln in lines if t0 - 0.1 <= t <= t1 + 0.1]
            lines = window or lines
        sm, mx, reasons = [], 0, set()
        for _, ln in lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 3:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
                bits = int(parts[2], 16)
            except ValueError:
                continue
            for b, name in self.REASONS.items():
                if bits & b and name != "gpu_idle":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------

def algorithmic_bytes(n, nb, P):
    """algorithmic bytes per frame: positions read by the topology, point
    attributes read by the splat, every active padded brick written once per
    channel, and the apron source voxels read once per channel"""
    ch_bytes = 4 + 16  # density float + velocity float3 stored as float4
    b_topo = 12 * n
    b_splat_pts = (12 + 12) * n
    b_atlas = nb * P ** 3 * ch_bytes
    b_apron = nb * (P ** 3 - (P - 2) ** 3) * ch_bytes
    return b_topo, b_splat_pts, b_atlas, b_apron


def load_traffic():
    """(DRAM bytes per active brick, per point) of the splat launch, from the summary of an
    ncu capture of the bench's timed frames (profiles/splat_cubic_sph4m_traffic.txt)"""
    p = os.path.join(ROOT, "profiles", "splat_cubic_sph4m_traffic.txt")
    if not os.path.exists(p):
        return None
    vals = {}
    for ln in open(p):
        if ":" in ln:
            k, v = ln.split(":", 1)
            try:
                vals[k.strip()] = float(v.split()[0])
            except (ValueError, IndexError):
                pass
    if "dram_bytes_per_brick" in vals and "dram_bytes_per_point" in vals:
        return vals["dram_bytes_per_brick"], vals["dram_bytes_per_point"]
    return None


def max_over_ranks(ms, dist=None, device=None):
    """The job's step time: the slowest rank's mean step time (every rank calls this;
    one process per GPU, each a replica of the frame on its own points)."""
    if dist is None:
        return ms
    import torch

    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_mpoints_s(world, n, ms):
    """Whole-job throughput: every rank splats n points per step, the step takes ms"""
    return world * n / (ms * 1e-3) / 1e6


def run_ours(args, rank, world, pool):
    import numpy as np
    import torch

    import gvx
    import workloads

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist_mod

        dist = dist_mod
        dist.init_process_group("nccl", device_id=dev)

    npts = args.points or N_POINTS
    box = (BOX[0], BOX[1], BOX[2] * npts / N_POINTS)  # smaller runs keep the point density
    pos0, vel = workloads.sph_slab(n=npts, seed=0, box=box)
    n = pos0.shape[0]
    vel_d = torch.from_numpy(vel).to(dev)
    pos_d = torch.from_numpy(pos0).to(dev)
    frames = [pos_d + (f * DT) * vel_d for f in range(FRAMES)]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)

    g = gvx.Grid(dev.index)
    g.configure(LOGDIM)
    g.add_channel(0, gvx.T_FLOAT, 1)
    g.add_channel(1, gvx.T_FLOAT3, 1)
    g.set_stream(stream.cuda_stream)

    def step(f, events=None):
        p = frames[f % FRAMES]
        g.set_points(n, p, 0, 12, vel_d, 0, 12)
        g.rebuild_topology(n, RADIUS, mode=gvx.TOPO_FULL)
        g.finish_topology()
        g.update_atlas()
        g.insert_points(n)
        if events:
            events[0].record(stream)
        g.splat(gvx.SPLAT_CUBIC, n, RADIUS, chan_density=0, chan_vel=1)
        if events:
            events[1].record(stream)
        g.update_apron(0, 0.0)
        g.update_apron(1, 0.0)

    with torch.cuda.stream(stream):
        for w in range(args.warmup):
            step(w)
        torch.cuda.synchronize()

        # ---- per-stage breakdown (untimed pass)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(7)]
        p = frames[0]
        g.set_points(n, p, 0, 12, vel_d, 0, 12)
        ev[0].record(stream)
        g.rebuild_topology(n, RADIUS, mode=gvx.TOPO_FULL)
        g.finish_topology()
        ev[1].record(stream)
        g.update_atlas()
        ev[2].record(stream)
        g.insert_points(n)
        ev[3].record(stream)
        g.splat(gvx.SPLAT_CUBIC, n, RADIUS, chan_density=0, chan_vel=1)
        ev[4].record(stream)
        g.update_apron(0, 0.0)
        ev[5].record(stream)
        g.update_apron(1, 0.0)
        ev[6].record(stream)
        torch.cuda.synchronize()
        names = ["topology", "update_atlas", "insert_points", "splat", "apron_density", "apron_velocity"]
        stage_ms = {k: round(ev[i].elapsed_time(ev[i + 1]), 4) for i, k in enumerate(names)}

        # ---- timed region
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        sp = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        clocks = ClockSampler(dev.index)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        clocks.start()
        launches0 = g.kernel_launches()
        t0 = time.perf_counter()
        for k in range(args.steps):
            flush.fill_(float(k))
            starts[k].record(stream)
            step(args.warmup + k, sp[k])
            ends[k].record(stream)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        wall = t1 - t0
        launches = g.kernel_launches() - launches0
        clk = clocks.stop(t0, t1)
        if dist:
            dist.barrier()
        step_ms = [starts[k].elapsed_time(ends[k]) for k in range(args.steps)]
        splat_ms = [sp[k][0].elapsed_time(sp[k][1]) for k in range(args.steps)]
        ms = max_over_ranks(sum(step_ms) / len(step_ms), dist, dev)

        inf = g.info()
        P = inf["brick_res"] + 2 * inf["apron"]
        # active bricks of each timed frame (the splat's bytes scale with them): the frames'
        # topologies rebuilt again outside the timed region
        nb_frames = []
        for k in range(args.steps):
            g.set_points(n, frames[(args.warmup + k) % FRAMES], 0, 12, vel_d, 0, 12)
            g.rebuild_topology(n, RADIUS, mode=gvx.TOPO_FULL)
            nb_frames.append(int(g.info()["used_leaves"]))
        nb = sum(nb_frames) / len(nb_frames)

        # ---- the reference's default rebuild semantics (RebuildTopology's state machine, VG.cpp:1195-1217):
        # after one full build, frames extend the tree incrementally; outside the timed region
        incremental = None
        if not args.no_extras and world == 1:
            g.request_full_rebuild(True)
            inc_ms, modes = [], []
            for f in range(min(FRAMES, 12)):
                flush.fill_(float(f))
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                p = frames[f % FRAMES]
                g.set_points(n, p, 0, 12, vel_d, 0, 12)
                e0.record(stream)
                g.rebuild_topology(n, RADIUS, mode=gvx.TOPO_AUTO)
                g.finish_topology()
                g.update_atlas()
                g.insert_points(n)
                g.splat(gvx.SPLAT_CUBIC, n, RADIUS, chan_density=0, chan_vel=1)
                g.update_apron(0, 0.0)
                g.update_apron(1, 0.0)
                e1.record(stream)
                torch.cuda.synchronize()
                inc_ms.append(e0.elapsed_time(e1))
                modes.append(g.info()["last_rebuild"])
            steady = [t for t, m in zip(inc_ms, modes) if m == 2]
            incremental = {"frames": len(inc_ms), "rebuilds": modes,
                           "ms_per_incremental_frame": round(sum(steady) / max(len(steady), 1), 4),
                           "mpoints_s": round(n / (sum(steady) / max(len(steady), 1) * 1e-3) / 1e6, 1) if steady else None,
                           "active_bricks_last": int(g.info()["used_leaves"])}

        # ---- end to end through the C ABI with host buffers (pinned)
        e2e_steps = 0 if args.no_e2e else max(3, min(args.steps, 10))
        e2e_wall, d2h = 1.0, 0
    if e2e_steps:
        host_pos = [torch.empty((n, 3), dtype=torch.float32, pin_memory=True) for _ in range(2)]
        host_pos[0].copy_(torch.from_numpy(pos0))
        host_pos[1].copy_(torch.from_numpy(workloads.advect(pos0, vel, DT)))
        host_vel = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
        host_vel.copy_(torch.from_numpy(vel))
        res = np.zeros(1 << 16, gvx.NODE_DTYPE)
        d2h = 0
        for k in range(2):  # warm
            g.commit_points_host(host_pos[k % 2], host_vel)
        torch.cuda.synchronize()

        def commit(k):
            g.lib.gvx_commit_points_host(g.h, n, host_pos[k % 2].data_ptr(), 12, host_vel.data_ptr(), 12, None,
                                         None)

        # step k: upload frame k's points (issued at the end of step k-1, so the copies overlap
        # that step's splat, as a simulation loop hands over its next frame), topology, insert,
        # splat, aprons, and the level-1 nodes read back to the host
        t0 = time.perf_counter()
        commit(0)
        for k in range(e2e_steps):
            g.rebuild_topology(n, RADIUS, mode=gvx.TOPO_FULL)
            g.finish_topology()
            g.update_atlas()
            g.insert_points(n)
            g.splat(gvx.SPLAT_CUBIC, n, RADIUS, chan_density=0, chan_vel=1)
            g.update_apron(0, 0.0)
            g.update_apron(1, 0.0)
            if k + 1 < e2e_steps:
                commit(k + 1)
            c1 = g.info()["node_count"][1]
            g._check(g.lib.gvx_read_nodes(g.h, 1, res.ctypes.data, len(res)))
            d2h = c1 * 64
        e2e_wall = time.perf_counter() - t0
    g.close()

    b_topo, b_pts, b_atlas, b_apron = algorithmic_bytes(n, nb, P)
    splat_bytes = b_pts + b_atlas
    splat_avg = sum(splat_ms) / len(splat_ms)
    achieved = splat_bytes / (splat_avg * 1e-3) / 1e9
    # per-brick and per-point DRAM bytes of the splat from an ncu capture of the same frames,
    # applied to this run's bricks and points
    tr = load_traffic()
    traffic = tr[0] * nb + tr[1] * n if tr else None
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        peak = float(json.load(open(peaks_path))["hbm_gbs"])
        peak_src = "measured"
    out = {
        "metric": METRIC, "value": job_mpoints_s(world, n, ms), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": config_dict(n),
        "wall_s_timed_region": wall,
        "stage_ms": stage_ms,
        "incremental": incremental,
        "hbm_gbs_step": (b_topo + b_pts + b_atlas + b_apron) / (ms * 1e-3) / 1e9,
        "active_bricks": nb,
        "active_bricks_per_frame": nb_frames,
        "roofline": {"kernel": "k_splat_slab (cubic, density+velocity)", "bound": "hbm", "achieved": achieved,
                     "peak": peak, "peak_source": peak_src, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "algorithmic_bytes": splat_bytes, "launch_ms": splat_avg,
                     "bytes_model": "24 B per point (position, velocity) + P^3 * 20 B per active brick (density "
                                    "float + velocity float4), bricks averaged over the timed frames; traffic = "
                                    "ncu DRAM bytes per brick and per point of the same frames, times this run's"},
        "gpu_launches": int(launches),
        "clocks": clk,
        "e2e": {"value": world * n * e2e_steps / e2e_wall / 1e6, "unit": UNIT, "h2d_bytes_per_step": n * 24,
                "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
                "readback": "the level-1 node pool only: the density and velocity atlases stay in HBM, where "
                            "GVDB's consumers (raycast, gathers, compute) read them"} if e2e_steps else None,
    }
    if dist:
        dist.destroy_process_group()
    return out


def run_differentiable(dev, iters=5):
    """Differentiable workload: 1M points U[8,504)^3, w ~ U(0,1), per-point R ~ U(1,3),
    cubic density splat (forward) and its adjoint gvx_splat_backward (backward) with
    G = rho - rho*, rho* the splat of p + N(0, 0.5).  CUDA-event times of both
    kernels' calls on the grid's stream, after warm-up."""
    import numpy as np
    import torch

    import gvx
    import workloads

    pos, w, r = workloads.differentiable(n=1_000_000, seed=1)
    tgt = np.clip(pos + np.random.default_rng(2).normal(0, 0.5, pos.shape), 8.0, 504.0).astype(np.float32)
    n = len(pos)
    stream = torch.cuda.Stream(device=dev)
    g = gvx.Grid(dev.index)
    g.configure(LOGDIM)
    g.add_channel(0, gvx.T_FLOAT, 1)
    g.set_stream(stream.cuda_stream)
    both = torch.from_numpy(np.vstack([pos, tgt])).to(dev)
    pd, td = both[:n], both[n:]
    wd, rd = torch.from_numpy(w).to(dev), torch.from_numpy(r).to(dev)
    with torch.cuda.stream(stream):
        g.set_points(2 * n, both)
        g.rebuild_topology(2 * n, 3.0, mode=gvx.TOPO_FULL)
        g.update_atlas()
        g.set_points(n, td)
        g.set_point_attribs(weight=wd, radius=rd)
        g.splat(gvx.SPLAT_CUBIC, n, 1.0, chan_density=0)
        ptr, nbytes = g.channel_device_ptr(0)
        rho_t = torch.empty(nbytes // 4, dtype=torch.float32, device=dev)
        g.sync()
        rho_t.copy_(torch.from_numpy(g.read_channel(0).reshape(-1)))
        g.set_points(n, pd)
        g.set_point_attribs(weight=wd, radius=rd)
        gp = torch.empty((n, 3), dtype=torch.float32, device=dev)
        gw = torch.empty(n, dtype=torch.float32, device=dev)
        gr = torch.empty(n, dtype=torch.float32, device=dev)
        G = torch.empty_like(rho_t)
        fwd, bwd, bwd_rc = [], [], []
        for k in range(iters + 3):
            e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            e[0].record(stream)
            g.splat(gvx.SPLAT_CUBIC, n, 1.0, chan_density=0)
            e[1].record(stream)
            if k == 0:
                g.sync()
                G.copy_(torch.from_numpy(g.read_channel(0).reshape(-1)) - rho_t.cpu())
            g.splat_backward(gvx.SPLAT_CUBIC, n, 1.0, G, gp, gw, gr)
            e[2].record(stream)
            # the adjoint with the sorted-key permutation recomputed from the positions
            g.splat_backward(gvx.SPLAT_CUBIC, n, 1.0, G, gp, gw, gr, recompute=True)
            e[3].record(stream)
            torch.cuda.synchronize()
            if k >= 3:
                fwd.append(e[0].elapsed_time(e[1]))
                bwd.append(e[1].elapsed_time(e[2]))
                bwd_rc.append(e[2].elapsed_time(e[3]))
        bricks = g.info()["used_leaves"]
    g.close()
    f, b, brc = sum(fwd) / len(fwd), sum(bwd) / len(bwd), sum(bwd_rc) / len(bwd_rc)
    return {"workload": "differentiable: 1M points U[8,504)^3 in 512^3, w~U(0,1), R~U(1,3), cubic density; "
                        "G = rho - rho*, rho* = splat of p + N(0,0.5)",
            "points": n, "active_bricks": bricks, "fwd_ms": round(f, 4), "bwd_ms": round(b, 4),
            "fwd_plus_bwd_ms": round(f + b, 4), "bwd_over_fwd": round(b / f, 4),
            "bwd_ms_recomputed": round(brc, 4), "bwd_recomputed_over_fwd": round(brc / f, 4),
            "bwd_note": "bwd_ms reuses the forward's sorted-key grouping; bwd_ms_recomputed re-keys, re-sorts and "
                        "re-partitions the points from their positions before the adjoint"}


def run_batched(dev, iters=5):
    """Batched workload: 64 uneven clouds (N_i = floor(exp(U(ln 1e4, ln 2e6))), seed 7, Gaussian
    mixtures in 1024^3, w ~ U(0.5, 1.5)), one grid each, TRILINEAR density.  Times, on one stream,
    the per-cloud loop of gvx_splat calls against one gvx_batch_splat replaying its captured graph
    (autotuned on its first call); the topologies, atlases and groupings are built beforehand."""
    import numpy as np
    import torch

    import gvx
    import workloads

    cl = workloads.batched_clouds(count=64, seed=7)
    stream = torch.cuda.Stream(device=dev)
    grids, keep = [], []
    with torch.cuda.stream(stream):
        for p, w in cl:
            g = gvx.Grid(dev.index)  # its own stream while the topologies are built
            g.configure(LOGDIM)
            g.add_channel(0, gvx.T_FLOAT, 1)
            pd, wd = torch.from_numpy(p).to(dev), torch.from_numpy(w).to(dev)
            keep.append((pd, wd))
            g.set_points(len(p), pd)
            g.set_point_attribs(weight=wd)
            grids.append(g)
        # the topologies (full rebuild, UpdateAtlas, InsertPoints of every cloud): host-orchestrated
        # builds, wall-clock timed (three times, the last kept: a grid's second full build runs under
        # the first one's plan and grows its buffers to the plan's capacities), from one host thread
        # and from 16
        tb = gvx.Batch(dev.index)
        tb.set_grids(grids)
        topo_ms = {}
        for label, th in (("one_thread", 1), ("16_threads", 16), ("staged", 0)):
            for rep in range(3):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                tb.topology(1.0, threads=th)
                torch.cuda.synchronize()
                topo_ms[label] = round((time.perf_counter() - t0) * 1e3, 3)
        own = [torch.cuda.Stream(device=dev) for _ in grids]
        for g, s_ in zip(grids, own):
            g.set_stream(s_.cuda_stream)
        for g in grids:
            g.set_stream(stream.cuda_stream)
        b = gvx.Batch(dev.index)
        b.set_stream(stream.cuda_stream)
        b.set_grids(grids)
        b.splat(gvx.SPLAT_TRILINEAR, 1.0, graph=True, tune=True)  # tunes, captures
        b.splat(gvx.SPLAT_TRILINEAR, 1.0, graph=True)
        for g, (p, _) in zip(grids, cl):
            g.splat(gvx.SPLAT_TRILINEAR, len(p), 1.0)
        torch.cuda.synchronize()
        seq, bat = [], []
        for k in range(iters):
            e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            e[0].record(stream)
            for g, (p, _) in zip(grids, cl):
                g.splat(gvx.SPLAT_TRILINEAR, len(p), 1.0)
            e[1].record(stream)
            b.splat(gvx.SPLAT_TRILINEAR, 1.0, graph=True)
            e[2].record(stream)
            torch.cuda.synchronize()
            seq.append(e[0].elapsed_time(e[1]))
            bat.append(e[1].elapsed_time(e[2]))
        tun = b.tuning()
        bricks = sum(g.info()["used_leaves"] for g in grids)
        # end to end, topology + splat (+ aprons, fused): the per-cloud loop on one stream against
        # the staged batch topology on the grids' own streams and the batch splat's graph
        e2e_seq, e2e_bat = [], []
        for k in range(3):
            for g in grids:
                g.set_stream(stream.cuda_stream)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for g, (p, _) in zip(grids, cl):
                g.rebuild_topology(len(p), 1.0, mode=gvx.TOPO_FULL)
                g.update_atlas()
                g.insert_points(len(p))
                g.splat(gvx.SPLAT_TRILINEAR, len(p), 1.0)
            torch.cuda.synchronize()
            e2e_seq.append((time.perf_counter() - t0) * 1e3)
            for g, s_ in zip(grids, own):
                g.set_stream(s_.cuda_stream)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            tb.topology(1.0, threads=0)
            b.splat(gvx.SPLAT_TRILINEAR, 1.0, graph=True)
            torch.cuda.synchronize()
            e2e_bat.append((time.perf_counter() - t0) * 1e3)
        # whole frames through gvx_batch_frame: the first unplanned (staged topology, plans made),
        # the second planned without a graph, then every grid's planned build and the splat as one
        # captured CUDA graph, replayed (the grids on their own streams, forked in the graph)
        for g, s_ in zip(grids, own):
            g.set_stream(s_.cuda_stream)
        fb = gvx.Batch(dev.index)
        fb.set_stream(stream.cuda_stream)
        fb.set_grids(grids)
        frame_first = []
        for k in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fb.frame(1.0, gvx.SPLAT_TRILINEAR, 1.0)
            torch.cuda.synchronize()
            frame_first.append(((time.perf_counter() - t0) * 1e3, fb.frame_path()))
        frame_ms, frame_paths = [], set()
        for k in range(max(iters, 5)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fb.frame(1.0, gvx.SPLAT_TRILINEAR, 1.0)
            torch.cuda.synchronize()
            frame_ms.append((time.perf_counter() - t0) * 1e3)
            frame_paths.add(fb.frame_path())
        frame_launches = fb.kernel_launches()
        fb.close()
        tb.close()
    b.close()
    for g in grids:
        g.close()
    s_ms, b_ms = sum(seq) / len(seq), sum(bat) / len(bat)
    npts = int(sum(len(p) for p, _ in cl))
    return {"workload": "batched: 64 Gaussian-mixture clouds, N_i = floor(exp(U(ln 1e4, ln 2e6))) seed 7, "
                        "1024^3, TRILINEAR density, one grid per cloud",
            "clouds": len(cl), "points": npts, "active_bricks": int(bricks),
            "sequential_ms": round(s_ms, 4), "batched_graph_ms": round(b_ms, 4),
            "speedup": round(s_ms / b_ms, 3), "batched_mpoints_s": round(npts / (b_ms * 1e-3) / 1e6, 1),
            "tuning": tun,
            "topology_ms": topo_ms,
            "end_to_end_sequential_ms": round(min(e2e_seq), 3), "end_to_end_batched_ms": round(min(e2e_bat), 3),
            "end_to_end_speedup": round(min(e2e_seq) / min(e2e_bat), 3),
            "frame_ms": round(min(frame_ms), 3), "frame_ms_mean": round(sum(frame_ms) / len(frame_ms), 3),
            "frame_speedup": round(min(e2e_seq) / min(frame_ms), 3),
            "frame_paths": sorted(frame_paths),
            "frame_first_ms": [[round(t, 3), list(pth)] for t, pth in frame_first],
            "frame_batch_stream_launches": int(frame_launches),
            "scope": "speedup: the splat alone, per-cloud gvx_splat loop vs one batched launch replayed from its "
                     "captured graph (aprons fused). end_to_end: topology (full rebuild, UpdateAtlas, InsertPoints) "
                     "+ splat, wall clock: the per-cloud loop on one stream vs gvx_batch_topology staged from one "
                     "host thread (two host waits per grid, the grids' streams overlapping) + the batched graph. "
                     "topology_ms: gvx_batch_topology alone, per-grid calls from 1 or 16 host threads, or staged. "
                     "frame_ms: gvx_batch_frame, wall clock per frame once its graph is captured: every grid's "
                     "planned full rebuild, UpdateAtlas and InsertPoints (forked onto the grids' streams) and the "
                     "batched splat replayed as one CUDA graph, one host wait; frame_paths (path, grids rebuilt): "
                     "2 = graph replay; frame_first_ms: the unplanned, the first planned and the capturing frame"}


def run_batched_frames(dev, frames=3, graph=False, clouds=64, cloud_max=2_000_000):
    """The batched workload's clouds through gvx_batch_frame alone: one grid per cloud on its own
    stream, `frames` frames (the first unplanned, then planned; with graph, captured from the
    third on).  Wall clock per frame and the path each took (for launch lists: graph=False keeps
    every planned build's launches visible to a profiler as separate launches)."""
    import torch

    import gvx
    import workloads

    cl = workloads.batched_clouds(count=clouds, seed=7, nmax=cloud_max)
    stream = torch.cuda.Stream(device=dev)
    grids, keep, own = [], [], []
    with torch.cuda.stream(stream):
        for p, w in cl:
            g = gvx.Grid(dev.index)
            g.configure(LOGDIM)
            g.add_channel(0, gvx.T_FLOAT, 1)
            pd, wd = torch.from_numpy(p).to(dev), torch.from_numpy(w).to(dev)
            keep.append((pd, wd))
            g.set_points(len(p), pd)
            g.set_point_attribs(weight=wd)
            own.append(torch.cuda.Stream(device=dev))
            g.set_stream(own[-1].cuda_stream)
            grids.append(g)
        b = gvx.Batch(dev.index)
        b.set_stream(stream.cuda_stream)
        b.set_grids(grids)
        out = []
        for f in range(frames):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            b.frame(1.0, gvx.SPLAT_TRILINEAR, 1.0, graph=graph)
            torch.cuda.synchronize()
            out.append({"ms": round((time.perf_counter() - t0) * 1e3, 3), "path": list(b.frame_path())})
        bricks = sum(g.info()["used_leaves"] for g in grids)
        b.close()
    for g in grids:
        g.close()
    return {"workload": "%d batched clouds (N_i <= %d) through gvx_batch_frame" % (clouds, cloud_max),
            "graph": graph, "points": int(sum(len(p) for p, _ in cl)), "active_bricks": int(bricks), "frames": out}


def run_scatter_frame(dev, frames=3):
    """libgvx on the work of the reference arm's `reference_cuda` frame: the same 4M SPH frames
    (advected 1..3), full RebuildTopology (radius 2), UpdateAtlas, ClearChannel, InsertPoints +
    ScatterDensity (radius 2, 7-voxel stencil) and UpdateApron of the density channel.  Positions
    on the device; CUDA-event time per stage on the grid's stream, frame 0 twice as warm-up (the
    second build runs under the first one's plan and grows the buffers to its capacities)."""
    import torch

    import gvx
    import workloads

    pos0, vel = workloads.sph_slab(n=N_POINTS, seed=0, box=BOX)
    stream = torch.cuda.Stream(device=dev)
    g = gvx.Grid(dev.index)
    g.configure(LOGDIM)
    g.add_channel(0, gvx.T_FLOAT, 1)
    g.set_stream(stream.cuda_stream)
    names = ("topology", "update_atlas", "clear_channel", "insert_points_scatter_density", "update_apron")
    tot, stages = [], []
    with torch.cuda.stream(stream):
        for i, f in enumerate([0] + list(range(frames + 1))):
            pd = torch.from_numpy(workloads.advect(pos0, vel, DT * f)).to(dev)
            n = pd.shape[0]
            torch.cuda.synchronize()
            e = [torch.cuda.Event(enable_timing=True) for _ in range(len(names) + 1)]
            e[0].record(stream)
            g.set_points(n, pd)
            g.rebuild_topology(n, RADIUS, mode=gvx.TOPO_FULL)
            e[1].record(stream)
            g.update_atlas()
            e[2].record(stream)
            g.clear_channel(0)
            e[3].record(stream)
            g.insert_points(n)
            g.scatter_density(n, RADIUS)
            e[4].record(stream)
            g.update_apron(0, 0.0)
            e[5].record(stream)
            torch.cuda.synchronize()
            if i > 1:
                tot.append(e[0].elapsed_time(e[-1]))
                stages.append([e[k].elapsed_time(e[k + 1]) for k in range(len(names))])
        used = g.info()["used_leaves"]
    g.close()
    ms = sum(tot) / len(tot)
    return {"workload": "the reference arm's reference_cuda frame through libgvx: ScatterDensity (7-voxel "
                        "stencil, radius 2) + UpdateApron of density on the 4M SPH frames 1..3",
            "ms_per_frame": round(ms, 4), "mpoints_s": round(N_POINTS / (ms * 1e-3) / 1e6, 1),
            "active_bricks": int(used),
            "stage_ms": {k: round(sum(x[i] for x in stages) / len(stages), 4) for i, k in enumerate(names)}}


def run_point_cloud(dev, reps=5):
    """Point-cloud level set, the sequence gPointCloud runs per frame: RebuildTopology (radius 2r,
    full) + UpdateAtlas + ClearChannel + InsertPointsSubcell_FP16 (subcell 4, r) +
    GatherLevelSet_FP16 + UpdateApron(0, 3) + Compute(FUNC_SMOOTH, 0, 1, (1, 0, 0), apron, packed, 3),
    on the surface points of the 30 fusion frames taken as one cloud (r = 1).  Points on the device
    before timing; CUDA-event time per stage on the grid's stream, median of `reps` runs."""
    import numpy as np
    import torch

    import gvx
    import workloads

    pos = np.concatenate([p for p, _ in workloads.depth_fusion(frames=30, seed=3)])
    n = len(pos)
    pd = torch.from_numpy(pos).to(dev)
    stream = torch.cuda.Stream(device=dev)
    g = gvx.Grid(dev.index)
    g.configure(LOGDIM)
    g.add_channel(0, gvx.T_FLOAT, 1)
    g.set_stream(stream.cuda_stream)
    g.set_points(n, pd)
    names = ("topology", "subcell_fp16", "gather_levelset_fp16", "apron", "smooth")
    runs = []
    with torch.cuda.stream(stream):
        for r in range(reps + 2):
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(names) + 1)]
            ev[0].record(stream)
            g.rebuild_topology(n, 2.0, mode=gvx.TOPO_FULL)
            g.update_atlas()
            g.clear_channel(0)
            ev[1].record(stream)
            sc = g.insert_points_subcell_fp16(4, n, 1.0)
            ev[2].record(stream)
            g.gather_levelset_fp16(4, n, 1.0, sc, chan=0)
            ev[3].record(stream)
            g.update_apron(0, 3.0)
            ev[4].record(stream)
            g.compute(gvx.FUNC_SMOOTH, 0, 1, (1.0, 0.0, 0.0), update_apron=True, skip_over_aprons=True, boundval=3.0)
            ev[5].record(stream)
            torch.cuda.synchronize()
            if r >= 2:
                runs.append([ev[k].elapsed_time(ev[k + 1]) for k in range(len(names))])
        inf = g.info()
    g.close()
    med = np.median(np.asarray(runs), axis=0)
    total = float(med.sum())
    return {"workload": "point_cloud: the 30 fusion frames' surface points as one cloud (%d points, 2048^3); "
                        "RebuildTopology r=2 + UpdateAtlas + ClearChannel + InsertPointsSubcell_FP16(4, r=1) + "
                        "GatherLevelSet_FP16 + UpdateApron(0, 3) + Compute(FUNC_SMOOTH, 1 iteration)" % n,
            "points": n, "active_bricks": int(inf["used_leaves"]), "subcell_entries": int(sc),
            "stage_ms": {k: round(float(v), 4) for k, v in zip(names, med)}, "ms_per_frame": round(total, 4),
            "mpoints_s": round(n / (total * 1e-3) / 1e6, 1)}


def run_fusion(dev, frames=30):
    """Surface-fusion workload: 30 depth frames (640x480, f = 525) of an analytic
    scene in 2048^3, each AccumulateTopology (radius 1) + UpdateAtlas + InsertPoints +
    accumulating TRILINEAR splats of density (w = 1) and of confidence-weighted
    density, then UpdateApron of both.  Frames are on the device before timing;
    CUDA-event time per frame on the grid's stream."""
    import numpy as np
    import torch

    import gvx
    import workloads

    fr = [(torch.from_numpy(p).to(dev), torch.from_numpy(c).to(dev)) for p, c in
          workloads.depth_fusion(frames=frames, seed=3)]
    stream = torch.cuda.Stream(device=dev)
    g = gvx.Grid(dev.index)
    g.configure(LOGDIM)
    g.add_channel(0, gvx.T_FLOAT, 1)
    g.add_channel(1, gvx.T_FLOAT, 1)
    g.set_stream(stream.cuda_stream)
    ms, pts = [], 0
    names = ("topology", "update_atlas", "insert_points", "splat_density", "splat_confidence", "aprons")
    stages = []
    with torch.cuda.stream(stream):
        for pd, cd in fr:
            n = pd.shape[0]
            e = [torch.cuda.Event(enable_timing=True) for _ in range(len(names) + 1)]
            e[0].record(stream)
            g.set_points(n, pd)
            g.set_point_attribs()
            g.rebuild_topology(n, 1.0, mode=gvx.TOPO_ACCUMULATE)
            e[1].record(stream)
            g.update_atlas()
            e[2].record(stream)
            g.insert_points(n)
            e[3].record(stream)
            g.splat(gvx.SPLAT_TRILINEAR, n, 1.0, chan_density=0, accum=True)
            e[4].record(stream)
            g.set_point_attribs(weight=cd)
            g.splat(gvx.SPLAT_TRILINEAR, n, 1.0, chan_density=1, accum=True)
            e[5].record(stream)
            g.update_apron(0, 0.0)
            g.update_apron(1, 0.0)
            e[6].record(stream)
            torch.cuda.synchronize()
            ms.append(e[0].elapsed_time(e[-1]))
            stages.append([e[k].elapsed_time(e[k + 1]) for k in range(len(names))])
            pts += n
        inf = g.info()
    g.close()
    steady = ms[2:]  # the first two AccumulateTopology calls are full rebuilds of a growing tree
    st_mean = [sum(x[k] for x in stages[2:]) / len(stages[2:]) for k in range(len(names))]
    return {"workload": "fusion: %d depth frames 640x480 (f=525) of 8 spheres + 2 planes in 2048^3, N(0,0.5) "
                        "noise; AccumulateTopology r=1, TRILINEAR density + confidence-weighted density (accum), "
                        "UpdateApron x2" % frames,
            "frames": frames, "points": int(pts), "active_bricks": int(inf["used_leaves"]),
            "ms_per_frame": round(sum(ms) / len(ms), 4), "ms_per_frame_incremental": round(sum(steady) / len(steady), 4),
            "stage_ms_incremental": {k: round(v, 4) for k, v in zip(names, st_mean)},
            "mpoints_s": round(pts / (sum(ms) * 1e-3) / 1e6, 1)}


def reference_cuda(frames=3):
    """The reference's own CUDA kernels (PTX compiled from its sources) driven by the
    restated host orchestration of oracle/ref_harness.cu, on the same SPH frame: full
    RebuildTopology (radius 2), UpdateAtlas, ClearChannel, InsertPoints +
    ScatterDensity (radius 2: the reference has no cubic splat) and UpdateApron of the
    density channel.  Wall-clock time per frame (the reference synchronises on the host
    many times per rebuild), positions already on the device."""
    sys.path.insert(0, ORACLE)
    try:
        import ref_harness as rh
        import torch
    except Exception as e:  # noqa: BLE001
        return {"unavailable": "harness not importable: %s" % e}
    if not rh.available() or not torch.cuda.is_available():
        return {"unavailable": "reference kernels not built or no GPU"}
    import workloads

    try:
        rh.load()
    except Exception as e:  # noqa: BLE001
        return {"unavailable": "harness not loadable: %s" % e}
    pos0, vel = workloads.sph_slab(n=N_POINTS, seed=0, box=BOX)
    r = rh.RefGrid(LOGDIM)
    r.add_channel(0, 3)
    names = ("topology", "update_atlas", "clear_channel", "insert_points_scatter_density", "update_apron")
    times, stages = [], []
    for f in range(frames + 1):
        r.set_points(workloads.advect(pos0, vel, DT * f))
        torch.cuda.synchronize()
        t = [time.perf_counter()]
        st = r.rebuild(RADIUS, mode=1)
        if st != 0:
            return {"unavailable": "reference rebuild failed: status %d" % st}
        torch.cuda.synchronize()
        t.append(time.perf_counter())
        r.update_atlas()
        torch.cuda.synchronize()
        t.append(time.perf_counter())
        r.clear_channel(0)
        torch.cuda.synchronize()
        t.append(time.perf_counter())
        r.scatter(RADIUS)
        torch.cuda.synchronize()
        t.append(time.perf_counter())
        r.update_apron(0, 0.0)
        torch.cuda.synchronize()
        t.append(time.perf_counter())
        if f > 0:
            times.append(t[-1] - t[0])
            stages.append([t[k + 1] - t[k] for k in range(len(names))])
    used = r.used_leaves()
    r.close()
    ms = 1e3 * sum(times) / len(times)
    st_ms = {k: round(1e3 * sum(x[i] for x in stages) / len(stages), 3) for i, k in enumerate(names)}
    return {"value": N_POINTS / (ms * 1e-3) / 1e6, "unit": UNIT, "ms_per_frame": ms, "frames": frames,
            "active_bricks": used, "stage_ms": st_ms,
            "path": "reference kernels (cuda_gvdb_module.cu as PTX, --use_fast_math) + restated host "
                    "orchestration: GetBoundingBox with thrust min/max on the device, thrust sort/unique; "
                    "ScatterDensity + UpdateApron of density; wall clock per stage with a device synchronisation "
                    "after each (the reference synchronises inside every stage)"}


def host_topology(frames=2):
    """The reference's host-side topology path (ActivateSpace per point, then
    FinishTopology; gvdb_volume_gvdb.cpp:2766-2855, 1579-1593) as the oracle
    restates it, on the full 4M-point frame: single-threaded, as the reference's
    host code is.  Points with a negative coordinate are left out, as the GPU path
    drops them."""
    import numpy as np
    import workloads

    sys.path.insert(0, ORACLE)
    import oracle as O

    pos0, vel = workloads.sph_slab(n=N_POINTS, seed=0, box=BOX)
    times, npts, leaves = [], 0, 0
    for f in range(frames):
        pos = workloads.advect(pos0, vel, DT * f)
        pos = pos[(pos >= 0.0).all(axis=1)]
        t0 = time.perf_counter()
        t = O.CpuTree(LOGDIM)
        t.activate(pos)
        leaves = int(t.lib.orc_cpu_tree_count(t.h, 0))
        times.append(time.perf_counter() - t0)
        npts = pos.shape[0]
        del t
    s = sum(times) / len(times)
    return {"value": npts / s / 1e6, "unit": UNIT, "ms_per_frame": 1e3 * s, "points": int(npts), "leaves": leaves,
            "frames": frames, "cores": 1, "host_cores": os.cpu_count(), "kind": "port",
            "path": "host ActivateSpace per point into the host pools (the oracle's restatement), one thread"}


def run_reference(args, world, rank):
    if rank != 0:
        return None
    workers = max(1, os.cpu_count() or 1)
    pool = cpu_pool(workers)
    jobs = [(SAMPLE_FRAC, 1000 + i) for i in range(workers)]
    for _ in range(args.warmup):
        pool.map(_cpu_sample, jobs)
    times, pts = [], 0
    for k in range(args.steps):
        t0 = time.perf_counter()
        r = pool.map(_cpu_sample, [(SAMPLE_FRAC, 2000 + k * workers + i) for i in range(workers)])
        times.append(time.perf_counter() - t0)
        pts = sum(x[0] for x in r)
    pool.close()
    ms = 1e3 * sum(times) / len(times)
    v = pts / (ms * 1e-3) / 1e6
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "config": config_dict(),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": workers, "kind": "port",
                             "sample": "%d independent sub-boxes of 1/128 of the slab per step (%d points, same "
                                       "density), one per host core" % (workers, pts)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "host_topology": host_topology() if not args.no_extras else None,
            "reference_cuda": reference_cuda() if not args.no_extras else None}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--points", type=int, default=0, help="smaller runs for profiling (same density)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the differentiable, batched, fusion and point-cloud workloads")
    ap.add_argument("--clouds", type=int, default=64, help="batched_frames: clouds (profiling a smaller case)")
    ap.add_argument("--cloud-max", type=int, default=2_000_000, help="batched_frames: largest cloud's points")
    ap.add_argument("--extra", choices=["differentiable", "batched", "batched_frames", "fusion", "point_cloud",
                                        "scatter_frame"],
                    help="run only this workload and print its JSON (for profiling)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.extra:
        import torch

        fn = {"differentiable": run_differentiable, "batched": run_batched, "batched_frames": run_batched_frames,
              "fusion": run_fusion, "point_cloud": run_point_cloud, "scatter_frame": run_scatter_frame}[args.extra]
        kw = {"clouds": args.clouds, "cloud_max": args.cloud_max} if args.extra == "batched_frames" else {}
        print(json.dumps(fn(torch.device("cuda", 0), **kw)))
        return
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference":
        out = run_reference(args, world, rank)
        if out is not None:
            print(json.dumps(out))
        return
    pool = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        pool = cpu_pool(1)  # spawned before the first CUDA call
    out = run_ours(args, rank, world, pool)
    if rank == 0 and world == 1 and not args.no_extras:
        import torch

        out["differentiable"] = run_differentiable(torch.device("cuda", 0))
        out["batched"] = run_batched(torch.device("cuda", 0))
        out["fusion"] = run_fusion(torch.device("cuda", 0))
        out["point_cloud"] = run_point_cloud(torch.device("cuda", 0))
        out["scatter_frame"] = run_scatter_frame(torch.device("cuda", 0))
    if rank == 0:
        if pool is not None:
            out["cpu_baseline"] = cpu_baseline(pool)
            pool.close()
        print(json.dumps(out))


if __name__ == "__main__":
    main()
