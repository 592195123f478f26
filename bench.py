"""Benchmark of the Livre rendering hot path on GB300.

Workload (the plain path at scale): a 2048^3 uint8 blob volume (256 blobs,
noise +-8) in 64^3 bricks with a 1-voxel overlap (6 LOD levels), rendered at
1920x1080 along a 64-frame orbit at 2.5x the volume diagonal, 256-entry RGBA
float32 transfer function with 4 Gaussian peaks, LOD threshold 2 px, step
0.5 voxel of the finest rendered level, trilinear sampling, early ray
termination at alpha 0.99.

One step = one frame of one view: LOD selection, residency (brick streaming
on a miss), leaf grid, ray cast. `value` is frames/s with every brick the
orbit needs already resident in HBM, timed per frame with CUDA events on the
rendering stream after an L2 flush (a 256 MiB write). `e2e` is the same
metric through the public C ABI with host buffers: the brick pool starts
empty, bricks stream host->device from a page-locked host store on a miss,
and each frame is converted to RGBA8 and copied back to host memory.

Frames: the timed steps visit orbit frames spread evenly over the whole
64-frame orbit (step i renders frame floor(i * 64 / steps)).

`--impl reference` times the CPU restatement of the reference path (the
reference itself needs an OpenGL context and cannot run here): per step one
whole frame, the FP32 LOD selection single-threaded as on the reference
render thread plus the FP64 ray cast of every row on every host thread,
with the host's CPU model and thread count stated.

Extra keys of the default line: `plain256` (the CPU-runnable plain workload:
256^3 uint8 in 32^3 bricks, 512x512), `parity` (device frames of both plain
workloads against the oracle on this host: per-ray mode, shader-order mode),
`batched`, `served`, `outofcore` (the 128-frame fly-through).
"""
import argparse
import json
import os
import platform
import subprocess
import sys
import threading
import time

# The serving mode keeps a few hundred CUDA streams busy (batches in flight,
# each with its view streams at several priority levels). With CUDA's default
# of 8 hardware work queues, an admission selection's first kernel can wait
# behind a ray cast queued on another stream that shares its queue; 32 (the
# maximum) spreads them out. Read when CUDA initialises, so set before any
# CUDA call of this process.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    "plain2048": dict(workload="plain_2048c_u8_64b_1080p_orbit64", voxels=2048, block=64,
                      overlap=1, n_blobs=256, noise=8, seed=2, width=1920, height=1080,
                      frames=64, sse=2.0, early=0.99, tf_entries=256, tf_seed=4,
                      pool_gib=24),
    "plain256": dict(workload="plain_256c_u8_32b_512sq_orbit64", voxels=256, block=32,
                     overlap=1, n_blobs=16, noise=0, seed=1, width=512, height=512,
                     frames=64, sse=1.0, early=0.999, tf_entries=256, tf_seed=None,
                     pool_gib=1),
}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=512)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--config", default="plain2048", choices=sorted(CONFIGS))
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--pool-gib", type=int, default=None,
                   help="brick pool size (default: the config's)")
    p.add_argument("--ooc-voxels", type=int, default=8192,
                   help="out-of-core volume edge (a smaller one for ncu captures)")
    p.add_argument("--ooc-pool-gib", type=int, default=64)
    p.add_argument("--ooc-host-frames", type=int, default=3,
                   help="host-generated frames after frame 0 in the outofcore_host mode")
    p.add_argument("--ooc-frames", type=int, default=128,
                   help="frames of the 128-frame out-of-core fly-through to render")
    p.add_argument("--modes", default="plain,plain256,parity,launches,batched,served,outofcore",
                   help="comma list: plain (headline), plain256 (the 256^3 / 512^2 plain "
                        "workload), parity (device frames against the oracle), launches "
                        "(ray-cast time of every lv_render launch shape), batched (64 "
                        "uneven views in one persistent launch), served (Poisson request "
                        "stream), outofcore (8192^3 u16 fly-through through a 64 GiB pool), "
                        "outofcore_host (the same with host-generated bricks; not in the "
                        "default list: host generation takes tens of seconds per frame)")
    p.add_argument("--cpu-frames", type=int, default=2,
                   help="whole frames the CPU baseline of the default line ray casts")
    p.add_argument("--serve-seconds", type=float, default=3.0,
                   help="request stream length per rate below 1000 req/s (half of it "
                        "from 1000 req/s: the saturated rates)")
    p.add_argument("--serve-rates", type=lambda t: [int(x) for x in t.split(",")],
                   default=[200, 250, 300, 350, 400, 450, 500, 550, 600, 2000],
                   help="Poisson request rates (req/s)")
    p.add_argument("--slo-ms", type=float, default=150.0,
                   help="p99 latency objective of the serving capacity figure")
    return p.parse_args()




def transfer_function(cfg):
    import livre_gb300 as lv
    if cfg["tf_seed"] is None:
        return lv.linear_ramp_tf(cfg["tf_entries"])
    return lv.gaussian_peaks_tf(cfg["tf_entries"], seed=cfg["tf_seed"])


def cameras(cfg, world_size):
    import livre_gb300 as lv
    return [lv.orbit_camera(k, cfg["frames"], world_size, cfg["width"], cfg["height"])
            for k in range(cfg["frames"])]


# ------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        import statistics
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


# ------------------------------------------------------ CPU baseline
def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.machine()


def orbit_frame(i, steps, n_frames):
    """Orbit frame of step i: steps spread evenly over the whole orbit."""
    return (i * n_frames) // max(steps, 1) % n_frames


class CpuFrames:
    """The oracle (CPU restatement of the reference path) on one workload:
    bricks generated once per node, then per frame the FP32 LOD selection on
    one thread (the reference's render thread) and the FP64 ray cast on every
    host thread."""

    def __init__(self, cfg):
        from oracle import pyoracle as O
        self.O, self.cfg = O, cfg
        self.ovol = O.volume(cfg["voxels"], cfg["block"], cfg["overlap"])
        self.bp = O.blob_params(cfg["n_blobs"], cfg["seed"], cfg["noise"], 1)
        self.tf = transfer_function(cfg)
        self.bricks = {}

    def camera(self, k):
        import livre_gb300 as lv
        c = self.cfg
        return lv.orbit_camera(k, c["frames"], tuple(self.ovol.world_size), c["width"],
                               c["height"])

    def inputs(self, k):
        """(mv, proj, visible ids, seconds of the selection)."""
        mv, proj = self.camera(k)
        t0 = time.perf_counter()
        ids, _ = self.O.select_visible(self.ovol, mv, proj, self.cfg["height"], self.cfg["sse"])
        return mv, proj, ids, time.perf_counter() - t0

    def brick_stack(self, ids):
        import concurrent.futures as cf
        import numpy as np
        miss = [int(i) for i in ids if int(i) not in self.bricks]
        with cf.ThreadPoolExecutor(os.cpu_count()) as ex:
            for i, b in zip(miss, ex.map(lambda n: self.O.blob_brick(self.ovol, self.bp, n),
                                         miss)):
                self.bricks[i] = b
        return np.stack([self.bricks[int(i)] for i in ids])

    def view(self, mv, proj, ids, early=None):
        c = self.cfg
        max_level = max(int(i) & 0xF for i in ids)
        n_samples = (2 * c["voxels"]) >> (self.ovol.depth - 1 - max_level)
        return self.O.make_view(mv, proj, c["width"], c["height"], n_samples,
                                early_exit=c["early"] if early is None else early)

    def frame(self, k, rows=None, mode=0, diagnostics=False):
        """Renders frame k: (result of the oracle's raycast, selection s,
        ray-cast s)."""
        mv, proj, ids, t_lod = self.inputs(k)
        bricks = self.brick_stack(ids)
        view = self.view(mv, proj, ids)
        t0 = time.perf_counter()
        res = self.O.raycast(self.ovol, 1, ids, bricks, self.tf, view, rows=rows, mode=mode,
                             diagnostics=diagnostics)
        return res, t_lod, time.perf_counter() - t0


def cpu_sample(cfg, frames):
    """Whole frames of the oracle: (seconds per frame, selection s per frame,
    frames rendered)."""
    cf_ = CpuFrames(cfg)
    tot, lod = 0.0, 0.0
    for k in frames:
        _, t_lod, t_ray = cf_.frame(k)
        tot += t_lod + t_ray
        lod += t_lod
    return tot / len(frames), lod / len(frames)


def workload_config(cfg, world):
    """The `config` object of both arms' JSON lines."""
    return {"workload": cfg["workload"], "volume": "%d^3 u8" % cfg["voxels"],
            "brick": "%d^3 + overlap %d" % (cfg["block"], cfg["overlap"]),
            "viewport": "%dx%d" % (cfg["width"], cfg["height"]), "frames": cfg["frames"],
            "lod_px": cfg["sse"], "step": "0.5 voxel of finest rendered level",
            "filter": "trilinear", "early_exit": cfg["early"],
            "tf": "%d-entry RGBA f32" % cfg["tf_entries"],
            "mode": "plain per-view launch (synchronous residency)",
            "l2": "flushed between frames (256 MiB write)",
            "parallelism": "replicas" if world > 1 else "single"}


def reference_arm(args, cfg):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import build as ob
    ob.build()
    cf_ = CpuFrames(cfg)
    H = cfg["height"]
    times, lods, samples = [], [], 0
    wall0 = time.perf_counter()
    for s_ in range(args.warmup + args.steps):
        timed = s_ >= args.warmup
        k = orbit_frame(s_ - args.warmup, args.steps, cfg["frames"]) if timed else \
            orbit_frame(s_, args.warmup, cfg["frames"])
        (img, ns), t_lod, t_ray = cf_.frame(k)
        if timed:
            times.append(t_lod + t_ray)
            lods.append(t_lod)
            samples += ns
    wall = time.perf_counter() - wall0
    ms = 1000.0 * sum(times) / len(times)
    fps = 1000.0 / ms
    cores = os.cpu_count()
    model = cpu_model()
    line = {"impl": "reference", "metric": "frames/s", "value": fps, "unit": "frames/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(cfg, 1),
            "note": "CPU restatement of the reference path (the reference renders through "
                    "OpenGL, unavailable on this box); every step one whole frame",
            "samples_per_s": samples / (sum(times)),
            "lod_select_ms_mean": 1000.0 * sum(lods) / len(lods),
            "wall_s": wall,
            "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": cores,
                             "cpu_model": model, "kind": "port",
                             "sample": "per step one whole %dx%d orbit frame (frames spread "
                                       "evenly over the orbit): FP32 LOD selection (1 thread) "
                                       "+ FP64 ray cast of all %d rows (%d threads)"
                                       % (cfg["width"], H, H, cores)},
            "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------- batched / served modes
BATCH_VIEWPORTS = [(256, 256), (512, 512), (1024, 768), (1920, 1080), (2048, 2048)]


def batched_mode(ctx, args, dev, seed=7):
    """64 views of uneven viewports over 4 resident volumes: plain per-view
    lv_render launches vs one lv_batch_render (persistent kernel, CUDA graph,
    autotuned tiles)."""
    import numpy as np
    import torch
    import livre_gb300 as lv
    rng = np.random.default_rng(seed)
    specs = [(512, lv.DT_UINT8, 64), (1024, lv.DT_UINT8, 160), (2048, lv.DT_UINT8, 512),
             (1024, lv.DT_UINT16, 128)]
    vols = []
    for k, (n, dt, blobs) in enumerate(specs):
        vi = lv.VolumeInformation(n, 64, 1, dtype=dt)
        vols.append((ctx.blob_volume(vi, blobs, 100 + k, noise=4), vi))
    tfs = [ctx.transfer_function(lv.gaussian_peaks_tf(256, seed=s_)) for s_ in range(4)]
    items = []
    for i in range(64):
        v, vi = vols[i % 4]
        W, H = BATCH_VIEWPORTS[int(rng.integers(0, len(BATCH_VIEWPORTS)))]
        mv, proj = lv.orbit_camera(int(rng.integers(0, 64)), 64, vi.world_size, W, H,
                                   radius_scale=float(rng.uniform(1.2, 2.5)))
        desc = ctx.render_desc(mv, proj, W, H, sse=float(rng.uniform(0.5, 4.0)),
                               early_exit=0.99, step_policy=lv.STEP_HALF_VOXEL)
        out = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
        items.append((v, tfs[i % 4], desc, out))
    for v, t, d, o in items:  # residency: every brick of every view
        ctx.render(v, t, d, o)
    ctx.last_stats()
    # plain: one lv_render per view
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * len(items))]
    reps = min(4, max(2, args.steps // 16))
    plain_ms, plain_done = [], []
    for r in range(reps + 1):
        for i, (v, t, d, o) in enumerate(items):
            ev[2 * i].record()
            ctx.render(v, t, d, o)
            ev[2 * i + 1].record()
        torch.cuda.synchronize()
        if r:
            plain_ms.extend(ev[2 * i].elapsed_time(ev[2 * i + 1]) for i in range(len(items)))
            # the 64 views submitted together: each one's completion time
            plain_done.extend(ev[0].elapsed_time(ev[2 * i + 1]) for i in range(len(items)))
    plain_ms = np.array(plain_ms)
    # batched: autotune, then graph replays
    batch = lv.Batch(ctx)
    t0 = time.time()
    cfg = batch.autotune(items, reps=2)
    tune_s = time.time() - t0
    table = batch.autotune_results()
    queue_names = {lv.QUEUE_CTA_TILES: "persistent_cta_tiles",
                   lv.QUEUE_VIEW_KERNELS: "per_view_kernels",
                   lv.QUEUE_WARP_REFILL: "persistent_warp_refill"}
    n = len(items)
    pixels = float(sum(d.width * d.height for _, _, d, _ in items))

    def timed(config, rounds):
        batch.set_config(**{k: config[k] for k in ("tile_w", "tile_h", "ctas_per_sm",
                                                   "tf_shared", "use_graph", "queue",
                                                   "samples_per_check", "order",
                                                   "lookahead")})
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ms, ray, dev_ms, host_ms = [], [], [], []
        cap0, rep0, _ = batch.graph_stats()
        for r in range(args.warmup + rounds):
            e0.record()
            h0 = time.perf_counter()
            batch.render(items)
            h1 = time.perf_counter()
            e1.record()
            st, total, ray_ms = batch.stats(n)
            if r >= args.warmup:
                ms.append(e0.elapsed_time(e1))
                ray.append(ray_ms)
                dev_ms.append(total)
                host_ms.append(1e3 * (h1 - h0))
        cap1, rep1, _ = batch.graph_stats()
        ms = np.array(ms)
        return {"queue": queue_names.get(config["queue"], str(config["queue"])),
                "config": config, "frames_per_s": 1000.0 * n / ms.mean(),
                "batch_ms_p50": float(np.percentile(ms, 50)),
                "batch_ms_p99": float(np.percentile(ms, 99)),
                "raycast_ms_mean": float(np.mean(ray)),
                # the batch's device time (its first to its last event) and the
                # host time of the lv_batch_render call that enqueued it
                "device_batch_ms_mean": float(np.mean(dev_ms)),
                "host_render_call_ms_mean": float(np.mean(host_ms)),
                "samples_per_batch": float(sum(x["n_samples"] for x in st)),
                "gpu_launches_per_batch": int(st[0]["n_launches"]),
                "graph_captures": int(cap1 - cap0), "graph_replays": int(rep1 - rep0),
                "graph_used": bool(rep1 > rep0)}

    reps = min(4, max(2, args.steps // 16))
    best = timed(cfg, reps * 4)
    # the best persistent-kernel configuration (one launch per voxel-type
    # group, replayed as a CUDA graph), timed the same way whatever won
    pers = [(c, ms) for c, ms in table if c["queue"] == lv.QUEUE_CTA_TILES]
    persistent = timed(min(pers, key=lambda x: x[1])[0], reps * 4) if pers else None
    out = {"views": n, "volumes": "512^3 u8, 1024^3 u8, 2048^3 u8, 1024^3 u16 (64^3 bricks)",
           "pixels_per_batch": pixels,
           "plain": {"frames_per_s": 1000.0 * len(plain_ms) / plain_ms.sum(),
                     "p50_ms": float(np.percentile(plain_ms, 50)),
                     "p99_ms": float(np.percentile(plain_ms, 99)),
                     # latency of a view when the set is submitted at once
                     # (the batched views all complete at the batch's end)
                     "completion_p50_ms": float(np.percentile(plain_done, 50)),
                     "completion_p99_ms": float(np.percentile(plain_done, 99))},
           "batched": best, "persistent": persistent, "autotune_s": tune_s,
           # every configuration the autotuner ran: queue kind, tile, order,
           # TF staging, look-ahead, refill interval -> mean ray-cast ms
           "autotune_table": [[queue_names.get(c["queue"], c["queue"]), c["tile_w"], c["tile_h"],
                               c["order"], c["tf_shared"], c["lookahead"],
                               c["samples_per_check"], round(ms, 3)] for c, ms in table]}
    out["speedup_frames_per_s"] = best["frames_per_s"] / out["plain"]["frames_per_s"]
    batch.close()
    for v, _ in vols:
        v.close()
    for t in tfs:
        t.close()
    return out


def served_mode(ctx, args, dev, seed=11):
    """Poisson request streams over 8 resident volumes: continuous-batching
    server vs the plain per-request server, p50/p99 latency and frames/s."""
    import numpy as np
    import torch
    import livre_gb300 as lv
    rng = np.random.default_rng(seed)
    # (edge, type, generator): blob volumes and two fBm volumes (device fBm)
    specs = [(256, lv.DT_UINT8, "blob"), (512, lv.DT_UINT8, "blob"), (512, lv.DT_UINT16, "fbm"),
             (1024, lv.DT_UINT8, "blob"), (1024, lv.DT_UINT16, "blob"),
             (2048, lv.DT_UINT8, "fbm"), (2048, lv.DT_UINT16, "blob"), (4096, lv.DT_UINT8, "blob")]
    vols = []
    for k, (n, dt, gen) in enumerate(specs):
        vi = lv.VolumeInformation(n, 64, 1, dtype=dt)
        if gen == "fbm":
            vols.append((ctx.fbm_volume(vi, 300 + k, octaves=6, frequency=8.0), vi))
        else:
            vols.append((ctx.blob_volume(vi, int(rng.integers(64, 513)), 300 + k, noise=4), vi))
    tfs = [ctx.transfer_function(lv.gaussian_peaks_tf(256, seed=100 + k)) for k in range(16)]
    viewports = [(512, 512), (1920, 1080), (3840, 2160)]

    def make_request():
        v, vi = vols[int(rng.integers(0, len(vols)))]
        W, H = viewports[int(rng.integers(0, 3))]
        mv, proj = lv.orbit_camera(int(rng.integers(0, 256)), 256, vi.world_size, W, H,
                                   radius_scale=float(rng.uniform(1.2, 2.5)))
        d = ctx.render_desc(mv, proj, W, H, sse=float(rng.uniform(0.5, 4.0)), early_exit=0.99)
        return v, tfs[int(rng.integers(0, 16))], d

    # Output frames: a ring of 8 buffers per viewport size (timing only; the
    # images of requests sharing a buffer are not inspected here, the server
    # tests check each result against lv_render).
    rings, ring_pos = {}, {}

    def take(W, H):
        ring = rings.setdefault((W, H), [torch.empty((H, W, 4), dtype=torch.float32,
                                                     device=dev) for _ in range(8)])
        k = ring_pos.get((W, H), 0)
        ring_pos[(W, H)] = (k + 1) % len(ring)
        return ring[k]

    # One request sequence and one sequence of unit-rate exponential gaps for
    # every rate and both modes (common random numbers): a rate's stream is a
    # prefix of the requests arriving at gaps / rate, so the two modes and
    # neighbouring rates see the same mix of volumes, viewports and LODs.
    counts = {rate: max(64, int(rate * args.serve_seconds * (0.5 if rate >= 1000 else 1.0)))
              for rate in args.serve_rates}
    pool = [make_request() for _ in range(max(counts.values()))]
    gaps = rng.exponential(1.0, len(pool))

    def run(mode, rate, reqs):
        srv = lv.Server(ctx, mode=mode, max_batch=64, max_pixels=16 << 20)
        # warm-up burst (graph captures, per-batch buffers), not timed
        for tk in [srv.submit(v, t, d, take(d.width, d.height)) for v, t, d in reqs[:64]]:
            srv.wait(tk, 600000)
        prof0 = srv.profile()
        arrivals = np.cumsum(gaps[:len(reqs)]) / rate
        tickets, outs = [], []
        t0 = time.perf_counter()
        for (v, t, d), at in zip(reqs, arrivals):
            now = time.perf_counter() - t0
            if at > now:
                time.sleep(at - now)
            o = take(d.width, d.height)
            tickets.append(srv.submit(v, t, d, o))
            outs.append(o)
        res = [srv.wait(tk, 600000) for tk in tickets]
        wall = time.perf_counter() - t0
        prof = srv.profile()
        srv.close()
        lat = np.array([r["latency_ms"] for r in res])
        queued = np.array([r["queue_ms"] for r in res])
        return {"rate_req_s": rate, "requests": len(reqs),
                "frames_per_s": len(reqs) / wall, "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)),
                "mean_batch": float(np.mean([r["batch_size"] for r in res])),
                "queue_p50_ms": float(np.percentile(queued, 50)),
                "queue_p99_ms": float(np.percentile(queued, 99)),
                "service_p50_ms": float(np.percentile(lat - queued, 50)),
                "service_p99_ms": float(np.percentile(lat - queued, 99)),
                "failed": int(sum(r["status"] != 0 for r in res)),
                "profile": {k: (round(v - prof0[k], 2) if isinstance(v, float)
                                else v - prof0[k]) for k, v in prof.items()}}

    # residency warm-up: one pass of requests through the plain path
    warm = [make_request() for _ in range(64)]
    for v, t, d in warm:
        ctx.render(v, t, d, take(d.width, d.height))
    ctx.last_stats()
    out = {"volumes": "8 volumes 256^3..4096^3 u8/u16, 64^3 bricks: 6 blob, 2 fBm "
                      "(512^3 u16, 2048^3 u8)",
           "pool_gib": args.pool_gib or 96, "brick_layout": "compact",
           "slo_p99_ms": args.slo_ms, "rates": []}
    for rate in args.serve_rates:
        reqs = pool[:counts[rate]]
        # every brick the stream needs made resident first, so neither mode
        # pays (or is spared) streaming the other mode already did
        for v, t, d in reqs:
            ctx.render(v, t, d, take(d.width, d.height))
        ctx.last_stats()
        served = run(0, rate, reqs)
        plain = run(1, rate, reqs)
        out["rates"].append({"served": served, "plain": plain})
    # capacity at the latency objective: the highest offered rate whose p99
    # stays within it, and the frames/s delivered there
    for mode in ("served", "plain"):
        ok = [r[mode] for r in out["rates"] if r[mode]["p99_ms"] <= args.slo_ms]
        top = max(ok, key=lambda r: r["rate_req_s"]) if ok else None
        out["capacity_%s" % mode] = ({"rate_req_s": top["rate_req_s"],
                                      "frames_per_s": top["frames_per_s"],
                                      "p99_ms": top["p99_ms"]} if top else None)
    # the same at several objectives, the rate interpolated linearly between
    # the last offered rate within the objective and the first beyond it
    def rate_at(mode, slo):
        pts = sorted((r[mode]["rate_req_s"], r[mode]["p99_ms"]) for r in out["rates"])
        prev = None
        for rate, p99 in pts:
            if p99 > slo:
                if prev is None:
                    return None
                r0, p0 = prev
                return round(r0 + (slo - p0) / (p99 - p0) * (rate - r0), 1)
            prev = (rate, p99)
        return prev[0] if prev else None

    out["rate_at_p99_slo"] = [{"slo_ms": slo, "served_req_s": rate_at("served", slo),
                               "plain_req_s": rate_at("plain", slo)}
                              for slo in (75, 100, 125, 150, 200, 300)]
    for v, _ in vols:
        v.close()
    for t in tfs:
        t.close()
    return out


def fly_through(k, n, W, H):
    """Camera of frame k of an n-frame straight fly-through entering the
    volume (world box +-0.5) near one corner and leaving near the opposite
    one; near plane 0.01."""
    import numpy as np
    import livre_gb300 as lv
    t = k / max(n - 1, 1)
    a, b = np.array([-0.45, -0.3, -0.8]), np.array([0.35, 0.25, 0.55])
    eye = a + (b - a) * t
    mv = lv.look_at(eye, eye + (b - a) / np.linalg.norm(b - a), (0.0, 1.0, 0.0))
    return mv, lv.perspective(45.0, W / H, 0.01, 15.0)


def outofcore_mode(local, args, dev):
    """8192^3 uint16 fBm volume (1 TiB logical) in 128^3 bricks streamed into
    a 64 GiB pool with LRU eviction, 1920x1080, LOD threshold 1 px,
    4096-entry transfer function: the first frames of a 128-frame
    fly-through, every brick generated when it first misses."""
    import numpy as np
    import torch
    import livre_gb300 as lv
    W, H, n_path = 1920, 1080, 128
    ctx = lv.Context(local, pool_bytes=args.ooc_pool_gib << 30)
    vi = lv.VolumeInformation(args.ooc_voxels, 128, 1, dtype=lv.DT_UINT16)
    vol = ctx.fbm_volume(vi, 3, octaves=6, frequency=8.0, placement=lv.FBM_DEVICE)
    tf = ctx.transfer_function(lv.gaussian_peaks_tf(4096, seed=12))
    out = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
    frames = max(2, min(args.ooc_frames, n_path))
    rows = []
    for k in range(frames):
        mv, proj = fly_through(k, n_path, W, H)
        d = ctx.render_desc(mv, proj, W, H, sse=1.0, step_policy=lv.STEP_REFERENCE,
                            early_exit=0.999)
        t0 = time.perf_counter()
        ctx.render(vol, tf, d, out)
        st = ctx.last_stats()  # synchronises
        rows.append((time.perf_counter() - t0, st))
    timed = rows[1:]  # frame 0 fills the empty pool
    # the same frames again from a purged pool, back to back with no wait
    # between frames: each frame's misses stream beside the previous
    # frame's ray cast
    ctx.purge()
    mv, proj = fly_through(0, n_path, W, H)
    d0 = ctx.render_desc(mv, proj, W, H, sse=1.0, step_policy=lv.STEP_REFERENCE,
                         early_exit=0.999)
    ctx.render(vol, tf, d0, out)
    ctx.last_stats()
    descs = []
    for k in range(1, frames):
        mv, proj = fly_through(k, n_path, W, H)
        descs.append(ctx.render_desc(mv, proj, W, H, sse=1.0, step_policy=lv.STEP_REFERENCE,
                                     early_exit=0.999))
    tot0 = ctx.totals()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for d in descs:
        ctx.render(vol, tf, d, out)
    ctx.last_stats()  # waits for the last frame; raises on a device error
    torch.cuda.synchronize()
    pipe_s = time.perf_counter() - t0
    tot1 = ctx.totals()
    wall = np.array([r[0] for r in timed]) * 1e3
    n = args.ooc_voxels
    res = {
        "workload": "outofcore_%dc_u16_128b_1080p_flythrough128" % n,
        "volume": "%d^3 u16 fBm (6 octaves), 128^3 bricks + overlap 1, %.0f GiB logical"
                  % (n, 2.0 * n ** 3 / 2 ** 30),
        "generator": "device fBm, bit-identical to the host generator a data-source "
                     "plugin runs (host generation: ~0.3 s per brick on 16 cores)",
        "pool_gib": args.ooc_pool_gib, "frames": frames, "timed_frames": len(timed),
        "frames_per_s": float(len(timed) / (wall.sum() / 1e3)),
        "p50_ms": float(np.percentile(wall, 50)), "p99_ms": float(np.percentile(wall, 99)),
        "first_frame_ms": rows[0][0] * 1e3,
        "visible_bricks_mean": float(np.mean([r[1]["n_visible"] for r in timed])),
        "passes_max": int(max(r[1]["n_passes"] for r in rows)),
        "streamed_bricks_per_frame": float(np.mean([r[1]["n_uploaded"] for r in timed])),
        "streamed_gb_per_frame": float(np.mean([r[1]["n_uploaded"] for r in timed])
                                       * vi.brick_bytes / 1e9),
        "samples_per_s": float(sum(r[1]["n_samples"] for r in timed) / (wall.sum() / 1e3)),
        "raycast_ms_mean": float(np.mean([r[1]["raycast_ms"] for r in timed])),
        "select_ms_mean": float(np.mean([r[1]["select_ms"] for r in timed])),
        "stream_ms_mean": float(np.mean([r[1]["stream_ms"] for r in timed])),
        # frames 1.. back to back (no host wait between frames), from a purged pool
        "back_to_back_frames_per_s": len(descs) / pipe_s,
        "back_to_back_streamed_bricks_per_frame":
            (tot1["bricks_uploaded"] - tot0["bricks_uploaded"]) / len(descs),
    }
    if not args.no_cpu_baseline:
        # the CPU restatement of the reference's LOD selection (one thread, as
        # on the reference's render thread) on frame 1's camera
        from oracle import pyoracle as O
        ovol = O.volume(args.ooc_voxels, 128, 1)
        mv, proj = fly_through(1, n_path, W, H)
        t0 = time.perf_counter()
        ids, visited = O.select_visible(ovol, mv, proj, H, 1.0)
        res["cpu_lod_select_ms"] = 1e3 * (time.perf_counter() - t0)
        res["cpu_lod_visited"] = int(visited)
        res["gpu_lod_visible_equal"] = int(len(ids)) == int(rows[1][1]["n_visible"])
    vol.close()
    tf.close()
    ctx.close()
    return res


# ------------------------------------------------------ launch sweep
def launch_sweep(ctx, vol, tf, descs, dev, frames=64):
    """Mean ray-cast time of the headline workload's orbit (every brick
    resident, no L2 flush) for each lv_render launch shape, then the default
    launch restored: {name: ms}."""
    import numpy as np
    import torch
    import livre_gb300 as lv
    default = ctx.render_launch()
    G, T, Q, W, R = (lv.LAUNCH_GRID, lv.LAUNCH_TILE_GRID, lv.LAUNCH_TILE_QUEUE,
                     lv.LAUNCH_WARP_TILES, lv.LAUNCH_WARP_REFILL)
    LF, RA = lv.ORDER_LONGEST_FIRST, lv.ORDER_RASTER
    shapes = [("tile_grid 8x16 longest-first look-ahead", T, 8, 16, 0, LF, 1),
              ("tile_grid 8x16 longest-first", T, 8, 16, 0, LF, 0),
              ("tile_grid 8x8 longest-first look-ahead", T, 8, 8, 0, LF, 1),
              ("tile_grid 8x4 longest-first look-ahead", T, 8, 4, 0, LF, 1),
              ("tile_grid 16x8 longest-first look-ahead", T, 16, 8, 0, LF, 1),
              ("tile_grid 16x16 longest-first look-ahead", T, 16, 16, 0, LF, 1),
              ("tile_grid 32x8 longest-first look-ahead", T, 32, 8, 0, LF, 1),
              ("tile_grid 8x16 raster look-ahead", T, 8, 16, 0, RA, 1),
              ("grid 8x16 (hardware-scheduled blocks) look-ahead", G, 8, 16, 0, RA, 1),
              ("warp_tiles 8x4 longest-first look-ahead", W, 8, 4, 0, LF, 1),
              ("tile_queue 8x16 longest-first look-ahead", Q, 8, 16, 0, LF, 1),
              ("warp_refill 8x4 every 8 samples", R, 8, 4, 8, RA, 0)]
    out = {}
    out_t = torch.empty((descs[0].height, descs[0].width, 4), dtype=torch.float32, device=dev)
    for name, kind, tw, th, spc, order, la in shapes:
        ctx.set_render_launch(kind, tw, th, spc, order, la)
        for d in descs[:4]:
            ctx.render(vol, tf, d, out_t)
            ctx.last_stats()
        ray = []
        for k in range(frames):
            ctx.render(vol, tf, descs[k % len(descs)], out_t)
            ray.append(ctx.last_stats()["raycast_ms"])
        out[name] = round(float(np.mean(ray)), 4)
    ctx.set_render_launch(default["kind"], default["tile_w"], default["tile_h"],
                          default["samples_per_check"], default["order"], default["lookahead"])
    return out


# ------------------------------------------------ plain 256^3 and parity
def plain256_mode(local, args, dev, steps=64):
    """The CPU-runnable plain workload (256^3 uint8, 32^3 bricks, 16 blobs,
    512x512, linear ramp, LOD 1 px, early termination 0.999): the 64 orbit
    frames with every brick resident, CUDA events per frame, L2 flushed."""
    import numpy as np
    import torch
    import livre_gb300 as lv
    cfg = CONFIGS["plain256"]
    W, H = cfg["width"], cfg["height"]
    ctx = lv.Context(local, pool_bytes=cfg["pool_gib"] << 30)
    vi = lv.VolumeInformation(cfg["voxels"], cfg["block"], cfg["overlap"])
    vol = ctx.blob_volume(vi, cfg["n_blobs"], cfg["seed"], cfg["noise"])
    tf = ctx.transfer_function(transfer_function(cfg))
    descs = [ctx.render_desc(mv, pr, W, H, sse=cfg["sse"], early_exit=cfg["early"],
                             step_policy=lv.STEP_HALF_VOXEL) for mv, pr in
             cameras(cfg, vi.world_size)]
    out = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    for d in descs + descs[: args.warmup]:
        ctx.render(vol, tf, d, out)
        ctx.last_stats()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    stats = []
    for i in range(steps):
        flush.fill_(i & 0xFF)
        ev[i][0].record(stream)
        ctx.render(vol, tf, descs[orbit_frame(i, steps, cfg["frames"])], out)
        ev[i][1].record(stream)
        stats.append(ctx.last_stats())
    torch.cuda.synchronize()
    ms = np.array([a.elapsed_time(b) for a, b in ev])
    ray = np.array([st["raycast_ms"] for st in stats])
    ns = np.array([st["n_samples"] for st in stats], np.float64)
    alg = ns * 8 + W * H * 16
    res = {"workload": cfg["workload"], "frames": steps, "frames_per_s": 1000.0 * steps / ms.sum(),
           "p50_ms": float(np.percentile(ms, 50)), "p99_ms": float(np.percentile(ms, 99)),
           "raycast_ms_mean": float(ray.mean()),
           "select_ms_mean": float(np.mean([st["select_ms"] for st in stats])),
           "samples_per_s": float(ns.sum() / (ms.sum() / 1000.0)),
           "visible_bricks_mean": float(np.mean([st["n_visible"] for st in stats])),
           "raycast_gbs": float(alg.sum() / (ray.sum() / 1000.0) / 1e9)}
    vol.close()
    tf.close()
    ctx.close()
    return res


def parity_mode(ctx, vol, tf, cfg, args, dev):
    """Device frames of both plain workloads against the oracle on this host:
    max per-channel error against the per-ray mode (the parity bar, 1/255),
    and against the shader-order mode (brick-by-brick, brick-centre distance
    order) the pixels over 1/255 and the sample-count difference."""
    import numpy as np
    import torch
    import livre_gb300 as lv
    res = {"tolerance": 1.0 / 255.0}

    def compare(cpu, img, k, st, rows=None, shader=True):
        (ref, ns), _, _ = cpu.frame(k, rows=rows)
        sl = slice(None) if rows is None else slice(rows[0], rows[1])
        r = {"frame": k, "rows": list(rows) if rows else "all",
             "max_err_255": float(np.abs(img[sl] - ref[sl]).max() * 255.0),
             "device_samples": int(st["n_samples"]) if rows is None else None,
             "oracle_samples": int(ns)}
        # the same oracle with its trilinear weights rounded to 1/256, the
        # fixed-point weights of a texture unit's linear filter: what bricks
        # in 3D textures with hardware filtering would cost in parity
        (q, _), _, _ = cpu.frame(k, rows=rows, mode=0x200)
        dq = np.abs(q[sl] - ref[sl]).max(axis=2)
        r["texture_filter_weights"] = {"max_err_255": float(dq.max() * 255.0),
                                       "pixels_over_1_255": int((dq > 1.0 / 255.0).sum())}
        if shader:
            (shd, nss, c_shd, flags), _, _ = cpu.frame(k, rows=rows, mode=1, diagnostics=True)
            d = np.abs(img[sl] - shd[sl]).max(axis=2)
            r["shader_order"] = {"max_err_255": float(d.max() * 255.0),
                                 "pixels_over_1_255": int((d > 1.0 / 255.0).sum()),
                                 "pixels": int(d.size), "samples": int(nss),
                                 "inverted_pixels": int(((flags[sl] & 2) != 0).sum())}
        return r

    # workload 1 (256^3 / 512^2), full frames
    c1 = CONFIGS["plain256"]
    c1ctx = lv.Context(dev.index or 0, pool_bytes=c1["pool_gib"] << 30)
    vi = lv.VolumeInformation(c1["voxels"], c1["block"], c1["overlap"])
    v1 = c1ctx.blob_volume(vi, c1["n_blobs"], c1["seed"], c1["noise"])
    t1 = c1ctx.transfer_function(transfer_function(c1))
    cpu1 = CpuFrames(c1)
    res["plain256"] = []
    for k in (0, 32):
        mv, pr = cpu1.camera(k)
        d = c1ctx.render_desc(mv, pr, c1["width"], c1["height"], sse=c1["sse"],
                              early_exit=c1["early"], step_policy=lv.STEP_HALF_VOXEL)
        img = c1ctx.render(v1, t1, d).cpu().numpy()
        res["plain256"].append(compare(cpu1, img, k, c1ctx.last_stats()))
    v1.close()
    t1.close()
    c1ctx.close()
    # workload 2 (the headline), row bands of two frames
    cpu2 = CpuFrames(cfg)
    res[args.config] = []
    for k in (0, 40):
        mv, pr = cpu2.camera(k)
        d = ctx.render_desc(mv, pr, cfg["width"], cfg["height"], sse=cfg["sse"],
                            early_exit=cfg["early"], step_policy=lv.STEP_HALF_VOXEL)
        img = ctx.render(vol, tf, d).cpu().numpy()
        st = ctx.last_stats()
        for r0 in (cfg["height"] * 3 // 8, cfg["height"] // 2):
            res[args.config].append(compare(cpu2, img, k, st, rows=(r0, r0 + 16)))
    res["max_err_255"] = max(r["max_err_255"] for key in ("plain256", args.config)
                             for r in res[key])
    res["texture_filter_weights_max_err_255"] = max(
        r["texture_filter_weights"]["max_err_255"] for key in ("plain256", args.config)
        for r in res[key])
    return res


def outofcore_host_mode(local, args, dev):
    """The out-of-core fly-through with its bricks generated on the host, as
    the configuration states: a callback volume (a data-source plugin's
    getData) served from a brick store that a producer thread fills ahead of
    the path with the host fBm generator (lv_fbm_brick, every host thread),
    one frame ahead of the frame being rendered. Frame 0 (about 7 000 bricks)
    is filled from the device generator, which produces the same bytes, so
    the timed frames 1.. measure the host-fed steady state."""
    import ctypes
    import queue as queue_
    import numpy as np
    import torch
    import livre_gb300 as lv
    W, H, n_path = 1920, 1080, 128
    frames = max(2, args.ooc_host_frames + 1)
    ctx = lv.Context(local, pool_bytes=args.ooc_pool_gib << 30)
    vi = lv.VolumeInformation(args.ooc_voxels, 128, 1, dtype=lv.DT_UINT16)
    seed = 3
    store, ready = {}, threading.Condition()
    stats = {"host_bricks": 0, "host_s": 0.0, "waits": 0, "served": 0}

    def put(nid, data):
        with ready:
            store[nid] = data
            ready.notify_all()

    def get_data(node_id, dst, nbytes):
        with ready:
            if node_id not in store:
                stats["waits"] += 1
                # the producer is on it; a brick it never schedules is
                # generated here after a bounded wait
                ready.wait_for(lambda: node_id in store, timeout=60.0)
            data = store.get(node_id)
            stats["served"] += 1
        if data is None:
            data = lv.fbm_brick(vi, node_id, seed, n_threads=1)
        ctypes.memmove(dst, data.ctypes.data, nbytes)
        return True

    vol = ctx.callback_volume(vi, get_data)
    vol.fetch_threads = 0
    tf = ctx.transfer_function(lv.gaussian_peaks_tf(4096, seed=12))
    out = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
    descs, visible = [], []
    for k in range(frames):
        mv, proj = fly_through(k, n_path, W, H)
        descs.append(ctx.render_desc(mv, proj, W, H, sse=1.0, step_policy=lv.STEP_REFERENCE,
                                     early_exit=0.999))
        ids, _ = ctx.select_visible(vi, mv, proj, H, 1.0)
        visible.append([int(i) for i in ids])
    # frame 0: device generator (same bytes), into the store
    first = visible[0]
    for a in range(0, len(first), 256):
        chunk = first[a:a + 256]
        dev_bricks = ctx.fbm_bricks(vi, chunk, seed).cpu().numpy()
        for nid, b in zip(chunk, dev_bricks):
            put(nid, b)
    jobs = queue_.Queue()

    def producer():
        while True:
            k = jobs.get()
            if k is None:
                return
            for nid in visible[k]:
                with ready:
                    have = nid in store
                if have:
                    continue
                t0 = time.perf_counter()
                b = lv.fbm_brick(vi, nid, seed, n_threads=0)
                stats["host_s"] += time.perf_counter() - t0
                stats["host_bricks"] += 1
                put(nid, b)

    th = threading.Thread(target=producer, daemon=True)
    th.start()
    jobs.put(1)  # prefetch one frame ahead of the path
    rows = []
    for k in range(frames):
        t0 = time.perf_counter()
        ctx.render(vol, tf, descs[k], out)
        st = ctx.last_stats()
        rows.append((time.perf_counter() - t0, st))
        if k + 2 < frames:
            jobs.put(k + 2)
    jobs.put(None)
    th.join()
    timed = rows[1:]
    wall = np.array([r[0] for r in timed])
    res = {"workload": "outofcore_%dc_u16_128b_1080p_flythrough128_hostgen" % args.ooc_voxels,
           "generator": "host fBm (lv_fbm_brick, %d threads) for frames 1..%d, prefetched one "
                        "frame ahead of the path; frame 0 from the device generator (same "
                        "bytes)" % (os.cpu_count(), frames - 1),
           "timed_frames": len(timed), "frames_per_s": float(len(timed) / wall.sum()),
           "frame_s": [round(float(x), 3) for x in wall],
           "streamed_bricks_per_frame": float(np.mean([r[1]["n_uploaded"] for r in timed])),
           "host_generated_bricks": stats["host_bricks"],
           "host_bricks_per_s": stats["host_bricks"] / max(stats["host_s"], 1e-9),
           "fetch_waits_for_producer": stats["waits"],
           "raycast_ms_mean": float(np.mean([r[1]["raycast_ms"] for r in timed]))}
    vol.close()
    tf.close()
    ctx.close()
    return res


# ------------------------------------------------------------ GPU arm
def gb300_arm(args, cfg):
    import numpy as np
    import torch
    import livre_gb300 as lv
    from livre_gb300 import build as nb
    from livre_gb300 import replicas

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    nb.build()
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    W, H = cfg["width"], cfg["height"]

    ctx = lv.Context(local, pool_bytes=(args.pool_gib or cfg["pool_gib"]) << 30)
    vi = lv.VolumeInformation(cfg["voxels"], cfg["block"], cfg["overlap"])
    t0 = time.time()
    vol = ctx.blob_volume(vi, cfg["n_blobs"], cfg["seed"], cfg["noise"], placement=lv.BLOB_HOST)
    gen_s = time.time() - t0
    tf = ctx.transfer_function(transfer_function(cfg))
    cams = cameras(cfg, vi.world_size)
    descs = [ctx.render_desc(mv, pr, W, H, sse=cfg["sse"], early_exit=cfg["early"],
                             step_policy=lv.STEP_HALF_VOXEL, filt=lv.FILTER_TRILINEAR,
                             synchronous=True) for mv, pr in cams]
    my_frames = replicas.shard(cfg["frames"], rank, world)
    out = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
    out8 = torch.empty((H, W, 4), dtype=torch.uint8, device=dev)
    host8 = torch.empty((H, W, 4), dtype=torch.uint8).pin_memory()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def frame_of(i):
        """Frame of timed step i: spread evenly over this rank's frames."""
        return my_frames[orbit_frame(i, args.steps, len(my_frames))]

    # ---- e2e: cold pool, bricks streamed from the host store, RGBA8 back.
    # Each frame's RGBA8 copy to the host runs on a copy stream while the
    # next frame renders (two RGBA8 buffers); the clock stops once the last
    # copy has landed.
    for i in range(args.warmup):
        ctx.render(vol, tf, descs[frame_of(i)], out)
        ctx.last_stats()
    ctx.purge()
    copy_stream = torch.cuda.Stream(dev)
    out8s = [out8, torch.empty_like(out8)]
    host8s = [host8, torch.empty_like(host8).pin_memory()]
    copied = [None, None]
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    tot0 = ctx.totals()
    t1 = time.perf_counter()
    for i in range(args.steps):
        b = i & 1
        if copied[b] is not None:
            copied[b].synchronize()  # the copy of frame i - 2 has landed
        ctx.render(vol, tf, descs[frame_of(i)], out)
        ctx.to_rgba8(out, out8s[b])
        ready = torch.cuda.Event()
        ready.record(stream)
        copy_stream.wait_event(ready)
        with torch.cuda.stream(copy_stream):
            host8s[b].copy_(out8s[b], non_blocking=True)
            copied[b] = torch.cuda.Event()
            copied[b].record(copy_stream)
    copy_stream.synchronize()
    e2e_total = time.perf_counter() - t1
    tot1 = ctx.totals()
    h2d = tot1["bytes_uploaded"] - tot0["bytes_uploaded"]
    launches_e2e = tot1["launches"] - tot0["launches"] + args.steps  # + RGBA8 conversions
    ctx.last_stats()  # raises if a frame reported a device error

    # ---- value: every brick of the orbit resident, L2 flushed between frames
    for k in my_frames:
        ctx.render(vol, tf, descs[k], out)
    ctx.last_stats()
    for i in range(args.warmup):
        ctx.render(vol, tf, descs[frame_of(i)], out)
        ctx.last_stats()
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    stats = []
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    with ClockSampler(local) as clocks:
        wall0 = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(i & 0xFF)
            ev0[i].record(stream)
            ctx.render(vol, tf, descs[frame_of(i)], out)
            ev1[i].record(stream)
            stats.append(ctx.last_stats())
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    if dist:
        dist.barrier()
    frame_ms = np.array([a.elapsed_time(b) for a, b in zip(ev0, ev1)])
    total_ms = float(frame_ms.sum())
    total_ms, e2e_total = replicas.max_over_ranks([total_ms, e2e_total], dist, dev)
    if rank != 0:
        return
    value = replicas.job_rate(args.steps, world, total_ms / 1000.0)
    ray_ms = np.array([s["raycast_ms"] for s in stats])
    n_samples = np.array([s["n_samples"] for s in stats], dtype=np.float64)
    bpv = vi.bytes_per_voxel
    alg_bytes = n_samples * 8 * bpv + W * H * 16
    achieved = float(alg_bytes.sum() / (ray_ms.sum() / 1000.0) / 1e9)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    line = {
        "metric": "frames/s", "value": value, "unit": "frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": workload_config(cfg, world),
        "p50_ms": float(np.percentile(frame_ms, 50)), "p99_ms": float(np.percentile(frame_ms, 99)),
        "samples_per_s": float(n_samples.sum() / (total_ms / 1000.0)),
        "raycast_ms_mean": float(ray_ms.mean()),
        "select_ms_mean": float(np.mean([s["select_ms"] for s in stats])),
        "wall_s": wall, "volume_generation_s": gen_s,
        "gpu_launches": int(sum(s["n_launches"] for s in stats)),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "traffic": None,
                     "traffic_note": "not yet captured with the voxel-quad brick layout; the "
                                     "last ncu capture of this launch (voxel pairs, 2 bytes "
                                     "per voxel) read 37.11 MB and wrote 2.35 MB: the visible "
                                     "bricks once, the 8-byte-per-sample gather served by "
                                     "L1/L2",
                     "algorithmic_bytes_per_launch": float(alg_bytes.mean()),
                     "kernel": "raycast_tiles_kernel<u8,trilinear>",
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6800"},
        "e2e": {"value": replicas.job_rate(args.steps, world, e2e_total), "unit": "frames/s",
                "h2d_bytes_per_step": int(h2d / args.steps),
                "d2h_bytes_per_step": W * H * 4,
                "note": "pool purged before the timed steps; bricks streamed from pinned host "
                        "memory; RGBA8 frame copied to host every step on a copy stream "
                        "overlapping the next frame; wall clock over all steps"},
        "e2e_gpu_launches": launches_e2e,
        "clocks": clocks.summary(),
        "visible_bricks_mean": float(np.mean([s["n_visible"] for s in stats])),
        "samples_per_ray": int(stats[-1]["samples_per_ray"]),
    }
    modes = set(args.modes.split(","))
    if "batched" in modes:
        bctx = lv.Context(local, pool_bytes=32 << 30)
        line["batched"] = batched_mode(bctx, args, dev)
        bctx.close()
    if "served" in modes:
        # the serving mix (8 volumes up to 4096^3 sharing 96 GiB) is sized for
        # one voxel per byte: with voxel pairs its uint8 working sets outgrow
        # the pool; served and plain requests share this context's layout
        sctx = lv.Context(local, pool_bytes=96 << 30, brick_layout=lv.BRICKS_COMPACT)
        line["served"] = served_mode(sctx, args, dev)
        sctx.close()
    if "outofcore" in modes:
        line["outofcore"] = outofcore_mode(local, args, dev)
    if "outofcore_host" in modes:
        line["outofcore_host"] = outofcore_host_mode(local, args, dev)
    if "launches" in modes:
        line["launch_sweep_raycast_ms"] = launch_sweep(ctx, vol, tf, descs, dev)
    if "plain256" in modes:
        line["plain256"] = plain256_mode(local, args, dev)
    if "parity" in modes:
        line["parity"] = parity_mode(ctx, vol, tf, cfg, args, dev)
    if world == 1 and not args.no_cpu_baseline:
        ks = [orbit_frame(j, args.cpu_frames, cfg["frames"]) for j in range(args.cpu_frames)]
        sec, t_lod = cpu_sample(cfg, ks)
        line["cpu_baseline"] = {"value": 1.0 / sec, "unit": "frames/s", "cores": os.cpu_count(),
                                "cpu_model": cpu_model(), "kind": "port",
                                "lod_select_ms": 1e3 * t_lod,
                                "sample": "orbit frames %s, whole %dx%d frames: FP32 LOD "
                                          "selection (1 thread) + FP64 ray cast of every row "
                                          "(%d threads), %.1f s per frame"
                                          % (ks, W, H, os.cpu_count(), sec)}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    cfg = CONFIGS[args.config]
    if args.impl == "reference":
        reference_arm(args, cfg)
    else:
        gb300_arm(args, cfg)


if __name__ == "__main__":
    main()
