#!/usr/bin/env python
"""Training-throughput benchmark of the SuperNormal hot path on GB300.

Workload (the reference-equivalent GPU configuration): a displaced torus
(R=0.5, r=0.2, amplitude 0.02, frequency 20) seen by 20 views of 612x512 on an
elevated ring; hash grid 16 levels x 2 features, 2^19 entries per level, base
resolution 16, scale 1.447; SDF MLP 35 -> 64 -> 16; 128^3 occupancy grid
(threshold 0.1, updated every 8 iterations with the post-warm-up cell
sampling); marching step 2/1024; 2048 patches of 3x3 per iteration; FP32;
all 16 levels active (the most expensive bandwidth of the schedule).  Data
are synthetic (no dataset is shipped).  A step is one full training
iteration: marching, culling, patch expansion, field forward, render + loss +
adjoint, field backward, learning-rate schedule and Adam, plus the amortised
occupancy update.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision fp32|mixed] [--eager] [--serve small|full|off] [--quality]

The timed region replays each iteration as a CUDA graph whose captured copies
carry the stage events (per-stage times and the roofline's kernel durations
come from those events; --eager times eager launches instead).  The
end-to-end figure feeds every iteration from pinned host memory through the
trainer's prefetcher and reads its loss back.  N > 1 runs as independent
replicas (one process per GPU via torchrun; the path has no exchange step),
value = all ranks' rays / max rank time.
--impl reference times the reference's CPU implementation of the path (the
float64 restatement in oracle/, the reference having no CPU path of its own)
on host cores over a bounded, proportional sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402
import torch  # noqa: E402

# The reference's own published training speed: about 50 s for 5000 iterations
# of 2048 3x3 patches on an RTX 4090 (README.md:60), i.e. 1.84 M rays/s end to end.
REFERENCE_RAYS_PER_S = 5000 * 2048 * 9 / 50.0
METRIC = "train_rays_per_s"
UNIT = "rays/s"
ENC = dict(otype="HashGrid", n_levels=16, n_features_per_level=2, log2_hashmap_size=19,
           base_resolution=16, per_level_scale=1.447)
WORKLOAD = "patch-NeuS training iteration, displaced torus 20x612x512, hashgrid L16 F2 T2^19, 128^3 grid, dt=2/1024"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--batch", type=int, default=2048)
    p.add_argument("--views", type=int, default=20)
    p.add_argument("--height", type=int, default=512)
    p.add_argument("--width", type=int, default=612)
    p.add_argument("--pretrain", type=int, default=200, help="untimed iterations before warm-up")
    p.add_argument("--cpu-sample-patches", type=int, default=8)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-clocks", action="store_true")
    p.add_argument("--precision", choices=["fp32", "mixed"], default="fp32",
                   help="mixed: FP16 hash-table copy and one-pass TF32 MLP products (config 3's path)")
    p.add_argument("--eager", action="store_true",
                   help="time eager launches instead of CUDA-graph replays of each iteration")
    p.add_argument("--no-encoding-cache", action="store_true",
                   help="field backward recomputes the encoding instead of reading the forward's")
    p.add_argument("--serve", choices=["small", "full", "off"], default="small",
                   help="serving-loop trace after the training measurement (p50/p99 latency)")
    p.add_argument("--quality", action="store_true",
                   help="instead of the throughput run: FP32 vs mixed precision reconstruction quality "
                        "on the sphere scene (angular error, mask IoU, Chamfer / F@0.01)")
    p.add_argument("--quality-iters", type=int, default=1000)
    return p.parse_args()


# ---------------------------------------------------------------------------
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(local)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, enabled: bool):
        self.proc = None
        self.gpu = gpu_index
        if enabled:
            try:
                self.proc = subprocess.Popen(
                    ["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.Q}",
                     "--format=csv,noheader,nounits", "-lms", "200"],
                    stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            except OSError:
                self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
def build_workload(args, device, seed):
    from supernormal_gb300 import scenes
    from supernormal_gb300.fields import SDFNetwork, SingleVarianceNetwork
    from supernormal_gb300.trainer import FusedTrainer, TrainConfig

    torch.manual_seed(seed)
    scene = scenes.displaced_torus(0.5, 0.2, 0.02, 20.0)
    rig = scenes.ring_cameras(args.views, args.height, args.width, radius=3.0, elevation_deg=30.0,
                              fov_deg=40.0)
    net = SDFNetwork(3, 16, 64, 1, skip_in=(-1,), bias=0.5, encoding_config=ENC,
                     input_concat=True).to(device)
    var = SingleVarianceNetwork(0.5).to(device)
    cfg = TrainConfig(batch_size=args.batch, step_size=2.0 / 1024, occ_update_freq=8,
                      occ_threshold=0.1, increase_bandwidth_every=0, end_iter=5000, seed=seed,
                      encoding_cache=not getattr(args, "no_encoding_cache", False),
                      precision=getattr(args, "precision", "fp32"))
    tr = FusedTrainer(net, var, cfg, device=device)
    net.bindwidth = ENC["n_levels"]
    return scene, rig, net, var, tr


def run_ours(args, world, rank, local):
    from supernormal_gb300 import scenes
    from supernormal_gb300._lib import lib
    from supernormal_gb300.trainer import GraphStep, HostPrefetcher

    dev = torch.device("cuda", local)
    scene, rig, net, var, tr = build_workload(args, dev, seed=1234 + rank)
    ds = scenes.SyntheticDataset(scene, rig, dev)
    g = torch.Generator(device=dev).manual_seed(99 + rank)
    pool = [ds.gen_random_patches(args.batch, generator=g) for _ in range(16)]
    # warm state: occupancy warm-up from the initial field, a short pre-training
    tr.occupancy_update(0)
    for i in range(args.pretrain):
        tr.train_step(*pool[i % len(pool)])
    tr.iter_step = max(tr.iter_step, tr.cfg.occ_warmup_steps)   # post-warm-up occupancy regime
    # iterations as CUDA-graph replays carrying the stage events (captured
    # before the warm-up), or eager launches with --eager
    gs = None if args.eager else GraphStep(tr, profile=True)
    if gs is not None:
        gs.prepare()
    for i in range(args.warmup):
        if gs is not None:
            gs.step(pool[i % len(pool)])
        else:
            tr.train_step(*pool[i % len(pool)])
    torch.cuda.synchronize()
    tr.check_status()
    if gs is not None:
        gs.flush()
        gs.stage_marks.clear()
        gs.points.clear()

    # ---------------- device-resident timed region ----------------
    K = args.steps
    if gs is None:
        tr.profile = True
        tr.marks.clear()
        tr.q_hist.clear()
    clocks = ClockSampler(local, not args.no_clocks and rank == 0)
    launches0 = gs.launches if gs is not None else lib().sn_kernel_launches()
    barrier(world)
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed")      # profiler filter: the timed steps only
    start.record()
    for i in range(K):
        if gs is not None:
            gs.step(pool[i % len(pool)])
        else:
            tr.train_step(*pool[i % len(pool)])
    end.record()
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    ms = start.elapsed_time(end)
    tr.check_status()
    if gs is not None:
        gs.flush()
        launches = gs.launches - launches0
        stages = stage_times([m for step in gs.stage_marks for m in step])
        q = np.asarray(gs.points, dtype=np.float64)
        samples = np.asarray(gs.samples, dtype=np.float64)
    else:
        samples = None
        launches = lib().sn_kernel_launches() - launches0
        stages = stage_times(tr.marks)
        q = torch.cat(tr.q_hist).double().cpu().numpy() if tr.q_hist else None
        tr.profile = False
    ms_max = max_over_ranks(ms, world)
    rays = args.batch * tr.P * K * world
    value = rays / (ms_max / 1e3)

    # ---------------- end-to-end through host buffers ----------------
    host = [tuple(t.cpu().pin_memory() for t in b) for b in pool[:8]]
    loss_host = torch.empty((5,), dtype=torch.float32).pin_memory()
    h2d = sum(t.numel() * t.element_size() for t in host[0])
    d2h = loss_host.numel() * loss_host.element_size()
    pf = HostPrefetcher(tr, host[0], graph=None if args.eager else GraphStep(tr))
    if pf.graph is not None:
        pf.graph.prepare()
        for i in range(3):              # replays of the fresh captures, untimed
            pf.graph.step(pool[i % len(pool)])
    barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    pf.put(host[0])                # every step's batch is copied inside the timed region
    for i in range(K):
        loss = pf.step(host[(i + 1) % len(host)] if i + 1 < K else None)
        loss_host.copy_(loss, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    barrier(world)
    e2e_ms = max_over_ranks(e0.elapsed_time(e1), world)
    e2e_value = rays / (e2e_ms / 1e3)

    if rank != 0:
        return None
    peaks, peak_kind = load_peaks()
    rl = roofline(stages, q, tr, peaks, peak_kind, K)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": ms_max / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": value / REFERENCE_RAYS_PER_S,
        "dtype": "f32" if tr.cfg.precision == "fp32" else "f32 with f16 table, tf32 mlp", "data": "synthetic",
        "config": {"workload": WORKLOAD, "patches_per_step": args.batch, "patch": "3x3",
                   "rays_per_step": args.batch * tr.P, "views": args.views,
                   "resolution": [args.height, args.width], "hash_levels": 16, "log2_table": 19,
                   "active_levels": net.active_levels(), "step_size": 2.0 / 1024,
                   "occupancy_update_every": 8, "encoding_cache": tr.enc_cache is not None,
                   "precision": tr.cfg.precision,
                   "samples_per_ray": float(tr.S.item()) / args.batch,
                   "l2": "step working set > L2: table + Adam state 4 x 64 MiB streamed every step",
                   "parallelism": f"replicas{world}"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "roofline": rl,
        "stages_ms_per_step": {k: v / K for k, v in stages.items()},
        "stage_roofline": stage_rooflines(stages, q, samples, tr, rl["peak"], K),
    }
    if clk:
        out["clocks"] = clk
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args, tr, scene, rig, budget_s=20.0)
    if args.serve != "off":
        del tr, ds, pool, host, pf, gs
        torch.cuda.empty_cache()
        out["serve"] = run_serve(args.serve, dev)
    return out


def run_quality(iters: int, dev) -> dict:
    """FP32 and mixed precision (FP16 table copy, one-pass TF32 MLP) trained
    from the same initialisation on the sphere scene of the small
    configuration, then measured against the analytic scene."""
    from supernormal_gb300 import quality, scenes
    from supernormal_gb300.fields import SDFNetwork, SingleVarianceNetwork
    from supernormal_gb300.nerfacc import OccupancyGrid
    from supernormal_gb300.trainer import FusedTrainer, TrainConfig

    scene = scenes.sphere(0.5)
    rig = scenes.ring_cameras(8, 128, 128, radius=3.0, elevation_deg=0.0)
    ds = scenes.SyntheticDataset(scene, rig, dev)
    enc = dict(otype="HashGrid", n_levels=16, n_features_per_level=2, log2_hashmap_size=15, base_resolution=16,
               per_level_scale=1.447)
    out = {"config": {"scene": "sphere r=0.5", "views": "8 x 128x128, ring radius 3", "hash": "L16 F2 T2^15",
                      "patches_per_iteration": 256, "samples_per_ray": 128, "iterations": iters,
                      "mixed": "FP16 table copy of FP32 master weights, FP32 gradients, one-pass TF32 MLP"}}
    for prec in ("fp32", "mixed"):
        torch.manual_seed(0)
        net = SDFNetwork(3, 16, 64, 1, skip_in=(-1,), bias=0.5, encoding_config=enc, input_concat=True).to(dev)
        var = SingleVarianceNetwork(0.3).to(dev)
        net.bindwidth = 16
        grid = OccupancyGrid(roi_aabb=[-1.0, -1.0, -1.0, 1.0, 1.0, 1.0], resolution=128).to(dev)
        grid._binary = torch.ones_like(grid._binary)
        cfg = TrainConfig(batch_size=256, step_size=1.0 / 64, occ_update_freq=0, increase_bandwidth_every=0,
                          learning_rate=1e-3, warm_up_end=50, end_iter=iters, precision=prec, seed=0)
        tr = FusedTrainer(net, var, cfg, occupancy_grid=grid, device=dev)
        g = torch.Generator(device=dev).manual_seed(7)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(iters):
            loss = tr.train_step(*ds.gen_random_patches(256, generator=g))
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        tr.check_status()
        m = quality.evaluate(net, var, grid, ds, scene, cfg.step_size)
        m["final_loss"] = float(loss[4].item())
        m["ms_per_iteration"] = 1e3 * dt / iters
        out[prec] = m
    return out


def run_serve(size: str, dev) -> dict:
    """The serving loop on a seeded request trace, served (CUDA graphs, short
    requests between reconstruction slices) and plain (one request at a time,
    eager), under an HBM budget that forces offloads."""
    from supernormal_gb300.serve import ServedObject, Server, object_specs, poisson_trace

    if size == "full":   # 32 objects, 8-100 views at 256^2-1024^2, tables 2^17-2^21
        cfg = dict(objects=32, views=(8, 100), res=(256, 1024), log2_table=(17, 21), duration=20.0, rate=4.0,
                   budget_frac=0.6)
    else:
        cfg = dict(objects=8, views=(8, 24), res=(192, 384), log2_table=(17, 19), duration=6.0, rate=10.0,
                   budget_frac=0.6)
    t0 = time.perf_counter()
    specs = object_specs(cfg["objects"], seed=5, views=cfg["views"], res=cfg["res"], log2_table=cfg["log2_table"])
    objs = [ServedObject(s, dev, batch=512) for s in specs]
    total = sum(o.nbytes() for o in objs)
    budget = int(cfg["budget_frac"] * total)
    setup_s = time.perf_counter() - t0
    trace = poisson_trace(len(objs), cfg["duration"], cfg["rate"], seed=11, recon_iters=100)
    out = {"config": {"objects": len(objs), "views": list(cfg["views"]), "resolution": list(cfg["res"]),
                      "log2_table": list(cfg["log2_table"]), "patches_per_iteration": 512,
                      "recon_block_iterations": 100, "query_grid": 256, "arrival_rate_per_s": cfg["rate"],
                      "trace_s": cfg["duration"], "requests": len(trace),
                      "hbm_budget_gb": budget / 1e9, "objects_total_gb": total / 1e9,
                      "setup_s": setup_s}}
    # capacity: a saturating burst of the same request mix (rays/s over its makespan)
    burst = poisson_trace(len(objs), 2.0, 40.0, seed=13, recon_iters=100)
    out["config"]["burst_requests"] = len(burst)
    for policy in ("served", "plain"):
        srv = Server(objs, budget, query_res=256, slice_iters=10)
        srv.fit_budget()
        r = srv.run(trace, policy)
        r["swaps"] = srv.swaps
        b = Server(objs, budget, query_res=256, slice_iters=10).run(burst, policy)
        r["burst"] = {"makespan_s": b["makespan_s"], "rays_per_s": b["rays_per_s"], "p50_ms": b["p50_ms"],
                      "p99_ms": b["p99_ms"]}
        out[policy] = r
    return out


def stage_times(marks):
    """Sum of event intervals per stage over all profiled steps (ms)."""
    pairs = {"march": ("step_begin", "march_end"),
             "cull": ("march_end", "cull_end"),
             "expand": ("cull_end", "field_fwd_begin"),
             "field_fwd": ("field_fwd_begin", "field_fwd_end"),
             "render": ("field_fwd_end", "render_end"),
             "field_bwd": ("field_bwd_begin", "field_bwd_end"),
             "adam": ("adam_begin", "adam_end"),
             "occupancy": ("occ_begin", "occ_end")}
    tot = {k: 0.0 for k in pairs}
    open_ev = {}
    for tag, ev in marks:   # ev: a CUDA event, or ms from the step's first mark (graph replays)
        for k, (b, e) in pairs.items():
            if tag == b:
                open_ev[k] = ev
            elif tag == e and k in open_ev:
                b_ev = open_ev.pop(k)
                tot[k] += ev - b_ev if isinstance(ev, float) else b_ev.elapsed_time(ev)
    return tot


def stage_rooflines(stages, q, samples, tr, peak, K):
    """Achieved algorithmic GB/s of the other stages (per-unit bytes as in the
    survey's measurement table): marcher 16 B per marched centre sample + 8 B
    per ray; patch render 36 B per patch-pixel sample + 16 B per pixel; Adam
    32 B per parameter; field kernels as in roofline()."""
    if samples is None or q is None or len(samples) == 0:
        return None
    L, F = tr.net.active_levels(), 2
    enc = L * F * 4 if tr.enc_cache is not None else 0
    marched, kept = samples[:, 0].sum(), samples[:, 1].sum()
    steps = len(samples)
    nbytes = {
        "march": marched * 16 + steps * tr.B * 8,
        "render": kept * tr.P * 36 + steps * tr.B * tr.P * 16,
        "adam": float(tr.n_params) * 32 * steps,
        "field_fwd": float(q.sum()) * (12 + L * 8 * F * 4 + 4 + enc),
        "field_bwd": float(q.sum()) * (12 + 4 + (enc if enc else L * 8 * F * 4) + L * 8 * F * 4),
    }
    out = {}
    for k, b in nbytes.items():
        ms = stages[k] * steps / K
        gbs = b / (ms / 1e3) / 1e9 if ms > 0 else None
        out[k] = {"achieved_gbs": gbs, "frac": gbs / peak if gbs else None,
                  "bytes_per_step": b / steps}
    return out


def roofline(stages, q, tr, peaks, peak_kind, K):
    """Dominant kernel's achieved algorithmic bandwidth vs the measured HBM peak."""
    L = tr.net.active_levels()
    F = 2
    enc = L * F * 4 if tr.enc_cache is not None else 0   # encoding cache, per point
    bytes_per = {
        # xyz + d sdf in, the encoding (cached: read back; else the gather of 8
        # corners x F fp32 per level recomputed), float2 gradient scatter
        "field_bwd": lambda: float(q.sum()) * (12 + 4 + (enc if enc else L * 8 * F * 4) + L * 8 * F * 4),
        # xyz in, gather, sdf out, encoding cache written
        "field_fwd": lambda: float(q.sum()) * (12 + L * 8 * F * 4 + 4 + enc),
        # p, g, m, v read; p, m, v, g(=0) written
        "adam": lambda: float(tr.n_params) * 32 * K,
    }
    top = max(bytes_per, key=lambda k: stages[k])   # single-kernel stages only
    achieved = bytes_per[top]() / (stages[top] / 1e3) / 1e9
    peak = float(peaks.get("hbm_gbs", 6800.0))
    traffic = None
    tpath = os.path.join(ROOT, "profiles", f"{top}_dram_traffic.json")
    if os.path.exists(tpath) and q is not None:
        with open(tpath) as f:
            t = json.load(f)
        # captured bytes per field point (or per parameter), scaled to this run's launch
        per_unit = t["dram_bytes_per_unit"]
        units = float(q.mean()) if top != "adam" else float(tr.n_params)
        traffic = per_unit * units
    return {"kernel": top, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
            "algorithmic_bytes_per_launch": bytes_per[top]() / K}


# ---------------------------------------------------------------------------
def cpu_step_factory(args, net_state, scene, rig, seed):
    """One proportional sample of a training iteration on host cores (float64 oracle)."""
    import numpy as np

    from oracle import field as OF
    from oracle import march as OM
    from oracle import renderer as OR
    from supernormal_gb300 import scenes

    B_s = args.cpu_sample_patches
    frac = B_s / args.batch
    prm, geom, variance, binary, n_params = net_state
    table = prm["table"]
    g = torch.Generator().manual_seed(seed)
    n_occ = max(1, int(round((128 ** 3 // 2) / 8 * frac)))      # amortised occupancy points
    n_adam = max(4, int(round(n_params * frac)))
    adam_p = torch.zeros(n_adam, dtype=torch.float64, requires_grad=True)
    opt = torch.optim.Adam([adam_p], lr=5e-4)
    roi = np.array([-1, -1, -1, 1, 1, 1], np.float32)
    fld = lambda x: OF.sdf_network(x, **prm, geom=geom, active_levels=16, out_cols=1)

    def step():
        ro, rd, pn, vinv, nrm, mask = scenes.sample_patches(scene, rig, B_s, generator=g)
        ro_c = ro[:, 1, 1].numpy()
        rd_c = rd[:, 1, 1].numpy()
        b = 2 * (ro_c * rd_c).sum(1)
        c = (ro_c * ro_c).sum(1) - 1
        a = (rd_c * rd_c).sum(1)
        disc = np.sqrt(np.maximum(b * b - 4 * a * c, 0))
        near = ((-b - disc) / (2 * a)).astype(np.float32)
        far = ((-b + disc) / (2 * a)).astype(np.float32)
        jit = torch.rand(B_s, generator=g).numpy().astype(np.float32)
        packed, ri, ts, te = OM.ray_marching(ro_c, rd_c, near, far, roi, binary, 2.0 / 1024, jitter=jit)
        if ri.size:
            vis, _ = OR.cull(fld, packed, ri, ts, te, ro_c, rd_c, variance.detach())
            ri, ts, te = ri[vis], ts[vis], te[vis]
        if ri.size:
            out = OR.patch_forward(fld, ri, ts, te, ro.numpy(), rd.numpy(), pn.numpy(), vinv.numpy(),
                                   variance)
            L = OR.losses(out["comp_normal"], out["weight_sum"], out["gradients"], nrm.numpy(),
                          mask.numpy())
            L["total"].backward()
        with torch.no_grad():
            x = torch.rand((n_occ, 3), generator=g, dtype=torch.float64) * 2 - 1
            torch.sigmoid(-fld(x) * 80.0)
        adam_p.grad = torch.randn(n_adam, generator=g, dtype=torch.float64)
        opt.step()
        for p in list(prm.values()) + [variance]:
            p.grad = None
        return B_s * 9

    return step


def cpu_state(tr):
    from oracle import field as OF

    prm = OF.params_from_module(tr.net)
    geom = OF.geometry_from_module(tr.net)
    variance = tr.dev_net.variance.detach().cpu().double().clone().requires_grad_(True)
    binary = tr.grid.binary.cpu().numpy().astype("uint8")
    return prm, geom, variance, binary, tr.n_params


def cpu_baseline(args, tr, scene, rig, budget_s=20.0):
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    step = cpu_step_factory(args, cpu_state(tr), scene, rig, seed=7)
    step()  # warm-up
    rays, t0 = 0, time.perf_counter()
    n = 0
    while time.perf_counter() - t0 < budget_s and n < 50:
        rays += step()
        n += 1
    dt = time.perf_counter() - t0
    return {"value": rays / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} iterations of {args.cpu_sample_patches} patches (1/{args.batch // args.cpu_sample_patches} "
                      f"of a step: patches, amortised occupancy points and Adam elements scaled alike), "
                      f"float64 oracle, {dt:.1f} s"}


def run_reference(args, world, rank, local):
    """CPU arm: the reference path's math (oracle port) on host cores."""
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    dev = torch.device("cuda", local) if torch.cuda.is_available() else torch.device("cpu")
    from supernormal_gb300 import scenes
    from supernormal_gb300.fields import SDFNetwork, SingleVarianceNetwork
    from oracle import field as OF

    torch.manual_seed(1234)
    scene = scenes.displaced_torus(0.5, 0.2, 0.02, 20.0)
    rig = scenes.ring_cameras(args.views, args.height, args.width, radius=3.0, elevation_deg=30.0,
                              fov_deg=40.0)
    net = SDFNetwork(3, 16, 64, 1, skip_in=(-1,), bias=0.5, encoding_config=ENC, input_concat=True)
    var = SingleVarianceNetwork(0.5)
    prm = OF.params_from_module(net)
    geom = OF.geometry_from_module(net)
    variance = var.variance.detach().double().clone().requires_grad_(True)
    # occupancy of the initial field (all cells) on host cores
    import numpy as np

    r = 128
    c = (np.stack(np.meshgrid(*[np.arange(r)] * 3, indexing="ij"), -1).reshape(-1, 3) + 0.5) / r * 2 - 1
    # the sphere-initialised SDF is |x| - 0.5 (+ small table terms): binarise its occupancy
    occ = 1.0 / (1.0 + np.exp(np.clip((np.linalg.norm(c, axis=1) - 0.5) * 80.0, -50, 50)))
    binary = (occ > min(occ.mean(), 0.1)).reshape(r, r, r).astype(np.uint8)
    n_params = net.encoding.params.numel() + sum(p.numel() for n_, p in net.named_parameters()
                                                 if not n_.startswith("encoding"))
    step = cpu_step_factory(args, (prm, geom, variance, binary, n_params), scene, rig, seed=11)
    for _ in range(max(args.warmup, 1)):
        step()
    rays, t0 = 0, time.perf_counter()
    for _ in range(args.steps):
        rays += step()
    dt = time.perf_counter() - t0
    value = rays / dt
    sample = (f"{args.steps} iterations of {args.cpu_sample_patches} patches each (1/"
              f"{args.batch // args.cpu_sample_patches} of a step, occupancy points and Adam elements "
              f"scaled alike), float64 restatement of the reference math, {threads} threads")
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": value / REFERENCE_RAYS_PER_S,
            "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "patches_per_step": args.batch,
                       "sampled_patches_per_step": args.cpu_sample_patches, "device": "host cores"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.quality:
        out = {"quality": run_quality(args.quality_iters, torch.device("cuda", local))} if rank == 0 else None
    elif args.impl == "reference":
        out = run_reference(args, world, rank, local)
    else:
        out = run_ours(args, world, rank, local)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
