#!/usr/bin/env python
"""Training-throughput benchmark of the SuperNormal hot path on GB300.

Workload (the reference-equivalent GPU configuration): a displaced torus
(R=0.5, r=0.2, amplitude 0.02, frequency 20) seen by 20 views of 612x512 on an
elevated ring (15 train; views 0, 4, 8, 12, 16 held out for evaluation as
config/diligent.conf:16 excludes them); hash grid 16 levels x 2 features,
2^19 entries per level, base resolution 16, scale 1.447; SDF MLP
35 -> 64 -> 16; 128^3 occupancy grid (threshold 0.1, updated every 8
iterations); marching step 2/1024; 2048 patches of 3x3 per iteration; FP32.
Data are synthetic (no dataset is shipped).

The run: (1) the configuration's whole training schedule from the seeded
initialisation (5000 iterations, one finer level every 300, occupancy
warm-up then sampled updates, warm-up + cosine learning rate), timed end to
end (``training_run``); (2) quality of the trained field on the held-out
views (normal angular error, mask IoU, Chamfer / F-score, ``quality``);
(3) W warm-up and K timed steps at the trained state with all 16 levels
active: a step is one full training iteration (marching, culling, patch
expansion, field forward, render + loss + adjoint, field backward,
learning-rate schedule and Adam, plus the amortised occupancy update).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--train-iters N] [--precision fp32|mixed] [--eager]
                  [--serve small|full|off] [--quality]

The timed region replays each iteration as a CUDA graph whose captured copies
carry the stage events (per-stage times and the roofline's kernel durations
come from those events; --eager times eager launches instead).  The
end-to-end figure feeds every iteration from pinned host memory through the
trainer's prefetcher and reads its loss back.  N > 1 runs as independent
replicas (one process per GPU via torchrun; the path has no exchange step),
value = all ranks' rays / max rank time.
Baselines: ``kernels_vs_reference`` times the reference's own marcher and
patch-weight kernels (built from its sources) against ours on the run's
inputs; ``cpu_baseline`` and --impl reference time the reference path's
math (the float32 restatement in oracle/, the reference having no CPU path
of its own) on host cores over a bounded, proportional sample of the same
workload, on a state both arms rebuild on the host.
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


def parse(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--batch", type=int, default=2048)
    p.add_argument("--views", type=int, default=20)
    p.add_argument("--height", type=int, default=512)
    p.add_argument("--width", type=int, default=612)
    p.add_argument("--train-iters", type=int, default=5000,
                   help="training run from the initialisation before the timed steps (the configuration's "
                        "5000-iteration schedule)")
    p.add_argument("--bandwidth-every", type=int, default=300, help="one finer hash level every N iterations")
    p.add_argument("--cpu-sample-patches", type=int, default=8)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-quality", action="store_true", help="skip the held-out-view quality evaluation")
    p.add_argument("--no-reference-kernels", action="store_true",
                   help="skip timing the reference's own marcher / patch-weight kernels")
    p.add_argument("--no-ad", action="store_true",
                   help="skip timing the iteration with the 'ad' gradient method")
    p.add_argument("--no-clocks", action="store_true")
    p.add_argument("--precision", choices=["fp32", "mixed"], default="fp32",
                   help="mixed: FP16 hash-table copy and one-pass TF32 MLP products (config 3's path)")
    p.add_argument("--eager", action="store_true",
                   help="time eager launches instead of CUDA-graph replays of each iteration")
    p.add_argument("--no-encoding-cache", action="store_true",
                   help="field backward recomputes the encoding instead of reading the forward's")
    p.add_argument("--serve", choices=["small", "full", "off"], default="full",
                   help="serving-loop trace after the training measurement (p50/p99 latency); full: 32 objects")
    p.add_argument("--quality", action="store_true",
                   help="instead of the throughput run: FP32 vs mixed precision reconstruction quality "
                        "on the sphere scene (angular error, mask IoU, Chamfer / F@0.01)")
    p.add_argument("--quality-iters", type=int, default=1000)
    return p.parse_args(argv)


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
TEST_VIEWS = (0, 4, 8, 12, 16)   # held out for evaluation, as config/diligent.conf:16 excludes them


def workload_config(args, world) -> dict:
    """The workload both arms run (identical dictionaries in both JSON lines)."""
    return {"workload": WORKLOAD, "scene": "displaced torus R=0.5 r=0.2 amp=0.02 freq=20",
            "patches_per_step": args.batch, "patch": "3x3", "rays_per_step": args.batch * 9,
            "views": args.views, "train_views": args.views - len([v for v in TEST_VIEWS if v < args.views]),
            "resolution": [args.height, args.width], "hash": "L16 F2 T2^19 base 16 scale 1.447",
            "mlp": "35-64-16 softplus(beta=100), weight norm", "hash_levels": 16, "log2_table": 19,
            "active_levels": 16, "occupancy": "128^3, threshold 0.1, updated every 8 iterations",
            "step_size": 2.0 / 1024, "precision": args.precision,
            "l2": "step working set > L2: table + Adam state 4 x 64 MiB streamed every step",
            "parallelism": f"replicas{world}"}


def build_workload(args, device, seed):
    from supernormal_gb300 import scenes
    from supernormal_gb300.fields import SDFNetwork, SingleVarianceNetwork
    from supernormal_gb300.trainer import FusedTrainer, TrainConfig

    torch.manual_seed(seed)
    scene = scenes.displaced_torus(0.5, 0.2, 0.02, 20.0)
    rig = scenes.ring_cameras(args.views, args.height, args.width, radius=3.0, elevation_deg=30.0,
                              fov_deg=40.0)
    test = [v for v in TEST_VIEWS if v < args.views]
    train = [v for v in range(args.views) if v not in test]
    pick = lambda vs: scenes.CameraRig(rig.poses[vs], rig.intrinsics[vs], rig.H, rig.W)
    net = SDFNetwork(3, 16, 64, 1, skip_in=(-1,), bias=0.5, encoding_config=ENC,
                     input_concat=True).to(device)
    var = SingleVarianceNetwork(0.5).to(device)
    cfg = TrainConfig(batch_size=args.batch, step_size=2.0 / 1024, occ_update_freq=8,
                      occ_threshold=0.1, increase_bandwidth_every=args.bandwidth_every,
                      end_iter=args.train_iters, seed=seed,
                      encoding_cache=not getattr(args, "no_encoding_cache", False),
                      precision=getattr(args, "precision", "fp32"))
    tr = FusedTrainer(net, var, cfg, device=device)
    return scene, pick(train), pick(test) if test else None, net, var, tr


def training_run(args, tr, ds, g) -> dict:
    """The benchmark configuration's whole training schedule from the seeded
    initialisation: fresh patches every iteration, occupancy warm-up sweeps
    for 256 iterations then sampled updates every 8, one finer level every
    ``bandwidth_every`` iterations, warm-up + cosine learning rate, each
    iteration a CUDA-graph replay (re-captured when the bandwidth changes).
    Timed end to end with CUDA events (captures and host waits included)."""
    from supernormal_gb300.trainer import GraphStep

    n = args.train_iters
    gs = GraphStep(tr)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(n):
        gs.step(ds.gen_random_patches(args.batch, generator=g))
    e1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    tr.check_status()
    ms = e0.elapsed_time(e1)
    rays = n * args.batch * tr.P
    return {"iterations": n, "seconds": ms / 1e3, "wall_seconds": wall, "rays_per_s": rays / (ms / 1e3),
            "graph_captures": gs.captures, "final_active_levels": tr.net.active_levels(),
            "loss": [float(x) for x in tr.loss_out.tolist()],
            "note": "whole schedule from initialisation: patch sampling, occupancy updates, bandwidth "
                    "schedule and graph captures inside the timed span"}


def run_ours(args, world, rank, local):
    from supernormal_gb300 import quality, scenes
    from supernormal_gb300._lib import lib
    from supernormal_gb300.trainer import GraphStep, HostPrefetcher

    dev = torch.device("cuda", local)
    t_setup = time.perf_counter()
    scene, rig, test_rig, net, var, tr = build_workload(args, dev, seed=1234 + rank)
    ds = scenes.SyntheticDataset(scene, rig, dev)
    g = torch.Generator(device=dev).manual_seed(99 + rank)
    pool = [ds.gen_random_patches(args.batch, generator=g) for _ in range(16)]
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t_setup
    # the training schedule from initialisation, then the state is measured
    train = training_run(args, tr, ds, g) if args.train_iters > 0 else None
    if args.train_iters <= 0:
        tr.occupancy_update(0)
    net.bindwidth = max(net.bindwidth, ENC["n_levels"])      # timed steps: all 16 levels
    tr.iter_step = max(tr.iter_step, tr.cfg.occ_warmup_steps)
    qual = None
    if rank == 0 and test_rig is not None and not args.no_quality:
        tq = time.perf_counter()
        test_ds = scenes.SyntheticDataset(scene, test_rig, dev)
        qual = quality.evaluate(net, var, tr.grid, test_ds, scene, tr.cfg.step_size)
        qual["after_iterations"] = tr.iter_step
        qual["views"] = f"held-out views {list(TEST_VIEWS)} of {args.views}"
        qual["seconds"] = time.perf_counter() - tq
    # iterations as CUDA-graph replays (captured before the warm-up), or eager
    # launches with --eager; a second set of captures carries the stage events
    gs = gp = None
    if not args.eager:
        gs, gp = GraphStep(tr), GraphStep(tr, profile=True)
        gs.prepare()
        gp.prepare()

    def step(graph, i):
        if graph is not None:
            graph.step(pool[i % len(pool)])
        else:
            tr.train_step(*pool[i % len(pool)])

    for i in range(args.warmup):
        step(gs, i)
    if gp is not None:
        for i in range(gp.n_copies):           # first replays of the profiled copies, untimed
            step(gp, i)
    torch.cuda.synchronize()
    tr.check_status()
    if gp is not None:
        gp.flush()
        gp.stage_marks.clear()
        gp.points.clear()
        gp.samples.clear()

    # ---------------- device-resident timed region ----------------
    K = args.steps
    clocks = ClockSampler(local, not args.no_clocks and rank == 0)
    launches0 = gs.launches if gs is not None else lib().sn_kernel_launches()
    barrier(world)
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed")      # profiler filter: the timed steps only
    start.record()
    for i in range(K):
        step(gs, i)
    end.record()
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    ms = start.elapsed_time(end)
    tr.check_status()
    launches = (gs.launches if gs is not None else lib().sn_kernel_launches()) - launches0

    # ---------------- the same K steps with stage events (roofline, stage times) ----------------
    if gp is None:
        tr.profile = True
        tr.marks.clear()
        tr.q_hist.clear()
    torch.cuda.synchronize()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record()
    for i in range(K):
        step(gp, i)
    p1.record()
    torch.cuda.synchronize()
    tr.check_status()
    profiled_ms = p0.elapsed_time(p1)
    if gp is not None:
        gp.flush()
        stages = stage_times([m for s_ in gp.stage_marks for m in s_])
        q = np.asarray(gp.points, dtype=np.float64)
        samples = np.asarray(gp.samples, dtype=np.float64)
    else:
        samples = None
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
    pf = HostPrefetcher(tr, host[0], graph=gs)
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
    spr = None
    if samples is not None and len(samples):
        spr = {"marched": float(samples[:, 0].mean()) / args.batch, "kept": float(samples[:, 1].mean()) / args.batch}
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": ms_max / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": value / REFERENCE_RAYS_PER_S,
        "dtype": "f32" if tr.cfg.precision == "fp32" else "f32 with f16 table, tf32 mlp", "data": "synthetic",
        "config": workload_config(args, world),
        "state": {"kind": "trained", "iterations": tr.iter_step if train else 0,
                  "samples_per_ray": spr, "encoding_cache": tr.enc_cache is not None,
                  "note": "timed after the training run from the seeded initialisation; "
                          "occupancy update every 8 iterations in its sampled regime"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "roofline": rl,
        "stages_ms_per_step": {k: v / K for k, v in stages.items()},
        "profiled_ms_per_step": profiled_ms / K,
        "stage_roofline": stage_rooflines(stages, q, samples, tr, rl["peak"], K),
        "setup_s": setup_s,
    }
    if train is not None:
        out["training_run"] = train
    if qual is not None:
        out["quality"] = qual
    if clk:
        out["clocks"] = clk
    if not args.no_reference_kernels:
        out["kernels_vs_reference"] = reference_kernels_leg(tr, pool[0])
    if not args.no_ad and tr.cfg.precision == "fp32":
        out["ad_step"] = ad_step_leg(args, tr, pool)
    if tr.cfg.precision == "fp32":
        out["mlp_precision"] = mlp_precision_leg(tr)
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args, budget_s=20.0)
    if args.serve != "off":
        del tr, ds, pool, host, pf, gs, gp
        torch.cuda.empty_cache()
        out["serve"] = run_serve(args.serve, dev)
    return out


def ad_step_leg(args, tr, pool, steps: int = 10) -> dict:
    """The same iteration with the gradients of the normals from
    SDFNetwork.gradient (the reference's 'ad' method, models/renderer.py:225-226)
    instead of dfd, on the trained state: the field's first- and second-order
    adjoint kernels run as well.  CUDA-graph replays, CUDA events."""
    from supernormal_gb300.trainer import FusedTrainer, GraphStep, TrainConfig

    c = tr.cfg
    cfg = TrainConfig(batch_size=c.batch_size, step_size=c.step_size, occ_update_freq=c.occ_update_freq,
                      occ_threshold=c.occ_threshold, increase_bandwidth_every=0, end_iter=c.end_iter, seed=c.seed,
                      gradient_method="ad", encoding_cache=tr.enc_cache is not None)
    tr_ad = FusedTrainer(tr.net, tr.dev_net, cfg, occupancy_grid=tr.grid, device=tr.device)
    tr_ad.iter_step = tr.iter_step
    gs = GraphStep(tr_ad, profile=True)
    gs.prepare()
    for i in range(3):
        gs.step(pool[i % len(pool)])
    gs.flush()
    gs.stage_marks.clear()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for i in range(steps):
        gs.step(pool[i % len(pool)])
    e1.record()
    torch.cuda.synchronize()
    tr_ad.check_status()
    gs.flush()
    ms = e0.elapsed_time(e1) / steps
    st = stage_times([m for step in gs.stage_marks for m in step])
    return {"ms_per_step": ms, "rays_per_s": args.batch * tr.P / (ms / 1e3), "steps": steps,
            "stages_ms_per_step": {k: v / steps for k, v in st.items()},
            "gradient_method": "ad (SDFNetwork.gradient with the second-order adjoint)"}


def mlp_precision_leg(tr, reps: int = 20, rounds: int = 3) -> dict:
    """The field forward over the last step's training points with the
    first layer's tensor-core products in FP32-accurate 3xTF32 (the training
    path), one TF32 pass (the mixed-precision path) and one BF16 pass, FP32
    table: CUDA-event time per launch (variants interleaved) and the sdf
    difference from 3xTF32."""
    import ctypes as Ct

    from supernormal_gb300._lib import SN_FIELD_MLP_BF16, SN_FIELD_MLP_TF32, call, stream_handle

    n = int(tr.q1.item())
    if n == 0:
        return {"points": 0}
    st = stream_handle()
    table = tr.views["table"]
    variants = {"fp32_3xtf32": 0, "tf32": SN_FIELD_MLP_TF32, "bf16": SN_FIELD_MLP_BF16}
    outs = {k: torch.empty((n, 1), device=tr.device) for k in variants}
    descs = {}
    for k, f in variants.items():
        d = tr._mlp()
        d.flags = f
        descs[k] = d
    times = {k: [] for k in variants}
    for r in range(rounds):
        for k in variants:
            for _ in range(3 if r == 0 else 0):
                call("sn_field_fwd", n, None, tr.xyz1, table, Ct.byref(tr.net.encoding.desc),
                     tr.net.active_levels(), Ct.byref(descs[k]), 1, outs[k], st)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                call("sn_field_fwd", n, None, tr.xyz1, table, Ct.byref(tr.net.encoding.desc),
                     tr.net.active_levels(), Ct.byref(descs[k]), 1, outs[k], st)
            e1.record()
            torch.cuda.synchronize()
            times[k].append(e0.elapsed_time(e1) / reps)
    tr.check_status()
    ref = outs["fp32_3xtf32"].double()
    out = {"points": n, "table": "fp32", "note": "field forward over the last step's training points; "
           "min over rounds of the mean launch time; sdf differences against the 3xTF32 launch"}
    for k in variants:
        diff = (outs[k].double() - ref).abs()
        out[k] = {"ms": min(times[k]), "max_abs_diff": float(diff.max()), "rms_diff": float(diff.pow(2).mean().sqrt())}
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
    """The serving loop on a seeded request trace under an HBM budget that
    forces offloads: served (mixed precision, CUDA-graph reconstruction
    slices on one stream, render / query requests on a second, ordered per
    object) against plain (FP32, one request at a time, eager)."""
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
                      "setup_s": setup_s,
                      "served": "mixed precision (FP16 table copy, one-pass TF32 MLP), graph replays, "
                                "requests on a second stream beside reconstruction slices",
                      "plain": "FP32, eager, one request at a time"}}
    # capacity: a saturating burst of the same request mix (rays/s over its makespan)
    burst = poisson_trace(len(objs), 2.0, 40.0, seed=13, recon_iters=100)
    out["config"]["burst_requests"] = len(burst)
    for policy in ("served", "plain"):
        for o in objs:
            o.set_precision("mixed" if policy == "served" else "fp32")
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
    if len(samples) != len(q):
        raise ValueError(f"stage_rooflines: sample counts of {len(samples)} steps against field points of {len(q)}")
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
# Baseline legs.  They run the reference's arithmetic outside the package:
# the host restatement in oracle/ on the CPU (cpu_baseline, --impl reference)
# and the reference's own kernels compiled from its sources (oracle/_ref) on
# the GPU (kernels_vs_reference).  Nothing on the timed path of our arm calls
# them.
HOST_STATE = ("seeded initialisation (torch seed 1234; the same parameters as the GPU arm's initial "
              "network) with the occupancy grid of the analytic torus (sigmoid(-80 sdf) at cell centres "
              "above min(mean, 0.1)): a state both arms rebuild exactly on host cores")


def host_step_factory(args, seed, dtype=torch.float32):
    """One proportional sample of a training iteration on host cores: the
    reference's math restated in oracle/ (marcher in C, field, culling,
    patch render, losses and their backward in torch on the CPU), on the
    host state above.  B_s of ``args.batch`` patches; the amortised
    occupancy update and the Adam elements are scaled by the same fraction.
    Batches are drawn before timing (the reference gathers them from images
    already in memory)."""
    from oracle import field as OF
    from oracle import march as OM
    from oracle import renderer as OR
    from oracle import scene as OS

    B_s = args.cpu_sample_patches
    frac = B_s / args.batch
    prm, geom = OS.sdf_network_init(1234, ENC)
    prm = {k: v.to(dtype).requires_grad_(True) for k, v in prm.items()}
    variance = torch.tensor(0.5, dtype=dtype, requires_grad=True)
    binary = OS.analytic_occupancy(OS.torus_sdf, 128, 0.1)
    n_params = sum(v.numel() for v in prm.values()) + 1
    poses, kinv = OS.ring_rig(args.views, args.height, args.width)
    train_views = [v for v in range(args.views) if v not in TEST_VIEWS]
    poses, kinv = poses[train_views], kinv[train_views]
    rng = np.random.default_rng(seed)
    pool = [OS.gen_random_patches(OS.torus_sdf, OS.torus_lipschitz(), poses, kinv, args.height, args.width,
                                  B_s, rng) for _ in range(4)]
    n_occ_cells = int(binary.sum())
    n_occ = max(1, int(round((128 ** 3 // 4 + min(n_occ_cells, 128 ** 3 // 4)) / 8 * frac)))
    n_adam = max(4, int(round(n_params * frac)))
    adam_p = torch.zeros(n_adam, dtype=dtype, requires_grad=True)
    opt = torch.optim.Adam([adam_p], lr=5e-4)
    roi = np.array([-1, -1, -1, 1, 1, 1], np.float32)
    fld = lambda x: OF.sdf_network(x, **prm, geom=geom, active_levels=16, out_cols=1, dtype=dtype)
    g = torch.Generator().manual_seed(seed)
    state = {"i": 0}

    def step():
        ro, rd, pn, vinv, nrm, mask = pool[state["i"] % len(pool)]
        state["i"] += 1
        ro_c, rd_c = ro[:, 1, 1], rd[:, 1, 1]
        near, far = OS.near_far(ro_c.astype(np.float64), rd_c.astype(np.float64))
        jit = torch.rand(B_s, generator=g).numpy().astype(np.float32)
        packed, ri, ts, te = OM.ray_marching(ro_c, rd_c, near.astype(np.float32), far.astype(np.float32), roi,
                                             binary, 2.0 / 1024, jitter=jit)
        marched, kept = ri.size, 0
        if ri.size:
            vis, _ = OR.cull(fld, packed, ri, ts, te, ro_c, rd_c, variance.detach(), dtype=dtype)
            ri, ts, te = ri[vis], ts[vis], te[vis]
            kept = ri.size
        if ri.size:
            out = OR.patch_forward(fld, ri, ts, te, ro, rd, pn, vinv, variance, dtype=dtype)
            L = OR.losses(out["comp_normal"], out["weight_sum"], out["gradients"], nrm, mask)
            L["total"].backward()
        with torch.no_grad():
            x = torch.rand((n_occ, 3), generator=g, dtype=dtype) * 2 - 1
            torch.sigmoid(-fld(x) * 80.0)
        adam_p.grad = torch.randn(n_adam, generator=g, dtype=dtype)
        opt.step()
        for p in list(prm.values()) + [variance]:
            p.grad = None
        return B_s * 9, marched, kept

    return step


def _host_sample(args, n, dt, marched, kept):
    return (f"{n} iterations of {args.cpu_sample_patches} patches (1/{args.batch // args.cpu_sample_patches} "
            f"of a step; amortised occupancy points and Adam elements scaled alike), float32 restatement of "
            f"the reference math in oracle/ on host cores, {dt:.1f} s; samples per ray marched "
            f"{marched:.1f}, kept {kept:.1f}; state: {HOST_STATE}")


def cpu_baseline(args, budget_s=20.0):
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    step = host_step_factory(args, seed=7)
    step()  # warm-up
    rays = marched = kept = n = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < budget_s and n < 50:
        r, m, k = step()
        rays, marched, kept, n = rays + r, marched + m, kept + k, n + 1
    dt = time.perf_counter() - t0
    B = n * args.cpu_sample_patches
    return {"value": rays / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": _host_sample(args, n, dt, marched / B, kept / B)}


def reference_kernels_leg(tr, batch, reps: int = 20) -> dict:
    """The reference's own marcher and patch-weight kernels (nerfacc 0.3.5
    compiled from its sources for sm_103a) against ours on this step's
    inputs, CUDA-event medians over ``reps`` repetitions: the marcher as the
    reference runs it (count pass, cumsum, the .item() sync, fill pass:
    NA/nerfacc/cuda/csrc/ray_marching.cu:194-289) against sn_march_padded +
    sn_pack_counts + sn_compact_padded; the patch weights forward and backward
    (render_weight.cu:502-626) against sn_weight_from_alpha_fwd/bwd on the
    NeuS alphas of the step's kept samples."""
    try:
        from oracle import refkernels
    except Exception as e:   # pragma: no cover
        return {"unavailable": f"reference kernel loader: {e}"}
    ref = refkernels.load()
    if isinstance(ref, Exception):
        return {"unavailable": f"reference kernels not built: {ref}"}
    from supernormal_gb300._lib import call, stream_handle

    st = stream_handle()
    rays_o, rays_d, plane_n, vinv, normal, mask = batch
    tr.forward_backward(rays_o, rays_d, plane_n, vinv, normal, mask, tr.step_key(tr.iter_step),
                        tr.net.active_levels())
    torch.cuda.synchronize()
    B, P, dt = tr.B, tr.P, tr.cfg.step_size
    ro, rd, near, far, jit = tr.ro_c.clone(), tr.rd_c.clone(), tr.near.clone(), tr.far.clone(), tr.jitter.clone()
    t_min = (near + jit * dt).contiguous()            # the reference adds the jitter in Python
    grid = tr.grid
    roi = grid._roi_aabb.contiguous().float()
    binary = grid._binary.contiguous()

    def timed(fn):
        ts = []
        for _ in range(reps + 2):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts[2:]))

    ref_out = {}

    def ref_march():
        ref_out["r"] = ref.ray_marching(ro, rd, t_min, far, roi, binary, dt)

    def our_march():
        call("sn_march_padded", B, ro, rd, near, far, jit, roi, binary.view(torch.uint8), *tr.res,
             grid._contraction_type.value, float(dt), None, 0.0, 0, tr.max_steps, tr.counts0, tr.ridx_pad,
             tr.ts_pad, tr.te_pad, tr.status, st)
        call("sn_pack_counts", B, tr.counts0, tr.packed0, tr.total0, tr.scan_ws, st)
        call("sn_compact_padded", B, tr.max_steps, tr.packed0, tr.ridx_pad, tr.ts_pad, tr.te_pad, tr.ridx0,
             tr.ts0, tr.te0, st)

    t_ref_m, t_our_m = timed(ref_march), timed(our_march)
    n0 = int(tr.total0.item())
    same = bool(torch.equal(ref_out["r"][1], tr.ridx0[:n0]))
    # NeuS alphas of the kept samples per patch pixel from the step's field values
    S = int(tr.S.item())
    packed = tr.packed1.contiguous()
    alphas = _patch_alphas(tr, S).contiguous()
    w_ref = ref.patch_weight_fwd(packed, alphas)
    w_our = torch.empty_like(alphas)
    g_w = torch.randn(alphas.shape, device=alphas.device, generator=torch.Generator(device=alphas.device).manual_seed(3))
    ga_our = torch.empty_like(alphas)
    t_ref_f = timed(lambda: ref.patch_weight_fwd(packed, alphas))
    t_our_f = timed(lambda: call("sn_weight_from_alpha_fwd", B, P, packed, alphas, w_our, st))
    t_ref_b = timed(lambda: ref.patch_weight_bwd(packed, alphas, w_ref, g_w))
    t_our_b = timed(lambda: call("sn_weight_from_alpha_bwd", B, P, packed, alphas, w_our, g_w, ga_our, st))
    ga_ref = ref.patch_weight_bwd(packed, alphas, w_ref, g_w)
    tr.grads.zero_()
    torch.cuda.synchronize()
    return {"march": {"reference_ms": t_ref_m, "ours_ms": t_our_m, "speedup": t_ref_m / t_our_m,
                      "rays": B, "samples": n0, "ray_indices_identical": same,
                      "reference": "count pass + cumsum + .item() + fill pass",
                      "ours": "single-pass warp-per-ray marcher + scan + compaction, no host sync"},
            "patch_weights_fwd": {"reference_ms": t_ref_f, "ours_ms": t_our_f, "speedup": t_ref_f / t_our_f,
                                  "samples": S, "identical": bool(torch.equal(w_ref, w_our))},
            "patch_weights_bwd": {"reference_ms": t_ref_b, "ours_ms": t_our_b, "speedup": t_ref_b / t_our_b,
                                  "identical": bool(torch.equal(ga_ref, ga_our))},
            "note": "inputs: this run's centre rays, jitter and occupancy grid, and the NeuS alphas of its kept "
                    "samples; the training iteration itself runs the weights fused into the patch render"}


def _patch_alphas(tr, S):
    """(S, P) NeuS alphas (models/renderer.py:164-179) of the last step's kept
    samples from its field values: the end value is the next start of the
    ray, or the separate end evaluation where t_end != next t_start."""
    P = tr.P
    sdf = tr.sdf1[:, 0]
    s0 = sdf[: S * P].view(S, P)
    s1 = torch.cat([s0[1:], s0[-1:]], 0).clone()
    ep = tr.endp1[:S]
    has_end = ep[:, 1] != 0
    slots = ep[has_end, 0].long()
    s1[has_end] = sdf.view(-1, P)[S + slots]
    inv_s = torch.exp(tr.dev_net.variance.detach() * 10.0).clip(1e-6, 1e6)
    prev, nxt = torch.sigmoid(s0 * inv_s), torch.sigmoid(s1 * inv_s)
    return (((prev - nxt) + 1e-5) / (prev + 1e-5)).clip(0.0, 1.0)


def run_reference(args, world, rank, local):
    """The reference path's math on host cores (float32 restatement in
    oracle/, the reference having no CPU path of its own), rank 0 only.
    Imports nothing from the package."""
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    step = host_step_factory(args, seed=11)
    for _ in range(max(args.warmup, 1)):
        step()
    rays = marched = kept = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r, m, k = step()
        rays, marched, kept = rays + r, marched + m, kept + k
    dt = time.perf_counter() - t0
    value = rays / dt
    B = args.steps * args.cpu_sample_patches
    sample = _host_sample(args, args.steps, dt, marched / B, kept / B)
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": value / REFERENCE_RAYS_PER_S,
            "dtype": "f32", "data": "synthetic", "config": workload_config(args, world),
            "state": {"kind": "host", "samples_per_ray": {"marched": marched / B, "kept": kept / B},
                      "note": HOST_STATE},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
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
