"""Serving loop over many resident reconstruction objects.

A stand-in for a reconstruction service: each object is one SuperNormal
reconstruction (an analytic scene seen by its own views, a hash-grid SDF, the
variance, Adam state and an occupancy grid) and requests arrive as a seeded
Poisson process:

* ``recon``  -- a block of training iterations (exp_runner.py:147-210),
* ``render`` -- a normal map of the current SDF at a new camera pose
  (NeuSRenderer.render in eval mode over the image's 3x3 patches),
* ``query``  -- the SDF on a regular grid, the input of mesh extraction
  (models/renderer.py:9-34 ``extract_fields``).

Objects are admitted under a fixed HBM budget: the least recently used
resident objects are offloaded (persistent state copied to pinned host
memory, every storage shrunk to zero bytes) to make room, and brought back on
their next request.  Two service policies run the same trace:

* ``plain``  -- one request at a time in arrival order, eager launches;
* ``served`` -- training iterations replayed as CUDA graphs in slices on a
  reconstruction stream, and render / query requests on a second stream, so
  a short request is admitted while a reconstruction block is on the GPU and
  runs alongside it instead of waiting behind it.

Ordering across the two streams is per object: every piece of work of an
object (its onload copies included) waits for the event its previous work
recorded and records a new one, and an object is offloaded only after the
host has waited for that event.  Latency = completion of the request's own
work (its object's event) minus arrival.
"""
from __future__ import annotations

import math
import time
from collections import deque
from contextlib import contextmanager
from dataclasses import dataclass
from typing import Optional

import torch

from . import scenes
from .fields import SDFNetwork, SingleVarianceNetwork
from .renderer import NeuSRenderer, near_far_from_sphere
from .trainer import FusedTrainer, GraphStep, TrainConfig


@dataclass
class ObjectSpec:
    index: int
    seed: int
    n_views: int
    res: int
    log2_table: int


def object_specs(n_objects: int, seed: int = 0, views=(8, 100), res=(256, 1024),
                 log2_table=(17, 21)) -> list:
    """Seeded object sizes: views, square resolution and table size drawn uniformly."""
    g = torch.Generator().manual_seed(seed)
    out = []
    for i in range(n_objects):
        nv = int(torch.randint(views[0], views[1] + 1, (1,), generator=g))
        r = int(torch.randint(res[0], res[1] + 1, (1,), generator=g)) // 3 * 3
        t = int(torch.randint(log2_table[0], log2_table[1] + 1, (1,), generator=g))
        out.append(ObjectSpec(i, seed * 1000 + i, nv, r, t))
    return out


class ServedObject:
    """One reconstruction: dataset views, field, optimiser state, occupancy grid."""

    def __init__(self, spec: ObjectSpec, device, batch: int = 512, step_size: float = 2.0 / 1024,
                 precision: str = "fp32"):
        self.spec = spec
        self.ready = None   # event after the object's last enqueued work (None: nothing pending)
        dev = torch.device(device)
        scene = scenes.random_scene(spec.seed)
        rig = scenes.ring_cameras(spec.n_views, spec.res, spec.res, radius=3.0, elevation_deg=20.0)
        self.ds = scenes.SyntheticDataset(scene, rig, dev)
        self.scene = scene
        enc = dict(otype="HashGrid", n_levels=16, n_features_per_level=2, log2_hashmap_size=spec.log2_table,
                   base_resolution=16, per_level_scale=1.447)
        torch.manual_seed(spec.seed)
        net = SDFNetwork(3, 16, 64, 1, skip_in=(-1,), bias=0.5, encoding_config=enc, input_concat=True).to(dev)
        var = SingleVarianceNetwork(0.3).to(dev)
        # no encoding cache: its n_levels x 8 bytes per point of step capacity
        # would more than double an object's device footprint
        cfg = TrainConfig(batch_size=batch, step_size=step_size, occ_update_freq=8, occ_warmup_steps=16,
                          increase_bandwidth_every=100, end_iter=5000, seed=spec.seed,
                          encoding_cache=False, precision=precision)
        self.tr = FusedTrainer(net, var, cfg, device=dev)
        self.graph = GraphStep(self.tr)
        self.renderer = NeuSRenderer(net, var)
        self.renderer.occupancy_grid = self.tr.grid
        self.renderer.sampling_step_size = step_size
        self.gen = torch.Generator(device=dev).manual_seed(spec.seed)
        self.resident = True
        self.last_used = 0.0
        self._host: dict = {}
        self._state, self._work = self._classify()
        self._sizes = [st.nbytes() for st in self._state], [st.nbytes() for st in self._work]
        self._nbytes = sum(self._sizes[0]) + sum(self._sizes[1])

    # ---- residency -------------------------------------------------------
    def _classify(self):
        """Storages holding persistent state (copied on offload) vs workspace."""
        tr, ds = self.tr, self.ds
        state_t = [tr.params, tr.exp_avg, tr.exp_avg_sq, tr.iter_dev, tr.lr_dev, tr.adam_step_dev,
                   tr.status, ds.normals, ds.masks, ds.kinv, ds.pose34, ds.pose_all, ds.intrinsics_all]
        state_t += list(tr.grid.buffers()) + list(tr.net.buffers())
        if tr.params_half is not None:
            state_t.append(tr.params_half)
        state, seen = [], set()
        for t in state_t:
            st = t.untyped_storage()
            if st.data_ptr() not in seen and t.is_cuda:
                seen.add(st.data_ptr())
                state.append(st)
        work = []
        for t in list(vars(tr).values()) + list(self.graph.inputs):
            if isinstance(t, torch.Tensor) and t.is_cuda:
                st = t.untyped_storage()
                if st.data_ptr() not in seen:
                    seen.add(st.data_ptr())
                    work.append(st)
        return state, work

    def nbytes(self) -> int:
        """Device bytes of the object when resident (fixed at construction)."""
        return self._nbytes

    def offload(self) -> None:
        if not self.resident:
            return
        if self.ready is not None:
            self.ready.synchronize()      # the object's own work, whichever stream ran it
        torch.cuda.current_stream().synchronize()
        for i, st in enumerate(self._state):
            if i not in self._host:     # pinned once per object, reused by every offload
                self._host[i] = torch.empty(st.nbytes(), dtype=torch.uint8, pin_memory=True)
            self._host[i].untyped_storage().copy_(st)
        for st in self._state + self._work:
            st.resize_(0)
        self.graph.invalidate()
        self.resident = False

    def onload(self) -> None:
        if self.resident:
            return
        ss, ws = self._sizes
        for st, n in zip(self._state, ss):
            st.resize_(n)
        for st, n in zip(self._work, ws):
            st.resize_(n)
        for i, st in enumerate(self._state):
            st.copy_(self._host[i].untyped_storage(), non_blocking=True)
        self.tr.grads.zero_()          # zero at rest (Adam consumes and clears them)
        self.graph.invalidate()
        self.resident = True

    def set_precision(self, precision: str) -> None:
        """Precision of the object's next training iterations (applied when it
        next trains, resident: the FP16 table copy is formed then)."""
        self._want_precision = precision

    def _apply_precision(self) -> None:
        want = getattr(self, "_want_precision", None)
        if want is None or want == self.tr.cfg.precision:
            return
        self.tr.set_precision(want)
        self.graph.invalidate()
        self._state, self._work = self._classify()
        self._sizes = [st.nbytes() for st in self._state], [st.nbytes() for st in self._work]
        self._nbytes = sum(self._sizes[0]) + sum(self._sizes[1])

    # ---- requests --------------------------------------------------------
    def train_iterations(self, n: int, graphs: bool) -> None:
        self._apply_precision()
        for _ in range(n):
            batch = self.ds.gen_random_patches(self.tr.B, generator=self.gen)
            if graphs:
                self.graph.step(batch)
            else:
                self.tr.train_step(*batch)

    @torch.no_grad()
    def render(self, pose_seed: int, chunk: int = 4096) -> torch.Tensor:
        """Normal map (H, W, 3) of the current field at a seeded new pose."""
        g = torch.Generator().manual_seed(pose_seed)
        az = float(torch.rand(1, generator=g)) * 2 * math.pi
        el = 10.0 + 30.0 * float(torch.rand(1, generator=g))
        rig = scenes.ring_cameras(1, self.spec.res, self.spec.res, radius=3.0, elevation_deg=el)
        c, s = math.cos(az), math.sin(az)
        rot = torch.tensor([[c, -s, 0.0, 0.0], [s, c, 0.0, 0.0], [0.0, 0.0, 1.0, 0.0], [0.0, 0.0, 0.0, 1.0]],
                           dtype=rig.poses.dtype)
        rig.poses = rot @ rig.poses
        dev = self.tr.device
        d, v = scenes.view_rays(rig, 0, dev)
        H = W = self.spec.res
        ph, pw = H // 3, W // 3
        blk = lambda t: t.reshape(ph, 3, pw, 3, *t.shape[2:]).transpose(1, 2).reshape(
            ph * pw, 3, 3, *t.shape[2:]).contiguous()
        rays_d = blk(d)
        vinv = blk(v)
        pose = rig.poses[0].to(dev).float()
        rays_o = pose[:3, 3].expand(rays_d.shape).contiguous()
        plane_n = pose[:3, 2].expand(rays_d.shape[0], 3).contiguous()
        out = torch.empty_like(rays_d)
        self.renderer.gradient_method = "dfd"
        jit = torch.Generator(device=dev).manual_seed(pose_seed)   # the request's own stratified jitter
        for a in range(0, rays_d.shape[0], chunk):
            b = min(a + chunk, rays_d.shape[0])
            near, far = near_far_from_sphere(rays_o[a:b, 1, 1].contiguous(), rays_d[a:b, 1, 1].contiguous())
            r = self.renderer.render(rays_o[a:b], rays_d[a:b], plane_n[a:b], near, far, vinv[a:b],
                                     mode="eval", generator=jit)
            out[a:b] = r["comp_normal"]
        return out.reshape(ph, pw, 3, 3, 3).transpose(1, 2).reshape(H, W, 3)

    @torch.no_grad()
    def query(self, res: int = 256) -> torch.Tensor:
        """SDF on a res^3 lattice over [-1, 1]^3 (models/renderer.py:9-24
        extract_fields; X first, Z fastest)."""
        return query_batch([self], res)[0]


@torch.no_grad()
def query_batch(objects: list, res: int = 256, slab_points: int = 1 << 22) -> list:
    """SDF lattices (res^3 over [-1, 1]^3) of several objects from shared
    lattice points, each slab one field launch over all objects' tables and
    MLPs (``sn_field_fwd_batch``, at most SN_FIELD_MAX_SEGMENTS objects)."""
    import ctypes as Ct

    import numpy as np

    from ._lib import SN_FIELD_MAX_SEGMENTS, FieldSegment, call, stream_handle

    if not 1 <= len(objects) <= SN_FIELD_MAX_SEGMENTS:
        raise ValueError(f"query_batch: 1..{SN_FIELD_MAX_SEGMENTS} objects")
    dev = objects[0].tr.device
    st = stream_handle()
    outs = [torch.empty((res, res, res), device=dev) for _ in objects]
    keep = []   # effective weights and descriptors live until the launches are enqueued
    for o in objects:
        net = o.tr.net
        w0, b0, w1, b1 = (t.detach().contiguous() for t in net.mlp_tensors())
        keep.append((w0, b0, w1, b1, net._mlp_desc(w0, b0, w1, b1)))
    per = max(1, slab_points // (res * res))
    x = torch.empty((min(per, res) * res * res, 3), device=dev)
    lo, hi = np.full(3, -1.0), np.full(3, 1.0)
    for i0 in range(0, res, per):
        ni = min(per, res - i0)
        n = ni * res * res
        call("sn_lattice_points", i0, ni, res, res, res, lo.ctypes.data, hi.ctypes.data, x, st)
        segs = (FieldSegment * len(objects))()
        for k, o in enumerate(objects):
            net = o.tr.net
            segs[k] = FieldSegment(n, x.data_ptr(), net.encoding.params.data_ptr(), Ct.pointer(net.encoding.desc),
                                   net.active_levels(), Ct.pointer(keep[k][4]), outs[k][i0:i0 + ni].data_ptr())
        call("sn_field_fwd_batch", len(objects), segs, 1, st)
    return outs


@dataclass
class Request:
    rid: int
    kind: str            # 'recon' | 'render' | 'query'
    obj: int
    arrival: float       # seconds after the start of the trace
    iters: int = 0       # recon: iterations left
    done_at: Optional[float] = None
    rays: int = 0


def poisson_trace(n_objects: int, duration: float, rate: float, seed: int = 0,
                  mix=(0.4, 0.35, 0.25), recon_iters: int = 100) -> list:
    """Seeded arrivals over ``duration`` seconds at ``rate`` per second."""
    g = torch.Generator().manual_seed(seed)
    t, out = 0.0, []
    while True:
        t += float(-math.log(1.0 - float(torch.rand(1, generator=g))) / rate)
        if t > duration:
            break
        u = float(torch.rand(1, generator=g))
        kind = "recon" if u < mix[0] else ("render" if u < mix[0] + mix[1] else "query")
        obj = int(torch.randint(0, n_objects, (1,), generator=g))
        out.append(Request(len(out), kind, obj, t, recon_iters if kind == "recon" else 0))
    return out


class Server:
    """Runs a request trace over ServedObjects under an HBM budget."""

    def __init__(self, objects: list, budget_bytes: int, query_res: int = 256, slice_iters: int = 10,
                 sync=None):
        self.objects = objects
        self.budget = budget_bytes
        self.query_res = query_res
        self.slice_iters = slice_iters
        self.swaps = 0
        self.max_batch = 4              # objects per batched SDF-grid query launch
        self.batched_queries = 0        # queries that joined another query's launches
        self.device = sync is None
        self.sync = torch.cuda.synchronize if sync is None else sync
        if self.device:
            self.mark = self._record_event
            self.wait = lambda ev: ev.synchronize()
            # requests on a higher-priority stream: when both streams have
            # work ready, the GPU schedules the request's blocks first, so a
            # render or query beside a reconstruction slice is slowed less
            self.recon_stream = torch.cuda.Stream(priority=0)
            self.req_stream = torch.cuda.Stream(priority=-1)
        else:                     # host-only tests: no device work to wait for
            self.mark = lambda: None
            self.wait = lambda ev: None
            self.recon_stream = self.req_stream = None

    @contextmanager
    def on(self, obj, stream):
        """Runs the enclosed work of ``obj`` on ``stream`` (None: the current
        stream) after the object's previous work, on any stream, and records
        the object's new event."""
        if not self.device:
            yield
            return
        stream = stream if stream is not None else torch.cuda.current_stream()
        with torch.cuda.stream(stream):
            if getattr(obj, "ready", None) is not None:
                stream.wait_event(obj.ready)
            yield
            ev = torch.cuda.Event()
            ev.record(stream)
            obj.ready = ev

    @contextmanager
    def on_many(self, objs, stream):
        """``on`` for work that reads several objects at once."""
        if not self.device:
            yield
            return
        with torch.cuda.stream(stream):
            for o in objs:
                if getattr(o, "ready", None) is not None:
                    stream.wait_event(o.ready)
            yield
            ev = torch.cuda.Event()
            ev.record(stream)
            for o in objs:
                o.ready = ev

    def done(self, obj) -> None:
        """Host waits for the object's last work (not for the other stream)."""
        if not self.device:
            self.sync()
        elif getattr(obj, "ready", None) is not None:
            obj.ready.synchronize()

    def query_batch(self, objs, res):
        if len(objs) == 1 or not self.device:
            for o in objs:
                o.query(res)
        else:
            query_batch(objs, res)

    @staticmethod
    def _record_event():
        ev = torch.cuda.Event()
        ev.record()
        return ev

    def resident_bytes(self) -> int:
        return sum(o.nbytes() for o in self.objects if o.resident)

    def admit(self, obj: ServedObject, now: float) -> None:
        """Make ``obj`` resident, offloading least recently used objects as needed."""
        obj.last_used = now
        if obj.resident:
            return
        need = obj.nbytes()
        for o in sorted((o for o in self.objects if o.resident), key=lambda o: o.last_used):
            if self.resident_bytes() + need <= self.budget:
                break
            o.offload()
            self.swaps += 1
        obj.onload()
        self.swaps += 1

    def fit_budget(self) -> None:
        """Initial admission: the first objects that fit stay resident."""
        used = 0
        for o in self.objects:
            if used + o.nbytes() <= self.budget:
                used += o.nbytes()
            else:
                o.offload()

    def run(self, trace: list, policy: str) -> dict:
        graphs = policy == "served"
        reqs = [Request(r.rid, r.kind, r.obj, r.arrival, r.iters) for r in trace]
        pending = deque(sorted(reqs, key=lambda r: r.arrival))
        recon_q: deque = deque()
        short_q: deque = deque()
        fifo: deque = deque()
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        busy = 0.0
        train_rays = render_rays = 0
        slice_done: list = []     # completion marks of queued reconstruction slices

        def arrive():
            while pending and pending[0].arrival <= now():
                r = pending.popleft()
                if policy == "plain":
                    fifo.append(r)
                elif r.kind == "recon":
                    recon_q.append(r)
                else:
                    short_q.append(r)

        def finish(r, obj):
            self.done(obj)
            r.done_at = now()

        while pending or recon_q or short_q or fifo:
            arrive()
            if policy == "plain":
                r = fifo.popleft() if fifo else None
            else:
                r = short_q.popleft() if short_q else (recon_q[0] if recon_q else None)
            if r is None:
                time.sleep(max(0.0, min(0.002, pending[0].arrival - now())) if pending else 0.0)
                continue
            s = now()
            obj = self.objects[r.obj]
            if policy != "plain" and r.kind == "query":
                # SDF-grid queries waiting for other resident objects join this
                # one's launches (one field launch per slab over all of them)
                group = [r]
                for q in list(short_q):
                    if (len(group) < self.max_batch and q.kind == "query" and self.objects[q.obj].resident
                            and all(self.objects[q.obj] is not self.objects[g.obj] for g in group)):
                        group.append(q)
                        short_q.remove(q)
                objs = [self.objects[g.obj] for g in group]
                with self.on_many(objs, self.req_stream):
                    for o in objs:
                        self.admit(o, s)
                    self.query_batch(objs, self.query_res)
                for g, o in zip(group, objs):
                    finish(g, o)
                self.batched_queries += len(group) - 1
                busy += now() - s
                continue
            if policy == "plain":
                stream = None                    # the current stream, one request at a time
            else:
                stream = self.recon_stream if r.kind == "recon" else self.req_stream
            with self.on(obj, stream):
                self.admit(obj, s)
                if r.kind == "recon":
                    k = r.iters if policy == "plain" else min(r.iters, self.slice_iters)
                    obj.train_iterations(k, graphs)
                    r.iters -= k
                    train_rays += k * obj.tr.B * obj.tr.P
                    if r.iters > 0 and policy != "plain":
                        # a slice ends without a host wait (the host looks at new
                        # arrivals while the GPU works), but at most two slices are
                        # queued on the reconstruction stream
                        slice_done.append(self.mark())
                        if len(slice_done) > 2:
                            self.wait(slice_done.pop(0))
                elif r.kind == "render":
                    img = obj.render(pose_seed=r.rid)
                    render_rays += img.shape[0] * img.shape[1]
                else:
                    obj.query(self.query_res)
            if r.kind != "recon" or r.iters == 0:
                finish(r, obj)
                if r.kind == "recon" and policy != "plain":
                    recon_q.popleft()
            busy += now() - s
        span = now()
        lat = {k: sorted(r.done_at - r.arrival for r in reqs if r.kind == k) for k in ("recon", "render", "query")}
        allv = sorted(r.done_at - r.arrival for r in reqs)

        def pct(v, p):
            if not v:
                return None
            i = min(len(v) - 1, max(0, int(math.ceil(p / 100.0 * len(v))) - 1))
            return 1e3 * v[i]

        return {
            "policy": policy, "requests": len(reqs), "makespan_s": span, "busy_s": busy,
            "batched_queries": self.batched_queries,
            "p50_ms": pct(allv, 50), "p99_ms": pct(allv, 99),
            "by_kind": {k: {"n": len(v), "p50_ms": pct(v, 50), "p99_ms": pct(v, 99)} for k, v in lat.items()},
            "rays_per_s": (train_rays + render_rays) / span if span > 0 else 0.0,
            "train_rays": train_rays, "render_rays": render_rays,
        }
