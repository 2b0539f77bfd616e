"""CUDA-graph training step and the serving loop (GPU)."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_graph_step_matches_eager(built_lib):
    """The captured iteration gives the eager iteration's loss (the forward is
    deterministic; later steps differ only by float atomics order)."""
    from supernormal_gb300 import scenes
    from supernormal_gb300.fields import SDFNetwork, SingleVarianceNetwork
    from supernormal_gb300.trainer import FusedTrainer, GraphStep, TrainConfig

    ds = scenes.SyntheticDataset(scenes.sphere(0.5), scenes.ring_cameras(6, 96, 96, elevation_deg=20),
                                 torch.device("cuda"))
    enc = dict(otype="HashGrid", n_levels=16, n_features_per_level=2, log2_hashmap_size=15,
               base_resolution=16, per_level_scale=1.447)

    def make():
        torch.manual_seed(0)
        net = SDFNetwork(3, 16, 64, 1, skip_in=(-1,), bias=0.5, encoding_config=enc, input_concat=True).cuda()
        var = SingleVarianceNetwork(0.3).cuda()
        cfg = TrainConfig(batch_size=128, step_size=1.0 / 96, occ_update_freq=4, occ_warmup_steps=4,
                          increase_bandwidth_every=0, end_iter=100, seed=3)
        net.bindwidth = 16
        return FusedTrainer(net, var, cfg)

    g = torch.Generator(device="cuda").manual_seed(1)
    batches = [ds.gen_random_patches(128, generator=g) for _ in range(12)]
    eager, graphed = make(), make()
    gs = GraphStep(graphed)
    le, lg = [], []
    for b in batches:
        le.append(eager.train_step(*b).clone())
        lg.append(gs.step(b).clone())
    torch.cuda.synchronize()
    eager.check_status()
    graphed.check_status()
    assert torch.equal(le[0], lg[0])
    for a, b in zip(le, lg):
        assert torch.allclose(a, b, rtol=2e-3, atol=1e-6), (a, b)
    assert gs._steps[0] is not None and gs._occ is not None


def test_graph_step_follows_step_size_schedule(built_lib):
    """The reference's log step-size schedule (exp_runner.py:81-83,149;
    1e-2 -> 1e-3) as graph replays: the marcher reads the step the schedule
    kernel writes from the device iteration counter, so 20 iterations need
    one captured iteration, and they train like the eager iterations, whose
    marcher takes the same device-side step."""
    from supernormal_gb300 import scenes
    from supernormal_gb300.fields import SDFNetwork, SingleVarianceNetwork
    from supernormal_gb300.trainer import FusedTrainer, GraphStep, TrainConfig

    ds = scenes.SyntheticDataset(scenes.sphere(0.5), scenes.ring_cameras(6, 96, 96, elevation_deg=20),
                                 torch.device("cuda"))
    enc = dict(otype="HashGrid", n_levels=16, n_features_per_level=2, log2_hashmap_size=15,
               base_resolution=16, per_level_scale=1.447)

    def make():
        torch.manual_seed(0)
        net = SDFNetwork(3, 16, 64, 1, skip_in=(-1,), bias=0.5, encoding_config=enc, input_concat=True).cuda()
        var = SingleVarianceNetwork(0.3).cuda()
        cfg = TrainConfig(batch_size=128, start_step_size=1e-2, end_step_size=1e-3, end_iter=20,
                          occ_update_freq=0, increase_bandwidth_every=0, warm_up_end=2, seed=3)
        net.bindwidth = 16
        tr = FusedTrainer(net, var, cfg)
        tr.grid._binary = torch.ones_like(tr.grid._binary)   # every cell occupied: no updates needed
        return tr

    g = torch.Generator(device="cuda").manual_seed(1)
    batches = [ds.gen_random_patches(128, generator=g) for _ in range(20)]
    eager, graphed = make(), make()
    gs = GraphStep(graphed)
    le, lg, marched, steps = [], [], [], []
    for i, b in enumerate(batches):
        le.append(eager.train_step(*b).clone())
        marched.append(int(eager.total0.item()))
        steps.append(float(eager.dt_dev.item()))
        lg.append(gs.step(b).clone())
    torch.cuda.synchronize()
    eager.check_status()
    graphed.check_status()
    assert gs.captures == 1
    # the device schedule is the host schedule rounded once to float
    import numpy as np

    want = [np.float32(eager.step_size(i)) for i in range(20)]
    assert steps == [float(w) for w in want]
    assert marched[-1] > 3 * marched[0]       # finer steps march more samples
    assert torch.equal(le[0], lg[0])
    for a, b in zip(le, lg):
        assert torch.allclose(a, b, rtol=2e-3, atol=1e-6), (a, b)


def test_graph_step_profile_marks(built_lib):
    """Profiled graph replays (three copies with captured stage events) report
    every step's stage marks in order, its field-point count and the kernels
    replayed, and train like the eager iteration."""
    from supernormal_gb300 import scenes
    from supernormal_gb300.fields import SDFNetwork, SingleVarianceNetwork
    from supernormal_gb300.trainer import FusedTrainer, GraphStep, TrainConfig

    ds = scenes.SyntheticDataset(scenes.sphere(0.5), scenes.ring_cameras(6, 96, 96, elevation_deg=20),
                                 torch.device("cuda"))
    enc = dict(otype="HashGrid", n_levels=16, n_features_per_level=2, log2_hashmap_size=15,
               base_resolution=16, per_level_scale=1.447)

    def make():
        torch.manual_seed(0)
        net = SDFNetwork(3, 16, 64, 1, skip_in=(-1,), bias=0.5, encoding_config=enc, input_concat=True).cuda()
        var = SingleVarianceNetwork(0.3).cuda()
        cfg = TrainConfig(batch_size=128, step_size=1.0 / 96, occ_update_freq=4, occ_warmup_steps=4,
                          increase_bandwidth_every=0, end_iter=100, seed=3)
        net.bindwidth = 16
        return FusedTrainer(net, var, cfg)

    g = torch.Generator(device="cuda").manual_seed(1)
    batches = [ds.gen_random_patches(128, generator=g) for _ in range(10)]
    eager, graphed = make(), make()
    for b in batches[:4]:                      # occupancy warm-up runs eagerly in both
        eager.train_step(*b)
        graphed.train_step(*b)
    gs = GraphStep(graphed, profile=True)
    gs.prepare()
    le, lg = [], []
    for b in batches[4:]:
        le.append(eager.train_step(*b).clone())
        lg.append(gs.step(b).clone())
    gs.flush()
    eager.check_status()
    graphed.check_status()
    for a, b in zip(le, lg):
        assert torch.allclose(a, b, rtol=2e-3, atol=1e-6), (a, b)
    steps = [m for m in gs.stage_marks if m[0][0] == "step_begin"]
    assert len(steps) == 6 and len(gs.points) == 6 and all(p > 0 for p in gs.points)
    tags = [t for t, _ in steps[0]]
    assert tags.index("field_fwd_begin") < tags.index("field_bwd_begin") < tags.index("adam_end")
    for m in steps:
        ts = [t for _, t in m]
        assert all(b >= a for a, b in zip(ts, ts[1:])) and ts[-1] > 0.0
    assert any(m[0][0] == "occ_begin" for m in gs.stage_marks)   # the occupancy graph's own marks
    assert gs.launches > 6 * 10


def test_host_prefetcher_matches_device_batches(built_lib):
    """Batches fed from pinned host memory through HostPrefetcher (copies on a
    side stream, two device slots) give the losses of device-resident batches."""
    from supernormal_gb300 import scenes
    from supernormal_gb300.fields import SDFNetwork, SingleVarianceNetwork
    from supernormal_gb300.trainer import FusedTrainer, HostPrefetcher, TrainConfig

    ds = scenes.SyntheticDataset(scenes.sphere(0.5), scenes.ring_cameras(6, 96, 96, elevation_deg=20),
                                 torch.device("cuda"))
    enc = dict(otype="HashGrid", n_levels=16, n_features_per_level=2, log2_hashmap_size=15,
               base_resolution=16, per_level_scale=1.447)

    def make():
        torch.manual_seed(0)
        net = SDFNetwork(3, 16, 64, 1, skip_in=(-1,), bias=0.5, encoding_config=enc, input_concat=True).cuda()
        var = SingleVarianceNetwork(0.3).cuda()
        cfg = TrainConfig(batch_size=128, step_size=1.0 / 96, occ_update_freq=4, occ_warmup_steps=4,
                          increase_bandwidth_every=0, end_iter=100, seed=3)
        net.bindwidth = 16
        return FusedTrainer(net, var, cfg)

    g = torch.Generator(device="cuda").manual_seed(1)
    batches = [ds.gen_random_patches(128, generator=g) for _ in range(7)]
    host = [tuple(t.cpu().pin_memory() for t in b) for b in batches]
    direct, fed = make(), make()
    pf = HostPrefetcher(fed, host[0])
    pf.put(host[0])
    ld, lf = [], []
    for i, b in enumerate(batches):
        ld.append(direct.train_step(*b).clone())
        lf.append(pf.step(host[i + 1] if i + 1 < len(host) else None).clone())
    torch.cuda.synchronize()
    direct.check_status()
    fed.check_status()
    assert torch.equal(ld[0], lf[0])
    for a, b in zip(ld, lf):
        assert torch.allclose(a, b, rtol=2e-3, atol=1e-6), (a, b)
    with pytest.raises(RuntimeError):
        pf.step()                      # every put() batch was consumed


def test_serving_loop_small_trace(built_lib):
    from supernormal_gb300.serve import ServedObject, Server, object_specs, poisson_trace

    specs = object_specs(3, seed=1, views=(6, 8), res=(96, 120), log2_table=(15, 16))
    objs = [ServedObject(s, "cuda", batch=128, step_size=1.0 / 96) for s in specs]
    budget = objs[0].nbytes() + objs[1].nbytes()         # two of three fit: forces offloads
    trace = poisson_trace(3, duration=1.5, rate=8.0, seed=2, recon_iters=12)
    assert len(trace) > 4
    srv = Server(objs, budget, query_res=64, slice_iters=4)
    srv.fit_budget()
    assert srv.resident_bytes() <= budget
    res = srv.run(trace, "served")
    assert res["requests"] == len(trace) and res["p50_ms"] is not None and res["p99_ms"] >= res["p50_ms"]
    assert srv.resident_bytes() <= budget
    assert srv.swaps > 0
    res_plain = Server(objs, budget, query_res=64).run(trace, "plain")
    assert res_plain["requests"] == len(trace)
    for o in objs:
        if o.resident:
            o.tr.check_status()
    # an offloaded object comes back with its state intact
    o = objs[0]
    if not o.resident:
        o.onload()
    p = o.tr.params.clone()
    o.offload()
    o.onload()
    assert torch.equal(p, o.tr.params)


def test_requests_same_alone_and_in_the_mix(built_lib):
    """A render (its stratified jitter seeded by the request) and an SDF query
    give bit-identical results alone and running on the request stream while
    another object's training slices run on the reconstruction stream, as the
    served policy runs them; training with those requests alongside matches
    training alone (atomics order aside)."""
    from supernormal_gb300.serve import ServedObject, object_specs

    specs = object_specs(2, seed=3, views=(6, 6), res=(96, 96), log2_table=(15, 15))
    a, b, b_alone = (ServedObject(s, "cuda", batch=128, step_size=1.0 / 96) for s in (specs[0], specs[1], specs[1]))
    for o in (a, b, b_alone):
        o.train_iterations(6, False)          # past the occupancy warm-up
    torch.cuda.synchronize()
    img_alone = a.render(pose_seed=7).clone()
    q_alone = a.query(48).clone()
    la, lb = [], []
    for _ in range(3):
        b_alone.train_iterations(4, True)
        la.append(b_alone.tr.loss_out.clone())
    # as the served policy runs them: b's slices on the reconstruction stream,
    # a's requests on the request stream, concurrently on the device
    from supernormal_gb300.serve import Server

    srv = Server([a, b], budget_bytes=1 << 50)
    for i in range(3):
        with srv.on(b, srv.recon_stream):
            b.train_iterations(4, True)
            lb.append(b.tr.loss_out.clone())
        if i == 0:
            with srv.on(a, srv.req_stream):
                img_mix = a.render(pose_seed=7)
                q_mix = a.query(48)
    torch.cuda.synchronize()
    assert torch.equal(img_alone, img_mix)
    assert torch.equal(q_alone, q_mix)
    assert torch.equal(a.render(pose_seed=7), img_alone)
    for x, y in zip(la, lb):
        assert torch.allclose(x, y, rtol=2e-3, atol=1e-6), (x, y)


def test_query_batch_matches_per_object(built_lib):
    """One field launch over several objects' tables and MLPs per slab
    (sn_field_fwd_batch) gives each object's SDF lattice bit for bit as its
    own launch does, including objects with different active levels and a
    lattice split over several slabs."""
    import numpy as np

    from supernormal_gb300._lib import call, stream_handle
    from supernormal_gb300.serve import ServedObject, object_specs, query_batch

    specs = object_specs(3, seed=5, views=(6, 6, 6), res=(64, 64, 64), log2_table=(14, 15, 15))
    objs = [ServedObject(s, "cuda", batch=128, step_size=1.0 / 64) for s in specs]
    objs[0].train_iterations(5, False)
    objs[2].train_iterations(9, False)
    objs[1].tr.net.bindwidth = 7
    res = 40
    x = torch.empty((res ** 3, 3), device="cuda")
    lo, hi = np.full(3, -1.0), np.full(3, 1.0)
    call("sn_lattice_points", 0, res, res, res, res, lo.ctypes.data, hi.ctypes.data, x, stream_handle())
    want = [o.tr.net.sdf_raw(x).reshape(res, res, res) for o in objs]
    got = query_batch(objs, res, slab_points=11 * res * res)     # 4 slabs, the last one ragged
    torch.cuda.synchronize()
    for o in objs:
        o.tr.net.check_status()
    for w, g in zip(want, got):
        assert torch.equal(w, g)
    assert not torch.equal(got[0], got[1])
    one = query_batch(objs[2:], res)
    assert torch.equal(one[0], want[2])


def test_trainer_check_status_reports_each_condition(built_lib):
    """The trainer's status word (OR-ed by its kernels) surfaces on the host:
    each SN_STATUS bit raises its own error from check_status, and a clean
    word raises nothing."""
    from supernormal_gb300._lib import SN_STATUS_CAPACITY, SN_STATUS_MARCH_LIMIT, SN_STATUS_TIMEOUT
    from supernormal_gb300.fields import SDFNetwork, SingleVarianceNetwork
    from supernormal_gb300.trainer import FusedTrainer, TrainConfig

    enc = dict(otype="HashGrid", n_levels=16, n_features_per_level=2, log2_hashmap_size=15,
               base_resolution=16, per_level_scale=1.447)
    net = SDFNetwork(3, 16, 64, 1, skip_in=(-1,), bias=0.5, encoding_config=enc, input_concat=True).cuda()
    tr = FusedTrainer(net, SingleVarianceNetwork(0.3).cuda(), TrainConfig(batch_size=32, step_size=1.0 / 64))
    tr.status.zero_()
    tr.check_status()
    for bit, words in ((SN_STATUS_MARCH_LIMIT, "iteration limit"), (SN_STATUS_CAPACITY, "capacity"),
                       (SN_STATUS_TIMEOUT, "timed out")):
        tr.status.fill_(bit)
        with pytest.raises(RuntimeError, match=words):
            tr.check_status()
    tr.status.zero_()
