"""Host-side helpers of bench.py: stage intervals from graph-replay marks and
the per-stage algorithmic byte model."""
import numpy as np

import bench


class _Net:
    def active_levels(self):
        return 16


class _Tr:
    B, P, n_params = 2048, 9, 1000
    net = _Net()
    enc_cache = object()


def test_stage_times_from_replay_offsets():
    step = [("step_begin", 0.0), ("march_end", 0.2), ("cull_end", 0.35), ("field_fwd_begin", 0.4),
            ("field_fwd_end", 0.8), ("render_end", 1.0), ("field_bwd_begin", 1.0), ("field_bwd_end", 2.1),
            ("adam_begin", 2.15), ("adam_end", 2.25)]
    occ = [("occ_begin", 0.0), ("occ_end", 0.4)]
    t = bench.stage_times(step + step + occ)
    assert np.isclose(t["march"], 0.4) and np.isclose(t["field_bwd"], 2.2)
    assert np.isclose(t["expand"], 0.1) and np.isclose(t["occupancy"], 0.4)
    assert np.isclose(t["adam"], 0.2) and np.isclose(t["render"], 0.4)


def test_stage_rooflines_byte_model():
    stages = {"march": 1.0, "render": 1.0, "adam": 1.0, "field_fwd": 2.0, "field_bwd": 4.0}
    q = np.array([1000.0, 1000.0])
    samples = np.array([[500.0, 100.0], [500.0, 100.0]])
    out = bench.stage_rooflines(stages, q, samples, _Tr(), 1000.0, 2)
    # 16 B per marched sample + 8 B per ray; 36 B per patch-pixel sample + 16 B per pixel
    assert np.isclose(out["march"]["bytes_per_step"], 500 * 16 + 2048 * 8)
    assert np.isclose(out["render"]["bytes_per_step"], 100 * 9 * 36 + 2048 * 9 * 16)
    assert np.isclose(out["adam"]["bytes_per_step"], 1000 * 32)
    # with the encoding cache both field kernels move 1,168 B per point at L=16
    assert np.isclose(out["field_fwd"]["bytes_per_step"], 1000 * 1168)
    assert np.isclose(out["field_bwd"]["bytes_per_step"], 1000 * 1168)
    gbs = out["field_bwd"]["achieved_gbs"]
    assert np.isclose(gbs, 2000 * 1168 / (4.0 / 1e3) / 1e9) and np.isclose(out["field_bwd"]["frac"], gbs / 1000.0)
    assert bench.stage_rooflines(stages, None, None, _Tr(), 1000.0, 2) is None


def test_stage_rooflines_rejects_mismatched_steps():
    """Sample counts and field points must cover the same steps (a warm-up
    step left in one of them would scale the byte model wrongly)."""
    import pytest

    stages = {"march": 1.0, "render": 1.0, "adam": 1.0, "field_fwd": 2.0, "field_bwd": 4.0}
    q = np.full(20, 1000.0)
    samples = np.full((25, 2), 100.0)
    with pytest.raises(ValueError):
        bench.stage_rooflines(stages, q, samples, _Tr(), 1000.0, 20)


def test_reference_arm_prints_its_line():
    """bench.py --impl reference (the CPU restatement on host cores) prints one
    JSON line with the contract's keys."""
    import json
    import os
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', "
            "'--cpu-sample-patches', '2']; runpy.run_path('bench.py', run_name='__main__'); "
            "print('PKG_LOADED', any(m.startswith('supernormal_gb300') for m in sys.modules))")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    assert "PKG_LOADED False" in r.stdout          # the reference arm imports nothing from the package
    assert line["impl"] == "reference" and line["metric"] == "train_rays_per_s" and line["value"] > 0
    assert line["dtype"] == "f32" and line["state"]["samples_per_ray"]["marched"] > 0
    assert line["config"] == bench.workload_config(bench.parse([]), 1)
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["higher_is_better"] is True and line["vs_baseline"] > 0
