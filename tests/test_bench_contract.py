"""bench.py on the CPU.

* The reference arm: one JSON line with the keys of the bench contract (metric, value,
  unit, n_gpus, steps, warmup, ms_per_step, higher_is_better, scaling, vs_baseline,
  dtype, data, config, e2e, cpu_baseline, impl) on a small bounded sample; ranks other
  than 0 print nothing and exit 0.
* The roofline helpers' arithmetic.
* The GPU arm's own Python with CUDA and the GPU API faked (contract keys only)."""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ["--impl", "reference", "--steps", "2", "--warmup", "1", "--points", "2000", "--pairs", "2",
        "--ref-sample-iters", "1"]


def _weights(tmp_path):
    """Network weights of the right size for the CPU pipeline (random: the contract only)."""
    sys.path.insert(0, ROOT)
    from oracle import proposal as op
    path = str(tmp_path / "w.npy")
    np.save(path, (np.random.default_rng(0).normal(size=op.NUM_PARAMS) * 0.05).astype(np.float32))
    return path


def _run(tmp_path, env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *ARGS, "--proposal-weights", _weights(tmp_path)],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return [l for l in r.stdout.splitlines() if l.strip()]


def test_reference_arm_prints_one_contract_line(tmp_path):
    """The reference arm: the workload's pipeline on the host cores through the oracle,
    with the GPU arm's config; ms_per_step is the measured wall time of a step, the value
    is derived from measured per-phase times, and the product library is never loaded."""
    lines = _run(tmp_path)
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "e2e", "cpu_baseline"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["unit"] == "registrations/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["steps"] == 2 and d["warmup"] == 1
    full = d["full_registrations"]
    assert len(full) == 2 and all(f["iterations"] >= 1 and f["seconds"] > 0 for f in full)
    assert abs(d["value"] - 2 / sum(f["seconds"] for f in full)) <= 1e-3 * d["value"]
    m = d["measured"]
    assert m["cos_angles_per_s"] > 0 and m["align_iterations_per_s"] > 0
    assert d["config"]["pairs_per_step"] == 2 and d["config"]["points_per_cloud"] == 2000
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert "workload" in d["config"]


def test_reference_arm_other_ranks_are_silent(tmp_path):
    assert _run(tmp_path, {"RANK": "1", "WORLD_SIZE": "2"}) == []


def test_reference_arm_loads_no_product_library(tmp_path):
    """The CPU pipeline of the reference arm maps the oracle's library, never the
    product's (parameters from the oracle's yaml reader, weights from a file)."""
    code = ("import sys, json, argparse; sys.path.insert(0, %r); import bench;"
            "a = argparse.Namespace(refine_ell=0.4, proposal_weights=%r);"
            "cl = bench.CpuLearned(a); from rkhs_ba_gb300 import scenes;"
            "pair = scenes.global_pair(1500, 7); T, it, t = cl.register(pair, max_iter=2);"
            "maps = open('/proc/self/maps').read();"
            "print(json.dumps({'product': 'libcvo_gb300' in maps, 'oracle': 'libcvo_oracle' in maps, 'it': it}))"
            % (ROOT, _weights(tmp_path)))
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert d["oracle"] and not d["product"] and 1 <= d["it"] <= 2


def test_issue_roofline_arithmetic():
    sys.path.insert(0, ROOT)
    import bench
    # 2 pair-passes over 1 launch of 1 ms, 1e6 warp instructions per pair; 152 SMs at 2000 MHz
    r = bench.issue_roofline(1e6, 2, 1, 1e-3, 152, 2000.0)
    assert r["warp_instructions_per_launch"] == 2000000
    assert r["achieved"] == 2.0                        # 2e6 / 1e-3 s = 2 G warp instructions / s
    assert r["peak"] == 1216.0                         # 152 x 4 x 2.0 GHz
    assert abs(r["frac"] - 2.0 / 1216.0) < 1e-4
    assert bench.issue_roofline(None, 2, 1, 1e-3, 152, 2000.0) is None
    assert bench.issue_roofline(1e6, 0, 1, 1e-3, 152, 2000.0) is None
    assert bench.issue_roofline(1e6, 2, 1, 1e-3, None, 2000.0) is None
    v = bench._capture_value("warp_instructions_per_pair_launch")
    assert v is not None and v > 1e8


_FAKE_GPU_CHILD = r"""
import json, sys
import numpy as np


def main():
    sys.path.insert(0, sys.argv[1])
    import torch
    import bench
    import rkhs_ba_gb300

    class FakeStream:
        cuda_stream = 0

    class FakeEvent:
        clock = 0.0

        def __init__(self, enable_timing=True):
            self.t = 0.0

        def record(self, stream=None):
            FakeEvent.clock += 25.0
            self.t = FakeEvent.clock

        def synchronize(self):
            pass

        def elapsed_time(self, other):
            return other.t - self.t

    class Props:
        multi_processor_count = 152

    torch.cuda.set_device = lambda i: None
    torch.cuda.Stream = lambda: FakeStream()
    torch.cuda.set_stream = lambda s: None
    torch.cuda.Event = FakeEvent
    torch.cuda.synchronize = lambda *a: None
    torch.cuda.get_device_properties = lambda i: Props()
    real_empty = torch.empty
    torch.empty = lambda *a, device=None, **k: real_empty(*a, **k)

    class FakeCloud:
        def __init__(self, c):
            self.c = c

        def free(self):
            pass

    class FakeNet:
        num_hyp, num_params = 8, 93704

        def hypotheses(self, gs, gt):
            return np.tile(np.eye(4, dtype=np.float32), (len(gs), 8, 1, 1))

        def weights(self):
            return np.zeros(self.num_params, np.float32)

    class FakeCvo:
        rotation_grid = staticmethod(rkhs_ba_gb300.CvoGPU.rotation_grid)

        def __init__(self, params=None):
            self.p, self.n = params, 0

        def set_stream(self, s):
            pass

        def upload(self, c):
            return FakeCloud(c)

        def register_learned_batch(self, net, gs, gt, n_refine=1, fallback_cos=0.0, refine_ell=0.0):
            self.n += 100
            k = len(gs)
            return np.tile(np.eye(4), (k, 1, 1)), np.ones(k), np.zeros(k, np.int32), np.full(k, 60), 0.1

        def get_nearest_init_pose(self, s, t, ell, num_guess, kind):
            return np.eye(4), 0.0

        def align_batch(self, gs, gt, inits):
            k = len(gs)
            return np.tile(np.eye(4), (k, 1, 1)), np.zeros(k, np.int32), np.full(k, 250), 0.1

        def inner_product_batch(self, s, t, Ts, ell):
            return np.ones(len(Ts), np.float32)

        def register_hypotheses(self, s, t, Ts, ell):
            return np.eye(4), 0, np.ones(len(Ts)), 0.1

        def autotune(self, s, t, T, ell=0.0, reps=3):
            return {"configs": [(4.0, 8.0, 0, 2.0), (6.0, 4.0, 0, 1.9), (6.0, 4.0, 2, 1.8)], "best": 2}

        def profile(self, on=True):
            pass

        def profile_reset(self):
            pass

        @property
        def kernel_launches(self):
            return self.n

        def profile_read(self):
            return {"assoc_ms": 400.0, "assoc_launches": 80, "assoc_bytes": 4.9e8 * 80, "iterations": 60,
                    "kernel_ms": {"transform": 1.0, "assoc": 400.0, "reduce": 5.0, "step": 50.0, "iteration": 456.0}}

    class FakeClocks:
        def __init__(self, index=0):
            pass

        def start(self):
            pass

        def stop(self):
            return {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 10}

    rkhs_ba_gb300.CvoGPU = FakeCvo
    bench._proposal = lambda args, cvo: (FakeNet(), {"fake": True})
    bench.ClockSampler = FakeClocks
    sys.argv = ["bench.py"] + (sys.argv[3:] or ["--pairs", "2", "--points", "2000", "--steps", "3", "--warmup", "3",
                                                "--all24-pairs", "1"]) + ["--proposal-weights", sys.argv[2]]
    bench.main()



if __name__ == "__main__":
    main()
"""


def test_ours_arm_json_with_a_faked_gpu(tmp_path):
    """bench.py's own Python for the GPU arm (timing loops, replica rate, e2e, roofline with
    traffic and issue fractions, CPU baseline, JSON) run with CUDA and the library's GPU
    API replaced by fakes: every contract key is present.  The numbers are meaningless;
    the kernels are covered by the gpu-marked tests."""
    script = tmp_path / "fake_gpu_bench.py"
    script.write_text(_FAKE_GPU_CHILD)
    r = subprocess.run([sys.executable, str(script), ROOT, _weights(tmp_path)], cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    d = json.loads([l for l in r.stdout.splitlines() if l.strip()][-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "e2e", "gpu_launches", "roofline", "cpu_baseline", "clocks"):
        assert k in d, k
    assert d["n_gpus"] == 1 and d["steps"] == 3 and d["warmup"] == 3
    roof = d["roofline"]
    assert roof["bound"] == "hbm" and roof["frac"] > 0 and roof["traffic"] > 0
    assert roof["issue"]["frac"] > 0 and roof["issue"]["peak"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] > 0 and d["e2e"]["d2h_bytes_per_step"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] > 0


def test_global_eval_component_with_a_faked_gpu(tmp_path):
    """bench.py --component global-eval (held-out evaluation, learned vs plain grid) runs
    its own Python end to end with the GPU faked: batches, success rates, JSON."""
    script = tmp_path / "fake_gpu_bench.py"
    script.write_text(_FAKE_GPU_CHILD)
    r = subprocess.run([sys.executable, str(script), ROOT, _weights(tmp_path), "--component", "global-eval", "--eval-pairs", "5",
                        "--pairs", "2", "--points", "2000"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    d = json.loads([l for l in r.stdout.splitlines() if l.strip()][-1])
    assert d["component"] == "global-eval" and d["pairs"] == 5
    assert d["config"]["seeds"] == [5000, 5004]
    for m in ("learned", "plain_grid"):
        assert d[m]["value"] > 0 and 0.0 <= d[m]["success_rate"] <= 1.0
    assert d["learned_over_plain_grid"] > 0


def test_batching_component_with_a_faked_gpu(tmp_path):
    """bench.py --component batching (one persistent batch against one call per
    registration, for uneven pairs and for the 24 grid hypotheses) with the GPU faked."""
    script = tmp_path / "fake_gpu_bench.py"
    script.write_text(_FAKE_GPU_CHILD)
    r = subprocess.run([sys.executable, str(script), ROOT, _weights(tmp_path), "--component", "batching", "--pairs", "2", "--points", "2000",
                        "--steps", "1", "--warmup", "1"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    d = json.loads([l for l in r.stdout.splitlines() if l.strip()][-1])
    assert d["component"] == "batching"
    assert d["legs"]["pairs"]["registrations"] == 2 and d["legs"]["hypotheses"]["registrations"] == 24
    assert all(20000 <= n <= 60000 for n in d["config"]["pairs_points"])
    for leg in d["legs"].values():
        assert leg["speedup"] > 0 and leg["identical_results"] is True
