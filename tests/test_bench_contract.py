"""bench.py's reference arm on the CPU: one JSON line with the keys of the bench
contract (metric, value, unit, n_gpus, steps, warmup, ms_per_step, higher_is_better,
scaling, vs_baseline, dtype, data, config, e2e, cpu_baseline, impl), on a small
bounded sample; ranks other than 0 print nothing and exit 0."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ["--impl", "reference", "--steps", "1", "--warmup", "0", "--points", "2000", "--cpu-rotations", "1",
        "--cpu-iters", "1"]


def _run(env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *ARGS], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    return [l for l in r.stdout.splitlines() if l.strip()]


def test_reference_arm_prints_one_contract_line():
    lines = _run()
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "e2e", "cpu_baseline"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["unit"] == "registrations/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and abs(d["ms_per_step"] - 1000.0 / d["value"]) <= 1e-3 * d["ms_per_step"] + 1e-3
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert "workload" in d["config"]


def test_reference_arm_other_ranks_are_silent():
    assert _run({"RANK": "1", "WORLD_SIZE": "2"}) == []


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
    v = bench._profile_value("k_assoc_cta_global50k.md", "warp_instructions_per_pair_launch")
    assert v is not None and v > 1e8
