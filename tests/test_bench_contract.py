"""bench.py's reference arm on the CPU: one JSON line with the contract's keys (the same metric,
unit and workload config as the GPU arm, impl "reference", cpu_baseline and e2e with no host
transfers), and under a multi-rank launch only rank 0 prints."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ["--impl", "reference", "--n", "32", "--nt", "2", "--n-gauss", "8", "--steps", "1",
        "--warmup", "0"]


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *ARGS], cwd=ROOT,
                          env=env, capture_output=True, text=True, timeout=600)


def test_reference_arm_prints_one_contract_line():
    r = _run({"WORLD_SIZE": "1", "RANK": "0"})
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["unit"] == "gradient evals/s" and d["steps"] == 1 and d["warmup"] == 0
    assert d["config"]["n"] == 32 and "workload" in d["config"]
    # the config is the workload only (the same dict the GPU arm prints), the arm is named outside
    sys.path.insert(0, ROOT)
    import bench

    class A:
        n, nt, n_gauss = 32, 2, 8
    assert d["config"] == bench.workload_config(A)
    assert "arm" not in d["config"] and d["arm"]
    # each step is one full oracle evaluation at nt_per_step steps; value extrapolates it
    ex = d["extrapolated"]
    assert ex["nt_per_step"] == 1 and ex["nt_per_evaluation"] == 2
    assert abs(1.0 / d["value"] - d["ms_per_step"] * 1e-3 * 2) <= 1e-9 / d["value"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_print_nothing():
    r = _run({"WORLD_SIZE": "2", "RANK": "1"})
    assert r.returncode == 0, r.stderr
    assert not [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
