"""The benchmark's JSON line, checked on the CPU through its reference arm
(the oracle timed on the host cores): one line with the metric, the
throughput, the step timing, the CPU-baseline and end-to-end objects, and the
workload it ran.  Under a multi-rank launch only rank 0 prints."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _run_reference_arm(env_extra=None):
    env = dict(os.environ, **(env_extra or {}))
    cmd = [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0",
           "--width", "48", "--height", "27", "--aa", "1"]
    return subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)


def test_reference_arm_prints_one_contract_line():
    p = _run_reference_arm()
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, p.stdout
    line = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["unit"] == "Mrays/s" and line["higher_is_better"] is True
    assert line["n_gpus"] == 1 and line["steps"] == 1 and line["warmup"] == 0
    assert line["value"] > 0 and line["ms_per_step"] > 0
    cfg = line["config"]
    assert (cfg["width"], cfg["height"], cfg["aa"]) == (48, 27, 1)
    assert cfg["workload"].endswith("_resized_to_48x27_aa1")
    cpu = line["cpu_baseline"]
    assert cpu["kind"] in ("port", "reference") and cpu["cores"] >= 1 and cpu["value"] == line["value"]
    assert cpu["unit"] == line["unit"] and cpu["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_without_work():
    p = _run_reference_arm({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.strip() == ""


def test_flop_model_against_hand_counts():
    """flop_count: each counted event times its FP32 operation count."""
    sys.path.insert(0, str(ROOT))
    import bench
    from forgedthoughts_gb300 import _native

    s = _native.RenderStatsC()
    s.box_tests, s.primitive_evals, s.march_steps = 3, 2, 5
    s.blend_ops, s.candidate_entries, s.hook_instrs = 1, 4, 7
    # 3 boxes x 15 + 2 primitives x 34 + 5 steps x 12 + 1 blend x 10 + 4 entries x 3 + 7 hook ops
    assert bench.flop_count(s) == 45 + 68 + 60 + 10 + 12 + 7
    s2 = _native.RenderStatsC()
    assert bench.flop_count(s2) == 0
