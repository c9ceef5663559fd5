"""The benchmark's reference arm runs on the host cores alone (the CPU restatement of the path on
the 256^3 headline workload), so its JSON contract is checked here without a GPU: one line with
the metric, unit, direction, config and the cpu_baseline / e2e objects; under a multi-rank
launch only rank 0 prints."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(extra_env=None, args=("--impl", "reference", "--steps", "3", "--warmup", "3")):
    env = dict(os.environ)
    env.update(extra_env or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=900)


def test_reference_arm_json_line():
    r = _run()
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.strip().splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"].startswith("D3Q19 MLUPS") and d["unit"] == "MLUPS" and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["steps"] == 3 and d["warmup"] >= 3 and d["dtype"] == "f32"
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["cells"] == 256 ** 3 and "256^3" in d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["unit"] == "MLUPS"
    assert d["e2e"] == {"value": d["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    r = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]


def test_help_lists_the_modes():
    r = _run(args=("--help",))
    assert r.returncode == 0
    for opt in ("--impl", "--gpus", "--steps", "--warmup", "--adjoint-only", "--precision-only", "--coupled-only",
                "--scale-only"):
        assert opt in r.stdout
