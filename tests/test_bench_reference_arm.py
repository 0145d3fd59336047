"""bench.py's reference arm (the CPU oracle of cctpy's field sum) on a tiny sample: the JSON
line it prints, and ranks other than 0 exiting without work."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_bench(env_extra, *args):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *args],
                          cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)


def test_reference_line():
    r = run_bench({}, "--steps", "2", "--warmup", "1", "--ref-points", "32")
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["steps"] == 2 and line["warmup"] == 1 and line["unit"] == "Gpairs/s"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["config"]["workload"].startswith("field_map")
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "Gpairs/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    # the rate follows from the sample: points x segments x steps over the timed seconds
    pairs = 32 * line["config"]["n_segments"] * 2
    assert abs(pairs / (2 * line["ms_per_step"] * 1e-3) / 1e9 - line["value"]) <= 1e-9 * line["value"]


def test_other_ranks_exit_without_work():
    r = run_bench({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}, "--gpus", "2", "--steps", "1",
                  "--warmup", "0", "--ref-points", "32")
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
