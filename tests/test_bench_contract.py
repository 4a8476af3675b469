"""bench.py's reference arm (no GPU needed): the reference's CPU path, timed as
the oracle restatement on the host cores, prints exactly one JSON line with
the same metric and unit as the GPU arm, `impl: reference`, a cpu_baseline
describing the run and an e2e object with no host-device traffic; ranks
other than 0 (torchrun) exit 0 without work or output."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(extra_env=None):
    env = dict(os.environ, **(extra_env or {}))
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                           "--workload", "plate_cavity_small", "--steps", "2", "--warmup", "3"],
                          capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)


def test_reference_arm_prints_one_contract_line():
    run = _run()
    assert run.returncode == 0, run.stderr
    lines = [ln for ln in run.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    sys.path.insert(0, ROOT)
    import bench
    assert (line["metric"], line["unit"], line["impl"]) == (bench.METRIC, bench.UNIT, "reference")
    assert line["higher_is_better"] is True and line["value"] > 0
    assert (line["steps"], line["warmup"]) == (2, 3)
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert "plate_cavity_20x14x10" in cb["sample"]
    e2e = line["e2e"]
    assert (e2e["value"], e2e["unit"], e2e["h2d_bytes_per_step"], e2e["d2h_bytes_per_step"]) == \
        (line["value"], line["unit"], 0, 0)
    assert line["config"]["workload"].startswith("plate_cavity_20x14x10")


def test_reference_arm_other_ranks_exit_quietly():
    run = _run({"RANK": "1", "WORLD_SIZE": "2"})
    assert run.returncode == 0, run.stderr
    assert run.stdout.strip() == ""
