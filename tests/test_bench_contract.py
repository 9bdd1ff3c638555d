"""The reference arm of bench.py (`--impl reference`, the CPU path on the
host's cores) prints one JSON line with the keys and types the bench contract
asks for, and a rank other than 0 prints nothing and exits 0. Runs on CPU with
a small sample."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(extra_env=None):
    env = dict(os.environ)
    env.update(extra_env or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                           "--steps", "2", "--warmup", "3", "--scale", "0.01", "--ref-mbp", "4"],
                          capture_output=True, text=True, env=env, cwd=ROOT, timeout=600)


def test_reference_arm_line():
    r = _run()
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key, typ in [("metric", str), ("value", float), ("unit", str), ("n_gpus", int), ("steps", int),
                     ("warmup", int), ("ms_per_step", float), ("higher_is_better", bool), ("scaling", str),
                     ("dtype", str), ("data", str), ("config", dict), ("cpu_baseline", dict), ("e2e", dict)]:
        assert isinstance(d[key], typ), (key, d[key])
    assert d["steps"] == 2 and d["warmup"] == 3 and d["value"] > 0 and d["vs_baseline"] is None
    assert d["unit"] == "Gbases/s" and d["higher_is_better"] is True
    assert "workload" in d["config"]
    # the same config object as the GB300 arm's line (bench.main_config), so the
    # two arms are on one workload
    sys.path.insert(0, ROOT)
    import bench
    assert d["config"] == bench.main_config(d["config"]["bases"], d["config"]["stream_bytes"], 1)
    assert d["config"]["bases"] == 31_000_000 and "same assembly" in d["cpu_baseline"]["sample"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"] and cb["value"] == d["value"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_are_silent():
    r = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
