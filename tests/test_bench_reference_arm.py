"""bench.py's reference arm on the CPU: one JSON line with the same metric,
unit and workload as the GPU arm, timed on the CPU restatement of the
reference's passes (the oracle), and nothing at all from ranks other than
0 under a multi-process launch."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_bench(extra_env):
    env = dict(os.environ, **extra_env)
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return [l for l in r.stdout.splitlines() if l.startswith("{")]


def test_reference_arm_line():
    import bench

    lines = run_bench({"RANK": "0", "WORLD_SIZE": "1"})
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 3
    assert d["config"]["workload"] == "pcss_1080p"
    assert d["value"] > 0 and abs(d["ms_per_step"] - 1000.0 / d["value"]) < 1e-6 * d["ms_per_step"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_print_nothing():
    assert run_bench({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}) == []


def test_reference_arm_loads_no_product_code():
    """The timed CPU restatement reads its inputs from oracle/pcss_1080p_inputs.npz:
    libgishadow.so is never mapped into the reference arm's process."""
    code = ("import sys, types, bench; "
            "a = types.SimpleNamespace(gpus=1, steps=1, warmup=0); "
            "bench.run_reference(a); "
            "maps = open('/proc/self/maps').read(); "
            "sys.exit(3 if 'libgishadow' in maps else 0)")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600,
                       env=dict(os.environ, RANK="0", WORLD_SIZE="1"))
    assert r.returncode == 0, (r.returncode, r.stderr[-2000:])
