"""bench.py --impl reference on the CPU: the reference algorithm (the oracle,
one single-threaded process per core) timed on the benchmark's workload, one
JSON line with the fields the bench contract asks of that arm -- its metric and
unit are the GPU arm's, it carries a cpu_baseline describing the run and an
e2e block with no host-device copies."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "1", "--cpu-cores", "2"], cwd=ROOT, env=env, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"].startswith("SCF+MP2 solves/s") and d["unit"] == "solves/s"
    assert d["higher_is_better"] is True and d["steps"] == 1
    assert d["value"] > 0.0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] == 2 and cb["value"] == d["value"] and cb["sample"]
    # the extrapolated stage times add up to the rate of a single process
    per = cb["extrapolated_s_per_solve_median"]
    assert set(per) == {"int1e", "int2e", "scf", "ao2mo", "mp2"} and all(v > 0 for v in per.values())
    assert d["e2e"] == {"value": d["value"], "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["molecule"] == "(H2O)32"
