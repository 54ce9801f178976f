"""bench.py's reference arm on the CPU: one JSON line with the keys its
contract names, on the small single-case workload (the isentropic vortex,
262,144 cells), with the rate, cpu_baseline and e2e values consistent."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", "vortex", "--steps", "2", "--warmup", "1"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert (d["n_gpus"], d["steps"], d["warmup"]) == (1, 2, 1)
    assert d["value"] > 0 and d["higher_is_better"] is True and d["vs_baseline"] is None
    assert d["unit"] == "cell-subiters/s" and "workload" in d["config"]
    assert d["config"]["cells"] == 262144
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference")
    assert cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}
    # the timed region is what ms_per_step x steps says: 2 sub-iterations of the case
    t = d["timed_sample"]
    assert t["cell_subiters"] == 2 * 262144
    assert abs(t["cell_subiters"] / (d["ms_per_step"] * d["steps"] / 1e3) - d["value"]) \
        <= 1e-6 * d["value"]
