"""bench.py's reference arm on the host cores: the CPU implementation of the
step timed on a bounded sample of the membrane workload, printed as one JSON
line with the engine line's metric, unit and workload, "impl": "reference",
a cpu_baseline describing the run and an e2e line without host-device bytes.
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "3"],
                         capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"].startswith("particle-steps/s")
    assert d["unit"] == "particle-steps/s" and d["higher_is_better"] is True
    assert d["config"]["workload"] == "membrane_1m"
    assert (d["n_gpus"], d["steps"], d["warmup"]) == (1, 1, 3)
    assert d["value"] > 0 and d["ms_per_step"] > 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    # the sample's pair density and the host it ran on are part of the record
    assert 50 < cb["pairs_per_bead"] < 400
    assert cb["nproc"] >= 1 and "cpu_model" in cb and "omp_num_threads" in cb
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
