"""bench.py's reference arm on the CPU: the reference algorithm (the oracle's
OpenMP restatement) on the host cores, at a small size, prints one JSON line
with the fields of the benchmark contract."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line(oracle):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--cells", "16",
                          "--particles", "20000", "--cpu-sample", "20000", "--clumps", "4", "--sigma", "2",
                          "--steps", "2", "--warmup", "1"],
                         capture_output=True, text=True, timeout=300, cwd=ROOT, check=True).stdout
    lines = [l for l in out.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "P2G+G2P particles/s" and d["unit"] == "particles/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["scaling"] == "weak"
    assert (d["n_gpus"], d["steps"], d["warmup"]) == (1, 2, 1)
    assert d["ms_per_step"] > 0 and d["vs_baseline"] is None
    assert "16^3 cells" in d["config"]["workload"] and d["config"]["particles"] == 20000
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "particles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
