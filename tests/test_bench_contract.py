"""The JSON line of bench.py's reference arm (the CPU oracle of the reference's FSILS
path, timed on measured samples of its units): the keys the benchmark contract names,
on a small pipe so that it runs in seconds without a GPU; the arm loads the oracle's
library and never the svgpu library."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "small",
                          "--steps", "2", "--warmup", "1", "--no-config1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["higher_is_better"] is False and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert set(cb["measured_s"]) == {"assembly_s", "precond_s", "cycle_s"}
    assert len(d["measured"]["per_sample_s"]) == 2
    libs = d["repo_libraries_loaded"]
    assert libs is not None and any("liboracle" in p for p in libs)
    assert not any("libsvgpu" in p for p in libs), libs
