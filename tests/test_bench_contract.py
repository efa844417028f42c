"""bench.py's reference arm on the small cantilever (48x24x24), on the host:
the JSON line carries the keys the benchmark contract names, it is a full
(not projected) CPU solve at this size, and the arm maps no library of this
package (it runs the oracle's restatement of the reference's CPU path)."""
import json
import pathlib
import subprocess
import sys

ROOT = pathlib.Path(__file__).resolve().parents[1]

RUNNER = r"""
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--config", "c1", "--steps", "1", "--warmup", "0",
            "--cpu-seconds", "2"]
try:
    runpy.run_path("bench.py", run_name="__main__")
finally:
    maps = open("/proc/self/maps").read()
    print("LIBHEXAGPU_MAPPED=" + str("libhexagpu" in maps), file=sys.stderr)
"""


def test_reference_arm_line_on_the_small_cantilever():
    r = subprocess.run([sys.executable, "-c", RUNNER], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "LIBHEXAGPU_MAPPED=False" in r.stderr
    line = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["unit"] == "s" and line["higher_is_better"] is False
    assert line["n_gpus"] == 1 and line["steps"] == 1 and line["warmup"] == 0
    assert "workload" in line["config"]
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["unit"] == "s" and cb["sample"]
    assert cb["value"] == line["value"] > 0
    assert not line["projected"] and not cb["projected"]  # a whole solve fits the sample at this size
    assert line["e2e"] == {"value": line["value"], "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
