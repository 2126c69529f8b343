"""bench.py --impl reference on the CPU: the line the reference arm prints."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_its_line(O):
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "ring2d",
                        "--steps", "3", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([x for x in r.stdout.splitlines() if x.startswith("{")][-1])
    assert line["impl"] == "reference" and line["unit"] == "iter/s" and line["value"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["one_thread_value"] > 0 and cb["cpu_model"]
    # every step runs on all host threads, also after the one-thread run
    assert cb["cores"] == O.max_threads() and len(cb["step_ms"]) == 3
    assert "full matrix" in cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "iter/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["workload"] == "ring2d" and line["config"]["rows"] == 8128
    assert "reference_cuda" in line
    # the inputs come from the oracle: the product library is never loaded
    libs = line["repo_libraries_mapped"]
    assert libs is not None and any("liboracle" in p for p in libs)
    assert not any("libmlem_gb300" in p for p in libs), libs
