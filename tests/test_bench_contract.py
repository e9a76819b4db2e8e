"""The benchmark's reference arm keeps its JSON contract (CPU only).

`bench.py --impl reference` times the reference's own CPU implementation of
the solve path on the host cores (the reference package built into
baseline/_ref, else the oracle port) on the benchmark's own workload, and
prints one JSON line that the round-end comparison reads beside the GPU arm's
line. One short step of it runs here: the line must parse, name the same
metric, unit and direction as the GPU arm, say what it timed, and never load
this repository's package (it has no GPU to load it for).
"""

from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_its_json_line() -> None:
    # run the arm in a child that reports, at exit, whether this repository's
    # package was imported
    probe = (
        "import runpy, sys\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0']\n"
        "try:\n"
        "    runpy.run_path('bench.py', run_name='__main__')\n"
        "finally:\n"
        "    loaded = sorted(m for m in sys.modules if m.split('.')[0] == 'darcy_cpp_gb300')\n"
        "    print('PACKAGE_MODULES=' + ','.join(loaded), file=sys.stderr)\n"
    )
    proc = subprocess.run([sys.executable, "-c", probe], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert proc.returncode == 0, proc.stderr[-2000:]
    lines = [ln for ln in proc.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, proc.stdout
    line = json.loads(lines[0])
    if "unavailable" in line:  # allowed by the contract, with its reason
        assert line["impl"] == "reference" and line["unavailable"]
        return
    sys.path.insert(0, str(ROOT))
    import bench

    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC
    assert line["unit"] == "ms/solve" and line["higher_is_better"] is False
    assert line["steps"] == 1 and line["value"] > 0
    assert line["config"]["workload"] == bench.WORKLOAD
    base = line["cpu_baseline"]
    assert base["kind"] in ("reference", "port") and base["cores"] >= 1 and base["sample"]
    assert base["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert "PACKAGE_MODULES=\n" in proc.stderr or proc.stderr.rstrip().endswith("PACKAGE_MODULES="), proc.stderr[-500:]
