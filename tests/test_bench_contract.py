"""The reference arm of ``bench.py`` on a small grid, on the CPU: the JSON line carries the keys the
measurement contract asks for, and the arm maps none of this package's compiled libraries (the
reference's CPU path is timed without the GB300 engine anywhere in the process)."""

from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

# Runs the reference arm in a fresh interpreter, then prints the libraries of this repository
# that the process mapped (from /proc/self/maps) after the bench's own JSON line.
SCRIPT = """
import json, sys
sys.argv = ["bench.py", "--impl", "reference", "--cells", "40,40,24", "--steps", "2", "--warmup", "1"]
sys.path.insert(0, {root!r})
import bench
bench.main()
maps = open("/proc/self/maps").read().splitlines()
mine = sorted({{ln.split()[-1] for ln in maps if ln.split() and ln.split()[-1].endswith(".so")
               and ln.split()[-1].startswith({root!r})}})
print(json.dumps({{"mapped": mine}}))
"""


def test_reference_arm_line_and_no_product_library() -> None:
    out = subprocess.run(
        [sys.executable, "-c", SCRIPT.format(root=str(ROOT))],
        capture_output=True, text=True, timeout=300, cwd=ROOT, check=True,
    ).stdout.strip().splitlines()
    line = json.loads(out[-2])
    mapped = json.loads(out[-1])["mapped"]
    assert mapped == [], mapped
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["metric"] == line["unit"] == "Gcell-updates/s"
    assert line["higher_is_better"] is True and line["steps"] == 2 and line["warmup"] == 1
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["config"]["workload"] == "via_transition_40x40x24"
    assert line["config"]["cells"] == [40, 40, 24] and line["config"]["batch"] == 2
    cpu = line["cpu_baseline"]
    assert cpu["kind"] == "port" and cpu["cores"] == 1 and cpu["value"] == line["value"] and cpu["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
