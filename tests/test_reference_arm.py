"""bench.py's reference arm runs the reference's own code and nothing of this
package: in a fresh process, `bench.py --impl reference` (a short run)
prints the same metric line with impl "reference" and kind "reference",
imports no singularity_gb300 module and maps no libsgx.so — only the
reference's kernel source compiled for the host (oracle/_ref)."""

from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

PROBE = """
import io, json, runpy, sys, contextlib
sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"]
out = io.StringIO()
with contextlib.redirect_stdout(out):
    runpy.run_path("bench.py", run_name="__main__")
maps = open("/proc/self/maps").read()
print(json.dumps({"line": out.getvalue().strip().splitlines()[-1],
                  "product_modules": sorted(m for m in sys.modules if m.startswith("singularity_gb300")),
                  "libsgx": "libsgx" in maps, "libref_host": "libref_host" in maps}))
"""


def test_reference_arm_runs_only_the_reference(oracle):
    if not oracle.ref_available():
        pytest.skip("no host build of the reference (no reference sources on this machine)")
    r = subprocess.run([sys.executable, "-c", PROBE], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    rep = json.loads(r.stdout.strip().splitlines()[-1])
    assert rep["product_modules"] == [] and not rep["libsgx"] and rep["libref_host"]
    line = json.loads(rep["line"])
    assert line["impl"] == "reference" and line["cpu_baseline"]["kind"] == "reference"
    assert line["metric"].startswith("Kerr geodesic Mrays/s") and line["value"] > 0
    assert "fixed_h0.4" in line["config"]["workload"]
