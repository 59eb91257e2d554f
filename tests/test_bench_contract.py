"""The reference arm of bench.py runs on host cores only, so its JSON line is checked here (CPU):
it reports the workload it actually ran, and its process never loads the product library."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# runs bench.py's main() in this interpreter, then reports whether the product package was
# imported or its shared library mapped
_PROBE = r"""
import json, runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--size", "40", "--steps", "1", "--warmup", "0"]
runpy.run_path("bench.py", run_name="__main__")
maps = open("/proc/self/maps").read()
print("PROBE " + json.dumps({"package": "peclet_pnm_gb300" in sys.modules,
                             "library": "libpnm_gb300" in maps}))
"""


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, "-c", _PROBE], cwd=ROOT, capture_output=True, text=True,
                         timeout=300, check=True)
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "Gvoxel/s" and d["value"] > 0
    assert d["higher_is_better"] is True and d["n_gpus"] == 1
    assert d["config"]["voxels"] == 40 ** 3  # the volume it ran, whole
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert "40^3" in cb["sample"]
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    probe = json.loads([ln for ln in out.stdout.splitlines() if ln.startswith("PROBE ")][0][6:])
    assert probe == {"package": False, "library": False}
