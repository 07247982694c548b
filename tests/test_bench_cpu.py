"""bench.py on the host (no GPU needed): the reference arm times the oracle
without loading libpflbm, and builds the same workload configuration from
the oracle's restatement of src/constants.cuh as the library's preset does."""
import ctypes
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

PRESETS = ("droplet64", "jet_d3q27", "jet_d3q19", "jet_precision", "jet_closure", "jet_closure_fine")


@pytest.mark.parametrize("name", PRESETS)
def test_preset_from_oracle_base_equals_library_preset(pflbm, oracle, name):
    a = pflbm.preset(name)
    b = pflbm.preset(name, base=oracle.config_reference)
    assert ctypes.string_at(ctypes.byref(a), ctypes.sizeof(a)) == ctypes.string_at(ctypes.byref(b), ctypes.sizeof(b))


def test_reference_arm_loads_no_library(oracle):
    """One reference-arm run on a short jet (128x128x8) in a fresh process,
    which then lists the shared objects it has mapped: the oracle's only."""
    code = f"""
import json, sys
sys.path.insert(0, {str(ROOT)!r})
import bench
args = type("A", (), dict(workload="jet_d3q27", storage="fp32", nz=8, steps=1, warmup=0))()
out = bench.run_reference(args, type("R", (), dict(rank=0, world=1))())
maps = open("/proc/self/maps").read()
print(json.dumps(dict(value=out["value"], impl=out["impl"], pflbm="libpflbm" in maps, oracle="liboracle" in maps)))
"""
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    import json

    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["impl"] == "reference" and res["value"] > 0
    assert res["oracle"] and not res["pflbm"], res
