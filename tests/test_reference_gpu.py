"""Parity against the reference's own CUDA build (oracle/_ref cubins run by
oracle/ref_runner on the GPU), at the reference's compile-time configurations
(src/constants.cuh:80-141): JET 64x64x128 (D=10) and DROPLET 128^3 (R=35,
ellipsoidal), D3Q19 and D3Q27, f stored FP32.

  * the CPU oracle reproduces the reference build  -> the oracle is pinned
  * the library reproduces the reference build     -> the product is pinned
Tolerance: rel. L2 <= 1e-5 on rho, ux, uy, uz, phi after the stated steps.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
FIELDS = ("rho", "ux", "uy", "uz", "phi")


def _manifest():
    import sys

    sys.path.insert(0, str(ROOT))
    from oracle import ref_build

    m = ref_build.manifest()
    if not m:
        pytest.skip("oracle/_ref has no reference cubins (built only where the reference sources are)")
    return ref_build, m


def run_reference(name, steps, tmp_path):
    ref_build, m = _manifest()
    v = m[name]
    exe = ref_build.build_runner()
    out = tmp_path / name
    out.mkdir()
    nx, ny, nz = v["dims"]
    subprocess.run([str(exe), str(ref_build.OUT / v["cubin"]), v["case"], str(v["q"]), str(nx), str(ny), str(nz),
                    str(v["fp16"]), str(steps), str(out)], check=True, timeout=600)
    return {f: np.fromfile(out / f"{f}.bin", np.float32).reshape(nz, ny, nx) for f in FIELDS}


CASES = [("jet_d3q19", 1, 19, 200), ("jet_d3q27", 1, 27, 200), ("droplet_d3q19", 0, 19, 100),
         ("droplet_d3q27", 0, 27, 100)]


@pytest.mark.parametrize("name,case,vs,steps", CASES, ids=[c[0] for c in CASES])
def test_library_and_oracle_match_reference_build(pflbm, oracle, tmp_path, name, case, vs, steps):
    ref = run_reference(name, steps, tmp_path)
    cfg = pflbm.config_reference(case, vs)
    with pflbm.Simulation(cfg) as s:
        s.step(steps)
        lib = {f: s.get_field(f) for f in FIELDS}
    o = oracle.OracleSim(cfg)
    o.step(steps)
    ora = {f: o.get_field(f) for f in FIELDS}
    e_lib = {f: rel_l2(lib[f], ref[f]) for f in FIELDS}
    e_ora = {f: rel_l2(ora[f], ref[f]) for f in FIELDS}
    print(name, "library", e_lib, "oracle", e_ora)
    assert max(e_ora.values()) <= 1e-5, e_ora
    assert max(e_lib.values()) <= 1e-5, e_lib
