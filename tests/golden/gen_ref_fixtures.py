"""Generates tests/golden/ref_*.npz: outputs of the reference's own CUDA build.

Runs on a GPU machine: oracle/ref_runner executes the reference's kernels
(cubins built by oracle/ref_build.py from the reference sources) at the
reference's compile-time configurations, and selected z-planes of rho, ux,
uy, uz and phi are stored as float32 (small enough to commit). The CPU test
tests/test_oracle_golden.py checks the oracle against them.

    python tests/golden/gen_ref_fixtures.py [outdir]
"""
from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

FIELDS = ("rho", "ux", "uy", "uz", "phi")
# name, steps, planes kept
JOBS = [
    ("jet_d3q19", 60, (1, 2, 64, 126, 127)),
    ("jet_d3q27", 60, (1, 64, 126)),
    ("droplet_d3q19", 10, (40, 88)),
]


def main():
    from oracle import ref_build

    out_dir = Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parent
    m = ref_build.manifest()
    exe = ref_build.build_runner()
    for name, steps, planes in JOBS:
        v = m[name]
        nx, ny, nz = v["dims"]
        with tempfile.TemporaryDirectory() as td:
            subprocess.run([str(exe), str(ref_build.OUT / v["cubin"]), v["case"], str(v["q"]), str(nx), str(ny),
                            str(nz), str(v["fp16"]), str(steps), td], check=True)
            data = {f: np.fromfile(Path(td) / f"{f}.bin", np.float32).reshape(nz, ny, nx)[list(planes)] for f in FIELDS}
        np.savez_compressed(out_dir / f"ref_{name}.npz", steps=steps, planes=np.array(planes), case=v["case"],
                            q=v["q"], dims=np.array(v["dims"]), **data)
        print("wrote", name)


if __name__ == "__main__":
    main()
