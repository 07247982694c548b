"""The CPU oracle against outputs of the reference's own CUDA build
(tests/golden/ref_*.npz, made by tests/golden/gen_ref_fixtures.py on a GPU
from cubins of the reference's src/main.cu), at the reference's
compile-time configurations. Jets: every field within 1e-5 relative L2 after
60 steps. Droplet: rho, phi within 1e-5 after 10 steps, u within
max(1e-5, 2 x the FP32 rounding floor measured on the same case)."""
from pathlib import Path

import numpy as np
import pytest

from conftest import rel_l2

GOLDEN = Path(__file__).resolve().parent / "golden"
FIELDS = ("rho", "ux", "uy", "uz", "phi")


def _load(name):
    p = GOLDEN / f"ref_{name}.npz"
    if not p.exists():
        pytest.skip(f"{p.name} not generated")
    return np.load(p)


@pytest.mark.parametrize("name", ["jet_d3q19", "jet_d3q27"])
def test_oracle_matches_reference_build_jet(oracle, name):
    d = _load(name)
    c = oracle.config_reference(1, int(d["q"]))
    o = oracle.OracleSim(c)
    o.step(int(d["steps"]))
    planes = list(d["planes"])
    for f in FIELDS:
        assert rel_l2(o.get_field(f)[planes], d[f]) <= 1e-5, f


def test_oracle_matches_reference_build_droplet(oracle):
    d = _load("droplet_d3q19")
    c = oracle.config_reference(0, int(d["q"]))
    steps, planes = int(d["steps"]), list(d["planes"])
    o = oracle.OracleSim(c)
    o.step(steps)
    o64 = oracle.OracleSim(c, fp64=True)
    o64.step(steps)
    for f in FIELDS:
        e = rel_l2(o.get_field(f)[planes], d[f])
        floor = rel_l2(o.get_field(f)[planes], o64.get_field(f)[planes])
        tol = max(1e-5, 2.0 * floor) if f in ("ux", "uy", "uz") else 1e-5
        assert e <= tol, (f, e, floor)
