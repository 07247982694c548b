"""Storage precision against the FP64 oracle at the precision study's error
grid: the D3Q19 jet, 128x128x512, D = 16, Re = 5000, We = 500, seeded
uniform inflow noise. After 200 steps:
  * the library's FP64 path equals the FP64 oracle (rel. L2 <= 1e-10),
  * FP16 storage (FP32 arithmetic) is within 1e-3 of the FP64 oracle on rho,
    the centreline u_z and phi, and so is BF16 on rho and phi,
  * FP32 storage is within 1e-4.
The oracle runs on the host cores (about two minutes for 200 steps)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

STEPS = 200


@pytest.fixture(scope="module")
def oracle_fields(pflbm, oracle):
    cfg = pflbm.preset("jet_d3q19")
    o = oracle.OracleSim(cfg, fp64=True)
    o.step(STEPS)
    return {f: o.get_field(f) for f in ("rho", "uz", "phi")}


def _run(pflbm, storage):
    cfg = pflbm.preset("jet_d3q19", storage=storage)
    with pflbm.Simulation(cfg) as s:
        s.step(STEPS)
        return {f: s.get_field(f, dtype=np.float64) for f in ("rho", "uz", "phi")}


def _errors(got, ref):
    ny, nx = ref["uz"].shape[1:]
    cy, cx = ny // 2, nx // 2
    return {"rho": rel_l2(got["rho"], ref["rho"]), "uz": rel_l2(got["uz"], ref["uz"]),
            "uz_centreline": rel_l2(got["uz"][:, cy, cx], ref["uz"][:, cy, cx]), "phi": rel_l2(got["phi"], ref["phi"])}


def test_fp64_path_is_the_oracle(pflbm, oracle_fields):
    e = _errors(_run(pflbm, pflbm.STORAGE_FP64), oracle_fields)
    print("fp64", e)
    assert max(e.values()) <= 1e-10, e


@pytest.mark.parametrize("name,storage,tol,fields", [
    ("fp32", 0, 1e-4, ("rho", "uz_centreline", "phi", "uz")),
    ("fp16", 1, 1e-3, ("rho", "uz_centreline", "phi", "uz")),
    ("bf16", 2, 1e-3, ("rho", "phi")),
])
def test_storage_error_against_fp64_oracle(pflbm, oracle_fields, name, storage, tol, fields):
    e = _errors(_run(pflbm, storage), oracle_fields)
    print(name, e)
    for f in fields:
        assert e[f] <= tol, (name, f, e)
