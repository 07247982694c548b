"""The configurations that are benchmarked, compared field by field with the
CPU oracle (oracle/oracle.cpp, the pass-by-pass restatement of
src/phaseField.cuh:31-219, src/lbm.cu:33-239, src/BoundaryConditions.cuh and
src/initialConditions.cu) at their full sizes:

  * the bench line's workload, the D3Q27 + D3Q7 jet preset (128x128x512,
    D = 16, Re = 5000, We = 500, gamma = 0.05, seeded uniform +-5% u_z
    inflow noise), 100 steps: FP64 storage against the FP64 oracle
    (rel. L2 <= 1e-10 on all 18 fields), FP32 against the FP32 oracle;
  * the droplet64 preset (64^3 periodic, R = 16, tau = 0.6, sigma = 0.01,
    gamma = 0.05, spherical) for its full 1000 steps, FP32;
  * boxes of the seeded droplet ensemble at their real 80 and 96 edges,
    advanced inside one batch together with two smaller boxes, FP32.

FP32 tolerances (rel. L2): every field (rho, phi, each velocity component
and the velocity vector field) within max(1e-5, 2 x floor), the floor being
the oracle's own FP32-vs-FP64 difference on the same case and horizon. The
velocity of a young jet is mostly inflow noise and that of a droplet
spurious currents, so its FP32 rounding floor lies near or above 1e-5; rho
and phi stay at 1e-5 on the jet and droplet64 (floors 3e-8 to 2e-6), while
on the seeded ensemble's 80-edge box (small sigma, noisy initial velocity)
the oracle's own FP32 phi is 4.9e-5 from its FP64 phi after 300 steps, and
no FP32 implementation can do better there.

The oracle runs on the host cores: about four minutes for the whole file on
a 16-core host."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

BASIC = ("rho", "ux", "uy", "uz", "phi")
ALL18 = ("rho", "ux", "uy", "uz", "pxx", "pyy", "pzz", "pxy", "pxz", "pyz",
         "phi", "normx", "normy", "normz", "ind", "fsx", "fsy", "fsz")
VEL = ("ux", "uy", "uz")


def _with_u(d):
    d = dict(d)
    d["u"] = np.stack([d[f] for f in VEL])
    return d


def _fp32_errors_against_floor(lib, ora32, ora64):
    lib, ora32, ora64 = _with_u(lib), _with_u(ora32), _with_u(ora64)
    e = {f: rel_l2(lib[f], ora32[f]) for f in BASIC + ("u",)}
    floor = {f: rel_l2(ora32[f], ora64[f]) for f in BASIC + ("u",)}
    bad = {f: e[f] for f in BASIC + ("u",) if not e[f] <= max(1e-5, 2.0 * floor[f])}
    return e, floor, bad


def _lib_run(pf, cfg, storage, steps, fields):
    c = cfg.copy()
    c.storage = storage
    with pf.Simulation(c) as s:
        s.step(steps)
        assert s.current_step == steps
        return {f: s.get_field(f, dtype=np.float64) for f in fields}


def _oracle_run(oracle, cfg, steps, fp64, fields):
    o = oracle.OracleSim(cfg, fp64=fp64)
    o.step(steps)
    out = {f: o.get_field(f) for f in fields}
    o.close()
    return out


def test_bench_jet_d3q27_preset_against_oracle(pflbm, oracle):
    steps = 100
    cfg = pflbm.preset("jet_d3q27")
    assert (cfg.nx, cfg.ny, cfg.nz, cfg.diam) == (128, 128, 512, 16)
    ora64 = _oracle_run(oracle, cfg, steps, True, ALL18)
    lib64 = _lib_run(pflbm, cfg, pflbm.STORAGE_FP64, steps, ALL18)
    e64 = {f: rel_l2(lib64[f], ora64[f]) for f in ALL18}
    print("jet_d3q27 preset FP64 vs FP64 oracle", e64)
    assert max(e64.values()) <= 1e-10, e64
    ora32 = _oracle_run(oracle, cfg, steps, False, BASIC)
    lib32 = _lib_run(pflbm, cfg, pflbm.STORAGE_FP32, steps, BASIC)
    e, floor, bad = _fp32_errors_against_floor(lib32, ora32, {f: ora64[f] for f in BASIC})
    print("jet_d3q27 preset FP32 vs FP32 oracle", e, "floor", floor)
    assert not bad, (bad, e, floor)


def test_droplet64_full_run_against_oracle(pflbm, oracle):
    steps = 1000
    cfg = pflbm.preset("droplet64")
    ora32 = _oracle_run(oracle, cfg, steps, False, BASIC)
    ora64 = _oracle_run(oracle, cfg, steps, True, BASIC)
    lib32 = _lib_run(pflbm, cfg, pflbm.STORAGE_FP32, steps, BASIC)
    e, floor, bad = _fp32_errors_against_floor(lib32, ora32, ora64)
    print("droplet64 1000 steps FP32 vs FP32 oracle", e, "floor", floor)
    assert not bad, (bad, e, floor)
    # phase mass of the oracle run conserved as the library's is
    m0 = float(np.sum(_oracle_run(oracle, cfg, 0, True, ("phi",))["phi"]))
    assert abs(float(np.sum(ora64["phi"])) / m0 - 1.0) < 1e-6


def test_ensemble_boxes_at_real_size_against_oracle(pflbm, oracle):
    steps = 300
    cfgs = pflbm.ensemble_configs(64)
    edges = [int(c.nx) for c in cfgs]
    pick = [edges.index(80), edges.index(96), edges.index(32), edges.index(48)]
    batch = [cfgs[k] for k in pick]
    with pflbm.Ensemble(batch) as ens:
        ens.step(steps)
        got = [{f: ens.get_field(k, f).astype(np.float64) for f in BASIC} for k in range(len(batch))]
    for k in range(2):  # the 80 and 96 boxes
        c = batch[k]
        ora32 = _oracle_run(oracle, c, steps, False, BASIC)
        ora64 = _oracle_run(oracle, c, steps, True, BASIC)
        e, floor, bad = _fp32_errors_against_floor(got[k], ora32, ora64)
        print(f"ensemble box {pick[k]} (edge {int(c.nx)}) FP32 vs FP32 oracle", e, "floor", floor)
        assert not bad, (int(c.nx), bad, e, floor)
