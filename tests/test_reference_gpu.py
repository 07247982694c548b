"""Parity against the reference's own CUDA build (oracle/_ref cubins run by
oracle/ref_runner on the GPU), at the reference's compile-time configurations
(src/constants.cuh:80-141): JET 64x64x128 (D=10) and DROPLET 128^3 (R=35,
ellipsoidal), D3Q19 and D3Q27, f stored FP32.

  * the CPU oracle reproduces the reference build  -> the oracle is pinned
  * the library reproduces the reference build     -> the product is pinned
Tolerances (relative L2):
  * short horizon (jets 30 steps, droplets 10 steps), oracle and library:
    rho, phi <= 1e-5; each velocity component within max(1e-5, 2 x the FP32
    floor), the floor being the oracle's own FP32-vs-FP64 difference on the
    same case (ux, uy of the jet are inflow noise only; the reference's
    default droplet, R = 35 stretched to 140 cells in x, spans the whole
    128-cell box and is strongly ill-conditioned);
  * long horizons (jets 200, droplets 100 steps): FP32 rounding differences
    have grown to the floor; the library must be no farther from the
    reference build than 2x the independent oracle is (and rho <= 1e-5).
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


def _errors(pflbm, oracle, tmp_path, name, case, vs, steps, with_floor=False):
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
    floor = None
    if with_floor:
        o64 = oracle.OracleSim(cfg, fp64=True)
        o64.step(steps)
        floor = {f: rel_l2(ora[f], o64.get_field(f)) for f in FIELDS}
    print(name, steps, "library", e_lib, "oracle", e_ora, "floor", floor)
    return e_lib, e_ora, floor


SHORT = [("jet_d3q19", 1, 19, 30), ("jet_d3q27", 1, 27, 30), ("droplet_d3q19", 0, 19, 10),
         ("droplet_d3q27", 0, 27, 10)]
LONG = [("jet_d3q19", 1, 19, 200), ("jet_d3q27", 1, 27, 200), ("droplet_d3q19", 0, 19, 100),
        ("droplet_d3q27", 0, 27, 100)]


@pytest.mark.parametrize("name,case,vs,steps", SHORT, ids=[c[0] for c in SHORT])
def test_match_reference_build_short(pflbm, oracle, tmp_path, name, case, vs, steps):
    e_lib, e_ora, floor = _errors(pflbm, oracle, tmp_path, name, case, vs, steps, with_floor=True)
    for e in (e_lib, e_ora):
        for f in FIELDS:
            tol = max(1e-5, 2.0 * floor[f]) if f in ("ux", "uy", "uz") else 1e-5
            assert e[f] <= tol, (f, e, floor)


@pytest.mark.parametrize("name,case,vs,steps", LONG, ids=[c[0] for c in LONG])
def test_match_reference_build_long(pflbm, oracle, tmp_path, name, case, vs, steps):
    e_lib, e_ora, _ = _errors(pflbm, oracle, tmp_path, name, case, vs, steps)
    assert e_lib["rho"] <= 1e-5 and e_ora["rho"] <= 1e-5
    for f in FIELDS:
        assert e_lib[f] <= 2.0 * max(1e-5, e_ora[f]), (f, e_lib, e_ora)


BENCH = [("jet_d3q19_128x128x512", 19), ("jet_d3q27_128x128x512", 27)]


@pytest.mark.parametrize("name,vs", BENCH, ids=[b[0] for b in BENCH])
def test_match_reference_build_at_benchmark_size(pflbm, tmp_path, name, vs):
    """The benchmark-size jet (128x128x512, D = 16, the reference's own
    physics and Gaussian inflow noise) after 100 steps: the FP32 library
    against the reference's build patched to that mesh. rho, phi <= 1e-5;
    velocity components within max(1e-5, 2x) the library's own FP32-vs-FP64
    difference on the same case."""
    steps = 100
    ref = run_reference(name, steps, tmp_path)
    cfg = pflbm.config_reference(pflbm.CASE_JET, vs)
    cfg.nx, cfg.ny, cfg.nz, cfg.diam, cfg.radius = 128, 128, 512, 16, 8
    cfg.sigma = float(np.float32(np.float32(np.float32(cfg.u_inf) * np.float32(cfg.u_inf)) * np.float32(16))
                      / np.float32(500.0))
    out = {}
    for st in (pflbm.STORAGE_FP32, pflbm.STORAGE_FP64):
        cfg.storage = st
        with pflbm.Simulation(cfg) as s:
            s.step(steps)
            out[st] = {f: s.get_field(f, dtype=np.float64) for f in FIELDS}
    lib, lib64 = out[pflbm.STORAGE_FP32], out[pflbm.STORAGE_FP64]
    e = {f: rel_l2(lib[f], ref[f]) for f in FIELDS}
    floor = {f: rel_l2(lib[f], lib64[f]) for f in FIELDS}
    print(name, "library vs reference", e, "FP32 floor", floor)
    for f in FIELDS:
        tol = max(1e-5, 2.0 * floor[f]) if f in ("ux", "uy", "uz") else 1e-5
        assert e[f] <= tol, (f, e, floor)


PRESETS = [("jet_d3q27_bench", "jet_d3q27"), ("jet_d3q19_bench", "jet_d3q19")]


@pytest.mark.parametrize("name,preset", PRESETS, ids=[p[1] for p in PRESETS])
def test_match_reference_build_on_bench_preset(pflbm, tmp_path, name, preset):
    """The benchmark presets themselves (128x128x512, D = 16, Re = 5000,
    We = 500, gamma = 0.05, seeded uniform +-5% u_z inflow noise) after 100
    steps: the FP32 library against the reference's own build with the
    preset's gamma and inflow noise patched in (oracle/ref_build.py). rho,
    phi <= 1e-5; velocity components within max(1e-5, 2x) the library's own
    FP32-vs-FP64 difference on the same case."""
    steps = 100
    ref = run_reference(name, steps, tmp_path)
    cfg = pflbm.preset(preset)
    out = {}
    for st in (pflbm.STORAGE_FP32, pflbm.STORAGE_FP64):
        cfg.storage = st
        with pflbm.Simulation(cfg) as s:
            s.step(steps)
            out[st] = {f: s.get_field(f, dtype=np.float64) for f in FIELDS}
    lib, lib64 = out[pflbm.STORAGE_FP32], out[pflbm.STORAGE_FP64]
    e = {f: rel_l2(lib[f], ref[f]) for f in FIELDS}
    floor = {f: rel_l2(lib[f], lib64[f]) for f in FIELDS}
    e64 = {f: rel_l2(ref[f], lib64[f]) for f in FIELDS}
    print(preset, "library vs reference build", e, "FP32 floor", floor, "reference build vs FP64 path", e64)
    for f in FIELDS:
        tol = max(1e-5, 2.0 * floor[f]) if f in ("ux", "uy", "uz") else 1e-5
        assert e[f] <= tol, (f, e, floor)


def test_fp16_storage_against_reference_fp16_build(pflbm, tmp_path):
    """16-bit storage accuracy at the benchmark jet size: the library's FP16
    path (f - w stored as (f - w)/w, per-direction scaling) and the
    reference's own FP16 build (f - w stored unscaled as __half,
    src/cuda/precision.cuh:26-56) against the library's FP64 path after 100
    steps. Both are within 1e-3; the library is at least as accurate on rho
    and the velocity (2/3 of the reference's rho error, 0.94-0.99 of its
    velocity errors) and within 10% on phi (1.08x: J, which carries phi, is
    FP32 in both, so phi only sees the velocity's rounding)."""
    steps = 100
    ref16 = run_reference("jet_d3q19_128x128x512_fp16", steps, tmp_path)
    cfg = pflbm.config_reference(pflbm.CASE_JET, pflbm.VS_D3Q19)
    cfg.nx, cfg.ny, cfg.nz, cfg.diam, cfg.radius = 128, 128, 512, 16, 8
    cfg.sigma = float(np.float32(np.float32(np.float32(cfg.u_inf) * np.float32(cfg.u_inf)) * np.float32(16))
                      / np.float32(500.0))
    out = {}
    for st in (pflbm.STORAGE_FP16, pflbm.STORAGE_FP64):
        cfg.storage = st
        with pflbm.Simulation(cfg) as s:
            s.step(steps)
            out[st] = {f: s.get_field(f, dtype=np.float64) for f in FIELDS}
    ref64 = out[pflbm.STORAGE_FP64]
    e_lib = {f: rel_l2(out[pflbm.STORAGE_FP16][f], ref64[f]) for f in FIELDS}
    e_ref = {f: rel_l2(ref16[f], ref64[f]) for f in FIELDS}
    print("FP16 storage vs FP64: library", e_lib, "reference build", e_ref)
    for f in FIELDS:
        assert e_lib[f] <= 1e-3, (f, e_lib)
        assert e_lib[f] <= (1.1 if f == "phi" else 1.0) * e_ref[f], (f, e_lib, e_ref)
