"""Index safety of the step kernels' global stores: a test build of the
library with -DPFLBM_CHECK_BOUNDS (every guarded store checks its index and
sets the device error word instead of writing out of range) runs the main
configurations; no guard may fire (a fired guard makes pflbm_step return
PFLBM_ERR_DEVICE) and the results equal the normal build's to rounding.
This stands in for a memory checker, which is not available on this GPU."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "ux", "uy", "uz", "phi")


def _cases(pf):
    out = []
    c = pf.config_reference(pf.CASE_JET, pf.VS_D3Q19)
    c.nx, c.ny, c.nz, c.diam, c.radius = 30, 34, 40, 8, 4          # unaligned rows: plain loads, scalar phase
    out.append(("jet19_odd_fp32", c))
    c = pf.preset("jet_d3q27", nx=64, ny=48, nz=64, diam=10, radius=5, storage=pf.STORAGE_FP16,
                  flags=pf.FLAG_TIME_AVERAGE | pf.FLAG_REYNOLDS_MOMENTS)
    out.append(("jet27_fp16_avg", c))
    c = pf.preset("jet_d3q19", nx=64, ny=64, nz=96, diam=12, radius=6, storage=pf.STORAGE_BF16)
    out.append(("jet19_bf16_pairs", c))                              # node-pair collide
    c = pf.preset("jet_d3q19", nx=72, ny=40, nz=48, diam=10, radius=5, storage=pf.STORAGE_FP16)
    out.append(("jet19_fp16_pairs_overhang", c))                     # node pairs, last tile past the grid
    c = pf.config_reference(pf.CASE_DROPLET, pf.VS_D3Q27)
    c.nx = c.ny = c.nz = 48
    c.radius, c.diam = 12, 24
    c.storage = pf.STORAGE_FP64
    out.append(("droplet27_fp64", c))
    c = pf.preset("droplet64")
    out.append(("droplet19_fp32", c))
    return out


def _run(pf, cfg, steps):
    with pf.Simulation(cfg) as s:
        s.step(steps)
        return {f: s.get_field(f, dtype=np.float64) for f in FIELDS}


def test_checked_build_fires_no_guard_and_matches(pflbm):
    from phasefieldlbm_gb300 import build

    checked = pflbm.load_library(str(build.build_checked()))
    normal = pflbm.load_library()
    steps = 23
    try:
        for name, cfg in _cases(pflbm):
            pflbm._LIB = checked
            got = _run(pflbm, cfg, steps)  # raises PflbmError (device error word) if a guard fired
            pflbm._LIB = normal
            ref = _run(pflbm, cfg, steps)
            for f in FIELDS:
                # the guards change the code around the stores, so the
                # compiler may contract a multiply-add differently: equal to
                # rounding, not bit for bit
                assert rel_l2(got[f], ref[f]) <= (1e-12 if cfg.storage == pflbm.STORAGE_FP64 else 1e-5), (name, f)
        cfgs = pflbm.ensemble_configs(n=4, seed=3)
        for c in cfgs:
            c.nx = c.ny = c.nz = min(int(c.nx), 48)
            c.radius = min(c.radius, int(c.nx) // 4)
            c.diam = 2 * c.radius
        pflbm._LIB = checked
        with pflbm.Ensemble(cfgs) as ens:
            ens.step(17)
            for k in range(len(cfgs)):
                assert int(ens.reduce(k).nonfinite) == 0
    finally:
        pflbm._LIB = normal


def test_checked_build_closure_step(pflbm):
    """The closure-coupled step (TMA collide with the network after the
    pipeline's shared memory, time averages on) under the bounds-checked
    build: no guard fires and the fields equal the normal build's to
    rounding."""
    from phasefieldlbm_gb300 import build

    rng = np.random.default_rng(5)
    feats = np.empty((2048, 8))
    feats[:, :6] = rng.normal(0.0, 1e-4, (2048, 6))
    feats[:, 6] = rng.uniform(0.0, 1.0, 2048)
    feats[:, 7] = rng.exponential(0.05, 2048)
    checked = pflbm.load_library(str(build.build_checked()))
    normal = pflbm.load_library()
    try:
        with pflbm.Closure(2048) as c:
            c.set_samples(feats, np.full(2048, 2e-3))
            c.init_params(seed=3)
            blob = c.blob.copy()
        cfg = pflbm.preset("jet_d3q19", nx=40, ny=36, nz=48, diam=10, radius=5, flags=pflbm.FLAG_TIME_AVERAGE)
        out = {}
        for name, lib in (("checked", checked), ("normal", normal)):
            pflbm._LIB = lib
            with pflbm.Simulation(cfg) as s:
                s.set_closure(blob, strength=1.0)
                s.step(17)  # raises PflbmError if a guard fired
                out[name] = {f: s.get_field(f, dtype=np.float64) for f in FIELDS + ("avg_uz",)}
        for f in out["normal"]:
            assert rel_l2(out["checked"][f], out["normal"][f]) <= 1e-5, f
    finally:
        pflbm._LIB = normal
