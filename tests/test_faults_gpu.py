"""Failure detection without a GPU fault: every failure is made on the host
(an allocation cap, an unwritable output path, a NaN planted in the initial
state) and must come back as a status code with a message, leaving the
process and the device usable."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _small_jet(pflbm):
    c = pflbm.config_reference(pflbm.CASE_JET, pflbm.VS_D3Q19)
    c.nx, c.ny, c.nz, c.diam, c.radius = 32, 32, 48, 8, 4
    return c


def test_allocation_cap_fails_cleanly(pflbm, monkeypatch):
    monkeypatch.setenv("PFLBM_ALLOC_LIMIT_BYTES", "1000000")
    with pytest.raises(pflbm.PflbmError) as e:
        pflbm.Simulation(_small_jet(pflbm))
    assert e.value.code == 3 and "PFLBM_ALLOC_LIMIT_BYTES" in str(e.value)
    monkeypatch.delenv("PFLBM_ALLOC_LIMIT_BYTES")
    with pflbm.Simulation(_small_jet(pflbm)) as s:  # the device is still usable
        s.step(5)


def test_output_io_error_is_reported(pflbm, tmp_path):
    blocker = tmp_path / "file"
    blocker.write_text("not a directory")
    with pflbm.Simulation(_small_jet(pflbm)) as s:
        s.step(3)
        with pytest.raises(pflbm.PflbmError) as e:
            s.write_output(blocker / "out", ("rho",))
        assert e.value.code == 7
        s.step(2)
        s.write_output(tmp_path / "ok", ("rho",))  # recovers
        assert (tmp_path / "ok" / "rho000004.bin").exists()


def test_watchdog_catches_nan(pflbm):
    c = pflbm.preset("droplet64")
    with pflbm.Simulation(c) as s:
        rho = s.get_field("rho")
        rho[32, 32, 32] = np.nan  # planted on the host
        s.set_initial_field("rho", rho)
        s.set_watchdog(10)
        with pytest.raises(pflbm.PflbmError) as e:
            s.step(40)
        assert e.value.code == 5
        assert s.current_step == 10  # stopped at the first check
        assert int(s.reduce().nonfinite) > 0


def test_watchdog_mass_drift(pflbm):
    c = pflbm.preset("droplet64")
    with pflbm.Simulation(c) as s:
        s.set_watchdog(25, max_phi_mass_drift=1e-4)
        s.step(100)  # FP32 drift ~1e-7: passes
    with pflbm.Simulation(c) as s:
        s.set_watchdog(25, max_phi_mass_drift=1e-15)  # stricter than FP32 rounding
        with pytest.raises(pflbm.PflbmError) as e:
            s.step(100)
        assert e.value.code == 5 and "drift" in str(e.value)


def test_bounded_tma_wait_runs_out_and_reports(pflbm):
    """A device-side wait that runs out. The test build _build/deadwait
    (-DPFLBM_TEST_DEAD_WAIT) makes every collide pipeline's per-plane wait
    poll an mbarrier that nothing arrives on, with a short limit. Each CTA
    then sets the device error word, waits (at the full limit) for its own
    TMA copies still in flight and returns: pflbm_step and
    pflbm_ensemble_step must return PFLBM_ERR_DEVICE (8), and the device must
    stay usable for a normal run in the same process afterwards. Covers the
    one-node TMA collide (FP32), the node-pair collide (FP16) and the
    persistent batch collide."""
    from phasefieldlbm_gb300 import build

    dead = pflbm.load_library(str(build.build_dead_wait()))
    normal = pflbm.load_library()
    jet32 = _small_jet(pflbm)
    jet16 = _small_jet(pflbm)
    jet16.storage = pflbm.STORAGE_FP16
    boxes = pflbm.ensemble_configs(3, seed=5)
    for c in boxes:
        c.nx = c.ny = c.nz = 32
        c.radius, c.diam = 6, 12
    try:
        pflbm._LIB = dead
        for cfg, variant in ((jet32, "tma"), (jet16, "tma_pairs")):
            with pflbm.Simulation(cfg) as s:
                assert s.collide_variant == variant
                with pytest.raises(pflbm.PflbmError) as e:
                    s.step(3)
                assert e.value.code == 8, e.value
        with pflbm.Ensemble(boxes) as ens:
            with pytest.raises(pflbm.PflbmError) as e:
                ens.step(2)
            assert e.value.code == 8, e.value
    finally:
        pflbm._LIB = normal
    # the context is intact: a normal run in the same process
    with pflbm.Simulation(jet32) as s:
        s.step(5)
        assert int(s.reduce().nonfinite) == 0


def test_ensemble_grid_barrier_runs_out_and_reports(pflbm):
    """The grid-wide barrier of the ensemble's fused step, made to run out:
    the test build _build/deadgrid (-DPFLBM_TEST_DEAD_GRID) polls a flag that
    nothing sets, with a short limit. Every CTA sets the device error word
    and returns; pflbm_ensemble_step returns PFLBM_ERR_DEVICE (8) and a
    normal ensemble in the same process runs afterwards."""
    from phasefieldlbm_gb300 import build

    dead = pflbm.load_library(str(build.build_dead_grid()))
    normal = pflbm.load_library()
    boxes = pflbm.ensemble_configs(3, seed=5)
    for c in boxes:
        c.nx = c.ny = c.nz = 32
        c.radius, c.diam = 6, 12
    try:
        pflbm._LIB = dead
        with pflbm.Ensemble(boxes) as ens:
            with pytest.raises(pflbm.PflbmError) as e:
                ens.step(2)
            assert e.value.code == 8, e.value
    finally:
        pflbm._LIB = normal
    with pflbm.Ensemble(boxes) as ens:
        ens.step(3)
        assert all(int(ens.reduce(k).nonfinite) == 0 for k in range(len(boxes)))
