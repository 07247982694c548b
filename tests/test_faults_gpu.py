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
