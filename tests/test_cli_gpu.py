"""The drop-in driver surface: pipeline.sh <JET|DROPLET> <D3Q19|D3Q27> <id>
builds (compile.sh) and runs pflbm_run, which writes the reference's layout
bin/<case>/<set>/<id>/{<id>_info.txt, <field><step06>.bin, step_<step06>.vti}
(src/main.cu:130-133, hostFunctions.cuh:33-46, PostProcess.cuh:43-261). The
arrays are exactly what the library API returns for the same run."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def test_pipeline_writes_reference_layout(pflbm):
    run_id = "T900"
    args = ["--steps", "20", "--save", "10", "--nx", "32", "--ny", "32", "--nz", "48", "--diam", "8"]
    r = subprocess.run(["bash", "pipeline.sh", "JET", "D3Q19", run_id, *args], cwd=ROOT, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    out = ROOT / "bin" / "JET" / "D3Q19" / run_id
    info = (out / f"{run_id}_info.txt").read_text()
    assert "NX:                    32" in info
    n = 32 * 32 * 48
    for step in (0, 10, 20):
        for f in ("rho", "uz"):
            p = out / f"{f}{step:06d}.bin"
            assert p.stat().st_size == 4 * n, p
        assert (out / f"step_{step:06d}.vti").exists()
    cfg = pflbm.config_reference(pflbm.CASE_JET, pflbm.VS_D3Q19)
    cfg.nx, cfg.ny, cfg.nz, cfg.diam, cfg.radius = 32, 32, 48, 8, 4
    with pflbm.Simulation(cfg) as s:
        s.step(21)  # output step 20 is written after 21 completed steps (step index 0 .. 20)
        for f in ("rho", "uz"):
            ref = s.get_field(f).reshape(-1)
            got = np.fromfile(out / f"{f}000020.bin", np.float32)
            assert np.array_equal(got, ref), f


def test_async_output_matches_sync(pflbm, tmp_path):
    """pflbm_write_output_async stages the fields before returning; stepping
    on while the writer thread runs leaves the written step unchanged."""
    cfg = pflbm.config_reference(pflbm.CASE_JET, pflbm.VS_D3Q19)
    cfg.nx, cfg.ny, cfg.nz, cfg.diam, cfg.radius = 32, 32, 48, 8, 4
    fields = ("rho", "uz", "phi")
    with pflbm.Simulation(cfg) as s:
        s.step(11)
        s.write_output(tmp_path / "sync", fields)
        s.write_output(tmp_path / "async", fields, wait=False)
        s.step(7)  # runs while the files are written
        s.synchronize()
    for f in fields:
        a = (tmp_path / "sync" / f"{f}000010.bin").read_bytes()
        b = (tmp_path / "async" / f"{f}000010.bin").read_bytes()
        assert a == b and len(a) == 4 * 32 * 32 * 48, f
    assert (tmp_path / "sync" / "step_000010.vti").read_bytes() == (tmp_path / "async" / "step_000010.vti").read_bytes()
