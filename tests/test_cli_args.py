"""pipeline.sh / compile.sh reject bad arguments before they build, run or
delete anything (no GPU needed). The id names the output directory that
pipeline.sh empties, so path-like ids must never get that far."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.parametrize("args,msg", [
    ([], "Insufficient arguments"),
    (["JET", "D3Q19", "../../x"], "Invalid id"),
    (["JET", "D3Q19", "a/b"], "Invalid id"),
    (["JET", "D3Q19", ""], "Insufficient arguments"),
    (["JET", "D3Q15", "000"], "Invalid velocity_set"),
    (["FOO", "D3Q19", "000"], "Invalid flow_case"),
])
def test_pipeline_rejects_bad_arguments(args, msg):
    r = subprocess.run(["bash", "pipeline.sh", *args], cwd=ROOT, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert msg in r.stdout
    assert "Compiling" not in r.stdout


def test_compile_rejects_path_like_id():
    r = subprocess.run(["bash", "compile.sh", "JET", "D3Q19", "../x"], cwd=ROOT, capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 1
    assert "Invalid ID" in r.stdout
