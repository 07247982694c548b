"""The user-facing documents cover the library's interface: every environment
switch the CUDA library reads is listed in README.md, and every C-ABI entry
point of include/pflbm.h appears in INTEGRATION.md (no GPU needed)."""
import re
from pathlib import Path

from test_abi import header_symbols

ROOT = Path(__file__).resolve().parent.parent


def test_every_environment_switch_is_documented():
    src = ROOT / "phasefieldlbm_gb300" / "csrc"
    names = set()
    for f in list(src.glob("*.cu")) + list(src.glob("*.cuh")) + list(src.glob("*.cpp")):
        names |= set(re.findall(r'getenv\("([A-Z_0-9]+)"\)', f.read_text()))
    assert names, "no switches found"
    readme = (ROOT / "README.md").read_text()
    missing = sorted(n for n in names if f"`{n}" not in readme)
    assert not missing, missing


def test_every_entry_point_is_in_the_integration_guide():
    guide = (ROOT / "INTEGRATION.md").read_text()
    missing = []
    for s in header_symbols():
        # the guide's table abbreviates families as `pflbm_ensemble_create` / `_init` / ...
        short = "_" + s.split("_", 2)[-1] if s.count("_") >= 2 else s
        if s not in guide and f"`{short}`" not in guide:
            missing.append(s)
    assert not missing, missing
