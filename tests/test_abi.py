"""The C-ABI library builds, loads and exports every symbol of include/pflbm.h,
and rejects bad configurations before touching the GPU (no GPU needed)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def header_symbols():
    text = (ROOT / "include" / "pflbm.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*|void)\s*\*?\s*(pflbm_\w+)\s*\(", text, re.M)))


def test_header_declares_api():
    syms = header_symbols()
    for s in ("pflbm_create", "pflbm_init", "pflbm_step", "pflbm_get_field", "pflbm_reduce", "pflbm_destroy"):
        assert s in syms


def test_library_exports_every_declared_symbol(pflbm):
    lib = pflbm.load_library()
    for s in header_symbols():
        assert hasattr(lib, s), s
        # the Python binding declares a ctypes signature for every entry point
        assert getattr(lib, s).argtypes is not None, s
    assert set(pflbm.EXPORTED_SYMBOLS) == set(header_symbols())
    assert lib.pflbm_abi_version() == 1


def test_config_struct_size(pflbm):
    # struct_size guards the binding against header skew
    c = pflbm.config_reference(pflbm.CASE_JET, pflbm.VS_D3Q19)
    assert c.struct_size == ctypes.sizeof(pflbm.Config)


@pytest.mark.parametrize(
    "field,value,msg",
    [
        ("velocity_set", 15, "velocity_set"),
        ("flow_case", 7, "flow_case"),
        ("storage", 9, "storage"),
        ("nx", 3, "nx"),
        ("nz", 8, "nz >= 12"),
        ("radius", 40, "inlet disc"),
        ("inflow_noise", 5, "inflow_noise"),
        ("struct_size", 12, "struct_size"),
    ],
)
def test_create_rejects_bad_config(pflbm, field, value, msg):
    lib = pflbm.load_library()
    c = pflbm.config_reference(pflbm.CASE_JET, pflbm.VS_D3Q19)
    setattr(c, field, value)
    h = ctypes.c_void_p()
    rc = lib.pflbm_create(ctypes.byref(c), ctypes.byref(h))
    assert rc == 1  # PFLBM_ERR_INVALID_ARG
    assert msg in lib.pflbm_last_error().decode()
    assert not h.value


def test_droplet_tau_validation(pflbm):
    lib = pflbm.load_library()
    c = pflbm.config_reference(pflbm.CASE_DROPLET, pflbm.VS_D3Q27)
    c.tau = 0.5
    h = ctypes.c_void_p()
    assert lib.pflbm_create(ctypes.byref(c), ctypes.byref(h)) == 1


def test_null_arguments(pflbm):
    lib = pflbm.load_library()
    assert lib.pflbm_create(None, None) == 1
    assert lib.pflbm_init(None) == 1
    assert lib.pflbm_step(None, 1) == 1
    assert lib.pflbm_destroy(None) == 0


def test_presets_are_valid_configs(pflbm):
    for name in ("droplet64", "jet_d3q27", "jet_d3q19", "jet_precision", "jet_closure"):
        c = pflbm.preset(name)
        assert c.struct_size == ctypes.sizeof(pflbm.Config)
    j = pflbm.preset("jet_d3q27")
    assert (j.nx, j.ny, j.nz, j.velocity_set, j.diam) == (128, 128, 512, 27, 16)
    assert abs(j.sigma - 8e-5) < 1e-9


def test_header_is_plain_c_and_links(tmp_path, pflbm):
    """include/pflbm.h compiles as C99 and a C program links libpflbm and
    calls it (no GPU needed: configuration defaults and validation only)."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = Path(pflbm.load_library()._name)
    src = tmp_path / "abi.c"
    src.write_text(r'''
#include <stdio.h>
#include "pflbm.h"
int main(void) {
    pflbm_config c;
    if (pflbm_abi_version() != PFLBM_ABI_VERSION) return 2;
    if (pflbm_config_reference(&c, PFLBM_CASE_JET, PFLBM_VS_D3Q19) != PFLBM_OK) return 3;
    c.nz = 8;  /* rejected before any device work */
    pflbm_sim *s = 0;
    if (pflbm_create(&c, &s) != PFLBM_ERR_INVALID_ARG || s) return 4;
    printf("%u %u %u %s\n", c.nx, c.ny, c.struct_size, pflbm_last_error());
    return 0;
}
''')
    exe = tmp_path / "abi"
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(src), "-o", str(exe),
                        "-L", str(lib.parent), "-lpflbm", f"-Wl,-rpath,{lib.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert "nz >= 12" in r.stdout


def test_create_rejects_grids_of_2_32_nodes(pflbm):
    # the step kernels index a node within one array with 32 bits
    lib = pflbm.load_library()
    c = pflbm.config_reference(pflbm.CASE_JET, pflbm.VS_D3Q19)
    c.nx, c.ny, c.nz = 2048, 2048, 1024
    h = ctypes.c_void_p()
    assert lib.pflbm_create(ctypes.byref(c), ctypes.byref(h)) == 1
    assert "2^32" in lib.pflbm_last_error().decode()
    assert not h.value
