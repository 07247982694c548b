"""Build of the CUDA library libpflbm.so (sm_103a) with nvcc.

The library is a plain C-ABI shared object (include/pflbm.h); it does not
link against PyTorch. Translation units are compiled in parallel, one per
population storage type, then linked with ``nvcc -shared``.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libpflbm.so"
DRIVER = BUILD / "pflbm_run"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++20", "-lineinfo", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr"]
SOURCES = ["api.cu", "engine_fp32.cu", "engine_fp64.cu", "engine_fp16.cu", "engine_bf16.cu", "ensemble.cu", "noalloc.cu", "closure.cu"]
HOST_SOURCES = ["driver_main.cpp"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpflbm.so")
    return exe


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(
        CSRC.glob("*.cpp")) + [
        PKG.parent / "include" / "pflbm.h"
    ]


STAMP = BUILD / ".arch"


def up_to_date() -> bool:
    if not LIB.exists() or not DRIVER.exists():
        return False
    # binaries built on another architecture are never reused
    if not STAMP.exists() or STAMP.read_text().strip() != platform.machine():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def build(verbose: bool = False, force: bool = False, jobs: int | None = None) -> Path:
    """Compiles libpflbm.so if a source is newer than it; returns its path."""
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    exe = nvcc()
    objs = []

    def compile_one(src: str) -> Path:
        obj = BUILD / (Path(src).stem + ".o")
        cmd = [exe, *ARCH, *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=jobs or min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [exe, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    # the drop-in driver executable (host C++ over the C ABI)
    cmd = ["g++", "-O2", "-std=c++20", str(CSRC / "driver_main.cpp"), "-o", str(DRIVER), f"-L{BUILD}", "-lpflbm",
           "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{r.stderr}")
    STAMP.write_text(platform.machine())
    return LIB


CHECKED = BUILD / "checked"


def build_variant(name: str, defines: list[str], jobs: int | None = None) -> Path:
    """A test build of the library with extra preprocessor definitions, in
    _build/<name>/libpflbm.so (rebuilt when a source is newer). Test builds
    are loaded only by the tests, beside the shipped library."""
    out = BUILD / name
    lib = out / "libpflbm.so"
    stamp = out / ".arch"
    if (lib.exists() and stamp.exists() and stamp.read_text().strip() == platform.machine()
            and all(p.stat().st_mtime <= lib.stat().st_mtime for p in _deps())):
        return lib
    out.mkdir(parents=True, exist_ok=True)
    exe = nvcc()

    def compile_one(src: str) -> Path:
        obj = out / (Path(src).stem + ".o")
        cmd = [exe, *ARCH, *NVCC_FLAGS, *defines, "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=jobs or min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = lib.with_suffix(".so.tmp")
    r = subprocess.run([exe, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"], capture_output=True,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, lib)
    stamp.write_text(platform.machine())
    return lib


def build_checked(jobs: int | None = None) -> Path:
    """A test build of the library with -DPFLBM_CHECK_BOUNDS: every guarded
    global store of the step kernels checks its index and reports a miss in
    the device error word instead of writing (see PFLBM_GUARD). Returns the
    path of _build/checked/libpflbm.so (rebuilt when a source is newer)."""
    return build_variant("checked", ["-DPFLBM_CHECK_BOUNDS"], jobs)


def build_dead_wait(jobs: int | None = None) -> Path:
    """A test build with -DPFLBM_TEST_DEAD_WAIT: the collide pipelines' first
    wait of every plane polls an mbarrier that nothing arrives on, with a
    short limit, so that the bounded wait runs out and the kernel reports
    through the device error word and returns (_build/deadwait/libpflbm.so)."""
    return build_variant("deadwait", ["-DPFLBM_TEST_DEAD_WAIT"], jobs)


def build_dead_grid(jobs: int | None = None) -> Path:
    """A test build with -DPFLBM_TEST_DEAD_GRID: the grid-wide barrier of the
    ensemble's fused step polls a flag that nothing sets, with a short limit,
    so that every CTA gives up, sets the device error word and returns
    (_build/deadgrid/libpflbm.so)."""
    return build_variant("deadgrid", ["-DPFLBM_TEST_DEAD_GRID"], jobs)


if __name__ == "__main__":
    print(build(verbose=True, force=True))
