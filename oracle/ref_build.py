"""Build recipe of oracle/_ref/: the reference's own CUDA build, as a checker.

TEST INFRASTRUCTURE ONLY. Two parts:

* cubins: the device code of the reference's src/main.cu, compiled with nvcc
  for sm_103a from the sources where they lie (read-only), one per variant,
  with the flags of the reference's compile.sh:58-75 except -DENABLE_FP16
  (0 for the FP32 checker, 1 for the reference's default half-precision f)
  and -DBENCHMARK=1. The reference's own build system is not run. Variants at
  sizes the reference does not hard-code are compiled from a copy of
  src/ in a temporary directory outside the repository whose mesh constants
  (src/constants.cuh:84-89) are replaced; the copy is deleted afterwards.
  Needs /root/reference (present only in the build container); the cubins
  then travel with the repository to the GPU machine (git-ignored).
* ref_runner: oracle/ref_runner.cpp, a driver-API host program that loads a
  cubin and replays src/main.cu's launch sequence. Built wherever it runs
  (g++ -lcuda), since host binaries are per-architecture.
"""
from __future__ import annotations

import json
import platform
import shutil
import subprocess
import tempfile
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
REFERENCE = Path("/root/reference")
CUDA = Path("/usr/local/cuda")

FLAGS = ["-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--restrict", "--extra-device-vectorization",
         "--fmad=true", "--extended-lambda", "-std=c++20", "-DBENCHMARK=1", "-DTIME_AVERAGE=0",
         "-DREYNOLDS_MOMENTS=0", "-DVORTICITY_FIELDS=0", "-DPASSIVE_SCALAR=0"]

# name -> (case, Q, fp16, (nx, ny, nz), mesh patch or None)
VARIANTS = {
    "jet_d3q19": ("JET", 19, 0, (64, 64, 128), None),
    "jet_d3q27": ("JET", 27, 0, (64, 64, 128), None),
    "droplet_d3q19": ("DROPLET", 19, 0, (128, 128, 128), None),
    "droplet_d3q27": ("DROPLET", 27, 0, (128, 128, 128), None),
    "jet_d3q19_fp16": ("JET", 19, 1, (64, 64, 128), None),
    # the benchmark jet size: 128x128x512, inlet diameter 16
    "jet_d3q27_128x128x512": ("JET", 27, 0, (128, 128, 512), {"res": 128, "nz": 512, "diam": 16}),
    "jet_d3q19_128x128x512": ("JET", 19, 0, (128, 128, 512), {"res": 128, "nz": 512, "diam": 16}),
    "jet_d3q19_128x128x512_fp16": ("JET", 19, 1, (128, 128, 512), {"res": 128, "nz": 512, "diam": 16}),
}


def _patch_jet_mesh(constants: Path, patch: dict):
    text = constants.read_text()
    repl = [
        ("static constexpr label_t res = 64;", f"static constexpr label_t res = {patch['res']};"),
        ("static constexpr label_t nz = res * 2;", f"static constexpr label_t nz = {patch['nz']};"),
        ("static constexpr int diam = 10;", f"static constexpr int diam = {patch['diam']};"),
    ]
    for a, b in repl:
        if text.count(a) != 1:
            raise RuntimeError(f"mesh constant not found once in constants.cuh: {a!r}")
        text = text.replace(a, b)
    constants.write_text(text)


def build_cubins(reference: Path = REFERENCE, names=None) -> dict:
    if not (reference / "src" / "main.cu").exists():
        return {}
    OUT.mkdir(parents=True, exist_ok=True)
    manifest = {}

    def one(name):
        case, q, fp16, dims, patch = VARIANTS[name]
        out = OUT / f"ref_{name}.cubin"
        with tempfile.TemporaryDirectory(prefix="pflbm_ref_") as td:
            src = reference / "src"
            if patch:
                src = Path(td) / "src"
                shutil.copytree(reference / "src", src)
                _patch_jet_mesh(src / "constants.cuh", patch)
            cmd = ["nvcc", *FLAGS, f"-DVS_D3Q{q}", f"-D{case}", f"-DENABLE_FP16={fp16}", "-I", str(src),
                   str(src / "main.cu"), "-o", str(out)]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"reference cubin {name} failed:\n{r.stderr[-2000:]}")
        return name, {"cubin": out.name, "case": case.lower(), "q": q, "fp16": fp16, "dims": list(dims)}

    with ThreadPoolExecutor(max_workers=4) as ex:
        for name, entry in ex.map(one, names or list(VARIANTS)):
            manifest[name] = entry
    (OUT / "manifest.json").write_text(json.dumps(manifest, indent=1))
    return manifest


def build_runner() -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    exe = OUT / "ref_runner"
    src = HERE / "ref_runner.cpp"
    stamp = OUT / ".arch"
    same_arch = stamp.exists() and stamp.read_text().strip() == platform.machine()
    if same_arch and exe.exists() and exe.stat().st_mtime >= src.stat().st_mtime:
        return exe
    lib = CUDA / "lib64"
    stubs = lib / "stubs"
    cmd = ["g++", "-O2", "-std=c++17", f"-I{CUDA / 'include'}", str(src), "-o", str(exe), f"-L{lib}", f"-L{stubs}",
           "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("ref_runner build failed:\n" + r.stderr)
    stamp.write_text(platform.machine())
    return exe


def manifest() -> dict:
    p = OUT / "manifest.json"
    return json.loads(p.read_text()) if p.exists() else {}


if __name__ == "__main__":
    print(json.dumps(build_cubins(), indent=1))
    print(build_runner())
