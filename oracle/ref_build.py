"""Build recipe of oracle/_ref/: the reference's own CUDA build, as a checker.

TEST INFRASTRUCTURE ONLY. Two parts:

* cubins: the device code of the reference's src/main.cu, compiled with nvcc
  for sm_103a from the sources where they lie (read-only), one per variant,
  with the flags of the reference's compile.sh:58-75 except -DENABLE_FP16
  (0 for the FP32 checker, 1 for the reference's default half-precision f)
  and -DBENCHMARK=1. The reference's own build system is not run. Variants at
  sizes the reference does not hard-code are compiled from a copy of
  src/ in a temporary directory outside the repository whose mesh constants
  (src/constants.cuh:84-89) are replaced, and for the benchmark presets also
  gamma (src/constants.cuh:108) and the inflow noise
  (src/BoundaryConditions.cuh:67-69); the copy is deleted afterwards.
  Needs the reference checkout (present only in the build container,
  PFLBM_REFERENCE_SRC); the cubins then travel with the repository to the
  GPU machine (git-ignored).
* ref_runner: oracle/ref_runner.cpp, a driver-API host program that loads a
  cubin and replays src/main.cu's launch sequence. Built wherever it runs
  (g++ -lcuda), since host binaries are per-architecture.
"""
from __future__ import annotations

import json
import os
import platform
import shutil
import subprocess
import tempfile
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
# the reference checkout (read-only); PFLBM_REFERENCE_SRC overrides the
# location of this build container's copy
REFERENCE = Path(os.environ.get("PFLBM_REFERENCE_SRC", "/root/reference"))
CUDA = Path("/usr/local/cuda")

FLAGS = ["-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--restrict", "--extra-device-vectorization",
         "--fmad=true", "--extended-lambda", "-std=c++20", "-DBENCHMARK=1", "-DTIME_AVERAGE=0",
         "-DREYNOLDS_MOMENTS=0", "-DVORTICITY_FIELDS=0", "-DPASSIVE_SCALAR=0"]

# name -> (case, Q, fp16, (nx, ny, nz), patch or None). A patch sets the jet
# mesh (res, nz, diam) and, with "preset", also the benchmark preset's
# physics: gamma = 0.05 instead of the derived 4 D / (W cs2), and the seeded
# uniform +-5% u_z inflow noise (seed 12345) instead of the Gaussian u_x, u_y
# noise, so that the build runs exactly the benchmark jet.
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
    # the benchmark presets themselves (jet_d3q27 / jet_d3q19)
    "jet_d3q27_bench": ("JET", 27, 0, (128, 128, 512),
                        {"res": 128, "nz": 512, "diam": 16, "preset": {"gamma": "0.05", "noise_amp": "0.05",
                                                                       "seed": 12345}}),
    "jet_d3q19_bench": ("JET", 19, 0, (128, 128, 512),
                        {"res": 128, "nz": 512, "diam": 16, "preset": {"gamma": "0.05", "noise_amp": "0.05",
                                                                       "seed": 12345}}),
}

# Uniform inflow noise of the benchmark presets, in the reference's own
# helpers (hash32, uniform01 of BoundaryConditions.cuh): u_z = u_inf (1 + a xi),
# xi = 2 uniform01(hash32(base)) - 1 with the base of white_noise salted by
# 0x2545F491 ^ seed, each operation rounded as written.
_UNIFORM_INFLOW = """            const uint32_t ubase = (0x9E3779B9u ^ (0x2545F491u ^ {seed}u)) ^ static_cast<uint32_t>(x) ^
                                   (static_cast<uint32_t>(y) * 0x85EBCA6Bu) ^ (static_cast<uint32_t>(t) * 0xC2B2AE35u);
            const float uxi = 2.0f * uniform01(hash32(ubase)) - 1.0f;
            const scalar_t ux = static_cast<scalar_t>(0);
            const scalar_t uy = static_cast<scalar_t>(0);
            const scalar_t uz = __fmul_rn(physics::u_inf, __fadd_rn(1.0f, __fmul_rn({amp}f, uxi)));
"""


def _replace_once(text: str, a: str, b: str, where: str) -> str:
    if text.count(a) != 1:
        raise RuntimeError(f"patch target not found exactly once in {where}: {a!r}")
    return text.replace(a, b)


def _patch_jet(src: Path, patch: dict):
    constants = src / "constants.cuh"
    text = constants.read_text()
    text = _replace_once(text, "static constexpr label_t res = 64;", f"static constexpr label_t res = {patch['res']};",
                         "constants.cuh")
    text = _replace_once(text, "static constexpr label_t nz = res * 2;",
                         f"static constexpr label_t nz = {patch['nz']};", "constants.cuh")
    text = _replace_once(text, "static constexpr int diam = 10;", f"static constexpr int diam = {patch['diam']};",
                         "constants.cuh")
    pre = patch.get("preset")
    if pre:
        # gamma of the JET section only (the DROPLET section has the same line)
        jet, sep, rest = text.partition("#elif defined(DROPLET)")
        jet = _replace_once(jet, "static constexpr scalar_t gamma = kappa / phase::velocitySet::cs2();",
                            f"static constexpr scalar_t gamma = static_cast<scalar_t>({pre['gamma']});",
                            "constants.cuh (JET)")
        text = jet + sep + rest
        bc = src / "BoundaryConditions.cuh"
        btext = bc.read_text()
        btext = _replace_once(btext, """            const scalar_t ux = sigma_u * zx;
            const scalar_t uy = sigma_u * zy;
            const scalar_t uz = physics::u_inf;
""", _UNIFORM_INFLOW.format(seed=pre["seed"], amp=pre["noise_amp"]), "BoundaryConditions.cuh")
        bc.write_text(btext)
    constants.write_text(text)


def build_cubins(reference: Path = REFERENCE, names=None) -> dict:
    if not (reference / "src" / "main.cu").exists():
        return {}
    OUT.mkdir(parents=True, exist_ok=True)
    # variants built earlier stay listed when only some are rebuilt
    entries = {k: v for k, v in manifest().items() if (OUT / v["cubin"]).exists()}

    def one(name):
        case, q, fp16, dims, patch = VARIANTS[name]
        out = OUT / f"ref_{name}.cubin"
        with tempfile.TemporaryDirectory(prefix="pflbm_ref_") as td:
            src = reference / "src"
            if patch:
                src = Path(td) / "src"
                shutil.copytree(reference / "src", src)
                _patch_jet(src, patch)
            cmd = ["nvcc", *FLAGS, f"-DVS_D3Q{q}", f"-D{case}", f"-DENABLE_FP16={fp16}", "-I", str(src),
                   str(src / "main.cu"), "-o", str(out)]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"reference cubin {name} failed:\n{r.stderr[-2000:]}")
        return name, {"cubin": out.name, "case": case.lower(), "q": q, "fp16": fp16, "dims": list(dims)}

    with ThreadPoolExecutor(max_workers=4) as ex:
        for name, entry in ex.map(one, names or list(VARIANTS)):
            entries[name] = entry
    (OUT / "manifest.json").write_text(json.dumps(entries, indent=1))
    return entries


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
    cmd = ["g++", "-O2", "-std=c++20", f"-I{CUDA / 'include'}", str(src), "-o", str(exe), f"-L{lib}", f"-L{stubs}",
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
