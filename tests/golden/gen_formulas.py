"""Generates tests/golden/formulas.json from the reference's own headers.

The reference's velocity sets (src/velocitySet/D3Q19.cuh, D3Q27.cuh,
D3Q7.cuh) and relaxation constants (src/functions/globalFunctions.cuh) are
__host__ __device__, so a small host program compiled by nvcc can call them
directly. This script writes that program to a temporary directory, compiles
it against the reference sources where they lie (read-only), runs it on
seeded inputs and stores the inputs and float32 outputs. Nothing of the
reference is copied into the repository; only the numbers are kept.

    python tests/golden/gen_formulas.py [--reference <checkout>]

The reference checkout defaults to PFLBM_REFERENCE_SRC, else the build
container's copy at /root/reference.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

PROGRAM = r"""
#include <cstdio>
#include <utility>
#include "velocitySet/VelocitySet.cuh"

template <class VS, label_t... Q>
void per_q(std::integer_sequence<label_t, Q...>, const float *in) {
    const float rho = in[0], ux = in[1], uy = in[2], uz = in[3];
    const float pxx = in[4], pyy = in[5], pzz = in[6], pxy = in[7], pxz = in[8], pyz = in[9];
    const float fx = in[10], fy = in[11], fz = in[12];
    const float uu = 1.5f * (ux * ux + uy * uy + uz * uz);
    auto one = [&](auto q) {
        constexpr label_t QQ = decltype(q)::value;
        constexpr float cx = static_cast<float>(VS::template cx<QQ>());
        constexpr float cy = static_cast<float>(VS::template cy<QQ>());
        constexpr float cz = static_cast<float>(VS::template cz<QQ>());
        const float cu = VS::as2() * (cx * ux + cy * uy + cz * uz);
        std::printf("%.9g %.9g %.9g ", VS::template f_eq<QQ>(rho, uu, cu),
                    VS::template f_neq<QQ>(pxx, pyy, pzz, pxy, pxz, pyz, ux, uy, uz),
                    VS::template force<QQ>(cu, ux, uy, uz, fx, fy, fz));
    };
    (one(std::integral_constant<label_t, Q>{}), ...);
}

template <label_t... Q>
void phase_q(std::integer_sequence<label_t, Q...>, const float *in) {
    const float phi = in[0], ux = in[1], uy = in[2], uz = in[3], sharp = in[4], nx = in[5], ny = in[6], nz = in[7];
    auto one = [&](auto q) {
        constexpr label_t QQ = decltype(q)::value;
        std::printf("%.9g %.9g ", lbm::D3Q7::g_eq<QQ>(phi, ux, uy, uz), lbm::D3Q7::anti_diffusion<QQ>(sharp, nx, ny, nz));
    };
    (one(std::integral_constant<label_t, Q>{}), ...);
}

int main() {
    float in[16];
    int kind;
    while (std::scanf("%d", &kind) == 1) {
        const int n = kind == 7 ? 8 : 13;
        for (int i = 0; i < n; ++i) std::scanf("%f", &in[i]);
        if (kind == 19) per_q<lbm::D3Q19>(std::make_integer_sequence<label_t, 19>{}, in);
        else if (kind == 27) per_q<lbm::D3Q27>(std::make_integer_sequence<label_t, 27>{}, in);
        else phase_q(std::make_integer_sequence<label_t, 7>{}, in);
        std::printf("\n");
    }
    return 0;
}
"""


RELAX_PROGRAM = r"""
#include <cstdio>
#include "functions/globalFunctions.cuh"
int main() {
#if defined(JET)
    std::printf("%.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g\n", relaxation::tau_water(), relaxation::tau_oil(),
                relaxation::omco_zmin(), sponge::z_start(), sponge::inv_nz_m1(), sponge::inv_sponge(), physics::sigma,
                physics::gamma, relaxation::omco_zmax(0.3f));
#else
    std::printf("%.9g %.9g %.9g\n", relaxation::omega_ref(), physics::sigma, physics::gamma);
#endif
    return 0;
}
"""


def relaxation_constants(src: Path, td: Path) -> dict:
    """Compile-time constants of the reference's two default cases."""
    prog = td / "relax.cu"
    prog.write_text(RELAX_PROGRAM)
    out = {}
    for case in ("JET", "DROPLET"):
        exe = td / f"relax_{case}"
        subprocess.run(["nvcc", "-std=c++20", "--extended-lambda", "-I", str(src), "-DVS_D3Q19", f"-D{case}",
                        "-DENABLE_FP16=0", str(prog), "-o", str(exe)], check=True)
        vals = [float(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
        if case == "JET":
            keys = ["tau_water", "tau_oil", "omco_zmin", "z_start", "inv_nz_m1", "inv_sponge", "sigma", "gamma",
                    "omco_zmax_phi0.3"]
        else:
            keys = ["omega_ref", "sigma", "gamma"]
        out[case.lower()] = dict(zip(keys, vals))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("PFLBM_REFERENCE_SRC", "/root/reference"))
    ap.add_argument("--cases", type=int, default=24)
    args = ap.parse_args()
    src = Path(args.reference) / "src"
    rng = np.random.default_rng(20261203)
    cases = []
    for vs in (19, 27):
        for _ in range(args.cases):
            rho = 1 + 0.02 * rng.standard_normal()
            u = 0.06 * rng.standard_normal(3)
            pi = 2e-3 * rng.standard_normal(6)
            pi[:3] -= pi[:3].mean()
            F = 2e-4 * rng.standard_normal(3)
            cases.append((vs, np.float32([rho, *u, *pi, *F])))
    for _ in range(args.cases):
        phi = rng.uniform()
        u = 0.06 * rng.standard_normal(3)
        n = rng.standard_normal(3)
        n /= np.linalg.norm(n)
        cases.append((7, np.float32([phi, *u, 0.05 * phi * (1 - phi), *n])))
    with tempfile.TemporaryDirectory() as td:
        prog = Path(td) / "formulas.cu"
        prog.write_text(PROGRAM)
        exe = Path(td) / "formulas"
        subprocess.run(["nvcc", "-std=c++20", "--extended-lambda", "-I", str(src), "-DENABLE_FP16=0",
                        str(prog), "-o", str(exe)], check=True)
        stdin = "".join(f"{vs} " + " ".join(repr(float(v)) for v in x) + "\n" for vs, x in cases)
        out = subprocess.run([str(exe)], input=stdin, capture_output=True, text=True, check=True).stdout
        relax = relaxation_constants(src, Path(td))
    rows = out.strip().split("\n")
    golden = []
    for (vs, x), row in zip(cases, rows):
        vals = [float(v) for v in row.split()]
        if vs == 7:
            golden.append({"set": 7, "in": [float(v) for v in x], "geq": vals[0::2], "antidiff": vals[1::2]})
        else:
            golden.append({"set": vs, "in": [float(v) for v in x], "feq": vals[0::3], "fneq": vals[1::3],
                           "force": vals[2::3]})
    (HERE / "formulas.json").write_text(json.dumps({
        "generator": "tests/golden/gen_formulas.py",
        "source": "src/velocitySet/{D3Q19,D3Q27,D3Q7}.cuh compiled host-side with nvcc, float32",
        "relaxation": relax, "cases": golden}, indent=0))
    print(f"wrote {len(golden)} cases")


if __name__ == "__main__":
    main()
