"""ctypes binding of the CPU oracle (oracle/oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py, as the checker. The product never uses it.
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
_LIB = None


def build(force: bool = False) -> Path:
    src = HERE / "oracle.cpp"
    hdr = HERE.parent / "include" / "pflbm.h"
    stamp = HERE / "_build" / ".arch"
    same_arch = stamp.exists() and stamp.read_text().strip() == platform.machine()
    if (not force and same_arch and LIB_PATH.exists()
            and LIB_PATH.stat().st_mtime >= max(src.stat().st_mtime, hdr.stat().st_mtime)):
        return LIB_PATH
    r = subprocess.run(["make", "-C", str(HERE), "-B"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    stamp.write_text(platform.machine())
    return LIB_PATH


def load() -> ctypes.CDLL:
    global _LIB
    if _LIB is not None:
        return _LIB
    build()
    lib = ctypes.CDLL(str(LIB_PATH))
    vp, i32, u32, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_size_t
    fp = ctypes.POINTER(ctypes.c_float)
    lib.ora_config_reference.argtypes = [vp, i32, i32]
    lib.ora_create.argtypes = [vp, i32]
    lib.ora_create.restype = vp
    lib.ora_destroy.argtypes = [vp]
    lib.ora_init.argtypes = [vp]
    lib.ora_step.argtypes = [vp, i32]
    lib.ora_current_step.argtypes = [vp]
    lib.ora_current_step.restype = ctypes.c_uint64
    lib.ora_get_field.argtypes = [vp, i32, vp, sz]
    lib.ora_get_pops.argtypes = [vp, i32, vp, sz]
    lib.ora_node_feq.argtypes = [i32, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, fp]
    lib.ora_node_fneq.argtypes = [i32, fp, ctypes.c_float, ctypes.c_float, ctypes.c_float, fp]
    lib.ora_node_force.argtypes = [i32] + [ctypes.c_float] * 6 + [fp]
    lib.ora_node_geq.argtypes = [ctypes.c_float] * 4 + [fp]
    lib.ora_node_antidiff.argtypes = [ctypes.c_float] * 4 + [fp]
    lib.ora_velocity_set.argtypes = [i32, vp, vp, vp, vp]
    lib.ora_hash32.argtypes = [u32]
    lib.ora_hash32.restype = u32
    lib.ora_white_noise.argtypes = [u32, u32, u32, u32]
    lib.ora_white_noise.restype = ctypes.c_float
    lib.ora_uniform_noise.argtypes = [u32, u32, u32, u32]
    lib.ora_uniform_noise.restype = ctypes.c_float
    lib.ora_sponge_ramp.argtypes = [vp, u32]
    lib.ora_sponge_ramp.restype = ctypes.c_float
    lib.ora_relaxation.argtypes = [vp, fp]
    dp = ctypes.POINTER(ctypes.c_double)
    lib.ora_mlp_num_params.restype = i32
    lib.ora_mlp_eval.argtypes = [vp, vp, vp, ctypes.c_double, vp, vp, i32, vp, vp]
    lib.ora_set_closure.argtypes = [vp, vp, vp, vp, ctypes.c_double, ctypes.c_double]
    lib.ora_set_closure_mixing.argtypes = [vp, ctypes.c_double]
    _LIB = lib
    return lib


FIELDS = [
    "rho", "ux", "uy", "uz", "pxx", "pyy", "pzz", "pxy", "pxz", "pyz",
    "phi", "normx", "normy", "normz", "ind", "fsx", "fsy", "fsz",
    "avg_phi", "avg_ux", "avg_uy", "avg_uz",
    "avg_uxux", "avg_uyuy", "avg_uzuz", "avg_uxuy", "avg_uxuz", "avg_uyuz",
    "vort_x", "vort_y", "vort_z", "vort_mag", "c",
]


class OracleSim:
    """CPU restatement of the reference's time loop; fields as float64 (nz, ny, nx)."""

    def __init__(self, config, fp64: bool = False, threads: int | None = None):
        self.lib = load()
        if threads is not None:
            os.environ["OMP_NUM_THREADS"] = str(threads)
        self.config = config
        self._h = self.lib.ora_create(ctypes.byref(config), 1 if fp64 else 0)
        if not self._h:
            raise ValueError("oracle rejected the configuration")
        self.shape = (int(config.nz), int(config.ny), int(config.nx))
        self.lib.ora_init(self._h)

    def step(self, n: int = 1):
        self.lib.ora_step(self._h, int(n))

    @property
    def current_step(self) -> int:
        return int(self.lib.ora_current_step(self._h))

    def get_field(self, name: str) -> np.ndarray:
        a = np.empty(self.shape, np.float64)
        if self.lib.ora_get_field(self._h, FIELDS.index(name), a.ctypes.data, a.size) != 0:
            raise ValueError(f"field {name} not available in the oracle")
        return a

    def set_closure(self, params, mean, inv_scale, out_scale, strength=1.0):
        p = np.ascontiguousarray(params, np.float64)
        mu = np.ascontiguousarray(mean, np.float64)
        sc = np.ascontiguousarray(inv_scale, np.float64)
        self.lib.ora_set_closure(self._h, p.ctypes.data, mu.ctypes.data, sc.ctypes.data, float(out_scale), float(strength))

    def set_closure_mixing(self, inv_schmidt):
        self.lib.ora_set_closure_mixing(self._h, float(inv_schmidt))

    def close(self):
        if self._h:
            self.lib.ora_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def config_reference(flow_case: int, velocity_set: int):
    """The oracle's own restatement of src/constants.cuh:80-141."""
    from phasefieldlbm_gb300 import Config

    c = Config()
    load().ora_config_reference(ctypes.byref(c), flow_case, velocity_set)
    return c


def node_feq(vs, rho, ux, uy, uz):
    out = (ctypes.c_float * vs)()
    load().ora_node_feq(vs, rho, ux, uy, uz, out)
    return np.array(out, np.float32)


def node_fneq(vs, pi6, ux, uy, uz):
    p = (ctypes.c_float * 6)(*pi6)
    out = (ctypes.c_float * vs)()
    load().ora_node_fneq(vs, p, ux, uy, uz, out)
    return np.array(out, np.float32)


def node_force(vs, ux, uy, uz, fx, fy, fz):
    out = (ctypes.c_float * vs)()
    load().ora_node_force(vs, ux, uy, uz, fx, fy, fz, out)
    return np.array(out, np.float32)


def node_geq(phi, ux, uy, uz):
    out = (ctypes.c_float * 7)()
    load().ora_node_geq(phi, ux, uy, uz, out)
    return np.array(out, np.float32)


def node_antidiff(sharp, nx, ny, nz):
    out = (ctypes.c_float * 7)()
    load().ora_node_antidiff(sharp, nx, ny, nz, out)
    return np.array(out, np.float32)


def velocity_set(vs):
    cx, cy, cz = (ctypes.c_int * vs)(), (ctypes.c_int * vs)(), (ctypes.c_int * vs)()
    w = (ctypes.c_float * vs)()
    load().ora_velocity_set(vs, cx, cy, cz, w)
    return np.array([list(cx), list(cy), list(cz)], np.int64).T, np.array(w, np.float32)


def hash32(x: int) -> int:
    return int(load().ora_hash32(x))


def white_noise(salt, x, y, t) -> float:
    return float(load().ora_white_noise(salt, x, y, t))


def uniform_noise(seed, x, y, t) -> float:
    return float(load().ora_uniform_noise(seed, x, y, t))


def sponge_ramp(config, z) -> float:
    return float(load().ora_sponge_ramp(ctypes.byref(config), z))


def relaxation(config) -> np.ndarray:
    out = (ctypes.c_float * 7)()
    load().ora_relaxation(ctypes.byref(config), out)
    return np.array(out, np.float32)


def mlp_eval(params, mean, inv_scale, out_scale, x, targets=None, with_grad=False):
    """FP64 forward (and summed training-loss gradient) of the closure MLP."""
    lib = load()
    p = np.ascontiguousarray(params, np.float64)
    mu = np.ascontiguousarray(mean, np.float64)
    sc = np.ascontiguousarray(inv_scale, np.float64)
    xx = np.ascontiguousarray(x, np.float64).reshape(-1, 8)
    n = xx.shape[0]
    t = np.ascontiguousarray(targets if targets is not None else np.zeros(n), np.float64)
    out = np.empty(n, np.float64)
    g = np.empty(lib.ora_mlp_num_params(), np.float64) if with_grad else None
    lib.ora_mlp_eval(p.ctypes.data, mu.ctypes.data, sc.ctypes.data, float(out_scale), xx.ctypes.data, t.ctypes.data, n,
                     out.ctypes.data, g.ctypes.data if g is not None else None)
    return (out, g) if with_grad else out
