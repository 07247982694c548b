"""GB300-native phase-field lattice-Boltzmann hot path (Python host mirror).

The compute path is the CUDA library ``libpflbm.so`` behind the C ABI of
``include/pflbm.h``; this module binds it with ctypes and mirrors the
reference's driver vocabulary (flow case, velocity set, field names of
src/fileIO/fields.cuh:33-68). There is no CPU fallback: if the library is
missing or no CUDA device is present, creating a Simulation raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import build as _build

__all__ = [
    "CASE_DROPLET", "CASE_JET", "VS_D3Q19", "VS_D3Q27",
    "STORAGE_FP32", "STORAGE_FP16", "STORAGE_BF16", "STORAGE_FP64",
    "NOISE_GAUSSIAN_UXY", "NOISE_UNIFORM_UZ",
    "FLAG_TIME_AVERAGE", "FLAG_REYNOLDS_MOMENTS", "FLAG_VORTICITY",
    "FIELDS", "Config", "Diag", "PflbmError", "Simulation",
    "load_library", "config_reference", "preset", "EXPORTED_SYMBOLS", "Ensemble", "ensemble_configs",
]

CASE_DROPLET, CASE_JET = 0, 1
VS_D3Q19, VS_D3Q27 = 19, 27
STORAGE_FP32, STORAGE_FP16, STORAGE_BF16, STORAGE_FP64 = 0, 1, 2, 3
NOISE_GAUSSIAN_UXY, NOISE_UNIFORM_UZ = 0, 1
FLAG_TIME_AVERAGE, FLAG_REYNOLDS_MOMENTS, FLAG_VORTICITY = 1, 2, 4

# pflbm_field_id, in the order of host::FieldID (src/fileIO/fields.cuh:33-68)
FIELDS = [
    "rho", "ux", "uy", "uz", "pxx", "pyy", "pzz", "pxy", "pxz", "pyz",
    "phi", "normx", "normy", "normz", "ind", "fsx", "fsy", "fsz",
    "avg_phi", "avg_ux", "avg_uy", "avg_uz",
    "avg_uxux", "avg_uyuy", "avg_uzuz", "avg_uxuy", "avg_uxuz", "avg_uyuz",
    "vort_x", "vort_y", "vort_z", "vort_mag", "c",
]
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}

EXPORTED_SYMBOLS = [
    "pflbm_abi_version", "pflbm_last_error", "pflbm_config_reference", "pflbm_create",
    "pflbm_init", "pflbm_set_initial_field", "pflbm_step", "pflbm_step_async",
    "pflbm_synchronize", "pflbm_step_profiled", "pflbm_current_step", "pflbm_get_field", "pflbm_get_field_f64",
    "pflbm_reduce", "pflbm_write_output", "pflbm_save_checkpoint", "pflbm_load_checkpoint",
    "pflbm_device_bytes", "pflbm_uses_tma", "pflbm_collide_variant", "pflbm_kernels_per_step",
    "pflbm_destroy",
    "pflbm_ensemble_create", "pflbm_ensemble_init", "pflbm_ensemble_step", "pflbm_ensemble_step_profiled",
    "pflbm_ensemble_get_field", "pflbm_ensemble_reduce", "pflbm_ensemble_set_tuning", "pflbm_ensemble_autotune",
    "pflbm_ensemble_info", "pflbm_ensemble_destroy", "pflbm_ensemble_set_tile", "pflbm_ensemble_get_tuning",
    "pflbm_reduce_fields_noalloc", "pflbm_write_output_async", "pflbm_set_watchdog",
    "pflbm_closure_create", "pflbm_closure_add_snapshot", "pflbm_closure_num_samples", "pflbm_closure_get_samples",
    "pflbm_closure_interface_scale",
    "pflbm_closure_set_samples", "pflbm_closure_init_params", "pflbm_closure_get_blob", "pflbm_closure_set_blob",
    "pflbm_closure_gradient", "pflbm_closure_train", "pflbm_closure_loss", "pflbm_closure_destroy",
    "pflbm_set_closure", "pflbm_set_closure_mixing",
]


class Config(ctypes.Structure):
    """pflbm_config (include/pflbm.h)."""

    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("flow_case", ctypes.c_int32),
        ("velocity_set", ctypes.c_int32),
        ("storage", ctypes.c_int32),
        ("nx", ctypes.c_uint32),
        ("ny", ctypes.c_uint32),
        ("nz", ctypes.c_uint32),
        ("radius", ctypes.c_int32),
        ("diam", ctypes.c_int32),
        ("droplet_x_stretch", ctypes.c_float),
        ("center_offset", ctypes.c_float * 3),
        ("u_inf", ctypes.c_float),
        ("reynolds_water", ctypes.c_float),
        ("reynolds_oil", ctypes.c_float),
        ("sigma", ctypes.c_float),
        ("interface_width", ctypes.c_float),
        ("gamma", ctypes.c_float),
        ("tau", ctypes.c_float),
        ("sponge_gain", ctypes.c_float),
        ("sponge_cells", ctypes.c_int32),
        ("inflow_noise", ctypes.c_int32),
        ("noise_amp", ctypes.c_float),
        ("seed", ctypes.c_uint32),
        ("init_noise", ctypes.c_float),
        ("flags", ctypes.c_uint32),
        ("device", ctypes.c_int32),
    ]

    def copy(self) -> "Config":
        c = Config()
        ctypes.memmove(ctypes.byref(c), ctypes.byref(self), ctypes.sizeof(Config))
        return c

    def as_dict(self) -> dict:
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v) if name == "center_offset" else v
        return d

    @property
    def nodes(self) -> int:
        return int(self.nx) * int(self.ny) * int(self.nz)


class Diag(ctypes.Structure):
    """pflbm_diag (include/pflbm.h)."""

    _fields_ = [
        ("step", ctypes.c_uint64),
        ("phi_mass", ctypes.c_double),
        ("rho_mass", ctypes.c_double),
        ("momentum", ctypes.c_double * 3),
        ("max_speed", ctypes.c_double),
        ("rho_in", ctypes.c_double),
        ("rho_out", ctypes.c_double),
        ("laplace_dp", ctypes.c_double),
        ("n_in", ctypes.c_uint64),
        ("n_out", ctypes.c_uint64),
        ("nonfinite", ctypes.c_uint64),
    ]


class PflbmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"pflbm error {code}: {msg}")
        self.code = code


_LIB = None


def load_library(path: str | os.PathLike | None = None, build_if_missing: bool = True) -> ctypes.CDLL:
    """Loads libpflbm.so (building it with nvcc first if it is absent)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else _build.LIB
    if not p.exists():
        if not build_if_missing:
            raise RuntimeError(f"{p} is missing; run phasefieldlbm_gb300.build.build()")
        _build.build()
    lib = ctypes.CDLL(str(p))
    vp, i32, u32, u64, sz = ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_size_t
    sig = {
        "pflbm_abi_version": ([], ctypes.c_int),
        "pflbm_last_error": ([], ctypes.c_char_p),
        "pflbm_config_reference": ([ctypes.POINTER(Config), i32, i32], ctypes.c_int),
        "pflbm_create": ([ctypes.POINTER(Config), ctypes.POINTER(vp)], ctypes.c_int),
        "pflbm_init": ([vp], ctypes.c_int),
        "pflbm_set_initial_field": ([vp, i32, vp, sz], ctypes.c_int),
        "pflbm_step": ([vp, u64], ctypes.c_int),
        "pflbm_step_async": ([vp, u64], ctypes.c_int),
        "pflbm_synchronize": ([vp], ctypes.c_int),
        "pflbm_current_step": ([vp, ctypes.POINTER(u64)], ctypes.c_int),
        "pflbm_step_profiled": ([vp, u64, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), i32],
                                ctypes.c_int),
        "pflbm_get_field": ([vp, i32, vp, sz], ctypes.c_int),
        "pflbm_get_field_f64": ([vp, i32, vp, sz], ctypes.c_int),
        "pflbm_reduce": ([vp, ctypes.POINTER(Diag)], ctypes.c_int),
        "pflbm_reduce_fields_noalloc": ([vp, vp, vp, vp, vp, i32, i32, i32, vp, vp], ctypes.c_int),
        "pflbm_write_output": ([vp, ctypes.c_char_p, ctypes.POINTER(i32), i32], ctypes.c_int),
        "pflbm_write_output_async": ([vp, ctypes.c_char_p, ctypes.POINTER(i32), i32], ctypes.c_int),
        "pflbm_set_watchdog": ([vp, u64, ctypes.c_double], ctypes.c_int),
        "pflbm_device_bytes": ([vp, ctypes.POINTER(u64)], ctypes.c_int),
        "pflbm_save_checkpoint": ([vp, ctypes.c_char_p], ctypes.c_int),
        "pflbm_load_checkpoint": ([vp, ctypes.c_char_p], ctypes.c_int),
        "pflbm_kernels_per_step": ([vp, ctypes.POINTER(i32)], ctypes.c_int),
        "pflbm_uses_tma": ([vp, ctypes.POINTER(i32)], ctypes.c_int),
        "pflbm_collide_variant": ([vp, ctypes.POINTER(i32)], ctypes.c_int),
        "pflbm_destroy": ([vp], ctypes.c_int),
        "pflbm_ensemble_create": ([ctypes.POINTER(Config), i32, ctypes.POINTER(vp)], ctypes.c_int),
        "pflbm_ensemble_init": ([vp], ctypes.c_int),
        "pflbm_ensemble_step": ([vp, u64], ctypes.c_int),
        "pflbm_ensemble_step_profiled": ([vp, u64, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
        "pflbm_ensemble_get_field": ([vp, i32, i32, vp, sz], ctypes.c_int),
        "pflbm_ensemble_reduce": ([vp, i32, ctypes.POINTER(Diag)], ctypes.c_int),
        "pflbm_ensemble_set_tuning": ([vp, i32, i32], ctypes.c_int),
        "pflbm_ensemble_autotune": ([vp, i32, ctypes.POINTER(i32), ctypes.POINTER(i32), ctypes.POINTER(ctypes.c_double)],
                                    ctypes.c_int),
        "pflbm_ensemble_info": ([vp, ctypes.POINTER(u64), ctypes.POINTER(i32), ctypes.POINTER(i32)], ctypes.c_int),
        "pflbm_ensemble_set_tile": ([vp, i32, i32], ctypes.c_int),
        "pflbm_ensemble_get_tuning": ([vp] + [ctypes.POINTER(i32)] * 4, ctypes.c_int),
        "pflbm_ensemble_destroy": ([vp], ctypes.c_int),
        "pflbm_closure_create": ([i32, u64, ctypes.POINTER(vp)], ctypes.c_int),
        "pflbm_closure_add_snapshot": ([vp, vp, i32, ctypes.POINTER(u64)], ctypes.c_int),
        "pflbm_closure_num_samples": ([vp, ctypes.POINTER(u64)], ctypes.c_int),
        "pflbm_closure_interface_scale": ([vp] + [ctypes.POINTER(ctypes.c_double)] * 3, ctypes.c_int),
        "pflbm_closure_get_samples": ([vp, u64, u64, vp, vp], ctypes.c_int),
        "pflbm_closure_set_samples": ([vp, vp, vp, u64], ctypes.c_int),
        "pflbm_closure_init_params": ([vp, u32], ctypes.c_int),
        "pflbm_closure_get_blob": ([vp, vp], ctypes.c_int),
        "pflbm_closure_set_blob": ([vp, vp], ctypes.c_int),
        "pflbm_closure_gradient": ([vp, u64, vp, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
        "pflbm_closure_train": ([vp, i32, i32, ctypes.c_float, u32, vp], ctypes.c_int),
        "pflbm_closure_loss": ([vp, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
        "pflbm_closure_destroy": ([vp], ctypes.c_int),
        "pflbm_set_closure": ([vp, vp, ctypes.c_float], ctypes.c_int),
        "pflbm_set_closure_mixing": ([vp, ctypes.c_float], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if lib.pflbm_abi_version() != 1:
        raise RuntimeError("libpflbm ABI version mismatch")
    if path is None:
        _LIB = lib
    return lib


def _check(lib, rc: int):
    if rc != 0:
        raise PflbmError(rc, lib.pflbm_last_error().decode(errors="replace"))


def config_reference(flow_case: int, velocity_set: int) -> Config:
    """The reference's compile-time configuration (src/constants.cuh:80-141)."""
    lib = load_library()
    c = Config()
    _check(lib, lib.pflbm_config_reference(ctypes.byref(c), flow_case, velocity_set))
    return c


@dataclass(frozen=True)
class Preset:
    name: str
    description: str


def preset(name: str, base=None, **overrides) -> Config:
    """Configurations of the benchmark workloads (seeded synthetic cases).

    droplet64        static droplet, D3Q19, 64^3 periodic, R=16, tau=0.6,
                     sigma=0.01, gamma=0.05, spherical
    jet_d3q27        turbulent jet, D3Q27, 128x128x512, D=16, u=0.05,
                     Re=5000, We=500, gamma=0.05, uniform +-5% uz noise
    jet_d3q19        the same jet in D3Q19
    jet_precision    D3Q19 256x256x1024, D=32
    jet_closure      D3Q19 128x128x512, D=16, Re=10000
    jet_closure_fine the same jet on the 2x finer grid: 256x256x1024, D=32

    `base(flow_case, velocity_set) -> Config` supplies the reference's
    compile-time configuration the preset starts from; by default the
    library's pflbm_config_reference. A caller that must not load the
    library passes another restatement of src/constants.cuh:80-141.
    """
    if base is None:
        base = config_reference
    if name == "droplet64":
        c = base(CASE_DROPLET, VS_D3Q19)
        c.nx = c.ny = c.nz = 64
        c.radius, c.diam = 16, 32
        c.tau, c.sigma, c.gamma = 0.6, 0.01, 0.05
        c.droplet_x_stretch = 1.0
    elif name in ("jet_d3q27", "jet_d3q19", "jet_precision", "jet_closure", "jet_closure_fine"):
        vs = VS_D3Q27 if name == "jet_d3q27" else VS_D3Q19
        c = base(CASE_JET, vs)
        if name in ("jet_precision", "jet_closure_fine"):
            c.nx, c.ny, c.nz, c.diam = 256, 256, 1024, 32
        else:
            c.nx, c.ny, c.nz, c.diam = 128, 128, 512, 16
        c.radius = c.diam // 2
        re = 10000.0 if name.startswith("jet_closure") else 5000.0
        c.reynolds_water = c.reynolds_oil = re
        c.u_inf = 0.05
        # sigma = u^2 D / We with We = 500, computed in float as constants.cuh:98
        c.sigma = float(np.float32(np.float32(np.float32(c.u_inf) * np.float32(c.u_inf)) * np.float32(c.diam)) / np.float32(500.0))
        c.gamma = 0.05
        c.inflow_noise = NOISE_UNIFORM_UZ
        c.noise_amp = 0.05
        c.seed = 12345
    else:
        raise ValueError(f"unknown preset {name!r}")
    for k, v in overrides.items():
        if k == "center_offset":
            for i in range(3):
                c.center_offset[i] = v[i]
        else:
            setattr(c, k, v)
    return c


def ensemble_configs(n: int = 64, seed: int = 2026, velocity_set: int = VS_D3Q19) -> list:
    """The seeded droplet ensemble: edges uniform in {32,48,64,80,96}, radius
    uniform in 15-30% of the edge, centre offset uniform within +-10%, sigma
    log-uniform in [1e-3, 1e-2], tau uniform in [0.55, 0.9], initial velocity
    seeded uniform +-1e-3, spherical droplets, D3Q19 + D3Q7, FP32."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        c = config_reference(CASE_DROPLET, velocity_set)
        e = int(rng.choice([32, 48, 64, 80, 96]))
        c.nx = c.ny = c.nz = e
        c.radius = max(2, int(round(rng.uniform(0.15, 0.30) * e)))
        c.diam = 2 * c.radius
        off = rng.uniform(-0.1, 0.1, 3) * e
        for i in range(3):
            c.center_offset[i] = float(off[i])
        c.sigma = float(10 ** rng.uniform(-3, -2))
        c.tau = float(rng.uniform(0.55, 0.9))
        c.droplet_x_stretch = 1.0
        c.init_noise = 1e-3
        c.seed = int(seed * 1000 + k)
        out.append(c)
    return out


class Ensemble:
    """A batch of droplet boxes advanced together (pflbm_ensemble_*)."""

    def __init__(self, configs, init: bool = True):
        self.lib = load_library()
        arr = (Config * len(configs))()
        for i, c in enumerate(configs):
            ctypes.memmove(ctypes.byref(arr[i]), ctypes.byref(c), ctypes.sizeof(Config))
            arr[i].struct_size = ctypes.sizeof(Config)
        self.configs = [c.copy() for c in configs]
        h = ctypes.c_void_p()
        _check(self.lib, self.lib.pflbm_ensemble_create(arr, len(configs), ctypes.byref(h)))
        self._h = h
        if init:
            self.init()

    def init(self):
        _check(self.lib, self.lib.pflbm_ensemble_init(self._h))

    def step(self, n: int = 1):
        _check(self.lib, self.lib.pflbm_ensemble_step(self._h, int(n)))

    def step_profiled(self, n: int) -> float:
        ms = ctypes.c_double()
        _check(self.lib, self.lib.pflbm_ensemble_step_profiled(self._h, int(n), ctypes.byref(ms)))
        return float(ms.value)

    def get_field(self, box: int, name: str) -> np.ndarray:
        c = self.configs[box]
        a = np.empty((int(c.nz), int(c.ny), int(c.nx)), np.float32)
        _check(self.lib, self.lib.pflbm_ensemble_get_field(self._h, box, FIELD_ID[name], a.ctypes.data, a.nbytes))
        return a

    def reduce(self, box: int) -> Diag:
        d = Diag()
        rc = self.lib.pflbm_ensemble_reduce(self._h, box, ctypes.byref(d))
        if rc not in (0, 5):
            _check(self.lib, rc)
        return d

    def set_tuning(self, zchunk: int, ctas_per_sm: int):
        _check(self.lib, self.lib.pflbm_ensemble_set_tuning(self._h, zchunk, ctas_per_sm))

    def set_tile(self, tile_x: int, tile_y: int):
        _check(self.lib, self.lib.pflbm_ensemble_set_tile(self._h, tile_x, tile_y))

    @property
    def tuning(self) -> dict:
        v = [ctypes.c_int32() for _ in range(4)]
        _check(self.lib, self.lib.pflbm_ensemble_get_tuning(self._h, *(ctypes.byref(x) for x in v)))
        return {"tile": (v[0].value, v[1].value), "zchunk": v[2].value, "ctas_per_sm": v[3].value}

    def autotune(self, trial_steps: int = 10) -> dict:
        z, c, ms = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_double()
        _check(self.lib, self.lib.pflbm_ensemble_autotune(self._h, trial_steps, ctypes.byref(z), ctypes.byref(c),
                                                          ctypes.byref(ms)))
        t = self.tuning
        return {"tile": t["tile"], "zchunk": z.value, "ctas_per_sm": c.value, "trial_ms": ms.value}

    @property
    def info(self) -> dict:
        n, b, it = ctypes.c_uint64(), ctypes.c_int32(), ctypes.c_int32()
        _check(self.lib, self.lib.pflbm_ensemble_info(self._h, ctypes.byref(n), ctypes.byref(b), ctypes.byref(it)))
        return {"nodes": n.value, "boxes": b.value, "work_items": it.value}

    def close(self):
        if getattr(self, "_h", None):
            self.lib.pflbm_ensemble_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Simulation:
    """One simulation on one GPU (pflbm_create ... pflbm_destroy)."""

    def __init__(self, config: Config, init: bool = True):
        self.lib = load_library()
        self.config = config.copy()
        self.config.struct_size = ctypes.sizeof(Config)
        h = ctypes.c_void_p()
        _check(self.lib, self.lib.pflbm_create(ctypes.byref(self.config), ctypes.byref(h)))
        self._h = h
        self.shape = (int(config.nz), int(config.ny), int(config.nx))
        if init:
            self.init()

    # -- lifecycle -------------------------------------------------------
    def init(self):
        _check(self.lib, self.lib.pflbm_init(self._h))

    def close(self):
        if getattr(self, "_h", None):
            self.lib.pflbm_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- stepping --------------------------------------------------------
    def step(self, n: int = 1):
        _check(self.lib, self.lib.pflbm_step(self._h, int(n)))

    def step_async(self, n: int = 1):
        _check(self.lib, self.lib.pflbm_step_async(self._h, int(n)))

    def step_profiled(self, n: int) -> tuple[float, list[float]]:
        """Runs n steps with CUDA events around every kernel on the library's
        stream; returns (total ms, [collide ms, phase ms])."""
        tot = ctypes.c_double()
        ks = (ctypes.c_double * 2)()
        _check(self.lib, self.lib.pflbm_step_profiled(self._h, int(n), ctypes.byref(tot), ks, 2))
        return float(tot.value), [float(ks[0]), float(ks[1])]

    def synchronize(self):
        _check(self.lib, self.lib.pflbm_synchronize(self._h))

    @property
    def current_step(self) -> int:
        v = ctypes.c_uint64()
        _check(self.lib, self.lib.pflbm_current_step(self._h, ctypes.byref(v)))
        return int(v.value)

    # -- fields ----------------------------------------------------------
    def set_initial_field(self, name: str, values: np.ndarray):
        a = np.ascontiguousarray(values, dtype=np.float32).reshape(-1)
        _check(self.lib, self.lib.pflbm_set_initial_field(self._h, FIELD_ID[name], a.ctypes.data, a.nbytes))

    def get_field(self, name: str, out: np.ndarray | None = None, dtype=np.float32) -> np.ndarray:
        """Field as the reference's array holds it after the last step, shape (nz, ny, nx)."""
        fid = FIELD_ID[name] if isinstance(name, str) else int(name)
        if dtype == np.float64:
            a = out if out is not None else np.empty(self.shape, np.float64)
            _check(self.lib, self.lib.pflbm_get_field_f64(self._h, fid, a.ctypes.data, a.nbytes))
        else:
            a = out if out is not None else np.empty(self.shape, np.float32)
            _check(self.lib, self.lib.pflbm_get_field(self._h, fid, a.ctypes.data, a.nbytes))
        return a

    def reduce(self) -> Diag:
        d = Diag()
        rc = self.lib.pflbm_reduce(self._h, ctypes.byref(d))
        if rc not in (0, 5):
            _check(self.lib, rc)
        return d

    def write_output(self, directory: str, fields=("rho", "uz"), wait: bool = True):
        """<field><step06>.bin + step_<step06>.vti; wait=False returns once the
        fields are staged and writes the files in the background (finished
        by synchronize() or the next write_output)."""
        ids = (ctypes.c_int32 * len(fields))(*[FIELD_ID[f] for f in fields])
        fn = self.lib.pflbm_write_output if wait else self.lib.pflbm_write_output_async
        _check(self.lib, fn(self._h, str(directory).encode(), ids, len(fields)))

    def save_checkpoint(self, path):
        _check(self.lib, self.lib.pflbm_save_checkpoint(self._h, str(path).encode()))

    def load_checkpoint(self, path):
        _check(self.lib, self.lib.pflbm_load_checkpoint(self._h, str(path).encode()))

    @property
    def device_bytes(self) -> int:
        v = ctypes.c_uint64()
        _check(self.lib, self.lib.pflbm_device_bytes(self._h, ctypes.byref(v)))
        return int(v.value)

    @property
    def uses_tma(self) -> bool:
        v = ctypes.c_int32()
        _check(self.lib, self.lib.pflbm_uses_tma(self._h, ctypes.byref(v)))
        return bool(v.value)

    @property
    def collide_variant(self) -> str:
        """Collide kernel of the plain step: "plain", "tma" or "tma_pairs"."""
        v = ctypes.c_int32()
        _check(self.lib, self.lib.pflbm_collide_variant(self._h, ctypes.byref(v)))
        return ("plain", "tma", "tma_pairs")[v.value]

    @property
    def kernels_per_step(self) -> int:
        v = ctypes.c_int32()
        _check(self.lib, self.lib.pflbm_kernels_per_step(self._h, ctypes.byref(v)))
        return int(v.value)

    def set_watchdog(self, interval: int, max_phi_mass_drift: float = 0.0):
        """FP64 NaN/Inf (and phi-mass drift) checks every `interval` steps of step()."""
        _check(self.lib, self.lib.pflbm_set_watchdog(self._h, int(interval), float(max_phi_mass_drift)))

    def set_closure(self, blob, strength: float = 1.0):
        """Attaches a closure network (PFLBM_MLP_BLOB floats; None detaches)."""
        if blob is None:
            _check(self.lib, self.lib.pflbm_set_closure(self._h, None, 0.0))
            return
        b = np.ascontiguousarray(blob, np.float32)
        if b.size != MLP_BLOB:
            raise ValueError(f"closure blob must hold {MLP_BLOB} floats")
        _check(self.lib, self.lib.pflbm_set_closure(self._h, b.ctypes.data, float(strength)))

    def set_closure_mixing(self, inv_schmidt: float):
        """Phase mixing of the attached closure: eddy diffusivity of phi
        D_t = inv_schmidt * strength * nu_t (0 switches it off)."""
        _check(self.lib, self.lib.pflbm_set_closure_mixing(self._h, float(inv_schmidt)))


MLP_PARAMS, MLP_BLOB = 1377, 1395


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round float32 values to BF16 precision (nearest even), as float32."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    finite = (u & 0x7F800000) != 0x7F800000
    r = np.where(finite, (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000, u & 0xFFFF0000)
    return r.astype(np.uint32).view(np.float32)


class Closure:
    """Learned eddy-viscosity closure: training data, forward/backward/Adam
    on the GPU (pflbm_closure_* in include/pflbm.h)."""

    def __init__(self, max_samples: int, device: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        _check(self.lib, self.lib.pflbm_closure_create(int(device), int(max_samples), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self.lib.pflbm_closure_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_snapshot(self, fine: "Simulation", stride: int = 2) -> int:
        n = ctypes.c_uint64()
        _check(self.lib, self.lib.pflbm_closure_add_snapshot(self._h, fine._h, int(stride), ctypes.byref(n)))
        return int(n.value)

    @property
    def num_samples(self) -> int:
        n = ctypes.c_uint64()
        _check(self.lib, self.lib.pflbm_closure_num_samples(self._h, ctypes.byref(n)))
        return int(n.value)

    def interface_scale(self) -> dict:
        """Interface widths of the snapshots (fine field in fine units,
        filtered field in coarse units) and gamma_scale = their ratio, the
        factor on a coarse run's interface sharpening gamma that gives it
        the filtered fine interface width."""
        g, wf, wc = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _check(self.lib, self.lib.pflbm_closure_interface_scale(self._h, ctypes.byref(g), ctypes.byref(wf),
                                                                 ctypes.byref(wc)))
        return {"gamma_scale": g.value, "width_fine": wf.value, "width_filtered": wc.value}

    def samples(self, first: int = 0, count: int | None = None):
        count = self.num_samples - first if count is None else count
        x = np.empty((count, 8), np.float32)
        y = np.empty(count, np.float32)
        _check(self.lib, self.lib.pflbm_closure_get_samples(self._h, first, count, x.ctypes.data, y.ctypes.data))
        return x, y

    def set_samples(self, x: np.ndarray, y: np.ndarray):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        _check(self.lib, self.lib.pflbm_closure_set_samples(self._h, x.ctypes.data, y.ctypes.data, len(y)))

    def init_params(self, seed: int = 1):
        _check(self.lib, self.lib.pflbm_closure_init_params(self._h, int(seed)))

    @property
    def blob(self) -> np.ndarray:
        b = np.empty(MLP_BLOB, np.float32)
        _check(self.lib, self.lib.pflbm_closure_get_blob(self._h, b.ctypes.data))
        return b

    @blob.setter
    def blob(self, b):
        b = np.ascontiguousarray(b, np.float32)
        _check(self.lib, self.lib.pflbm_closure_set_blob(self._h, b.ctypes.data))

    def gradient(self, count: int):
        g = np.empty(MLP_PARAMS, np.float64)
        loss = ctypes.c_double()
        _check(self.lib, self.lib.pflbm_closure_gradient(self._h, int(count), g.ctypes.data, ctypes.byref(loss)))
        return g, float(loss.value)

    def train(self, iterations: int, batch: int = 8192, lr: float = 1e-3, seed: int = 7) -> np.ndarray:
        hist = np.empty(iterations, np.float64)
        _check(self.lib, self.lib.pflbm_closure_train(self._h, int(iterations), int(batch), float(lr), int(seed),
                                                      hist.ctypes.data))
        return hist

    def loss(self) -> float:
        v = ctypes.c_double()
        _check(self.lib, self.lib.pflbm_closure_loss(self._h, ctypes.byref(v)))
        return float(v.value)
