"""Benchmark of the phase-field LBM hot path on GB300.

One bench "step" = `--inner` lattice time steps (each one full pass of the
hot path over the domain: k_collide + k_phase). The workload is the turbulent
jet, D3Q27 + D3Q7, FP32, 128x128x512 (D=16, Re=5000, We=500, seeded uniform
+-5% inflow noise): synthetic, seeded. MLUPS counts every node of the grid,
ghost shell included, as the reference does (src/main.cu:201-205).

Timing: W warm-up bench steps, then K timed ones between a barrier and a
device sync; the time is taken with CUDA events recorded on the library's
own stream (pflbm_step_profiled), max over ranks. The populations (2 x 906 MB)
are far larger than the 129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the CPU transcription of the reference's kernels
(oracle/, OpenMP, all host cores) on the same workload: the reference itself
has no CPU path, and its CUDA build is a GPU baseline, reported separately.
Multi-GPU runs are independent replicas (one simulation per GPU, no
exchange); scaling is weak.

  python bench.py --study precision [--checkpoints 500,1000,...]

prints the storage-precision study (FP32/FP16/BF16 storage against the FP64
path on the 128x128x512 D3Q19 jet, MLUPS on 256x256x1024) instead.

  python bench.py --study closure

trains the learned closure on filtered 256x256x1024 snapshots and judges it
against plain constant-tau on the 128x128x512 grid (time-averaged u_z, phi).

  python bench.py --study ensemble

times the 64-box droplet ensemble (batched, autotuned) against the same boxes
run sequentially.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# algorithmic bytes per lattice update (canonical accounting):
# 2*Q*s_f (f read+write) + 2*7*s_g (g read+write) + 2*4 (phi write+read).
# The collide kernel owns f read+write, the g write and the phi read;
# the phase kernel owns the g read and the phi write.
def b_alg(q: int, s_f: int, s_g: int) -> dict:
    total = 2 * q * s_f + 2 * 7 * s_g + 8
    collide = 2 * q * s_f + 7 * s_g + 4
    return {"total": total, "collide": collide, "phase": total - collide}


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


# ---------------------------------------------------------------- ranks
class Ranks:
    def __init__(self):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            # bench plumbing only (barrier, max/sum of timings): the replicas
            # exchange no data, so the process group is gloo on the host
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def reduce(self, v: float, op: str) -> float:
        if not self.pg:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX if op == "max" else self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# --------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self._t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------ CPU legs
def cpu_oracle_mlups(cfg, steps: int, warm: int = 1) -> tuple[float, float, int]:
    from oracle import pyoracle

    o = pyoracle.OracleSim(cfg)
    o.step(warm)
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    o.close()
    return cfg.nodes * steps / dt / 1e6, dt, os.cpu_count() or 1


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of one k_collide
# launch, from ncu. jet_d3q27 (the bench workload): measured on the
# 128x128x512 workload itself, mean of two launches
# (profiles/k_collide_tma_jet_d3q27_fp32_traffic_128x128x512.md). jet_d3q19:
# measured on the 128x128x128 profiling case and scaled to 128x128x512 by the
# interior planes swept (510 / 126;
# profiles/k_collide_tma_jet_d3q19_fp32_128x128x128.md).
NCU_COLLIDE_TRAFFIC = {
    "jet_d3q27": ((1026.005248e6 + 938.875136e6) + (1026.161664e6 + 935.919616e6)) / 2,
    "jet_d3q19": (179.217664e6 + 127.435776e6) * 510 / 126,
}
NCU_TRAFFIC_SOURCE = {
    "jet_d3q27": "ncu on this 128x128x512 workload (mean of 2 launches)",
    "jet_d3q19": "ncu on 128x128x128, scaled by interior planes 510/126",
}


def traffic_for(workload: str):
    v = NCU_COLLIDE_TRAFFIC.get(workload)
    return {"collide_bytes_per_launch": int(v), "source": NCU_TRAFFIC_SOURCE[workload]} if v else None


# ---------------------------------------------------------------- arms
def workload_config(args, base=None):
    """The bench workload; --nz shortens the jet for profiling captures.
    `base` supplies the reference configuration the preset starts from (the
    reference arm passes the oracle's own, so that it loads no library)."""
    import phasefieldlbm_gb300 as pf

    st = {"fp32": pf.STORAGE_FP32, "fp16": pf.STORAGE_FP16, "bf16": pf.STORAGE_BF16, "fp64": pf.STORAGE_FP64}
    kw = {"storage": st[args.storage]}
    if args.nz:
        kw["nz"] = args.nz
    return pf.preset(args.workload, base=base, **kw)


def reference_build_mlups(workload: str, steps: int, nz: int = 0):
    """GPU baseline: the reference's own CUDA build (its src/main.cu compiled
    for sm_103a with the benchmark preset's physics patched in, run by
    oracle/ref_runner with src/main.cu's launch sequence and per-step sync),
    timed on the host wall clock around the step loop as src/main.cu:199-205
    does. None when the cubins were not built (they come from the reference
    sources, present only where the repository was prepared)."""
    from oracle import ref_build

    name = {"jet_d3q27": "jet_d3q27_bench", "jet_d3q19": "jet_d3q19_bench"}.get(workload)
    entry = ref_build.manifest().get(name) if name else None
    if not entry or nz or not (ref_build.OUT / entry["cubin"]).exists():
        return None
    try:
        exe = ref_build.build_runner()
        nx, ny, nzz = entry["dims"]
        r = subprocess.run([str(exe), str(ref_build.OUT / entry["cubin"]), entry["case"], str(entry["q"]), str(nx),
                            str(ny), str(nzz), str(entry["fp16"]), str(steps), "-", "time"],
                           capture_output=True, text=True, timeout=300)
        if r.returncode != 0:
            return {"value": None, "error": (r.stderr or r.stdout)[-200:]}
        line = json.loads(r.stdout.strip().splitlines()[-1])
    except Exception as ex:  # a baseline leg: report why it is missing
        return {"value": None, "error": str(ex)[:200]}
    return {"value": round(line["ref_mlups"], 2), "unit": "MLUPS", "kind": "reference_cuda_build",
            "steps": steps, "seconds": round(line["seconds"], 4),
            "sample": f"the reference's own kernels (src/main.cu built for sm_103a, FP32 f, preset physics patched "
                      f"in: gamma 0.05, uniform u_z noise seed 12345) on {nx}x{ny}x{nzz}, {steps} steps of its "
                      "5-kernel graph + inflow + outflow + stream sync, host wall clock (src/main.cu:199-205)"}


def run_gpu(args, ranks: Ranks) -> dict:
    import phasefieldlbm_gb300 as pf

    cfg = workload_config(args)
    cfg.device = ranks.local
    N = cfg.nodes
    q = int(cfg.velocity_set)
    s_f = {pf.STORAGE_FP32: 4, pf.STORAGE_FP64: 8, pf.STORAGE_FP16: 2, pf.STORAGE_BF16: 2}[int(cfg.storage)]
    # canonical bytes per lattice update: g counted at the storage width of f
    # for 16-bit runs (FP16/BF16 f and g, 112 B/LU for D3Q19), FP32 otherwise
    ba = b_alg(q, s_f, s_f if s_f in (2, 8) else 4)
    sim = pf.Simulation(cfg)
    inner = args.inner
    # warm-up
    sim.step(args.warmup * inner)
    sim.synchronize()
    ranks.barrier()
    sim.synchronize()
    clocks = ClockSampler(cfg.device)
    clocks.start()
    total_ms, kms = sim.step_profiled(args.steps * inner)
    sim.synchronize()
    ranks.barrier()
    clk = clocks.stop()
    t_local = total_ms / 1e3
    t = ranks.reduce(t_local, "max")
    lattice_steps = args.steps * inner
    units = ranks.reduce(float(N) * lattice_steps, "sum")
    value = units / t / 1e6
    d = sim.reduce()
    diverged = int(d.nonfinite) > 0

    # roofline of the dominant kernel (k_collide), CUDA-event durations
    pk = peaks()
    launches = lattice_steps
    collide_s = kms[0] / 1e3 / launches
    phase_s = kms[1] / 1e3 / launches
    achieved = ba["collide"] * N / collide_s / 1e9
    step_achieved = ba["total"] * N / ((kms[0] + kms[1]) / 1e3 / launches) / 1e9
    tr = None if (args.nz or args.storage != "fp32") else traffic_for(args.workload)
    roofline = {
        "bound": "hbm", "kernel": "k_collide", "achieved": round(achieved, 1), "peak": pk["hbm_gbs"],
        "unit": "GB/s", "frac": round(achieved / pk["hbm_gbs"], 4),
        "traffic": tr.get("collide_bytes_per_launch") if tr else None,
        "traffic_source": tr.get("source") if tr else None,
        "algorithmic_bytes_per_launch": ba["collide"] * N,
        "avg_launch_ms": round(collide_s * 1e3, 4),
        "peak_source": pk["source"],
        "step": {"kernels": ["k_collide", "k_phase"], "achieved": round(step_achieved, 1),
                 "frac": round(step_achieved / pk["hbm_gbs"], 4), "bytes_per_lu": ba["total"],
                 "phase_avg_launch_ms": round(phase_s * 1e3, 4)},
    }

    # end to end through the C ABI with pinned host buffers: per bench step,
    # upload the initial state (rho, ux, uy, uz, phi), run `inner` steps,
    # read back rho, uz and phi
    e2e = None
    try:
        import torch

        def pinned():
            return torch.empty(N, dtype=torch.float32, pin_memory=True).numpy()

        host_in = {f: pinned() for f in ("rho", "ux", "uy", "uz", "phi")}
        host_out = {f: pinned() for f in ("rho", "uz", "phi")}
        sim.init()
        for f in host_in:
            host_in[f][:] = sim.get_field(f).reshape(-1)
        ranks.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            sim.init()
            for f, a in host_in.items():
                sim.set_initial_field(f, a)
            sim.step(inner)
            for f, a in host_out.items():
                sim.get_field(f, out=a.reshape(sim.shape))
        te = time.perf_counter() - t0
        te = ranks.reduce(te, "max")
        e2e = {"value": round(units / te / 1e6, 2), "unit": "MLUPS",
               "h2d_bytes_per_step": 4 * N * len(host_in), "d2h_bytes_per_step": 4 * N * len(host_out),
               "per_step": f"{inner} lattice steps + upload of the initial rho,u,phi + readback of rho,uz,phi"}
    except Exception as ex:  # the CUDA path must not fall back; report why e2e is missing
        e2e = {"value": None, "unit": "MLUPS", "error": str(ex)[:200]}
    tma = sim.uses_tma
    sim.close()

    # other lattices / storage precisions on the same jet (informational)
    # other lattices / storage precisions on the same jet, each with its error
    # against the FP64 path after the same number of steps (rel. L2 of rho,
    # the centreline u_z and phi)
    variants = {}
    if not args.no_variants:
        vsteps = 3 * inner // 2 + 2 * inner
        fp64_ref = {}

        def errors(wl, s2):
            if wl not in fp64_ref:
                with pf.Simulation(pf.preset(wl, storage=pf.STORAGE_FP64, device=cfg.device)) as s64:
                    s64.step(vsteps)
                    fp64_ref[wl] = {f: s64.get_field(f, dtype=np.float64) for f in ("rho", "uz", "phi")}
            ref = fp64_ref[wl]
            cy, cx = ref["uz"].shape[1] // 2, ref["uz"].shape[2] // 2
            got = {f: s2.get_field(f, dtype=np.float64) for f in ("rho", "uz", "phi")}
            rl2 = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
            return {"rho": rl2(got["rho"], ref["rho"]), "uz_centreline": rl2(got["uz"][:, cy, cx], ref["uz"][:, cy, cx]),
                    "phi": rl2(got["phi"], ref["phi"])}

        for name, wl, st in (("jet_d3q19_fp32", "jet_d3q19", pf.STORAGE_FP32),
                             ("jet_d3q19_fp16", "jet_d3q19", pf.STORAGE_FP16),
                             ("jet_d3q19_bf16", "jet_d3q19", pf.STORAGE_BF16),
                             ("jet_d3q27_fp16", "jet_d3q27", pf.STORAGE_FP16)):
            c2 = pf.preset(wl, storage=st, device=cfg.device)
            with pf.Simulation(c2) as s2:
                s2.step(3 * inner // 2)
                s2.synchronize()
                tot2, k2 = s2.step_profiled(2 * inner)
                variants[name] = {"mlups": round(c2.nodes * 2 * inner / (tot2 / 1e3) / 1e6, 1),
                                  "collide_ms": round(k2[0] / (2 * inner), 4), "phase_ms": round(k2[1] / (2 * inner), 4),
                                  "steps": vsteps, "rel_l2_vs_fp64": errors(wl, s2)}

        # the batched droplet ensemble (64 seeded boxes, 2000 steps, autotuned,
        # one cooperative launch per step) against the same boxes run one
        # after another as single simulations
        variants["ensemble64_d3q19_fp32"] = run_ensemble_study(args, device=cfg.device)

    cpu = None
    if ranks.rank == 0 and ranks.world == 1 and not args.no_cpu_baseline:
        # a bounded sample of about 10 s of host work: as many full-grid steps
        # as one timed step suggests, at least 2
        m1, d1, _ = cpu_oracle_mlups(cfg, 1)
        csteps = max(2, min(40, int(10.0 / max(d1, 1e-3))))
        mlups, dt, cores = cpu_oracle_mlups(cfg, csteps)
        cpu = {"value": round(mlups, 3), "unit": "MLUPS", "cores": cores, "kind": "port",
               "sample": f"{csteps} time steps of the full {cfg.nx}x{cfg.ny}x{cfg.nz} D3Q{q} jet (FP32) after 1 warm-up "
                         f"step, OpenMP transcription of the reference kernels, {dt:.1f} s"}

    # the reference's own CUDA build on the same GPU and workload (rank 0, N = 1)
    gpu_base = None
    if ranks.rank == 0 and ranks.world == 1 and not args.no_cpu_baseline:
        gpu_base = reference_build_mlups(args.workload, 1000, args.nz)

    return {
        "metric": "MLUPS", "value": round(value, 2), "unit": "MLUPS", "n_gpus": ranks.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": {"fp32": "f32", "fp16": "f16-storage/f32-math", "bf16": "bf16-storage/f32-math", "fp64": "f64"}[args.storage],
        "data": "synthetic",
        "config": {"workload": f"jet D3Q{q}+D3Q7 {args.storage.upper()} {cfg.nx}x{cfg.ny}x{cfg.nz}, D={cfg.diam}, Re=5000, We=500, "
                               "gamma=0.05, uniform 5% inflow noise (seed 12345)",
                   "preset": args.workload, "nodes": N, "lattice_steps_per_step": inner,
                   "l2": "inputs larger than L2 (f ping-pong 2x{:.0f} MB)".format(q * s_f * N / 1e6),
                   "parallelism": f"replicas x{ranks.world}"},
        "roofline": roofline, "cpu_baseline": cpu, "gpu_baseline": gpu_base, "e2e": e2e,
        "gpu_launches": 2 * lattice_steps, "clocks": clk, "diverged": diverged, "tma": tma,
        "variants": variants,
    }


def run_reference(args, ranks: Ranks) -> dict | None:
    if ranks.rank != 0:
        return None
    from oracle import pyoracle

    # the oracle's own restatement of src/constants.cuh: this arm loads the
    # oracle library only, never libpflbm
    cfg = workload_config(args, base=pyoracle.config_reference)
    o = pyoracle.OracleSim(cfg)
    o.step(args.warmup)
    t0 = time.perf_counter()
    o.step(args.steps)
    dt = time.perf_counter() - t0
    v = cfg.nodes * args.steps / dt / 1e6
    cores = os.cpu_count() or 1
    return {
        "impl": "reference", "metric": "MLUPS", "value": round(v, 3), "unit": "MLUPS", "n_gpus": ranks.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"jet D3Q{cfg.velocity_set}+D3Q7 FP32 {cfg.nx}x{cfg.ny}x{cfg.nz}", "preset": args.workload,
                   "nodes": cfg.nodes, "lattice_steps_per_step": 1},
        "cpu_baseline": {"value": round(v, 3), "unit": "MLUPS", "cores": cores, "kind": "port",
                         "sample": f"1 time step of the full grid per bench step, {args.steps} steps after {args.warmup} "
                                   "warm-up; OpenMP transcription of the reference's kernels (the reference has no CPU path)"},
        "e2e": {"value": round(v, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_precision_study(args) -> dict:
    """Storage-precision study of the D3Q19 jet: FP32, FP16 and BF16 storage
    against the FP64 path on the 128x128x512 (D=16) instance, all four runs
    advanced in lockstep on the GPU and compared at checkpoints (relative L2
    of rho, of u_z on the centreline x = nx/2, y = ny/2, and of phi), plus
    the MLUPS of each storage on the 256x256x1024 (D=32) configuration."""
    import numpy as np

    import phasefieldlbm_gb300 as pf

    def rl2(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    names = {"fp64": pf.STORAGE_FP64, "fp32": pf.STORAGE_FP32, "fp16": pf.STORAGE_FP16, "bf16": pf.STORAGE_BF16}
    checkpoints = [int(c) for c in args.checkpoints.split(",")]
    sims = {k: pf.Simulation(pf.preset("jet_d3q19", storage=v)) for k, v in names.items()}
    errors, done = [], 0
    for cp in checkpoints:
        for s in sims.values():
            s.step(cp - done)
        done = cp
        c = sims["fp64"].config
        cx, cy = int(c.nx) // 2, int(c.ny) // 2
        ref = {f: sims["fp64"].get_field(f, dtype=np.float64) for f in ("rho", "uz", "phi")}
        row = {"step": cp}
        for k in ("fp32", "fp16", "bf16"):
            got = {f: sims[k].get_field(f, dtype=np.float64) for f in ("rho", "uz", "phi")}
            row[k] = {"rho": rl2(got["rho"], ref["rho"]),
                      "uz_centreline": rl2(got["uz"][:, cy, cx], ref["uz"][:, cy, cx]),
                      "uz": rl2(got["uz"], ref["uz"]), "phi": rl2(got["phi"], ref["phi"]),
                      "phi_mass_drift": float(sims[k].reduce().phi_mass / sims["fp64"].reduce().phi_mass - 1.0)}
        errors.append(row)
        print(json.dumps(row), file=sys.stderr, flush=True)
    for s in sims.values():
        s.close()
    mlups = {}
    for k in ("fp32", "fp16", "bf16"):
        c = pf.preset("jet_precision", storage=names[k])
        with pf.Simulation(c) as s:
            s.step(50)
            tot, _ = s.step_profiled(200)
            mlups[k] = round(c.nodes * 200 / (tot / 1e3) / 1e6, 1)
    return {"study": "precision", "case": "jet D3Q19+D3Q7, Re=5000, We=500, uniform 5% inflow noise (seed 12345)",
            "error_grid": "128x128x512, D=16, against the FP64 path", "mlups_grid": "256x256x1024, D=32",
            "errors": errors, "mlups": mlups}


def restrict_filtered(a):
    """3x3x3 box filter around fine node 2X, sampled at coarse node X."""
    nz, ny, nx = a.shape
    acc = np.zeros((nz // 2, ny // 2, nx // 2))
    for dz in (-1, 0, 1):
        zi = np.clip(np.arange(nz // 2) * 2 + dz, 0, nz - 1)
        for dy in (-1, 0, 1):
            yi = np.clip(np.arange(ny // 2) * 2 + dy, 0, ny - 1)
            for dx in (-1, 0, 1):
                xi = np.clip(np.arange(nx // 2) * 2 + dx, 0, nx - 1)
                acc += a[np.ix_(zi, yi, xi)]
    return acc / 27.0


def run_closure_study(args) -> dict:
    """Learned closure on the D3Q19 jet at Re = 10000: a 256x256x1024 (D=32)
    run gives 20 snapshots (every 500 steps) that are box-filtered and
    restricted to the 128x128x512 (D=16) grid; the MLP is trained on them on
    the GPU; plain constant-tau and closure runs on the coarse grid are then
    judged by the relative L2 error of their time-averaged u_z and phi
    against the filtered time average of the fine run over the same
    physical time (coarse steps = fine steps / 2)."""
    import phasefieldlbm_gb300 as pf

    t0 = time.perf_counter()
    n_snap, every = args.snapshots, args.snapshot_every
    fine_steps = n_snap * every
    coarse_steps = fine_steps // 2
    fx, fy, fz, fd = (int(v) for v in args.fine_grid.split(","))
    fine_cfg = pf.preset("jet_closure_fine", flags=pf.FLAG_TIME_AVERAGE, nx=fx, ny=fy, nz=fz, diam=fd, radius=fd // 2)
    fd2 = fd // 2
    coarse_cfg = pf.preset("jet_closure", flags=pf.FLAG_TIME_AVERAGE, nx=fx // 2, ny=fy // 2, nz=fz // 2, diam=fd2,
                           radius=fd2 // 2)
    # sigma = u^2 D / We (We = 500) on each grid, as the presets compute it
    for c in (fine_cfg, coarse_cfg):
        c.sigma = float(np.float32(np.float32(np.float32(c.u_inf) * np.float32(c.u_inf)) * np.float32(c.diam)) /
                        np.float32(500.0))
    stride = args.sample_stride
    per_snap = ((fine_cfg.nx // 2 - 3) // stride + 1) * ((fine_cfg.ny // 2 - 3) // stride + 1) * (fine_cfg.nz // 2 - 4)
    out = {"study": "closure", "fine": f"{fx}x{fy}x{fz} D={fd} Re=10000",
           "coarse": f"{fx // 2}x{fy // 2}x{fz // 2} D={fd2} Re=10000",
           "fine_steps": fine_steps, "coarse_steps": coarse_steps, "snapshots": n_snap, "sample_stride": stride}
    with pf.Closure(per_snap * n_snap) as cl:
        with pf.Simulation(fine_cfg) as fine:
            for k in range(n_snap):
                fine.step(every)
                cl.add_snapshot(fine, stride=stride)
            ref = {f: restrict_filtered(fine.get_field(f)) for f in ("avg_uz", "avg_phi")}
        out["samples"] = cl.num_samples
        out["interface"] = {k: round(v, 4) for k, v in cl.interface_scale().items()}
        out["t_fine_s"] = round(time.perf_counter() - t0, 1)
        cl.init_params(seed=args.seed)
        loss0 = cl.loss()
        t1 = time.perf_counter()
        hist = cl.train(args.train_iters, batch=args.train_batch, lr=args.train_lr, seed=args.seed)
        out["train"] = {"iterations": args.train_iters, "batch": args.train_batch, "lr": args.train_lr,
                        "loss_init": loss0, "loss_final": cl.loss(), "minibatch_last": float(hist[-1]),
                        "seconds": round(time.perf_counter() - t1, 2)}
        blob = cl.blob

    def coarse_run(strength, mixing=0.0, gamma_scale=1.0):
        c = coarse_cfg.copy()
        c.gamma = float(np.float32(c.gamma * gamma_scale))
        with pf.Simulation(c) as s:
            if strength > 0:
                s.set_closure(blob, strength)
                s.set_closure_mixing(mixing)
            ta = time.perf_counter()
            s.step(coarse_steps)
            dt = time.perf_counter() - ta
            return {f: s.get_field(f).astype(np.float64) for f in ("avg_uz", "avg_phi")}, c.nodes * coarse_steps / dt / 1e6

    def errors(res):
        sl = (slice(2, -2), slice(2, -2), slice(2, -2))
        cz, cy, cx = [n // 2 for n in res["avg_uz"].shape]
        e = {}
        for f in ("avg_uz", "avg_phi"):
            a, b = res[f][sl], ref[f][sl]
            e[f] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
            e[f + "_centreline"] = float(np.linalg.norm(res[f][2:-2, cy, cx] - ref[f][2:-2, cy, cx]) /
                                         np.linalg.norm(ref[f][2:-2, cy, cx]))
        return e

    # the closure: the learned eddy viscosity and the interface sharpening
    # scaled to the filtered fine interface width; each part alone as well
    gs = out["interface"]["gamma_scale"]
    runs = {}
    cases = [("plain", 0.0, 0.0, 1.0), ("closure", 1.0, 0.0, gs), ("closure_nu_only", 1.0, 0.0, 1.0),
             ("plain_sharpened", 0.0, 0.0, gs)]
    cases += [(f"closure_x{v:g}", v, 0.0, gs) for v in args.extra_strengths]
    cases += [(f"closure_nu_only_mix{m:g}", 1.0, m, 1.0) for m in args.mixing]
    for g in args.gamma_scales:
        cases += [(f"plain_gamma{g:g}", 0.0, 0.0, g), (f"closure_gamma{g:g}", 1.0, 0.0, g)]
    for name, strength, mixing, gs in cases:
        res, mlups = coarse_run(strength, mixing, gs)
        runs[name] = {"strength": strength, "mixing": mixing, "gamma_scale": gs, "mlups": round(mlups, 1),
                      **errors(res)}
    out["runs"] = runs
    out["seconds"] = round(time.perf_counter() - t0, 1)
    return out


def run_ensemble_study(args, device: int = 0) -> dict:
    """The batched droplet ensemble: 64 seeded periodic boxes (edges in
    {32,48,64,80,96}), autotuned (tile shape, z chunk, resident CTAs), `steps`
    steps of one persistent cooperative launch each, graph-captured, against
    the same boxes run one after another as single simulations (each with
    its own captured graph)."""
    import phasefieldlbm_gb300 as pf

    steps = args.ensemble_steps
    cfgs = pf.ensemble_configs(64)
    for c in cfgs:
        c.device = device
    total_nodes = sum(c.nodes for c in cfgs)
    with pf.Ensemble(cfgs) as ens:
        if getattr(args, "ensemble_tuning", ""):
            # a fixed tuning "TXxTY,zchunk,ctas" instead of the autotuner
            t, zc, ctas = args.ensemble_tuning.split(",")
            ens.set_tile(*(int(v) for v in t.split("x")))
            ens.set_tuning(int(zc), int(ctas))
            tune = {**ens.tuning, "trial_ms": None}
        else:
            tune = ens.autotune(10)
        ens.step(10)
        ms = ens.step_profiled(steps)
        diverged = [b for b in range(len(cfgs)) if int(ens.reduce(b).nonfinite) > 0]
    seq_ms = None
    if not getattr(args, "ensemble_no_sequential", False):
        seq_ms = 0.0
        for c in cfgs:
            with pf.Simulation(c) as s:
                s.step(10)
                tot, _ = s.step_profiled(steps)
                seq_ms += tot
    tune["tile"] = list(tune["tile"])
    return {"study": "ensemble", "boxes": len(cfgs), "nodes": total_nodes, "steps": steps, "autotune": tune,
            "batched_mlups": round(total_nodes * steps / (ms / 1e3) / 1e6, 1),
            "sequential_mlups": round(total_nodes * steps / (seq_ms / 1e3) / 1e6, 1) if seq_ms else None,
            "speedup": round(seq_ms / ms, 3) if seq_ms else None, "diverged_boxes": diverged,
            "launches_per_step": 1}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--inner", type=int, default=100, help="lattice steps per bench step")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="jet_d3q27")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--nz", type=int, default=0, help="override the workload's z extent (profiling captures)")
    ap.add_argument("--storage", choices=["fp32", "fp16", "bf16", "fp64"], default="fp32",
                    help="population storage of the workload")
    ap.add_argument("--study", choices=["precision", "closure", "ensemble"], help="run a study instead of the bench line")
    ap.add_argument("--ensemble-steps", type=int, default=2000)
    ap.add_argument("--ensemble-tuning", default="", help="ensemble study: fixed tuning TXxTY,zchunk,ctas (no autotune)")
    ap.add_argument("--ensemble-no-sequential", action="store_true",
                    help="ensemble study: skip the sequential single-box comparison (profiling captures)")
    ap.add_argument("--fine-grid", default="256,256,1024,32", help="closure study: fine nx,ny,nz,D")
    ap.add_argument("--snapshots", type=int, default=20)
    ap.add_argument("--snapshot-every", type=int, default=500)
    ap.add_argument("--sample-stride", type=int, default=2)
    ap.add_argument("--train-iters", type=int, default=3000)
    ap.add_argument("--train-batch", type=int, default=16384)
    ap.add_argument("--train-lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=2026)
    ap.add_argument("--extra-strengths", type=float, nargs="*", default=[0.5, 2.0])
    ap.add_argument("--mixing", type=float, nargs="*", default=[1.0],
                    help="closure study: inverse turbulent Schmidt numbers of the phase mixing")
    ap.add_argument("--gamma-scales", type=float, nargs="*", default=[],
                    help="closure study: coarse-grid multipliers of the interface sharpening gamma")
    ap.add_argument("--checkpoints", default="500,1000,2000,5000,10000")
    args = ap.parse_args()
    if args.study:
        run = {"precision": run_precision_study, "closure": run_closure_study, "ensemble": run_ensemble_study}[args.study]
        print(json.dumps(run(args)), flush=True)
        return
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    ranks = Ranks()
    try:
        out = run_reference(args, ranks) if args.impl == "reference" else run_gpu(args, ranks)
        if out is not None and ranks.rank == 0:
            print(json.dumps(out), flush=True)
    finally:
        ranks.close()


if __name__ == "__main__":
    main()
