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


def traffic_for(workload: str):
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    try:
        return json.loads(p.read_text()).get(workload)
    except (ValueError, OSError):
        return None


# ---------------------------------------------------------------- arms
def run_gpu(args, ranks: Ranks) -> dict:
    import phasefieldlbm_gb300 as pf

    cfg = pf.preset(args.workload)
    cfg.device = ranks.local
    N = cfg.nodes
    q = int(cfg.velocity_set)
    s_f = {pf.STORAGE_FP32: 4, pf.STORAGE_FP64: 8, pf.STORAGE_FP16: 2, pf.STORAGE_BF16: 2}[int(cfg.storage)]
    ba = b_alg(q, s_f, 4 if s_f != 8 else 8)
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
    tr = traffic_for(args.workload)
    roofline = {
        "bound": "hbm", "kernel": "k_collide", "achieved": round(achieved, 1), "peak": pk["hbm_gbs"],
        "unit": "GB/s", "frac": round(achieved / pk["hbm_gbs"], 4),
        "traffic": tr.get("collide_bytes_per_launch") if tr else None,
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
    variants = {}
    if not args.no_variants:
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
                                  "collide_ms": round(k2[0] / (2 * inner), 4), "phase_ms": round(k2[1] / (2 * inner), 4)}

    cpu = None
    if ranks.rank == 0 and ranks.world == 1 and not args.no_cpu_baseline:
        csteps = 2
        mlups, dt, cores = cpu_oracle_mlups(cfg, csteps)
        cpu = {"value": round(mlups, 3), "unit": "MLUPS", "cores": cores, "kind": "port",
               "sample": f"{csteps} time steps of the full {cfg.nx}x{cfg.ny}x{cfg.nz} D3Q{q} jet (FP32) after 1 warm-up "
                         f"step, OpenMP transcription of the reference kernels, {dt:.1f} s"}

    return {
        "metric": "MLUPS", "value": round(value, 2), "unit": "MLUPS", "n_gpus": ranks.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32" if s_f == 4 else str(s_f),
        "data": "synthetic",
        "config": {"workload": f"jet D3Q{q}+D3Q7 FP32 {cfg.nx}x{cfg.ny}x{cfg.nz}, D={cfg.diam}, Re=5000, We=500, "
                               "gamma=0.05, uniform 5% inflow noise (seed 12345)",
                   "preset": args.workload, "nodes": N, "lattice_steps_per_step": inner,
                   "l2": "inputs larger than L2 (f ping-pong 2x{:.0f} MB)".format(q * s_f * N / 1e6),
                   "parallelism": f"replicas x{ranks.world}"},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": 2 * lattice_steps, "clocks": clk, "diverged": diverged, "tma": tma,
        "variants": variants,
    }


def run_reference(args, ranks: Ranks) -> dict | None:
    if ranks.rank != 0:
        return None
    import phasefieldlbm_gb300 as pf
    from oracle import pyoracle

    cfg = pf.preset(args.workload)
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
    args = ap.parse_args()
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
