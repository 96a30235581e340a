#!/usr/bin/env python3
"""Throughput of the GB300 kinetic step: particle-steps/s on one GB300.

Workload (configs[1] shape, "Plain GPU scale-up"): a population of electrons
drawn from that case's seed distribution (K log-uniform 1-20 MeV, isotropic
in the -E hemisphere, uniform in a 5 m x 10 m disk), air at 1.225 kg/m^3,
uniform E_z = -500 kV/m, 256 x 2048 grid over 200 m x 2 km, dt = 0.5 ns,
10 keV tracking cut.  One step = one outer dt of the electron transport
phase over the whole resident population.  Synthetic seeds; no dataset.

  value       particle-steps/s with the tile resident in HBM (device-timed)
  e2e         the same through the drop-in C-ABI entry point with host
              buffers: H2D of the tile, the step, D2H of tile + secondaries
  roofline    transport kernel vs measured HBM bandwidth (112 B algorithmic
              traffic per particle-step: read r,z,theta,ux,uy,uz,w,id, write
              r,z,theta,ux,uy,uz)
  cpu_baseline the oracle (CPU restatement, all host threads) on a bounded
              sample of the same workload

--impl reference times the CPU restatement of the reference path (the
WarpX/AMReX build itself cannot be built here) on the host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CASE = "scaleup_c1"
DT_S = 5.0e-10
BYTES_PER_PARTICLE_STEP = 112
METRIC = "particle-steps/s (electron transport phase, configs[1] workload)"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--population", type=int, default=1 << 21)
    p.add_argument("--cpu-sample", type=int, default=32768)
    p.add_argument("--e2e-steps", type=int, default=3)
    p.add_argument("--threads", type=int, default=128)
    p.add_argument("--blocks-per-sm", type=int, default=5)
    return p.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def read_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def read_traffic_per_particle_step():
    """dram bytes per particle-step of the transport kernel from the committed
    ncu summary (profiles/electron_step_kernel_scaleup_c1.md), if present."""
    path = os.path.join(ROOT, "profiles", "electron_step_kernel_scaleup_c1.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.strip().startswith("dram_bytes_per_particle_step:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=5)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for k, n in enumerate(names):
                if s[5 + k].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def cpu_oracle_rate(cfg, field, n, seed, steps=1):
    """Oracle particle-steps/s on n electrons for `steps` steps (all threads)."""
    from oracle import oracle
    from rrea_feedback_warpx_amrex_geant4_gb300 import DEFAULT_TABLES, workloads

    oracle.load_tables(DEFAULT_TABLES)
    arr = workloads.make_electrons(CASE, n, seed=seed)
    moved = 0
    t0 = time.perf_counter()
    for s in range(steps):
        moved += int((arr["id"] > 0).sum())
        oracle.electron_step(cfg, field, s, DT_S, arr)
        workloads.capture_prev(arr)
    dt = time.perf_counter() - t0
    return moved / dt, moved, dt


def run_reference(args, rank, world):
    if rank != 0:
        return
    from rrea_feedback_warpx_amrex_geant4_gb300 import gpu, workloads

    cfg = workloads.make_config(gpu, CASE)
    field = workloads.make_field(CASE)
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    for w in range(args.warmup):
        cpu_oracle_rate(cfg, field, 1024, seed=99 + w)
    rates, total_moved, total_t = [], 0, 0.0
    for s in range(args.steps):
        r, moved, dt = cpu_oracle_rate(cfg, field, args.cpu_sample, seed=1000 + s)
        rates.append(r)
        total_moved += moved
        total_t += dt
    value = total_moved / total_t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "particle-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * total_t / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (configs[1] seed distribution)",
        "config": {"workload": f"{CASE}: electron phase, {args.cpu_sample} electrons per timed step",
                   "grid": "256x2048", "dt_s": DT_S},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{args.cpu_sample} electrons x {args.steps} steps, OpenMP chunks of 64"},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gb300(args, rank, world, local):
    import torch

    from rrea_feedback_warpx_amrex_geant4_gb300 import DEFAULT_TABLES, gpu, workloads

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist_mod

        dist_mod.init_process_group("nccl")
        dist = dist_mod

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    n = args.population
    cfg = workloads.make_config(gpu, CASE)
    ctx = gpu.RreaGpuContext(cfg, n)
    ctx.load_tables(DEFAULT_TABLES)
    field = workloads.make_field(CASE)
    ctx.set_field(**field)
    ctx.set_launch(args.threads, args.blocks_per_sm, diagnostics=False)
    arr = workloads.make_electrons(CASE, n, seed=777 + rank)
    ctx.stage_electrons(arr)
    stream = torch.cuda.ExternalStream(ctx.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    step = 0
    for _ in range(args.warmup):
        ctx.step_electrons_resident(step, DT_S)
        step += 1
    barrier()

    clocks = ClockSampler(local)
    clocks.start()
    total_ms = 0.0
    kernel_ms = 0.0
    moved = 0
    launches = 0
    secondaries = 0
    for _ in range(args.steps):
        flush.zero_()  # L2 flush between timed steps (256 MiB write)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        nsec = ctx.step_electrons_resident(step, DT_S)
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
        t, s, kms = ctx.last_step_stats()
        kernel_ms += kms
        moved += t
        secondaries += nsec
        launches += 1 + 3 + (1 if nsec > 0 else 0)
        step += 1
    barrier()
    clocks.stop()

    # max over ranks of the device time; total work summed
    t_local = torch.tensor([total_ms, float(moved), kernel_ms], dtype=torch.float64, device="cuda")
    if dist is not None:
        tmax = t_local.clone()
        dist.all_reduce(tmax[0:1], op=dist.ReduceOp.MAX)
        dist.all_reduce(tmax[1:2], op=dist.ReduceOp.SUM)
        t_local = tmax
    total_ms_max = float(t_local[0])
    moved_all = float(t_local[1])
    value = moved_all / (total_ms_max / 1000.0)

    # ---- e2e through the drop-in C-ABI (host buffers, copies in the timed region)
    ctx2_n = n
    pinned = {}
    for k, v in workloads.make_electrons(CASE, ctx2_n, seed=4242 + rank).items():
        tt = torch.from_numpy(v).pin_memory()
        pinned[k] = tt.numpy()
    for f in ("r", "z", "theta", "ux", "uy", "uz"):
        pinned["prev_" + f] = pinned[f]  # the captured state is the current state
    e2e_moved = 0
    e2e_t = 0.0
    sec_bytes = 0
    ctx.apply_electrons(pinned, step, DT_S, want_secondaries=True)  # warm
    step += 1
    barrier()
    for _ in range(args.e2e_steps):
        live = int((pinned["id"] > 0).sum())
        t0 = time.perf_counter()
        sec = ctx.apply_electrons(pinned, step, DT_S, want_secondaries=True)
        e2e_t += time.perf_counter() - t0
        e2e_moved += live
        sec_bytes += len(sec) * gpu.SECONDARY_DTYPE.itemsize
        step += 1
    e2e_value = e2e_moved / e2e_t
    h2d = ctx2_n * (13 * 8 + 8 + 4)
    d2h = ctx2_n * (6 * 8 + 8) + sec_bytes // max(args.e2e_steps, 1)

    if rank == 0:
        peak, peak_kind = read_peaks()
        achieved = (moved * BYTES_PER_PARTICLE_STEP) / (kernel_ms / 1000.0) / 1.0e9 if kernel_ms > 0 else 0.0
        traffic_pps = read_traffic_per_particle_step()
        launches_per_step = launches / max(args.steps, 1)
        traffic = traffic_pps * (moved / max(args.steps, 1)) if traffic_pps else None
        cores = os.cpu_count() or 1
        cpu_n = min(args.cpu_sample, 16384)
        cpu_rate, cpu_moved, cpu_t = cpu_oracle_rate(cfg, field, cpu_n, seed=31337)
        line = {
            "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (configs[1] seed distribution, seeded numpy PRNG)",
            "config": {"workload": f"{CASE}: electron transport phase over a resident population of {n} e- "
                                   f"per GPU (configs[1] seeds/geometry/field), dt 0.5 ns",
                       "grid": "256x2048", "population_per_gpu": n, "dt_s": DT_S,
                       "l2": "flushed between timed steps (256 MiB write)",
                       "parallelism": f"dp{world} (independent particle shards)"},
            "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": args.e2e_steps,
                    "path": "rrea_gpu_apply_electrons (pinned host tile -> HBM -> host)"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": traffic, "kernel": "electron_step_kernel",
                         "algorithmic_bytes_per_particle_step": BYTES_PER_PARTICLE_STEP,
                         "kernel_ms_per_step": kernel_ms / args.steps},
            "cpu_baseline": {"value": cpu_rate, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                             "sample": f"{cpu_n} electrons x 1 step of the same workload, OpenMP chunks of 64"},
            "gpu_launches": launches,
            "gpu_launches_per_step": launches_per_step,
            "secondaries_per_step": secondaries / max(args.steps, 1),
            "clocks": clocks.summary(),
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


def main():
    args = parse()
    rank, world, local = dist_info()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gb300(args, rank, world, local)


if __name__ == "__main__":
    main()
