#!/usr/bin/env python3
"""Throughput of the GB300 kinetic step: particle-steps/s on one GB300.

Workload: the plain GPU scale-up case with its self-consistent field.
Electrons drawn from its seed distribution (K log-uniform 1-20 MeV,
isotropic in the -E hemisphere, uniform in a 5 m x 10 m disk), a photon
population (E log-uniform 50 keV-20 MeV, +z hemisphere, same disk; half as
many) and a positron population (the electron distribution; 1/16 as many),
air at 1.225 kg/m^3, initial uniform E_z = -500 kV/m, 256 x 2048 grid over
200 m x 2 km, dt = 0.5 ns, 10 keV tracking cut.  One step is the whole
kinetic step in the reference's order: the electron, photon and positron
phases over the resident populations, the transient FIFO that flies every
secondary through the rest of its step (newborn residual legs), the
net-chord current of all charged flights, and the Maxwell TM-RZ field update
driven by it.  A particle-step is one live macroparticle advanced through
one dt, its newborn residual legs included.  Synthetic seeds; no dataset.

  value       particle-steps/s with the tiles resident in HBM (device-timed)
  e2e         the same through the drop-in C-ABI entry points with host
              buffers: H2D of the tiles, the three phases, H2D of their
              secondaries into the drain, D2H of tiles, secondaries and
              survivors
  roofline    electron transport kernel (the dominant one) vs measured HBM
              bandwidth (112 B algorithmic traffic per particle-step: read
              r,z,theta,ux,uy,uz,w,id, write r,z,theta,ux,uy,uz)
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
PHOTON_FRACTION = 0.5  # photons per electron in the resident populations
POSITRON_FRACTION = 0.0625  # positrons per electron
FIELD_SUBSTEPS = 2  # material substeps of the Maxwell update
METRIC = ("particle-steps/s on 1 GB300 (plain kinetic step: electron, photon and positron phases, "
          "newborn FIFO, net-chord current and field update)")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--population", type=int, default=1 << 21)
    p.add_argument("--cpu-sample", type=int, default=131072)
    p.add_argument("--cpu-baseline-sample", type=int, default=1 << 19)
    p.add_argument("--cpu-baseline-steps", type=int, default=4)
    p.add_argument("--e2e-steps", type=int, default=3)
    p.add_argument("--threads", type=int, default=128)
    p.add_argument("--blocks-per-sm", type=int, default=16)
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


def make_photons(n, seed):
    from rrea_feedback_warpx_amrex_geant4_gb300 import workloads

    rng = np.random.default_rng(seed)
    e = np.exp(rng.uniform(np.log(5.0e4), np.log(2.0e7), n))
    r = 5.0 * np.sqrt(rng.uniform(0.0, 1.0, n))
    theta = rng.uniform(-np.pi, np.pi, n)
    z = rng.uniform(0.0, 10.0, n)
    mu = rng.uniform(0.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    sn = np.sqrt(1.0 - mu * mu)
    arr = {"r": r, "z": z, "theta": theta, "ux": e * sn * np.cos(phi), "uy": e * sn * np.sin(phi), "uz": e * mu,
           "w": np.ones(n), "id": np.arange(1, n + 1, dtype=np.int64), "cpu": np.zeros(n, dtype=np.int32)}
    for f in ("r", "z", "theta", "ux", "uy", "uz"):
        arr[f] = np.ascontiguousarray(arr[f], dtype=np.float64)
        arr["prev_" + f] = arr[f].copy()
    workloads.push_photons(arr, DT_S)
    return arr


def cpu_populations(n, seed):
    """Electron, photon and positron tiles of the workload (n electrons)."""
    from rrea_feedback_warpx_amrex_geant4_gb300 import workloads

    arr = workloads.make_electrons(CASE, n, seed=seed)
    pho = make_photons(int(n * PHOTON_FRACTION), seed + 1)
    pos = workloads.make_electrons(CASE, max(1, int(n * POSITRON_FRACTION)), seed=seed + 2)
    return arr, pho, pos


def commit_and_compact(tile, survivors, species):
    """DrainAndCommitSecondaries' commit on a host tile: the species'
    survivors become particles (oracle.commit_survivors), and the particles
    that ended the step leave the tile."""
    from oracle import oracle

    keep = tile["id"] > 0
    add = oracle.commit_survivors(survivors, species, int(np.abs(tile["id"]).max(initial=0)) + 1)
    out = {}
    for k, v in tile.items():
        if k == "cpu":
            extra = np.zeros(len(add["id"]), dtype=v.dtype)
        else:
            extra = add[k[5:] if k.startswith("prev_") else k]
        out[k] = np.ascontiguousarray(np.concatenate([v[keep], extra.astype(v.dtype)]))
    return out


def cpu_oracle_rate(cfg, field, n, seed, steps=1):
    """Oracle particle-steps/s of the whole kinetic step (three phases, FIFO
    drain and commit, net-chord current, field update) on n electrons, the
    photon and positron fractions, for `steps` steps (all threads)."""
    from oracle import oracle
    from rrea_feedback_warpx_amrex_geant4_gb300 import DEFAULT_TABLES, workloads

    if not getattr(cpu_oracle_rate, "_loaded", False):
        oracle.load_tables(DEFAULT_TABLES)
        cpu_oracle_rate._loaded = True
    arr, pho, pos = cpu_populations(n, seed)
    fld = {k: np.array(v, dtype=np.float64) for k, v in field.items()}
    dr = (cfg.r_hi - cfg.r_lo) / cfg.nr
    dz = (cfg.z_hi - cfg.z_lo) / cfg.nz
    moved = 0
    t0 = time.perf_counter()
    for s in range(steps):
        moved += int((arr["id"] > 0).sum()) + int((pho["id"] > 0).sum()) + int((pos["id"] > 0).sum())
        oe = oracle.electron_step(cfg, fld, s, DT_S, arr)
        og = oracle.photon_step(cfg, s, DT_S, pho)
        op = oracle.positron_step(cfg, fld, s, DT_S, pos)
        pending = np.concatenate([oe["secondaries"], og["secondaries"], op["secondaries"]])
        od = oracle.drain(cfg, fld, s, DT_S, pending)
        arr = commit_and_compact(arr, od["survivors"], 0)
        pos = commit_and_compact(pos, od["survivors"], 1)
        pho = commit_and_compact(pho, od["survivors"], 2)
        rows = np.concatenate([oracle.segment_rows(r) for r in (oe, op, od)])
        cur = oracle.deposit_segments(cfg, DT_S, rows)
        fld["er"], fld["ez"], fld["bt"] = oracle.advance_maxwell(cfg.nr, cfg.nz, dr, dz, DT_S, FIELD_SUBSTEPS,
                                                                 fld["er"], fld["ez"], fld["bt"], cur["jr_phys"],
                                                                 cur["jz_phys"])
        for t in (arr, pho, pos):
            workloads.capture_prev(t)
        workloads.push_photons(pho, DT_S)
    dt = time.perf_counter() - t0
    return moved / dt, moved, dt


def population_text(n):
    return (f"{n} e-, {int(n * PHOTON_FRACTION)} photons, {max(1, int(n * POSITRON_FRACTION))} e+")


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
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (scale-up case seed distribution)",
        "config": {"workload": f"{CASE}: whole kinetic step (three phases, newborn FIFO and commit, net-chord current, "
                               f"field update), {population_text(args.cpu_sample)} per timed step",
                   "grid": "256x2048", "dt_s": DT_S, "field_substeps": FIELD_SUBSTEPS},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{population_text(args.cpu_sample)} x {args.steps} steps (a fresh draw of the "
                                   f"workload each step), OpenMP chunks of 64"},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gb300(args, rank, world, local):
    import torch

    from rrea_feedback_warpx_amrex_geant4_gb300 import DEFAULT_TABLES, distributed, gpu, workloads

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
    n_g = int(n * PHOTON_FRACTION)
    n_p = max(1, int(n * POSITRON_FRACTION))
    cfg = workloads.make_config(gpu, CASE)
    # room for the committed survivors: the populations grow from step to step
    ctx = gpu.RreaGpuContext(cfg, n + n // 4)
    ctx.load_tables(DEFAULT_TABLES)
    field = workloads.make_field(CASE)
    ctx.set_field(**field)
    ctx.set_launch(args.threads, args.blocks_per_sm, diagnostics=False)
    arr = workloads.make_electrons(CASE, n, seed=777 + rank)
    pho = make_photons(n_g, seed=778 + rank)
    for f in ("r", "z", "theta"):
        pho[f][:] = pho["prev_" + f]  # the resident photon step pushes by itself
    pos = workloads.make_electrons(CASE, n_p, seed=779 + rank)
    ctx.stage_electrons(arr)
    ctx.stage_photons(pho)
    ctx.stage_positrons(pos)
    stream = torch.cuda.ExternalStream(ctx.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def one_step(step):
        ctx.reset_current()  # the net-chord current is per step (ResetNetChordStep)
        ne = ctx.step_electrons_resident(step, DT_S)
        te, _, kme = ctx.last_step_stats()
        ng = ctx.step_photons_resident(step, DT_S)
        tg, _, kmg = ctx.last_step_stats()
        npos = ctx.step_positrons_resident(step, DT_S)
        tp, _, kmp = ctx.last_step_stats()
        ctx.drain_resident(step, DT_S)  # newborn residual legs of every secondary
        items, surv = ctx.last_drain_stats()
        # DrainAndCommitSecondaries' commit: survivors become resident particles,
        # and the particles that ended this step leave the tiles
        committed = ctx.commit_survivors_resident()
        for species in (gpu.SPECIES_ELECTRON, gpu.SPECIES_POSITRON, gpu.SPECIES_PHOTON):
            ctx.compact_resident(species)
        # Maxwell TM-RZ with this step's J, summed over the ranks' shards
        distributed.exchange_current_and_advance(ctx, dist, DT_S, FIELD_SUBSTEPS)
        return {"te": te, "tg": tg, "tp": tp, "kme": kme, "kmg": kmg, "kmp": kmp,
                "secondaries": ne + ng + npos, "fifo_items": items, "survivors": surv,
                "committed": int(committed.sum())}

    step = 0
    for _ in range(args.warmup):
        one_step(step)
        step += 1
    barrier()

    clocks = ClockSampler(local)
    clocks.start()
    total_ms = 0.0
    acc = {k: 0 for k in ("te", "tg", "tp", "kme", "kmg", "kmp", "secondaries", "fifo_items", "survivors",
                          "committed")}
    launches = 0
    for _ in range(args.steps):
        flush.zero_()  # L2 flush between timed steps (256 MiB write)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        l0 = gpu.kernel_launches()
        e0.record(stream)
        r = one_step(step)
        e1.record(stream)
        e1.synchronize()
        launches += gpu.kernel_launches() - l0  # this library's kernels only
        total_ms += e0.elapsed_time(e1)
        for k in acc:
            acc[k] += r[k]
        step += 1
    barrier()
    clocks.stop()
    moved_e, moved_g, moved_p = acc["te"], acc["tg"], acc["tp"]
    kernel_ms_e, kernel_ms_g, kernel_ms_p = acc["kme"], acc["kmg"], acc["kmp"]

    # max over ranks of the device time; total work summed
    moved = moved_e + moved_g + moved_p
    total_ms_max, moved_all = distributed.reduce_step_time(total_ms, moved, dist, "cuda")
    value = moved_all / (total_ms_max / 1000.0)

    # ---- e2e through the drop-in C-ABI (host buffers, copies in the timed region)
    def pinned_tile(src):
        out = {}
        for k, v in src.items():
            out[k] = torch.from_numpy(np.ascontiguousarray(v)).pin_memory().numpy()
        return out

    pe = pinned_tile(workloads.make_electrons(CASE, n, seed=4242 + rank))
    for f in ("r", "z", "theta", "ux", "uy", "uz"):
        pe["prev_" + f] = pe[f]  # the captured state is the current state
    pg = pinned_tile(make_photons(n_g, seed=4243 + rank))
    pp = pinned_tile(workloads.make_electrons(CASE, n_p, seed=4244 + rank))
    for f in ("r", "z", "theta", "ux", "uy", "uz"):
        pp["prev_" + f] = pp[f]
    rec = gpu.SECONDARY_DTYPE.itemsize

    def e2e_step(step):
        """The overlay's step through the drop-in entry points: Apply's three
        phases on host tiles, then DrainAndCommitSecondaries on their host
        secondaries, then the field update."""
        ctx.reset_current()
        sec_e = ctx.apply_electrons(pe, step, DT_S, want_secondaries=True)
        sec_g = ctx.apply_photons(pg, step, DT_S, want_secondaries=True)
        sec_p = ctx.apply_positrons(pp, step, DT_S, want_secondaries=True)
        pending = np.concatenate([sec_e, sec_g, sec_p])
        surv = ctx.drain_secondaries(pending, step, DT_S)
        distributed.exchange_current_and_advance(ctx, dist, DT_S, FIELD_SUBSTEPS)
        return len(pending), len(surv)

    e2e_moved = 0
    e2e_t = 0.0
    sec_bytes = 0
    surv_bytes = 0
    e2e_step(step)  # warm
    step += 1
    barrier()
    for _ in range(args.e2e_steps):
        # photons: the host captures the start and pushes (WarpX's part of the step)
        for f in ("r", "z", "theta", "ux", "uy", "uz"):
            np.copyto(pg["prev_" + f], pg[f])
        workloads.push_photons(pg, DT_S)
        live = int((pe["id"] > 0).sum()) + int((pg["id"] > 0).sum()) + int((pp["id"] > 0).sum())
        t0 = time.perf_counter()
        n_pending, n_surv = e2e_step(step)
        e2e_t += time.perf_counter() - t0
        e2e_moved += live
        sec_bytes += n_pending * rec
        surv_bytes += n_surv * rec
        step += 1
    e2e_value = e2e_moved / e2e_t
    k = max(args.e2e_steps, 1)
    h2d = (n + n_g + n_p) * (13 * 8 + 8 + 4) + sec_bytes // k
    d2h = (n + n_g + n_p) * (6 * 8 + 8) + sec_bytes // k + surv_bytes // k

    if rank == 0:
        peak, peak_kind = read_peaks()
        achieved = (moved_e * BYTES_PER_PARTICLE_STEP) / (kernel_ms_e / 1000.0) / 1.0e9 if kernel_ms_e > 0 else 0.0
        achieved_g = (moved_g * BYTES_PER_PARTICLE_STEP) / (kernel_ms_g / 1000.0) / 1.0e9 if kernel_ms_g > 0 else 0.0
        achieved_p = (moved_p * BYTES_PER_PARTICLE_STEP) / (kernel_ms_p / 1000.0) / 1.0e9 if kernel_ms_p > 0 else 0.0
        traffic_pps = read_traffic_per_particle_step()
        launches_per_step = launches / max(args.steps, 1)
        traffic = traffic_pps * (moved_e / max(args.steps, 1)) if traffic_pps else None
        cores = os.cpu_count() or 1
        cpu_n = args.cpu_baseline_sample
        cpu_rate, cpu_moved, cpu_t = cpu_oracle_rate(cfg, field, cpu_n, seed=31337, steps=args.cpu_baseline_steps)
        line = {
            "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (scale-up case seed distribution, seeded numpy PRNG)",
            "config": {"workload": f"{CASE}: whole kinetic step (electron, photon, positron phases, newborn "
                                   f"FIFO and commit, net-chord current, field update) over resident populations of "
                                   f"{population_text(n)} per GPU (256x2048 cells over 200 m x 2 km, initial "
                                   f"uniform E_z = -500 kV/m), dt 0.5 ns",
                       "grid": "256x2048",
                       "population_per_gpu": {"electrons": n, "photons": n_g, "positrons": n_p},
                       "dt_s": DT_S, "field_substeps": FIELD_SUBSTEPS,
                       "l2": "flushed between timed steps (256 MiB write)",
                       "parallelism": f"dp{world} (independent particle shards)"},
            "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": args.e2e_steps,
                    "path": "rrea_gpu_apply_electrons/_photons/_positrons (pinned host tiles -> HBM -> host), "
                            "rrea_gpu_drain_secondaries (host records in, survivors out), "
                            "rrea_gpu_current_device + rrea_gpu_advance_field_from_current"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": traffic, "kernel": "electron_step_kernel",
                         "algorithmic_bytes_per_particle_step": BYTES_PER_PARTICLE_STEP,
                         "kernel_ms_per_step": kernel_ms_e / args.steps,
                         "photon_kernel": {"kernel": "photon_step_kernel", "achieved": achieved_g,
                                           "frac": achieved_g / peak, "kernel_ms_per_step": kernel_ms_g / args.steps},
                         "positron_kernel": {"kernel": "positron_step_kernel", "achieved": achieved_p,
                                             "frac": achieved_p / peak,
                                             "kernel_ms_per_step": kernel_ms_p / args.steps}},
            "phases": {"electron_steps": moved_e, "photon_steps": moved_g, "positron_steps": moved_p,
                       "secondaries_per_step": acc["secondaries"] / args.steps,
                       "fifo_items_per_step": acc["fifo_items"] / args.steps,
                       "survivors_per_step": acc["survivors"] / args.steps,
                       "committed_per_step": acc["committed"] / args.steps,
                       "transport_kernels_ms_per_step": (kernel_ms_e + kernel_ms_g + kernel_ms_p) / args.steps},
            "cpu_baseline": {"value": cpu_rate, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                             "sample": f"{population_text(cpu_n)} x {args.cpu_baseline_steps} steps of the same "
                                       f"whole kinetic step ({cpu_moved} particle-steps in {cpu_t:.1f} s), "
                                       f"OpenMP chunks of 64"},
            "gpu_launches": launches,
            "gpu_launches_per_step": launches_per_step,
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
