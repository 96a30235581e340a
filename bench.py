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
net-chord current of all charged flights and the ionization sources, and the
coupled low-energy carrier fluid + Maxwell TM-RZ field update they drive
(production dry-air closures, adaptive material substeps).  A particle-step is one live macroparticle advanced through
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
  scaleup_run the scale-up case run from its seeds with field feedback and
              the merge cap (800 steps, host wall clock)
  profiled_atmosphere  the largest case's geometry (512x4096 cells, 6-14 km,
              density profile, altitude-dependent E_z) with an entering
              column of 2e6 e- and 5e5 e+ and the coupled fluid update
  batched     the batched pattern: 64 independent uniform-field instances
              advanced by one set of launches per step against the same 64
              run one after another (stepping wall time, results identical)
  adjoint     seconds per pathwise field gradient of the adjoint pattern
              (1e6 electrons, 2000 steps, checkpoints every 32 steps)

--impl reference times the CPU restatement of the reference path (the
WarpX/AMReX build itself cannot be built here) on the host cores, on the same
populations and the same evolution (warm-up steps untimed, then the timed
steps), without loading the GPU library.
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
FIELD_SUBSTEPS = 2  # minimum material substeps of the coupled update (the reference's default)
METRIC = ("particle-steps/s on 1 GB300 (plain kinetic step: electron, photon and positron phases, "
          "newborn FIFO, net-chord current, carrier fluid and field update)")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--population", type=int, default=1 << 21)
    p.add_argument("--cpu-baseline-steps", type=int, default=3)
    p.add_argument("--e2e-steps", type=int, default=5)
    p.add_argument("--e2e-warmup", type=int, default=1, help="untimed drop-in steps before the timed e2e steps")
    p.add_argument("--c0-steps", type=int, default=1000)
    p.add_argument("--ensemble-scale", type=float, default=0.05,
                   help="duration scale of the batched 64-instance ensemble line (0: skip it)")
    p.add_argument("--adjoint-steps", type=int, default=2000, help="steps of the adjoint line (0: skip it)")
    p.add_argument("--c1-run-steps", type=int, default=800,
                   help="steps of the scale-up avalanche run line (0: skip it)")
    p.add_argument("--profiled-steps", type=int, default=8,
                   help="timed steps of the profiled-atmosphere line (0: skip it)")
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


TRAFFIC_RECORD = os.path.join(ROOT, "profiles", "electron_step_kernel_traffic.json")


def read_fp64_pipe_pct():
    """The electron kernel's FP64-pipe utilisation from the same record
    (None when the record is absent, of another build, or lacks it)."""
    from rrea_feedback_warpx_amrex_geant4_gb300 import build

    if not os.path.exists(TRAFFIC_RECORD):
        return None
    with open(TRAFFIC_RECORD) as f:
        rec = json.load(f)
    if rec.get("source_digest") != build.source_digest():
        return None
    return rec.get("fp64_pipe_pct")


def read_traffic_per_particle_step():
    """DRAM bytes (read + write) per particle-step of the electron transport
    kernel, from the ncu capture recorded for THIS build: the record carries
    the library's source digest, and a record of another build is not used
    (returns (None, reason)).  ncu cannot run inside a timed bench, so the
    counter comes from a capture of the same build on the same workload."""
    from rrea_feedback_warpx_amrex_geant4_gb300 import build

    if not os.path.exists(TRAFFIC_RECORD):
        return None, "no ncu capture recorded"
    with open(TRAFFIC_RECORD) as f:
        rec = json.load(f)
    digest = build.source_digest()
    if rec.get("source_digest") != digest:
        return None, f"the recorded capture is of build {rec.get('source_digest')}, not {digest}"
    return float(rec["dram_bytes_per_particle_step"]), (f"ncu capture of this build ({digest}): "
                                                        f"{rec.get('capture', '')}")


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


def gpu_arm_populations(n, rank=0):
    """The resident populations both arms start from: n electrons from the
    case's seed distribution, n/2 photons and n/16 positrons (seeded), with
    photons at their start point (the resident photon step pushes them)."""
    from rrea_feedback_warpx_amrex_geant4_gb300 import workloads

    n_g = int(n * PHOTON_FRACTION)
    n_p = max(1, int(n * POSITRON_FRACTION))
    arr = workloads.make_electrons(CASE, n, seed=777 + rank)
    pho = make_photons(n_g, seed=778 + rank)
    for f in ("r", "z", "theta"):
        pho[f][:] = pho["prev_" + f]
    pos = workloads.make_electrons(CASE, n_p, seed=779 + rank)
    return arr, pho, pos


def oracle_whole_steps(n, warmup, steps, rank=0):
    """The oracle (CPU restatement, all host threads) running the bench's
    whole kinetic step on the bench's populations: `warmup` untimed steps,
    then `steps` timed ones, the populations evolving with commit and field
    feedback exactly as on the GPU.  Returns (particle-steps, seconds, cores).
    Loads no part of the GPU library."""
    from oracle import avalanche as oav, oracle
    from rrea_feedback_warpx_amrex_geant4_gb300 import DEFAULT_TABLES, workloads

    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    from oracle import fluid as ofl
    from rrea_feedback_warpx_amrex_geant4_gb300 import DEFAULT_CLOSURE

    oracle.load_tables(DEFAULT_TABLES)
    ofl.load_closure(DEFAULT_CLOSURE)
    cfg = workloads.make_config(oracle, CASE)
    arr, pho, pos = gpu_arm_populations(n, rank)
    run = oav.AvalancheRun(cfg, workloads.make_field(CASE), arr, photons=pho, positrons=pos, feedback=True,
                           field_substeps=FIELD_SUBSTEPS,
                           fluid=ofl.default_config(**workloads.fluid_overrides()))
    for _ in range(warmup):
        run.advance(DT_S)
    moved = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        moved += run.advance(DT_S)
    return moved, time.perf_counter() - t0, cores


DATA = "synthetic (scale-up case seed distribution, seeded numpy PRNG)"


def workload_config(n, world):
    """The workload both arms time (the same populations, evolution and field)."""
    return {"workload": f"{CASE}: whole kinetic step (electron, photon, positron phases, newborn FIFO and commit, "
                        f"net-chord current and ionization sources, coupled carrier-fluid + Maxwell update) over "
                        f"resident populations of {population_text(n)} per "
                        f"GPU (256x2048 cells over 200 m x 2 km, initial uniform E_z = -500 kV/m), dt 0.5 ns",
            "grid": "256x2048",
            "population_per_gpu": {"electrons": n, "photons": int(n * PHOTON_FRACTION),
                                   "positrons": max(1, int(n * POSITRON_FRACTION))},
            "dt_s": DT_S, "field": "coupled carrier fluid (en_table_flux_v1, en_table_attachment_v1) + Maxwell, "
                                   "adaptive material substeps (min 2)",
            "l2": "flushed between timed steps (256 MiB write)",
            "parallelism": f"dp{world} (independent particle shards)"}


def population_text(n):
    return (f"{n} e-, {int(n * PHOTON_FRACTION)} photons, {max(1, int(n * POSITRON_FRACTION))} e+")


def run_reference(args, rank, world):
    if rank != 0:
        return
    n = args.population
    moved, secs, cores = oracle_whole_steps(n, args.warmup, args.steps)
    value = moved / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "particle-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * secs / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": DATA,
        "config": workload_config(n, world),
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                         "sample": f"the whole workload: {population_text(n)} evolving over {args.warmup} untimed "
                                   f"and {args.steps} timed steps ({moved} particle-steps in {secs:.1f} s), "
                                   f"OpenMP chunks of 64, -O3"},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def profiled_column(n_e, n_p, seed=2026):
    """The profiled case's entering column: e- and e+ at 12 km altitude
    (z = 6 km above the 6 km floor) over r <= 1 km, K from E^-1.5 on
    1-100 MeV, moving down with zenith angle density ~ cos^2."""
    from rrea_feedback_warpx_amrex_geant4_gb300 import workloads

    def tile(n, s):
        rng = np.random.default_rng(s)
        a = 1.0 - 1.5
        k = (1.0e6 ** a + rng.uniform(0.0, 1.0, n) * (1.0e8 ** a - 1.0e6 ** a)) ** (1.0 / a)
        mu = rng.uniform(0.0, 1.0, n) ** (1.0 / 3.0)
        phi = rng.uniform(0.0, 2.0 * np.pi, n)
        sn = np.sqrt(1.0 - mu * mu)
        u = workloads.proper_velocity(k)
        t = workloads.make_electrons("profiled_c2", n, seed=s)
        t["r"][:] = 1000.0 * np.sqrt(rng.uniform(0.0, 1.0, n))
        t["theta"][:] = rng.uniform(-np.pi, np.pi, n)
        t["z"][:] = 6000.0 - 10.0 * rng.uniform(0.0, 1.0, n)
        t["ux"][:] = u * sn * np.cos(phi)
        t["uy"][:] = u * sn * np.sin(phi)
        t["uz"][:] = -u * mu
        workloads.capture_prev(t)
        return t

    return tile(n_e, seed), tile(n_p, seed + 1)


def profiled_line(args, gpu, workloads, distributed, tables, closure):
    import torch

    n_e, n_p = 2_000_000, 500_000
    cfg = workloads.make_config(gpu, "profiled_c2")
    ctx = gpu.RreaGpuContext(cfg, 4_000_000)
    try:
        ctx.load_tables(tables)
        alt, dens, alt0, field = workloads.profiled_atmosphere()
        ctx.set_field(**field)
        ctx.set_density_profile(alt, dens, alt0, workloads.TABLE_DENSITY)
        ctx.fluid_configure(**workloads.fluid_overrides())
        ctx.fluid_load_closure(closure)
        ctx.set_launch(args.threads, args.blocks_per_sm, diagnostics=False)
        e, pos = profiled_column(n_e, n_p)
        ctx.stage_electrons(e)
        ctx.stage_positrons(pos)
        ctx.stage_photons(workloads.make_electrons("profiled_c2", 0))
        stream = torch.cuda.ExternalStream(ctx.stream())
        moved = 0
        total_ms = 0.0
        for k in range(args.warmup + args.profiled_steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            ctx.reset_current()
            ctx.reset_sources()
            step_moved = 0
            for sp, fn in ((gpu.SPECIES_ELECTRON, ctx.step_electrons_resident),
                           (gpu.SPECIES_PHOTON, ctx.step_photons_resident),
                           (gpu.SPECIES_POSITRON, ctx.step_positrons_resident)):
                if ctx.resident_count(sp) == 0:
                    continue
                fn(k, DT_S)
                step_moved += ctx.last_step_stats()[0]
            ctx.drain_resident(k, DT_S)
            ctx.commit_survivors_resident()
            for sp in (gpu.SPECIES_ELECTRON, gpu.SPECIES_POSITRON, gpu.SPECIES_PHOTON):
                ctx.compact_resident(sp)
            distributed.exchange_and_advance_coupled(ctx, None, DT_S)
            e1.record(stream)
            e1.synchronize()
            if k >= args.warmup:
                total_ms += e0.elapsed_time(e1)
                moved += step_moved
        counts = [ctx.resident_count(sp) for sp in (gpu.SPECIES_ELECTRON, gpu.SPECIES_PHOTON, gpu.SPECIES_POSITRON)]
    finally:
        ctx.close()
    return {"workload": "profiled atmosphere: 512x4096 cells over r 0-1 km, altitudes 6-14 km, density 1.225 "
                        "exp(-h/7.2 km) as the transport's altitude profile, E_z 1.3 x threshold at 10 km; "
                        f"{n_e} e- and {n_p} e+ entering at 12 km (K ~ E^-1.5 on 1-100 MeV, zenith ~ cos^2); "
                        "three phases, drain, commit, compaction and the coupled carrier fluid + Maxwell update",
            "value": moved / (total_ms / 1000.0), "unit": "particle-steps/s",
            "ms_per_step": total_ms / args.profiled_steps, "steps": args.profiled_steps, "warmup": args.warmup,
            "final_counts": {"electrons": counts[0], "photons": counts[1], "positrons": counts[2]}}


def run_gb300(args, rank, world, local):
    import torch

    from rrea_feedback_warpx_amrex_geant4_gb300 import DEFAULT_CLOSURE, DEFAULT_TABLES, distributed, gpu, workloads

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
    # the carrier fluid of the feedback case (production closures)
    ctx.fluid_configure(**workloads.fluid_overrides())
    ctx.fluid_load_closure(DEFAULT_CLOSURE)
    ctx.set_launch(args.threads, args.blocks_per_sm, diagnostics=False)
    arr, pho, pos = gpu_arm_populations(n, rank)
    ctx.stage_electrons(arr)
    ctx.stage_photons(pho)
    ctx.stage_positrons(pos)
    stream = torch.cuda.ExternalStream(ctx.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def one_step(step):
        ctx.reset_current()  # the net-chord current is per step (ResetNetChordStep)
        ctx.reset_sources()  # and so are the ionization sources the fluid takes
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
        # the coupled carrier-fluid + Maxwell TM-RZ update with this step's
        # kinetic J and ionization sources, summed over the ranks' shards
        distributed.exchange_and_advance_coupled(ctx, dist, DT_S)
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

    # ---- e2e through the drop-in C-ABI (host buffers, copies in the timed
    # region) on the populations the resident steps reached
    def pinned_tile(src):
        out = {}
        for k, v in src.items():
            out[k] = torch.from_numpy(np.ascontiguousarray(v)).pin_memory().numpy()
        return out

    def fetched(species, fetch):
        m = ctx.resident_count(species)
        t = {k: np.ascontiguousarray(v[:m]) for k, v in workloads.make_electrons(CASE, max(m, 1)).items()}
        fetch(t)
        for f in ("r", "z", "theta", "ux", "uy", "uz"):
            t["prev_" + f][:] = t[f]  # the captured state is the current state
        return pinned_tile(t)

    pe = fetched(gpu.SPECIES_ELECTRON, ctx.fetch_electrons)
    pg = fetched(gpu.SPECIES_PHOTON, ctx.fetch_photons)
    pp = fetched(gpu.SPECIES_POSITRON, ctx.fetch_positrons)
    rec = gpu.SECONDARY_DTYPE.itemsize

    e2e_calls = {}

    def timed(name, fn, *a, **kw):
        t = time.perf_counter()
        out = fn(*a, **kw)
        e2e_calls[name] = e2e_calls.get(name, 0.0) + time.perf_counter() - t
        return out

    def e2e_step(step):
        """The overlay's step through the drop-in entry point: Apply in one
        call (the three phases on host tiles and DrainAndCommitSecondaries'
        transient FIFO, survivors back to the host), then the coupled fluid
        and field update."""
        ctx.reset_current()
        ctx.reset_sources()
        surv = timed("apply_step", ctx.apply_step, pe, pg, pp, step, DT_S)
        timed("field_update", distributed.exchange_and_advance_coupled, ctx, dist, DT_S)
        return 0, len(surv)

    e2e_moved = 0
    e2e_t = 0.0
    sec_bytes = 0
    surv_bytes = 0
    barrier()
    for i in range(args.e2e_warmup + args.e2e_steps):
        # photons: the host captures the start and pushes (WarpX's part of the step)
        for f in ("r", "z", "theta", "ux", "uy", "uz"):
            np.copyto(pg["prev_" + f], pg[f])
        workloads.push_photons(pg, DT_S)
        live = int((pe["id"] > 0).sum()) + int((pg["id"] > 0).sum()) + int((pp["id"] > 0).sum())
        t0 = time.perf_counter()
        n_pending, n_surv = e2e_step(step)
        step += 1
        if i < args.e2e_warmup:
            e2e_calls.clear()
            continue  # first use of the drop-in path's buffers, untimed
        e2e_t += time.perf_counter() - t0
        e2e_moved += live
        sec_bytes += n_pending * rec
        surv_bytes += n_surv * rec
    e2e_value = e2e_moved / e2e_t if e2e_t > 0 else None
    k = max(args.e2e_steps, 1)
    tiles_n = len(pe["id"]) + len(pg["id"]) + len(pp["id"])
    h2d = tiles_n * (13 * 8 + 8 + 4) + sec_bytes // k
    d2h = tiles_n * (6 * 8 + 8) + sec_bytes // k + surv_bytes // k

    # ---- the plain uniform-field case at its own small populations (1e4
    # seeds, the first c0 steps of its 4000): launch- and latency-bound
    c0 = None
    if rank == 0 and args.c0_steps > 0:
        from rrea_feedback_warpx_amrex_geant4_gb300 import avalanche

        c0_ctx = avalanche.make_context("uniform_c0", 1 << 20, 1, blocks_per_sm=args.blocks_per_sm)
        torch.cuda.synchronize()
        res = avalanche.AvalancheRun(c0_ctx, workloads.make_electrons("uniform_c0", 10_000)).run(
            args.c0_steps, census_every=args.c0_steps)
        c0_ctx.close()
        c0 = {"workload": f"uniform_c0: 10000 seeds at 7.2 MeV, E_z = -400 kV/m, 32x256 cells over 50 m x 500 m, "
                          f"first {args.c0_steps} of its 4000 steps (the resident loop: three phases, drain, "
                          f"commit, compaction; no field feedback)",
              "value": res["particle_steps_per_s"], "unit": "particle-steps/s",
              "ms_per_step": 1000.0 * res["wall_s"] / args.c0_steps,
              "particle_steps": res["particle_steps"],
              "launches_per_step": res["kernel_launches"] / args.c0_steps,
              "final_electrons": res["history"][-1]["electron_count"],
              "timing": "host wall clock around the steps (each step ends in a stream synchronisation)"}

    # ---- the scale-up case run from its seeds: 1e5 electrons (K log-uniform
    # 1-20 MeV), field feedback through the coupled carrier fluid, every step
    # committed, each species capped at 1e6 macroparticles by the
    # weight-doubling merge
    c1_run = None
    if rank == 0 and world == 1 and args.c1_run_steps > 0:
        from rrea_feedback_warpx_amrex_geant4_gb300 import avalanche

        try:
            run_ctx = avalanche.make_context(CASE, 3_000_000, 1, blocks_per_sm=args.blocks_per_sm)
            try:
                run_ctx.fluid_configure(**workloads.fluid_overrides())
                run_ctx.fluid_load_closure(DEFAULT_CLOSURE)
                res = avalanche.AvalancheRun(run_ctx, workloads.make_electrons(CASE, 100_000), feedback=True,
                                             fluid=True, merge_cap=1_000_000).run(args.c1_run_steps,
                                                                                 census_every=args.c1_run_steps)
            finally:
                run_ctx.close()
            last = res["history"][-1]
            c1_run = {"workload": f"scale-up case from its 1e5 seeds (K log-uniform 1-20 MeV), field feedback through the "
                                  f"coupled carrier fluid, {args.c1_run_steps} steps of 0.5 ns, every step committed, each "
                                  f"species capped at 1e6 macroparticles by the weight-doubling merge",
                      "value": res["particle_steps_per_s"], "unit": "particle-steps/s",
                      "ms_per_step": 1000.0 * res["wall_s"] / args.c1_run_steps,
                      "particle_steps": res["particle_steps"], "merged": res["population_merged"],
                      "multiplication": res["multiplication"],
                      "final": {"electrons": last["electron_count"], "electron_weight": last["electron_weight"],
                                "photons": last["photon_count"], "positrons": last["positron_count"]},
                      "timing": "host wall clock around the steps (each step ends in a stream synchronisation)"}
        except gpu.RreaGpuError as exc:  # reported in the line, the headline stands
            c1_run = {"error": str(exc)}

    # ---- the profiled atmosphere (the largest case's geometry): 512x4096
    # cells over r 0-1 km and altitudes 6-14 km, density 1.225 exp(-h/7.2 km)
    # bound as the transport's altitude profile, E_z peaking at 1.3 x the
    # local threshold at 10 km, a column of 2e6 e- and 5e5 e+ entering at
    # 12 km over r <= 1 km (K ~ E^-1.5 on 1-100 MeV, zenith ~ cos^2), with
    # the coupled carrier fluid and field update
    profiled = None
    if rank == 0 and world == 1 and args.profiled_steps > 0:
        try:
            profiled = profiled_line(args, gpu, workloads, distributed, DEFAULT_TABLES, DEFAULT_CLOSURE)
        except gpu.RreaGpuError as exc:  # reported in the line, the headline stands
            profiled = {"error": str(exc)}

    # ---- the batched pattern: 64 independent uniform-field instances in one
    # set of launches per step against the same 64 run one after another
    # (identical per-instance results, so the statistics match exactly)
    batched = None
    if rank == 0 and world == 1 and args.ensemble_scale > 0:
        from rrea_feedback_warpx_amrex_geant4_gb300 import ensemble

        inst = ensemble.batched_instances(64, duration_scale=args.ensemble_scale)
        b = ensemble.run_batched(inst, control_every=16)
        q = ensemble.run_sequential(inst, control_every=16)
        same = all(x["multiplication"] == y["multiplication"] and x["electron_count"] == y["electron_count"]
                   for x, y in zip(b["results"], q["results"]))
        batched = {"workload": f"64 uniform-field instances (E_z 300-1000 kV/m, 1e3-1e5 seeds at 7.2 MeV, 32x256 "
                               f"cells each), durations 0.5-4 us scaled by {args.ensemble_scale} "
                               f"({min(i.steps for i in inst)}-{max(i.steps for i in inst)} steps)",
                   "batched_s": b["stepping_s"], "sequential_s": q["stepping_s"],
                   "speedup": q["stepping_s"] / b["stepping_s"],
                   "batched_particle_steps_per_s": b["particle_steps"] / b["stepping_s"],
                   "sequential_particle_steps_per_s": q["particle_steps"] / q["stepping_s"],
                   "particle_steps": b["particle_steps"], "identical_results": same,
                   "launch_shape": b["autotune"][0] if b["autotune"] else None,
                   "timing": "host wall clock of the steps (set-up and table loads excluded; every step ends in a "
                             "stream synchronisation)"}

    # ---- the adjoint pattern: seconds per pathwise field gradient
    adjoint_line = None
    if rank == 0 and world == 1 and args.adjoint_steps > 0:
        from rrea_feedback_warpx_amrex_geant4_gb300 import adjoint

        a = adjoint.measure(1_000_000, repeats=1, steps=args.adjoint_steps)
        adjoint_line = {"workload": f"1e6 seed electrons at 7.2 MeV, E_z(z) on 256 nodes over 0-500 m (450 kV/m "
                                    f"plus a 20 kV/m, 20 m correlated perturbation), {a['steps']} steps of 0.5 ns "
                                    f"in {a['substeps']} substeps, checkpoints every {a['checkpoint_every']} steps, "
                                    f"FP64",
                        "s_per_grad": a["s_per_grad"], "forward_s": a["forward_s"], "reverse_s": a["reverse_s"],
                        "reverse_over_forward": a["reverse_over_forward"], "unit": "s/grad",
                        "higher_is_better": False}

    if rank == 0:
        peak, peak_kind = read_peaks()
        achieved = (moved_e * BYTES_PER_PARTICLE_STEP) / (kernel_ms_e / 1000.0) / 1.0e9 if kernel_ms_e > 0 else 0.0
        achieved_g = (moved_g * BYTES_PER_PARTICLE_STEP) / (kernel_ms_g / 1000.0) / 1.0e9 if kernel_ms_g > 0 else 0.0
        achieved_p = (moved_p * BYTES_PER_PARTICLE_STEP) / (kernel_ms_p / 1000.0) / 1.0e9 if kernel_ms_p > 0 else 0.0
        traffic_pps, traffic_source = read_traffic_per_particle_step()
        launches_per_step = launches / max(args.steps, 1)
        traffic = traffic_pps * (moved_e / max(args.steps, 1)) if traffic_pps else None
        cpu_moved, cpu_t, cores = (oracle_whole_steps(n, 0, args.cpu_baseline_steps, rank)
                                   if args.cpu_baseline_steps > 0 else (0, 0.0, os.cpu_count() or 1))
        cpu_rate = cpu_moved / cpu_t if cpu_t > 0 else None
        line = {
            "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": DATA,
            "config": workload_config(n, world),
            "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": args.e2e_steps, "warmup": args.e2e_warmup,
                    "ms_per_step": 1000.0 * e2e_t / max(args.e2e_steps, 1),
                    "calls_ms_per_step": {k: 1000.0 * v / max(args.e2e_steps, 1) for k, v in e2e_calls.items()},

                    "path": "rrea_gpu_apply_step (pinned host tiles -> HBM; the three phases and the transient "
                            "FIFO on the device; tiles and FIFO-ordered survivors back to the host), "
                            "rrea_gpu_current_device + rrea_gpu_fluid_take_sources + "
                            "rrea_gpu_advance_field_coupled_from_current"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": traffic, "traffic_source": traffic_source, "kernel": "electron_step_kernel",
                         "fp64_pipe_pct_of_peak": read_fp64_pipe_pct(),
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
                             "sample": f"{population_text(n)} (the GPU arm's starting populations) x "
                                       f"{args.cpu_baseline_steps} steps of the same whole kinetic step "
                                       f"({cpu_moved} particle-steps in {cpu_t:.1f} s), OpenMP chunks of 64, -O3"},
            "small_population": c0,
            "scaleup_run": c1_run,
            "profiled_atmosphere": profiled,
            "batched": batched,
            "adjoint": adjoint_line,
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
