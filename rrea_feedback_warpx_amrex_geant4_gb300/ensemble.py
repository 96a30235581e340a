"""Batched ensemble of independent uniform-field avalanche instances on one
GPU (the batched pattern of the kinetic step): the particles of every
instance share the resident species tiles, so one launch sequence per step
advances all of them, where the sequential way runs one launch sequence per
instance and step.

An instance is a particle's cpu ordinal (rrea_gpu_ensemble_configure): its
streams, ids and field are its own, and the ensemble evolves every instance
exactly as that instance alone with cpu = k would evolve (the sequential
reference below), including the per-instance population control, which both
apply to the same slice at the same steps.  Each instance runs for its own
number of steps; at its end its census (the multiplication factor of
electrons at or above 1 MeV and the e-/photon spectra) is taken and its
particles are retired.

The launch shape of the transport kernels (threads per block and resident
blocks per SM, i.e. block shape and particles per thread) and the
scheduling order of the charged tiles (the per-step sort by |u|) are picked
by `autotune`, which times live steps: no result depends on them.

Instances of the batched configuration come from `batched_instances`:
E_z evenly spaced 300-1000 kV/m, seed counts log-uniform 1e3-1e5 (seeded),
durations mapped linearly in 1/(E - 280 kV/m) onto 0.5-4 us, the air,
tables, grid and seeds of the plain uniform-field case."""
import argparse
import json
import time
from dataclasses import dataclass

import numpy as np

from . import avalanche, gpu, workloads
from .gpu import DEFAULT_TABLES

DT_S = avalanche.DT_S
CASE = "uniform_c0"


@dataclass
class Instance:
    field_v_per_m: float   # |E_z|; the field points along -z, the seeds along +z
    n_seeds: int
    steps: int
    target: int = 0        # per-species population target of the thinning (0: none)


def batched_instances(n=64, seed=7, duration_scale=1.0, target=0):
    """The batched configuration: n instances; durations scaled by
    duration_scale (1 = 0.5-4 us); target > 0 adds a per-instance population
    control (the configuration itself has none)."""
    e = np.linspace(3.0e5, 1.0e6, n)
    rng = np.random.default_rng(seed)
    seeds = np.exp(rng.uniform(np.log(1.0e3), np.log(1.0e5), n)).astype(np.int64)
    inv = 1.0 / (e - 2.8e5)
    dur = 0.5e-6 + 3.5e-6 * (inv - inv.min()) / (inv.max() - inv.min())
    steps = np.maximum(1, np.round(dur * duration_scale / DT_S)).astype(np.int64)
    return [Instance(float(e[k]), int(seeds[k]), int(steps[k]), int(target)) for k in range(n)]


def seed_tile(instances, only=None):
    """The seed electrons of every instance (or only those listed): the plain
    uniform-field seeds, ids 1..n_k and cpu k per instance."""
    parts = []
    for k, inst in enumerate(instances):
        if only is not None and k not in only:
            continue
        t = workloads.make_electrons(CASE, inst.n_seeds)
        t["id"][:] = np.arange(1, inst.n_seeds + 1)
        t["cpu"][:] = k
        parts.append(t)
    if not parts:
        return workloads.make_electrons(CASE, 0)
    return {key: np.concatenate([p[key] for p in parts]) for key in parts[0]}


class EnsembleRun:
    """Runs the instances (all, or `only` some of them: the sequential
    reference runs one) to their ends on one context."""

    SPECIES = (gpu.SPECIES_ELECTRON, gpu.SPECIES_PHOTON, gpu.SPECIES_POSITRON)

    def __init__(self, instances, capacity=1 << 22, rng_seed=1, only=None, control_every=1, one_pass=True,
                 tables=DEFAULT_TABLES, edges=avalanche.SPECTRUM_EDGES_EV, thresholds=avalanche.THRESHOLDS_EV):
        self.instances = list(instances)
        self.active = sorted(range(len(self.instances)) if only is None else only)
        self.edges, self.thresholds = edges, thresholds
        self.control_every = control_every
        self.one_pass = one_pass
        cfg = workloads.make_config(gpu, CASE, rng_seed=rng_seed)
        self.ctx = ctx = gpu.RreaGpuContext(cfg, capacity)
        ctx.load_tables(tables)
        ctx.ensemble_configure([-inst.field_v_per_m for inst in self.instances])
        ctx.set_launch(128, 16, diagnostics=False)
        empty = workloads.make_electrons(CASE, 0)
        ctx.stage_electrons(seed_tile(self.instances, self.active))
        ctx.stage_photons(empty)
        ctx.stage_positrons(empty)
        self.step = 0
        self.results = {}
        self.thinned = 0
        self.particle_steps = 0

    def close(self):
        self.ctx.close()

    def _phases(self):
        ctx = self.ctx
        ms = 0.0
        for sp, fn in ((gpu.SPECIES_ELECTRON, ctx.step_electrons_resident),
                       (gpu.SPECIES_PHOTON, ctx.step_photons_resident),
                       (gpu.SPECIES_POSITRON, ctx.step_positrons_resident)):
            if ctx.resident_count(sp) == 0:
                continue
            fn(self.step, DT_S)
            moved, _, kernel_ms = ctx.last_step_stats()
            self.particle_steps += moved
            if sp == gpu.SPECIES_ELECTRON:
                ms = kernel_ms / max(moved, 1)
        return ms

    def advance(self):
        """One step of every live instance; returns the electron kernel's ms
        per transported electron."""
        ctx = self.ctx
        per_particle_ms = self._phases()
        ctx.drain_resident(self.step, DT_S)
        ctx.commit_survivors_resident()
        for sp in self.SPECIES:
            ctx.compact_resident(sp)
        self.step += 1
        ending = [k for k in self.active if self.instances[k].steps == self.step]
        controlled = [k for k in self.active if self.instances[k].target > 0 and k not in ending]
        if controlled and self.step % self.control_every == 0:
            self._control(controlled)
        if ending:
            for sp in self.SPECIES:
                ctx.ensemble_partition(sp)
            for k in ending:
                self.results[k] = self._census(k)
                ctx.ensemble_retire(k)
                self.active.remove(k)
        return per_particle_ms

    def _control(self, controlled):
        """Population control of the listed instances: one plan over all of
        them per species, or (one_pass=False) one per instance slice."""
        ctx = self.ctx
        if self.one_pass:
            targets = np.zeros(len(self.instances), dtype=np.int64)
            for k in controlled:
                targets[k] = self.instances[k].target
            for sp in (gpu.SPECIES_ELECTRON, gpu.SPECIES_POSITRON):
                removed, _ = ctx.ensemble_population_thin_all(sp, targets, self.step)
                self.thinned += int(removed.sum())
            return
        for sp in (gpu.SPECIES_ELECTRON, gpu.SPECIES_POSITRON):
            counts = ctx.ensemble_partition(sp)
            for k in controlled:
                t = self.instances[k].target
                if counts[k] > t + t // 4:
                    self.thinned += ctx.ensemble_population_thin(sp, k, t, self.step)["removed"]

    def _census(self, k):
        ctx = self.ctx
        e = ctx.ensemble_census(gpu.SPECIES_ELECTRON, k, self.edges, self.thresholds)
        g = ctx.ensemble_census(gpu.SPECIES_PHOTON, k, self.edges)
        p = ctx.ensemble_census(gpu.SPECIES_POSITRON, k, self.edges)
        inst = self.instances[k]
        return {"instance": k, "field_v_per_m": inst.field_v_per_m, "n_seeds": inst.n_seeds, "steps": inst.steps,
                "multiplication": float(e["above"][1]) / inst.n_seeds,
                "electron_weight": e["sum_w"], "photon_weight": g["sum_w"], "positron_weight": p["sum_w"],
                "electron_count": e["count"], "photon_count": g["count"],
                "spectra": {"electron": e["hist"], "photon": g["hist"]}}

    def autotune(self, shapes=((128, 16), (128, 8), (128, 4), (64, 16), (128, 12)), steps_each=2,
                 orders=(True, False)):
        """Times live steps under each launch shape and scheduling order and
        keeps the fastest (ms per transported electron); returns the choice
        and the timings.  Steps taken here are ordinary steps of the run."""
        timings = []
        for order in orders:
            for threads, blocks in shapes:
                if not self.active:
                    break
                self.ctx.set_launch(threads, blocks, diagnostics=False)
                self.ctx.set_schedule(order)
                ms = [self.advance() for _ in range(steps_each)]
                timings.append(((threads, blocks, order), float(np.median(ms))))
        best = min(timings, key=lambda t: t[1])[0] if timings else (128, 16, True)
        self.ctx.set_launch(best[0], best[1], diagnostics=False)
        self.ctx.set_schedule(best[2])
        return best, timings

    def run(self, autotune=False):
        """Advances every instance to its end; `stepping_s` is the wall time
        of the steps (the autotuner's steps included, set-up excluded: every
        step ends in a stream synchronisation)."""
        t0 = time.perf_counter()
        tuned = self.autotune() if autotune else None
        while self.active:
            self.advance()
        return {"results": [self.results[k] for k in sorted(self.results)], "steps": self.step,
                "particle_steps": self.particle_steps, "thinned": self.thinned, "autotune": tuned,
                "stepping_s": time.perf_counter() - t0}


def run_batched(instances, capacity=1 << 22, autotune=True, **kw):
    run = EnsembleRun(instances, capacity=capacity, **kw)
    try:
        return run.run(autotune=autotune)
    finally:
        run.close()


def run_sequential(instances, capacity=1 << 20, **kw):
    """Every instance alone on its own context (cpu = k)."""
    out, steps, particle_steps, thinned, stepping = [], 0, 0, 0, 0.0
    for k in range(len(instances)):
        run = EnsembleRun(instances, capacity=capacity, only=[k], **kw)
        try:
            res = run.run(autotune=False)
        finally:
            run.close()
        out += res["results"]
        steps += res["steps"]
        particle_steps += res["particle_steps"]
        thinned += res["thinned"]
        stepping += res["stepping_s"]
    return {"results": out, "steps": steps, "particle_steps": particle_steps, "thinned": thinned,
            "stepping_s": stepping}


def main():
    p = argparse.ArgumentParser(description="batched ensemble of uniform-field avalanches")
    p.add_argument("--instances", type=int, default=64)
    p.add_argument("--duration-scale", type=float, default=1.0)
    p.add_argument("--target", type=int, default=0, help="per-instance population target (0: no control)")
    p.add_argument("--control-every", type=int, default=16, help="steps between population-control checks")
    p.add_argument("--sequential", action="store_true", help="also run the instances one by one")
    p.add_argument("--json", default=None)
    args = p.parse_args()
    inst = batched_instances(args.instances, duration_scale=args.duration_scale, target=args.target)
    t0 = time.perf_counter()
    batched = run_batched(inst, control_every=args.control_every)
    t_b = time.perf_counter() - t0
    summary = {"instances": args.instances, "duration_scale": args.duration_scale, "target": args.target,
               "control_every": args.control_every, "batched_s": t_b,
               "batched_stepping_s": batched["stepping_s"], "batched_steps": batched["steps"],
               "thinned": batched["thinned"], "batched_particle_steps": batched["particle_steps"],
               "autotune": batched["autotune"][0] if batched["autotune"] else None,
               "multiplication": [r["multiplication"] for r in batched["results"]]}
    if args.sequential:
        t0 = time.perf_counter()
        seq = run_sequential(inst, control_every=args.control_every)
        summary["sequential_s"] = time.perf_counter() - t0
        summary["sequential_stepping_s"] = seq["stepping_s"]
        summary["sequential_steps"] = seq["steps"]
        summary["sequential_particle_steps"] = seq["particle_steps"]
        summary["speedup"] = summary["sequential_s"] / t_b
        # the steps alone: 64 context set-ups and table loads left out
        summary["speedup_stepping"] = seq["stepping_s"] / batched["stepping_s"]
    print(json.dumps(summary))
    if args.json:
        with open(args.json, "w") as f:
            json.dump(summary, f)


if __name__ == "__main__":
    main()
