"""End-to-end avalanche runs through the resident C-ABI.

One run is what the overlay's WarpX loop does to the RREA species over many
steps (native_amrex_rrea/warpx_overlay/Source/Rrea/RreaParticleInteraction.cpp:12-62
for the transport, RreaSecondaryCommit.cpp for the drain and commit), with
every particle kept in HBM between steps:

  per step: ResetNetChordStep, the electron, photon and positron phases on
  the resident tiles (photons pushed straight on the device), the transient
  FIFO of every secondary's residual leg, the commit of the survivors into
  the tiles (new ids in FIFO order), the removal of the particles that ended
  the step, and, with feedback on, the Maxwell TM-RZ update driven by the
  step's net-chord current.

Every `census_every` steps (and after the last) the tiles are reduced on the
device (rrea_gpu_census_resident): counts, weights, the weight at or above
100 keV and 1 MeV (the reduced diagnostics' N_kinetic_e_ge_100keV and
N_kinetic_e_ge_1MeV_real probes, O/RreaCouplingDiagnostics.cpp:334-351) and
the weighted e-/photon/e+ energy spectra.

The multiplication factor of a run is the weight of electrons at or above
1 MeV at the end over the seed weight (a runaway-electron count ratio).

Run from the command line for a whole case:
  python -m rrea_feedback_warpx_amrex_geant4_gb300.avalanche --case uniform_c0 --seeds 10000 --steps 4000
"""
import argparse
import csv
import json
import os
import time

import numpy as np

from . import DEFAULT_TABLES, gpu, workloads

DT_S = 5.0e-10
# 10 keV to 1 GeV, 20 bins per decade: the spectra the statistical checks compare
SPECTRUM_EDGES_EV = np.logspace(4.0, 9.0, 101)
# the reduced diagnostics' energy probes (100 keV, 1 MeV)
THRESHOLDS_EV = np.array([1.0e5, 1.0e6])
SPECIES_NAMES = ("electron", "positron", "photon")


def c0_like_case(field_v_per_m=None, case="uniform_c0"):
    """Geometry, air and field of the plain uniform-field case; a different
    uniform field magnitude may be given."""
    p = dict(workloads.CASES[case])
    if field_v_per_m is not None:
        p["field_v_per_m"] = float(field_v_per_m)
    return p


def make_context(case="uniform_c0", capacity=1 << 20, rng_seed=1, field_v_per_m=None, tables=DEFAULT_TABLES,
                 blocks_per_sm=16):
    """A context for `case` with the uniform ambient E_z of the case (or the
    given magnitude) and a zero scattered field."""
    cfg = workloads.make_config(gpu, case, rng_seed=rng_seed)
    ctx = gpu.RreaGpuContext(cfg, capacity)
    ctx.load_tables(tables)
    field = workloads.make_field(case)
    if field_v_per_m is not None:
        field["amb_ez"][:] = -float(field_v_per_m)
    ctx.set_field(**field)
    ctx.set_launch(128, blocks_per_sm, diagnostics=False)
    return ctx


def census_row(ctx, step, edges=SPECTRUM_EDGES_EV, thresholds=THRESHOLDS_EV):
    """One census of all three resident tiles."""
    row = {"step": int(step), "time_s": step * DT_S}
    spectra = {}
    for sp, name in enumerate(SPECIES_NAMES):
        c = ctx.census(sp, edges, thresholds)
        row[f"{name}_count"] = c["count"]
        row[f"{name}_weight"] = c["sum_w"]
        row[f"{name}_energy_eV"] = c["sum_wk"]
        row[f"{name}_ge_100keV"] = float(c["above"][0])
        row[f"{name}_ge_1MeV"] = float(c["above"][1])
        spectra[name] = c["hist"]
    return row, spectra


class AvalancheRun:
    """A plain avalanche run on one GPU: seeds staged as the resident
    electron tile, then `steps` whole kinetic steps."""

    def __init__(self, ctx, electrons, photons=None, positrons=None, feedback=False, field_substeps=2,
                 population_target=None, split_min_weight=0.0, control_interval=1, controller_salt=0,
                 fluid=False, merge_cap=None):
        """feedback: the field follows the step's current; fluid (with
        feedback): through the coupled carrier-fluid + Maxwell step (the
        context's fluid must be configured) instead of the kinetic-only one;
        merge_cap: the weight-doubling merge of every species tile above
        that many live particles after each commit."""
        self.ctx = ctx
        self.feedback = feedback
        self.fluid = fluid
        self.field_substeps = field_substeps
        # adaptive_resample_v1: e- and e+ macro targets, the split floor, the
        # control interval in steps and the controller's RNG salt
        self.population_target = population_target
        self.split_min_weight = split_min_weight
        self.control_interval = control_interval
        self.controller_salt = controller_salt
        self.thinned = 0
        self.split = 0
        self.merge_cap = merge_cap
        self.merged = 0
        empty = workloads.make_electrons("uniform_c0", 0)
        ctx.stage_electrons(electrons)
        ctx.stage_photons(photons if photons is not None else empty)
        ctx.stage_positrons(positrons if positrons is not None else empty)
        self.seed_weight = float(np.sum(electrons["w"][electrons["id"] > 0]))
        self.step = 0

    def advance(self, dt_s=DT_S):
        """One whole kinetic step; returns the particle-steps it moved and
        the drain's (FIFO items, survivors)."""
        ctx = self.ctx
        if self.feedback:
            ctx.reset_current()
        ctx.reset_sources()
        moved = 0
        for sp, fn in ((gpu.SPECIES_ELECTRON, ctx.step_electrons_resident),
                       (gpu.SPECIES_PHOTON, ctx.step_photons_resident),
                       (gpu.SPECIES_POSITRON, ctx.step_positrons_resident)):
            if ctx.resident_count(sp) == 0:
                continue
            fn(self.step, dt_s)
            moved += ctx.last_step_stats()[0]
        ctx.drain_resident(self.step, dt_s)
        drained = ctx.last_drain_stats()
        control = bool(self.population_target) and self.step % self.control_interval == 0
        if control:
            # global thinning over the live particles and the staged survivors,
            # inside the commit transaction (PreflightAndApplySecondaryPopulationControl)
            for sp in (gpu.SPECIES_ELECTRON, gpu.SPECIES_POSITRON):
                self.thinned += ctx.population_thin(sp, self.population_target, self.step,
                                                    self.controller_salt)["removed"]
        ctx.commit_survivors_resident()
        if self.merge_cap:
            # weight-doubling merge above the cap (merged partners leave at the compaction)
            for sp in (gpu.SPECIES_ELECTRON, gpu.SPECIES_POSITRON, gpu.SPECIES_PHOTON):
                self.merged += ctx.population_merge(sp, self.merge_cap, self.step)["merged"]
        for sp in (gpu.SPECIES_ELECTRON, gpu.SPECIES_POSITRON, gpu.SPECIES_PHOTON):
            ctx.compact_resident(sp)
        if control and self.split_min_weight > 0.0:
            # split refill at the step boundary (ApplyAdaptivePopulationControl)
            for sp in (gpu.SPECIES_ELECTRON, gpu.SPECIES_POSITRON):
                self.split += ctx.population_split(sp, self.population_target, self.split_min_weight)
        if self.feedback and self.fluid:
            ctx.fluid_take_sources(dt_s)
            ctx.advance_field_coupled(dt_s)
        elif self.feedback:
            ctx.advance_field(dt_s, self.field_substeps)
        self.step += 1
        return moved, drained

    def run(self, steps, census_every=100, dt_s=DT_S, plane_csv=None):
        """Advances `steps` steps; returns a result dict with the census
        history, the final spectra, the multiplication factor and the
        device-side throughput.  plane_csv (a PlaneFluxCsv over the planes
        set on the context) writes the plane rows on its cadence and once
        more, forced, after the last step."""
        history = []
        moved_total = 0
        fifo_total = 0
        row, _ = census_row(self.ctx, self.step)
        history.append(row)
        l0 = gpu.kernel_launches()
        t0 = time.perf_counter()
        for k in range(steps):
            moved, drained = self.advance(dt_s)
            moved_total += moved
            fifo_total += drained[0]
            if plane_csv is not None:
                plane_csv.maybe_write(self.ctx, self.step, self.step * dt_s, force=k + 1 == steps)
            if (k + 1) % census_every == 0 or k + 1 == steps:
                row, spectra = census_row(self.ctx, self.step)
                row["particle_steps"] = moved_total
                if self.fluid:
                    row.update(self.ctx.fluid_reductions(dt_s))
                    row["N_inst_e_real"] = row["electron_weight"] + row["N_low_e_real"]
                history.append(row)
        wall = time.perf_counter() - t0
        launches = gpu.kernel_launches() - l0
        final = history[-1]
        return {
            "history": history, "spectra": spectra, "edges_eV": SPECTRUM_EDGES_EV.tolist(),
            "seed_weight": self.seed_weight,
            "multiplication": final["electron_ge_1MeV"] / self.seed_weight if self.seed_weight > 0 else 0.0,
            "particle_steps": moved_total, "fifo_items": fifo_total, "wall_s": wall,
            "particle_steps_per_s": moved_total / wall if wall > 0 else 0.0,
            "kernel_launches": launches, "steps": steps,
            "population_thinned": self.thinned, "population_split": self.split, "population_merged": self.merged,
        }


def avalanche_length_m(history, lo_frac=0.3, hi_frac=0.6, dt_s=DT_S, key="electron_ge_1MeV"):
    """Avalanche (e-folding) length of the runaway population along the
    drift: the log-slope of N(>= 1 MeV) between the census rows at lo_frac
    and hi_frac of the run, converted to distance at the speed of light
    (runaway electrons move at ~c)."""
    steps = np.array([h["step"] for h in history], dtype=np.float64)
    n = np.array([h[key] for h in history], dtype=np.float64)
    t_end = steps[-1]
    sel = (steps >= lo_frac * t_end) & (steps <= hi_frac * t_end) & (n > 0)
    if sel.sum() < 2:
        return float("nan")
    slope = np.polyfit(steps[sel] * dt_s * workloads.C_LIGHT, np.log(n[sel]), 1)[0]
    return 1.0 / slope if slope > 0 else float("inf")


def coleman_dwyer_length_m(field_v_per_m, density_kg_m3, threshold_kv_per_m=276.0, anchor_density=1.293):
    """Coleman-Dwyer avalanche length lambda = 7300 kV / (E - E_th n/n0),
    with the threshold scaled by the density over the 1.293 kg/m^3 anchor
    (scripts/test_cd_science.py:341-382, scripts/rrea_profiled_atmosphere.py)."""
    e_kv = field_v_per_m / 1000.0
    return 7300.0 / (e_kv - threshold_kv_per_m * density_kg_m3 / anchor_density)


REDUCED_COLUMNS = (  # our census fields under the reduced CSV's column names
    ("step", "step"), ("time_s", "time_s"),
    ("N_kinetic_e_real", "electron_weight"), ("N_kinetic_e_ge_1MeV_real", "electron_ge_1MeV"),
    ("N_kinetic_e_ge_100keV_real", "electron_ge_100keV"), ("N_photon_real", "photon_weight"),
    ("N_positron_real", "positron_weight"), ("N_positron_ge_100keV_real", "positron_ge_100keV"),
)
# with the carrier fluid: its totals (O/RreaCouplingDiagnostics.cpp:318-354, 469-471, 730-736)
FLUID_REDUCED_COLUMNS = tuple((c, c) for c in gpu.FLUID_REDUCED_COLUMNS) + (("N_inst_e_real", "N_inst_e_real"),)


def write_reduced_csv(path, history):
    """The census history as rrea_reduced.csv-style rows (the columns the
    census provides, under the reduced diagnostics' names,
    O/RreaCouplingDiagnostics.cpp:950-980)."""
    columns = REDUCED_COLUMNS + (FLUID_REDUCED_COLUMNS if history and "total_ne_low" in history[-1] else ())
    with open(path, "w", newline="") as f:
        w = csv.writer(f)
        w.writerow([c for c, _ in columns])
        for h in history:
            if all(k in h for _, k in columns):
                w.writerow([h[k] for _, k in columns])


class PlaneFluxCsv:
    """rrea_cd_plane_flux.csv of RreaWarpXCoupling::MaybeWriteCdPlaneFlux
    (O/RreaCouplingPlaneWriter.cpp:31-207) with the write cadence of
    RreaPlaneFluxState (I/RreaPlaneFlux.H:288-436): at the first step at or
    past each multiple of interval_s (within 32 ulps of the time), or when
    forced, one row per plane with the device's cumulative crossing
    accumulators (rrea_gpu_plane_flux) and the area-weighted mean of the
    cell-centred E_z over the core disc r <= core_radius_m at the plane (the
    plane between its bracketing cell-centre rows, clamped at the edges),
    beside the same mean of the ambient E_z and their relative difference."""

    HEADER = ("format_version", "write_index", "step", "time_s", "plane_index", "altitude_m",
              *gpu.RreaGpuContext.PLANE_VALUES,
              "core_total_ez_v_per_m", "core_ambient_ez_v_per_m", "core_field_perturbation_fraction")

    def __init__(self, path, planes, interval_s, core_radius_m, ambient_ez, altitude_at_z0_m=0.0):
        planes = np.asarray(planes, dtype=np.float64)
        if (planes.size == 0 or not np.all(np.isfinite(planes)) or np.any(np.diff(planes) <= 0.0)
                or not np.isfinite(interval_s) or not interval_s > 0.0
                or not np.isfinite(core_radius_m) or not core_radius_m > 0.0):
            raise ValueError("plane diagnostics need finite increasing planes, a positive output interval "
                             "and a positive core radius")
        self.path, self.planes = path, planes
        self.interval_s, self.core_radius_m = float(interval_s), float(core_radius_m)
        self.ambient_ez = np.asarray(ambient_ez, dtype=np.float64)   # the ambient face vector (nr x (nz+1))
        self.altitude_at_z0_m = float(altitude_at_z0_m)
        self.next_time_s = self.interval_s
        self.writes = 0
        self.last_step, self.last_time_s = -1, -np.inf

    def _tolerance(self, time_s):
        return 32.0 * np.finfo(np.float64).eps * max(1.0, abs(time_s), abs(self.next_time_s))

    def due(self, step, time_s, force=False):
        if step < 0 or not np.isfinite(time_s):
            return False
        if step == self.last_step and time_s == self.last_time_s:
            return False
        return force or time_s + self._tolerance(time_s) >= self.next_time_s

    def mark_written(self, step, time_s):
        if not self.due(step, time_s, True):
            raise ValueError("invalid or duplicate plane write")
        tol = self._tolerance(time_s)
        self.writes += 1
        self.last_step, self.last_time_s = step, time_s
        if time_s + tol >= self.next_time_s:
            # a forced write before the boundary keeps the schedule; an accepted
            # one moves past the boundary it was accepted at
            nxt = np.longdouble(self.next_time_s)
            intervals = np.floor((np.longdouble(time_s + tol) - nxt) / np.longdouble(self.interval_s)) + 1
            self.next_time_s = float(nxt + max(np.longdouble(1), intervals) * np.longdouble(self.interval_s))

    def core_means(self, cfg, scattered_ez):
        """Per plane: (total, ambient) area-weighted core means of E_z."""
        nr, nz = cfg.nr, cfg.nz
        dr, dz = (cfg.r_hi - cfg.r_lo) / nr, (cfg.z_hi - cfg.z_lo) / nz
        faces = (np.asarray(scattered_ez) + self.ambient_ez).reshape(nz + 1, nr)
        cell = 0.5 * (faces[:-1] + faces[1:])
        amb_faces = self.ambient_ez.reshape(nz + 1, nr)
        out = []
        for z in self.planes:
            x = (z - cfg.z_lo) / dz - 0.5        # RreaCellCenteredGatherIndexCoordinate
            if x <= 0.0:
                rows = [(0, 1.0)]
            elif x >= nz - 1:
                rows = [(nz - 1, 1.0)]
            else:
                lo = int(np.floor(x))
                rows = [(lo, 1.0 - (x - lo)), (lo + 1, x - lo)]
            total = ambient = area = 0.0
            # the ambient at the plane itself: linear between its bracketing E_z faces
            fz = min(max((z - cfg.z_lo) / dz, 0.0), float(nz))
            f0 = min(int(np.floor(fz)), nz - 1)
            amb_at_plane = amb_faces[f0] + (fz - f0) * (amb_faces[f0 + 1] - amb_faces[f0])
            for j, coefficient in rows:
                if not coefficient > 0.0:
                    continue
                for i in range(nr):
                    r_lo = max(0.0, cfg.r_lo + i * dr)
                    r_hi = min(self.core_radius_m, cfg.r_lo + (i + 1) * dr)
                    a = r_hi * r_hi - r_lo * r_lo if r_hi > r_lo else 0.0   # RreaCoreAnnulusArea
                    if not a > 0.0:
                        continue
                    wgt = coefficient * a
                    total += wgt * cell[j, i]
                    ambient += wgt * amb_at_plane[i]
                    area += wgt
            if not area > 0.0:
                raise ValueError("plane core field average has zero area")
            out.append((total / area, ambient / area))
        return out

    def maybe_write(self, ctx, step, time_s, force=False):
        if not self.due(step, time_s, force):
            return False
        flux = ctx.plane_flux()
        _, ez, _ = ctx.field()
        means = self.core_means(ctx.config, ez)
        fresh = self.writes == 0
        if fresh and os.path.exists(self.path) and os.path.getsize(self.path) > 0:
            raise ValueError("a fresh plane stream refuses to overwrite a non-empty CSV")
        with open(self.path, "w" if fresh else "a", newline="") as f:
            w = csv.writer(f)
            if fresh:
                w.writerow(self.HEADER)
            for p, z in enumerate(self.planes):
                total, ambient = means[p]
                perturbation = abs(total - ambient) / max(abs(ambient), 1.0e-30)
                w.writerow([1, self.writes, step, repr(float(time_s)), p, repr(self.altitude_at_z0_m + z)]
                           + [repr(float(v)) for v in flux[p]] + [repr(total), repr(ambient), repr(perturbation)])
        self.mark_written(step, time_s)
        return True


def main():
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("--case", default="uniform_c0", choices=["uniform_c0", "scaleup_c1"])
    p.add_argument("--feedback", action="store_true", help="the field follows the step's current")
    p.add_argument("--fluid", action="store_true",
                   help="with --feedback: the coupled carrier fluid (production closures) and Maxwell update")
    p.add_argument("--seeds", type=int, default=10_000)
    p.add_argument("--steps", type=int, default=4000)
    p.add_argument("--rng-seed", type=int, default=1)
    p.add_argument("--field", type=float, default=None, help="uniform |E_z| in V/m (default: the case's)")
    p.add_argument("--capacity", type=int, default=1 << 24)
    p.add_argument("--census-every", type=int, default=100)
    p.add_argument("--population-target", type=int, default=0,
                   help="adaptive_resample_v1 e-/e+ macro target (0: no population control)")
    p.add_argument("--split-min-weight", type=float, default=0.0)
    p.add_argument("--merge-cap", type=int, default=0,
                   help="weight-doubling merge of each species above this many live particles (0: off)")
    p.add_argument("--json", default=None)
    p.add_argument("--csv", default=None)
    p.add_argument("--planes", default=None, help="comma-separated plane z [m] of the crossing diagnostic")
    p.add_argument("--plane-interval", type=float, default=1.0e-7, help="plane CSV output interval [s]")
    p.add_argument("--plane-core-radius", type=float, default=5.0, help="core radius of the plane field mean [m]")
    p.add_argument("--plane-csv", default="rrea_cd_plane_flux.csv")
    a = p.parse_args()
    import torch

    torch.cuda.set_device(0)
    ctx = make_context(a.case, a.capacity, a.rng_seed, a.field)
    if a.feedback and a.fluid:
        from . import DEFAULT_CLOSURE
        ctx.fluid_configure(**workloads.fluid_overrides())
        ctx.fluid_load_closure(DEFAULT_CLOSURE)
    seeds = workloads.make_electrons(a.case, a.seeds)
    planes = None
    if a.planes:
        z = [float(v) for v in a.planes.split(",")]
        ctx.set_planes(z)
        amb = workloads.make_field(a.case)["amb_ez"]
        if a.field is not None:
            amb[:] = -float(a.field)
        planes = PlaneFluxCsv(a.plane_csv, z, a.plane_interval, a.plane_core_radius, amb)
    res = AvalancheRun(ctx, seeds, population_target=a.population_target or None,
                       split_min_weight=a.split_min_weight, merge_cap=a.merge_cap or None,
                       feedback=a.feedback, fluid=a.feedback and a.fluid).run(a.steps, census_every=a.census_every,
                                                                plane_csv=planes)
    p_case = c0_like_case(a.field, a.case)
    res["case"] = a.case
    res["seeds"] = a.seeds
    res["field_v_per_m"] = p_case["field_v_per_m"]
    res["avalanche_length_m"] = avalanche_length_m(res["history"])
    res["coleman_dwyer_length_m"] = [coleman_dwyer_length_m(p_case["field_v_per_m"], workloads.AIR_DENSITY, t)
                                     for t in (276.0, 284.0)]
    res["spectra"] = {k: v.tolist() for k, v in res["spectra"].items()}
    if a.csv:
        write_reduced_csv(a.csv, res["history"])
    text = json.dumps(res)
    if a.json:
        os.makedirs(os.path.dirname(os.path.abspath(a.json)), exist_ok=True)
        with open(a.json, "w") as f:
            f.write(text)
    print(json.dumps({k: res[k] for k in ("case", "seeds", "steps", "multiplication", "particle_steps", "wall_s",
                                          "particle_steps_per_s", "kernel_launches", "avalanche_length_m",
                                          "coleman_dwyer_length_m", "population_thinned", "population_split",
                                          "population_merged")}))
    ctx.close()


if __name__ == "__main__":
    main()
