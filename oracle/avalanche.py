"""ORACLE: test infrastructure only.

The CPU restatement of a whole avalanche run, step for step the sequence
rrea_feedback_warpx_amrex_geant4_gb300.avalanche drives on the GPU: the
electron, photon and positron phases of RreaParticleInteraction::Apply
(O/RreaParticleInteraction.cpp:12-62), the transient FIFO of
DrainAndCommitSecondaries (O/RreaSecondaryCommit.cpp:9-638), the overlay's
particle creation for the survivors (O/RreaCouplingSources.cpp:240-330) with
ids from a per-species counter in FIFO order, removal of the particles that
ended, CaptureRreaPositionsBeforePush (O/RreaWarpXCoupling.cpp:151-208) and
WarpX's straight photon push.  The census restates
rrea_gpu_census_resident in numpy.  Used by tests/ and bench.py's CPU legs
to check and time the GPU path; the product never imports it.
"""
import time

import numpy as np

from . import oracle as _oracle

ME_C2_EV = 510998.95000   # I/RreaConstants.H:9
C_M_PER_S = 299792458.0   # I/RreaConstants.H:10
TILE_KEYS = ("r", "z", "theta", "ux", "uy", "uz", "w", "prev_r", "prev_z", "prev_theta", "prev_ux", "prev_uy",
             "prev_uz", "id", "cpu")


def empty_tile():
    t = {k: np.zeros(0) for k in TILE_KEYS}
    t["id"] = np.zeros(0, dtype=np.int64)
    t["cpu"] = np.zeros(0, dtype=np.int32)
    return t


def commit_and_compact(tile, survivors, species, first_id):
    """The species' survivors become particles appended in FIFO order with
    ids first_id, first_id + 1, ... (oracle.commit_survivors); the particles
    that ended the step (id <= 0) leave the tile, the others keep their
    order.  Returns (tile, particles added)."""
    keep = tile["id"] > 0
    add = _oracle.commit_survivors(survivors, species, first_id)
    out = {}
    for k, v in tile.items():
        if k == "cpu":
            extra = np.zeros(len(add["id"]), dtype=v.dtype)
        else:
            extra = add[k[5:] if k.startswith("prev_") else k]
        out[k] = np.ascontiguousarray(np.concatenate([v[keep], np.asarray(extra).astype(v.dtype)]))
    return out, len(add["id"])


def capture_prev(t):
    for f in ("r", "z", "theta", "ux", "uy", "uz"):
        np.copyto(t["prev_" + f], t[f])


def push_photons(t, dt_s):
    """x += c dt u/|u| on the Cartesian image of the captured RZ point."""
    e = np.sqrt(t["ux"] ** 2 + t["uy"] ** 2 + t["uz"] ** 2)
    f = np.where(e > 0.0, C_M_PER_S * dt_s / np.where(e > 0.0, e, 1.0), 0.0)
    x = t["prev_r"] * np.cos(t["prev_theta"]) + t["ux"] * f
    y = t["prev_r"] * np.sin(t["prev_theta"]) + t["uy"] * f
    t["z"][:] = t["prev_z"] + t["uz"] * f
    t["r"][:] = np.hypot(x, y)
    t["theta"][:] = np.arctan2(y, x)


def census(tile, species, edges, thresholds):
    """rrea_gpu_census_resident restated: K from the proper velocity
    (RreaKineticEnergyEvFromProperVelocity, O/RreaParticleInteraction.H:1494-1505)
    or |u| for photons, in the same operation order."""
    valid = tile["id"] > 0
    ux, uy, uz, w = (tile[k][valid] for k in ("ux", "uy", "uz", "w"))
    u2 = ux * ux + uy * uy + uz * uz
    if species == 2:
        k = np.sqrt(u2)
    else:
        c2 = C_M_PER_S * C_M_PER_S
        gamma = np.sqrt(1.0 + u2 / c2)
        k = (u2 * ME_C2_EV) / (c2 * (gamma + 1.0))
    edges = np.asarray(edges, dtype=np.float64)
    inside = (k >= edges[0]) & (k < edges[-1])
    b = np.searchsorted(edges, k[inside], side="right") - 1
    hist = np.bincount(b, weights=w[inside], minlength=edges.size - 1)
    return {"count": int(valid.sum()), "max_weight": float(w.max()) if w.size else 0.0, "sum_w": float(w.sum()),
            "sum_w2": float((w * w).sum()), "sum_wk": float((w * k).sum()), "under": float(w[k < edges[0]].sum()),
            "over": float(w[k >= edges[-1]].sum()),
            "above": np.array([w[k >= t].sum() for t in thresholds]), "hist": hist, "energy": k}


class AvalancheRun:
    """The oracle's whole-run loop over host tiles (electron seeds)."""

    def __init__(self, cfg, field, electrons, photons=None, positrons=None, feedback=False, field_substeps=2,
                 fluid=None):
        """fluid: an oracle.fluid.FluidConfig to run the coupled fluid/Maxwell
        step (feedback=True) in place of the kinetic-only field update."""
        self.cfg = cfg
        self.feedback = feedback
        self.fluid = fluid
        n_cells = cfg.nr * cfg.nz
        self.fluid_state = {k: np.zeros(n_cells) for k in ("ne", "np", "nn", "rho", "se", "sp", "sn")}
        self.field_substeps = field_substeps
        self.field = {k: np.array(v, dtype=np.float64) for k, v in field.items()}
        self.tiles = {0: {k: np.array(v) for k, v in electrons.items()},
                      1: positrons if positrons is not None else empty_tile(),
                      2: photons if photons is not None else empty_tile()}
        for t in self.tiles.values():
            capture_prev(t)
        self.next_id = {s: int(np.abs(t["id"]).max(initial=0)) + 1 for s, t in self.tiles.items()}
        self.seed_weight = float(self.tiles[0]["w"][self.tiles[0]["id"] > 0].sum())
        self.step = 0

    def advance(self, dt_s):
        cfg, fld, t = self.cfg, self.field, self.tiles
        moved = sum(int((t[s]["id"] > 0).sum()) for s in t)
        push_photons(t[2], dt_s)
        phases = []
        if len(t[0]["id"]):
            phases.append(_oracle.electron_step(cfg, fld, self.step, dt_s, t[0]))
        if len(t[2]["id"]):
            phases.append(_oracle.photon_step(cfg, self.step, dt_s, t[2]))
        if len(t[1]["id"]):
            phases.append(_oracle.positron_step(cfg, fld, self.step, dt_s, t[1]))
        parts = [r["secondaries"] for r in phases]
        pending = np.concatenate(parts) if parts else np.zeros(0, dtype=_oracle.SECONDARY_DTYPE)
        od = _oracle.drain(cfg, fld, self.step, dt_s, pending)
        surv = od["survivors"]
        if self.feedback:
            # the step's net-chord current (charged phases and newborn legs)
            # drives the Maxwell TM-RZ update of the scattered field
            rows = np.concatenate([_oracle.segment_rows(r) for r in phases + [od]])
            cur = _oracle.deposit_segments(cfg, dt_s, rows)
            dr = (cfg.r_hi - cfg.r_lo) / cfg.nr
            dz = (cfg.z_hi - cfg.z_lo) / cfg.nz
            if self.fluid is None:
                fld["er"], fld["ez"], fld["bt"] = _oracle.advance_maxwell(
                    cfg.nr, cfg.nz, dr, dz, dt_s, self.field_substeps, fld["er"], fld["ez"], fld["bt"],
                    cur["jr_phys"], cur["jz_phys"])
            else:
                from . import fluid as _fluid
                # NormalizeAndSync of the step's sources into the fluid's rates
                cells = sum(r["cells"] for r in phases + [od]).reshape(5, -1)
                r_in = cfg.r_lo + (np.arange(cfg.nr * cfg.nz) % cfg.nr) * dr
                vol = np.pi * ((r_in + dr) ** 2 - r_in ** 2) * dz
                st = self.fluid_state
                for k, key in enumerate(("se", "sp", "sn")):
                    st[key] = np.where(vol * dt_s > 0, cells[k] / (vol * dt_s), 0.0)
                (fld["er"], fld["ez"], fld["bt"]), new, _ = _fluid.coupled_step(
                    self.fluid, cfg.nr, cfg.nz, cfg.z_lo, dr, dz, dt_s, (fld["er"], fld["ez"], fld["bt"]),
                    (fld["amb_er"], fld["amb_ez"]), (cur["jr_phys"], cur["jz_phys"]), st)
                self.fluid_state = {k: new[k] for k in st}
        for s in (0, 1, 2):
            t[s], added = commit_and_compact(t[s], surv, s, self.next_id[s])
            self.next_id[s] += added
            capture_prev(t[s])
        self.step += 1
        return moved

    def census_row(self, edges, thresholds, dt_s):
        names = {0: "electron", 1: "positron", 2: "photon"}
        row = {"step": self.step, "time_s": self.step * dt_s}
        spectra = {}
        for s, name in names.items():
            c = census(self.tiles[s], s, edges, thresholds)
            row[f"{name}_count"] = c["count"]
            row[f"{name}_weight"] = c["sum_w"]
            row[f"{name}_energy_eV"] = c["sum_wk"]
            row[f"{name}_ge_100keV"] = float(c["above"][0])
            row[f"{name}_ge_1MeV"] = float(c["above"][1])
            spectra[name] = c["hist"]
        return row, spectra

    def run(self, steps, dt_s, edges, thresholds, census_every=100):
        history = []
        row, spectra = self.census_row(edges, thresholds, dt_s)
        history.append(row)
        moved_total = 0
        t0 = time.perf_counter()
        for k in range(steps):
            moved_total += self.advance(dt_s)
            if (k + 1) % census_every == 0 or k + 1 == steps:
                row, spectra = self.census_row(edges, thresholds, dt_s)
                row["particle_steps"] = moved_total
                history.append(row)
        wall = time.perf_counter() - t0
        final = history[-1]
        return {"history": history, "spectra": spectra, "seed_weight": self.seed_weight,
                "multiplication": final["electron_ge_1MeV"] / self.seed_weight if self.seed_weight else 0.0,
                "particle_steps": moved_total, "wall_s": wall}
