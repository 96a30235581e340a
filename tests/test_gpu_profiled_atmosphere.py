"""The profiled-atmosphere workload run through the resident loop: seeds from
a seed schedule (rrea_gpu_inject_seeds_resident), transport through the
altitude density profile (rrea_gpu_set_density_profile) in an ambient E_z
that varies with altitude, the FIFO drain, the survivor commit and the
compaction, for three steps on the 512x4096 grid over r 0-1 km and
altitudes 6-14 km.  The oracle runs the same phases, drain and commit
from the GPU's tiles after each injection (lockstep), bound to the same
profile and field.

Tolerances as in the resident-loop test: sizes, ids and weights exact, FP64
state within 1e-12 relative (at most 0.1 % of the entries within 1e-11)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, TABLES

pytestmark = pytest.mark.gpu

CASE, DT_S = "profiled_c2", 5.0e-10
NAMES = {0: "electrons", 1: "positrons", 2: "photons"}


@pytest.fixture(scope="module")
def mods():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu, workloads
    from oracle import compare, oracle
    build.build()
    oracle.load_tables(TABLES)
    yield gpu, workloads, oracle, compare
    oracle.set_density_profile()


def _empty(workloads):
    t = workloads.make_electrons("uniform_c0", 1)
    return {k: np.ascontiguousarray(v[:0]) for k, v in t.items()}


def _fetch(ctx, workloads, species):
    n = ctx.resident_count(species)
    t = workloads.make_electrons("uniform_c0", max(n, 1))
    t = {k: np.ascontiguousarray(v[:n]) for k, v in t.items()}
    getattr(ctx, "fetch_" + NAMES[species])(t)
    for f in ("r", "z", "theta", "ux", "uy", "uz"):
        t["prev_" + f] = t[f].copy()
    return t


def _commit(oracle, tile, survivors, species, first_id):
    keep = tile["id"] > 0
    add = oracle.commit_survivors(survivors, species, first_id)
    out = {}
    for k, v in tile.items():
        extra = np.zeros(len(add["id"]), dtype=v.dtype) if k == "cpu" else add[k[5:] if k.startswith("prev_") else k]
        out[k] = np.ascontiguousarray(np.concatenate([v[keep], extra.astype(v.dtype)]))
    return out, len(add["id"])


def test_profiled_atmosphere_loop_matches_oracle(mods):
    gpu, workloads, oracle, compare = mods
    cfg = workloads.make_config(gpu, CASE)
    alt, dens, alt0, field = workloads.profiled_atmosphere(CASE)
    ctx = gpu.RreaGpuContext(cfg, 8192)
    ctx.load_tables(TABLES)
    ctx.set_field(**field)
    ctx.set_density_profile(alt, dens, alt0, workloads.TABLE_DENSITY)
    oracle.set_density_profile(alt, dens, alt0, workloads.TABLE_DENSITY)
    sched = gpu.SeedSchedule(os.path.join(GOLDEN, "ref_seed_schedule_input.csv"), "C2")
    sched.validate(1.0e4, 1.0e9, 0.0, cfg.r_hi, 0.0, cfg.z_hi)
    for s in NAMES:
        getattr(ctx, "stage_" + NAMES[s])(_empty(workloads))
    next_id = {0: 1, 1: 1, 2: 1}
    window = 2.0e-6 / 3.0
    injected_total, committed_total = 0, 0
    for step in range(3):
        injected = ctx.inject_seeds(sched, step * window, window)
        injected_total += int(injected.sum())
        next_id[0] += int(injected[0])
        next_id[1] += int(injected[1])
        start = {s: _fetch(ctx, workloads, s) for s in NAMES}
        workloads.push_photons(start[2], DT_S)
        ctx.reset_current()
        ctx.step_electrons_resident(step, DT_S)
        ctx.step_photons_resident(step, DT_S)
        ctx.step_positrons_resident(step, DT_S)
        ctx.drain_resident(step, DT_S)
        committed = ctx.commit_survivors_resident()
        for s in NAMES:
            ctx.compact_resident(s)
        oe = oracle.electron_step(cfg, field, step, DT_S, start[0])
        og = oracle.photon_step(cfg, step, DT_S, start[2])
        op = oracle.positron_step(cfg, field, step, DT_S, start[1])
        pending = np.concatenate([oe["secondaries"], og["secondaries"], op["secondaries"]])
        surv = oracle.drain(cfg, field, step, DT_S, pending)["survivors"]
        for s in NAMES:
            want, added = _commit(oracle, start[s], surv, s, next_id[s])
            assert committed[s] == added, f"step {step} {NAMES[s]} committed"
            next_id[s] += added
            got = _fetch(ctx, workloads, s)
            np.testing.assert_array_equal(got["id"], want["id"], err_msg=f"step {step} {NAMES[s]} ids")
            np.testing.assert_array_equal(got["w"], want["w"], err_msg=f"step {step} {NAMES[s]} weights")
            umag = np.sqrt(want["ux"] ** 2 + want["uy"] ** 2 + want["uz"] ** 2)
            for f in ("r", "z", "ux", "uy", "uz"):
                scale = np.abs(want[f]) + 1.0 if f in ("r", "z") else umag
                ok, n_over = compare.entries_ok(got[f], want[f], compare.RTOL * scale)
                assert ok, f"step {step} {NAMES[s]} {f}: {n_over} outside tolerance"
        committed_total += int(committed.sum())
    assert injected_total > 100
    assert ctx.resident_count(0) > 0
    ctx.close()
