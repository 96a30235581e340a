"""Two steps of the resident loop (the three resident phases, the FIFO drain,
the survivor commit and the tile compaction; rrea_gpu_step_*_resident,
rrea_gpu_drain_resident, rrea_gpu_commit_survivors_resident,
rrea_gpu_compact_resident) against the oracle's same sequence with its
restatement of the overlay's particle creation.

The oracle starts every step from the GPU's fetched tiles (lockstep), so a
one-ulp difference of one step cannot grow into a different history in the
next.  Tolerances: tile sizes, ids and their order, and weights exact; FP64
state within 1e-12 relative (at most 0.1 % of the entries within 1e-11),
as in the phase tests."""
import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu

CASE, N, DT_S = "scaleup_c1", 2048, 1.0e-8
NAMES = {0: "electrons", 1: "positrons", 2: "photons"}


@pytest.fixture(scope="module")
def mods():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu, workloads
    from oracle import compare, oracle
    build.build()
    oracle.load_tables(TABLES)
    return gpu, workloads, oracle, compare


def _fetch(ctx, workloads, species):
    n = ctx.resident_count(species)
    t = workloads.make_electrons("uniform_c0", max(n, 1))
    t = {k: np.ascontiguousarray(v[:n]) for k, v in t.items()}
    getattr(ctx, "fetch_" + NAMES[species])(t)
    for f in ("r", "z", "theta", "ux", "uy", "uz"):
        t["prev_" + f] = t[f].copy()  # the resident captured state is the current state
    return t


def _commit(oracle, tile, survivors, species, first_id):
    keep = tile["id"] > 0
    add = oracle.commit_survivors(survivors, species, first_id)
    out = {}
    for k, v in tile.items():
        extra = np.zeros(len(add["id"]), dtype=v.dtype) if k == "cpu" else add[k[5:] if k.startswith("prev_") else k]
        out[k] = np.ascontiguousarray(np.concatenate([v[keep], extra.astype(v.dtype)]))
    return out, len(add["id"])


def test_two_resident_steps_with_commit_match_oracle(mods):
    gpu, workloads, oracle, compare = mods
    cfg = workloads.make_config(gpu, CASE)
    field = workloads.make_field(CASE)
    ctx = gpu.RreaGpuContext(cfg, 4 * N)
    ctx.load_tables(TABLES)
    ctx.set_field(**field)
    e = workloads.make_electrons(CASE, N, seed=101)
    g = workloads.make_photons(CASE, N // 2, DT_S, seed=102, e_lo=5.0e4, e_hi=2.0e7)
    for f in ("r", "z", "theta"):
        g[f][:] = g["prev_" + f]
    p = workloads.make_electrons(CASE, N // 8, seed=103)
    ctx.stage_electrons(e)
    ctx.stage_photons(g)
    ctx.stage_positrons(p)
    next_id = {0: N + 1, 1: N // 8 + 1, 2: N // 2 + 1}
    committed_total = 0
    for step in range(2):
        start = {s: _fetch(ctx, workloads, s) for s in NAMES}
        workloads.push_photons(start[2], DT_S)  # the oracle's photon tile carries the pushed end point
        # GPU: the resident loop
        ctx.reset_current()
        ctx.step_electrons_resident(step, DT_S)
        ctx.step_photons_resident(step, DT_S)
        ctx.step_positrons_resident(step, DT_S)
        ctx.drain_resident(step, DT_S)
        committed = ctx.commit_survivors_resident()
        for s in NAMES:
            ctx.compact_resident(s)
        # oracle: the same sequence from the same start
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
            assert len(got["id"]) == len(want["id"]), f"step {step} {NAMES[s]} size"
            np.testing.assert_array_equal(got["id"], want["id"], err_msg=f"step {step} {NAMES[s]} ids")
            np.testing.assert_array_equal(got["w"], want["w"], err_msg=f"step {step} {NAMES[s]} weights")
            umag = np.sqrt(want["ux"] ** 2 + want["uy"] ** 2 + want["uz"] ** 2)
            for f in ("r", "z", "ux", "uy", "uz"):
                scale = np.abs(want[f]) + 1.0 if f in ("r", "z") else umag
                ok, n_over = compare.entries_ok(got[f], want[f], compare.RTOL * scale)
                assert ok, f"step {step} {NAMES[s]} {f}: {n_over} outside tolerance"
        committed_total += int(committed.sum())
    assert committed_total > 0, "no survivors were committed: the workload does not exercise the commit"
    ctx.close()
