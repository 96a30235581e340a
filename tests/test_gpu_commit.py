"""Resident commit of the FIFO survivors into the species tiles
(rrea_gpu_commit_survivors_resident) and the compaction of invalid
particles (rrea_gpu_compact_resident), through the C-ABI, against the
oracle's restatement of the overlay's particle creation
(oracle.commit_survivors, O/RreaCouplingSources.cpp:240-330).

Tolerances: counts, order, ids and weights exact; r, theta and momenta
within 1e-14 relative (device hypot/atan2/sqrt vs the host libm, a few
ulps); the compaction moves rows and is exact."""
import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu

SPECIES = ((0, "electrons"), (1, "positrons"), (2, "photons"))


@pytest.fixture(scope="module")
def mods():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu, workloads
    from oracle import oracle
    build.build()
    return gpu, workloads, oracle


def _fetch(gpu, ctx, workloads, species):
    n = ctx.resident_count(species)
    t = workloads.make_electrons("uniform_c0", max(n, 1))
    t = {k: np.ascontiguousarray(v[:n]) for k, v in t.items()}
    getattr(ctx, "fetch_" + dict(SPECIES)[species])(t)
    return t


def _resident_step(gpu, workloads, capacity, n=1024, step=2, dt_s=1.0e-7):
    case = "scaleup_c1"
    cfg = workloads.make_config(gpu, case)
    ctx = gpu.RreaGpuContext(cfg, capacity)
    ctx.load_tables(TABLES)
    ctx.set_field(**workloads.make_field(case))
    e = workloads.make_electrons(case, n, seed=81)
    g = workloads.make_photons(case, n, dt_s, seed=82, e_lo=5.0e4, e_hi=1.0e8)
    for f in ("r", "z", "theta"):
        g[f][:] = g["prev_" + f]
    p = workloads.make_electrons(case, n // 4, seed=83)
    ctx.stage_electrons(e)
    ctx.stage_photons(g)
    ctx.stage_positrons(p)
    ctx.step_electrons_resident(step, dt_s)
    ctx.step_photons_resident(step, dt_s)
    ctx.step_positrons_resident(step, dt_s)
    ctx.drain_resident(step, dt_s)
    return ctx, {0: e, 1: p, 2: g}


def test_commit_appends_survivors_as_the_overlay_creates_them(mods):
    gpu, workloads, oracle = mods
    ctx, staged = _resident_step(gpu, workloads, capacity=16384)
    surv = ctx.fetch_survivors()
    assert len(surv) > 0
    before = {s: _fetch(gpu, ctx, workloads, s) for s, _ in SPECIES}
    committed = ctx.commit_survivors_resident()
    for s, _ in SPECIES:
        n0 = len(before[s]["id"])
        after = _fetch(gpu, ctx, workloads, s)
        assert len(after["id"]) == n0 + committed[s]
        for k in ("r", "z", "theta", "ux", "uy", "uz", "w", "id"):
            np.testing.assert_array_equal(after[k][:n0], before[s][k], err_msg=f"species {s} {k} (old rows)")
        ref = oracle.commit_survivors(surv, s, int(np.abs(staged[s]["id"]).max()) + 1)
        assert committed[s] == len(ref["id"]), f"species {s}"
        new = {k: v[n0:] for k, v in after.items()}
        np.testing.assert_array_equal(new["id"], ref["id"])
        np.testing.assert_array_equal(new["w"], ref["w"])
        np.testing.assert_array_equal(new["z"], ref["z"])
        np.testing.assert_array_equal(new["cpu"], 0)
        for k in ("r", "theta", "ux", "uy", "uz"):
            scale = np.maximum(np.abs(ref[k]), 1e-300 if k != "theta" else 1e-15)
            assert np.all(np.abs(new[k] - ref[k]) <= 1e-14 * scale), f"species {s} {k}"
    assert committed.sum() > 0
    # a second commit has nothing left to add
    assert ctx.commit_survivors_resident().sum() == 0
    ctx.close()


def test_committed_particles_step_on(mods):
    """The committed particles are ordinary resident particles of the next
    step: it runs and moves them."""
    gpu, workloads, oracle = mods
    ctx, _ = _resident_step(gpu, workloads, capacity=16384)
    committed = ctx.commit_survivors_resident()
    n0 = ctx.resident_count(0) - committed[0]
    before = _fetch(gpu, ctx, workloads, 0)
    ctx.step_electrons_resident(3, 5.0e-10)
    after = _fetch(gpu, ctx, workloads, 0)
    moved = (after["z"][n0:] != before["z"][n0:]) | (after["id"][n0:] < 0)
    assert moved.all()
    ctx.close()


def test_compaction_keeps_the_valid_rows_in_order(mods):
    gpu, workloads, oracle = mods
    ctx, _ = _resident_step(gpu, workloads, capacity=16384)
    ctx.commit_survivors_resident()
    for s, _ in SPECIES:
        before = _fetch(gpu, ctx, workloads, s)
        keep = before["id"] > 0
        if s != 1:  # few positrons end within one step
            assert (~keep).any(), f"species {s}: nothing to remove"
        n_live = ctx.compact_resident(s)
        assert n_live == int(keep.sum())
        after = _fetch(gpu, ctx, workloads, s)
        for k in ("r", "z", "theta", "ux", "uy", "uz", "w", "id", "cpu"):
            np.testing.assert_array_equal(after[k], before[k][keep], err_msg=f"species {s} {k}")
        assert ctx.compact_resident(s) == n_live
    ctx.close()


def test_commit_beyond_capacity_changes_no_tile(mods):
    gpu, workloads, oracle = mods
    ctx, _ = _resident_step(gpu, workloads, capacity=520, n=512, dt_s=3.0e-8)
    sizes = [ctx.resident_count(s) for s, _ in SPECIES]
    surv = ctx.fetch_survivors()
    assert int((surv["species"] == 0).sum()) + sizes[0] > 520
    with pytest.raises(gpu.RreaGpuError) as e:
        ctx.commit_survivors_resident()
    assert e.value.status == 8  # RREA_GPU_ERR_CAPACITY
    assert [ctx.resident_count(s) for s, _ in SPECIES] == sizes
    ctx.close()


def test_scheduled_seeds_join_the_resident_tiles(mods):
    """InjectScheduledSeeds on the resident tiles: the window's events are
    appended per species with the reference's normalised momentum
    (tests/golden/ref_seed_schedule_events.npy, computed by the reference);
    stale events are skipped, later ones wait for their window."""
    import os

    from conftest import GOLDEN

    gpu, workloads, oracle = mods
    ref = np.load(os.path.join(GOLDEN, "ref_seed_schedule_events.npy"))
    windows = np.load(os.path.join(GOLDEN, "ref_seed_schedule_windows.npy"))
    sched = gpu.SeedSchedule(os.path.join(GOLDEN, "ref_seed_schedule_input.csv"), "C2")
    cfg = workloads.make_config(gpu, "scaleup_c1")
    ctx = gpu.RreaGpuContext(cfg, 4096)
    ctx.load_tables(TABLES)
    ctx.set_field(**workloads.make_field("scaleup_c1"))
    e = workloads.make_electrons("scaleup_c1", 64, seed=90)
    ctx.stage_electrons(e)
    ctx.stage_positrons(workloads.make_electrons("scaleup_c1", 8, seed=91))
    injected_total = np.zeros(2, dtype=np.int64)
    # windows as the golden: [0, 5e-7), then (skipping) [1e-6, 1.0005e-6), then [1.5e-6, 2.5e-6)
    for w, (t0, t1) in enumerate(((0.0, 5.0e-7), (1.0e-6, 1.0005e-6), (1.5e-6, 2.5e-6))):
        n0 = [ctx.resident_count(0), ctx.resident_count(1)]
        got = ctx.inject_seeds(sched, t0, t1 - t0)
        sel = windows[:, w] == 0
        want = ref[sel]
        assert got[0] == int((want[:, 1] == 1).sum()) and got[1] == int((want[:, 1] == 2).sum()), w
        injected_total += got
        for k, species in ((0, 0), (1, 1)):
            rows = want[want[:, 1] == k + 1]
            t = _fetch(gpu, ctx, workloads, species)
            new = {c: v[n0[k]:] for c, v in t.items()}
            np.testing.assert_array_equal(new["z"], rows[:, 5])
            np.testing.assert_array_equal(new["w"], rows[:, 11])
            np.testing.assert_array_equal(new["ux"], rows[:, 12])
            np.testing.assert_array_equal(new["uy"], rows[:, 13])
            np.testing.assert_array_equal(new["uz"], rows[:, 14])
            np.testing.assert_array_equal(new["r"], np.hypot(rows[:, 3], rows[:, 4]))
            np.testing.assert_array_equal(new["theta"], np.arctan2(rows[:, 4], rows[:, 3]))
            assert (np.diff(new["id"]) == 1).all() and (new["id"] > 0).all()
    # events between the windows were stale when their window passed
    assert injected_total.sum() == int((windows == 0).sum())
    ctx.close()
