"""Adaptive population control on the device (rrea_gpu_population_thin_resident,
rrea_gpu_population_split_resident) against the reference.

tests/golden/ref_population_*.npy come from oracle/_ref/ref_golden: the
reference's RreaPlanGlobalCicThinning, RreaCicResampleRemovalCapacity and
RreaAdaptiveResampleCicUniform (I/RreaCicConservingResample.H, O/RreaRng.H)
driven on one rank the way PreflightAndApplySecondaryPopulationControl
(O/RreaCouplingPopulation.cpp:175-640) drives them, over 3200-4000 live
particles (a third crowded into three cells, so supports hold well over 64
particles) and 800 staged candidates, for electrons (1500 target: every
support thinned to its floor until 3300 are gone) and positrons (3000
target: 1000 removed, the last support partly).  Exact: the plan's member,
support, capacity, request and removal counts, which particles reach weight
zero, and the invalidation of those; weights within 1e-12 relative (the
device solves each support's CIC constraints in double-double, the
reference in x87 long double; a few conditioned supports leave ~1e-13).  The four
CIC cell charges of every cell are kept to round-off.  The split refill is
checked on its own rule: halved weights, identical clones in tile order with
the next ids."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu, workloads
    from oracle import oracle
    build.build()
    return gpu, workloads, oracle


def _golden(tag, what):
    return np.load(os.path.join(GOLDEN, f"ref_population_{tag}_{what}.npy"))


def _fetch(ctx, workloads, species):
    n = ctx.resident_count(species)
    t = {k: np.ascontiguousarray(v[:n]) for k, v in workloads.make_electrons("uniform_c0", max(n, 1)).items()}
    (ctx.fetch_electrons if species == 0 else ctx.fetch_positrons)(t)
    return t


@pytest.mark.parametrize("tag", ["electron", "positron"])
def test_global_thinning_plan_matches_reference(mods, tag):
    gpu, workloads, oracle = mods
    setup = _golden(tag, "setup")[0]
    nr, nz, dr, dz, r_lo, z_lo, seed, salt, step, positron = setup
    species = 1 if positron else 0
    cfg = gpu.default_config(r_lo=r_lo, r_hi=r_lo + nr * dr, z_lo=z_lo, z_hi=z_lo + nz * dz, nr=int(nr), nz=int(nz),
                             rng_seed=int(seed))
    live = _golden(tag, "live")
    cand_in = _golden(tag, "candidates")
    want_w = _golden(tag, "weights")[:, 0]
    plan = _golden(tag, "plan")[0]
    n_live = len(live)
    ctx = gpu.RreaGpuContext(cfg, 2 * n_live)
    tile = workloads.make_electrons("uniform_c0", n_live)
    for k, col in zip(("r", "z", "theta", "ux", "uy", "uz", "w"), range(7)):
        tile[k][:] = live[:, col]
    tile["id"][:] = live[:, 7].astype(np.int64)
    tile["cpu"][:] = live[:, 8].astype(np.int32)
    workloads.capture_prev(tile)
    (ctx.stage_electrons if species == 0 else ctx.stage_positrons)(tile)
    cand = np.zeros(len(cand_in), dtype=gpu.SECONDARY_DTYPE)
    cand["species"] = species
    for k, col in zip(("x", "y", "z", "dir_x", "dir_y", "dir_z", "energy_eV", "weight"), range(8)):
        cand[k] = cand_in[:, col]
    cand["root_key"] = (cand_in[:, 8].astype(np.uint64) << np.uint64(32)) | cand_in[:, 9].astype(np.uint64)
    cand["lineage"] = cand_in[:, 10].astype(np.uint64)
    cand["root_species"] = cand_in[:, 11].astype(np.int32)
    before = cand.copy()
    stats = ctx.population_thin(species, int(plan[7]), int(step), int(salt), candidates=cand)
    assert stats["members"] == plan[0] and stats["live"] == plan[1] and stats["candidates"] == plan[2]
    assert stats["supports"] == plan[3] and stats["capacity"] == plan[4]
    assert stats["requested"] == plan[5] and stats["removed"] == plan[6]
    got = _fetch(ctx, workloads, species)
    ctx.close()
    got_w = np.concatenate([got["w"], cand["weight"]])
    np.testing.assert_array_equal(got_w == 0.0, want_w == 0.0)
    np.testing.assert_allclose(got_w, want_w, rtol=1e-12, atol=0)
    np.testing.assert_array_equal(got["id"] < 0, want_w[:n_live] == 0.0)
    assert (want_w == 0.0).sum() >= plan[6]
    # the CIC charge of every cell is kept
    r = np.concatenate([live[:, 0], np.hypot(before["x"], before["y"])])
    z = np.concatenate([live[:, 1], before["z"]])
    w0 = np.concatenate([live[:, 6], before["weight"]])
    q0 = oracle.deposit_charge_cic(int(nr), int(nz), dr, dz, r_lo, z_lo, r, z, w0)
    q1 = oracle.deposit_charge_cic(int(nr), int(nz), dr, dz, r_lo, z_lo, r, z, got_w)
    np.testing.assert_allclose(q1, q0, rtol=0, atol=1e-12 * np.abs(q0).max())


def test_nothing_happens_inside_the_band(mods):
    gpu, workloads, oracle = mods
    cfg = gpu.default_config(r_hi=10.0, z_hi=24.0, nr=10, nz=12, rng_seed=1)
    ctx = gpu.RreaGpuContext(cfg, 4096)
    tile = workloads.make_electrons("uniform_c0", 1000)
    rng = np.random.default_rng(3)
    tile["r"][:] = rng.uniform(0, 10, 1000)
    tile["z"][:] = rng.uniform(0, 24, 1000)
    workloads.capture_prev(tile)
    ctx.stage_electrons(tile)
    stats = ctx.population_thin(0, 800, 1)           # 1000 <= 800 * 1.25: no thinning
    assert stats["requested"] == 0 and stats["removed"] == 0 and stats["members"] == 1000
    assert ctx.population_split(0, 1500, 0.25) == 0  # 1000 >= 1500 / 2: no split
    got = _fetch(ctx, workloads, 0)
    np.testing.assert_array_equal(got["w"], tile["w"])
    ctx.close()


def test_split_refill_halves_and_clones_in_order(mods):
    gpu, workloads, oracle = mods
    cfg = gpu.default_config(r_hi=10.0, z_hi=24.0, nr=10, nz=12, rng_seed=1)
    ctx = gpu.RreaGpuContext(cfg, 2048)
    n = 1000
    tile = workloads.make_electrons("uniform_c0", n)
    rng = np.random.default_rng(4)
    tile["r"][:] = rng.uniform(0, 10, n)
    tile["z"][:] = rng.uniform(0, 24, n)
    tile["w"][:] = rng.uniform(0.5, 3.0, n)
    tile["id"][::10] *= -1                            # invalid particles neither split nor count
    tile["cpu"][:] = 3
    workloads.capture_prev(tile)
    ctx.stage_electrons(tile)
    floor = 0.75
    added = ctx.population_split(0, 2 * n + 10, floor)
    split = (tile["id"] > 0) & (tile["w"] >= 2 * floor)
    assert added == int(split.sum()) > 0
    got = _fetch(ctx, workloads, 0)
    assert len(got["id"]) == n + added
    np.testing.assert_array_equal(got["w"][:n], np.where(split, 0.5 * tile["w"], tile["w"]))
    clones = slice(n, n + added)
    for k in ("r", "z", "theta", "ux", "uy", "uz"):
        np.testing.assert_array_equal(got[k][clones], tile[k][split])
    np.testing.assert_array_equal(got["w"][clones], 0.5 * tile["w"][split])
    np.testing.assert_array_equal(got["id"][clones], n + 1 + np.arange(added))
    np.testing.assert_array_equal(got["cpu"][clones], 3)
    assert got["w"][got["id"] > 0].sum() == pytest.approx(tile["w"][tile["id"] > 0].sum(), rel=1e-15)
    with pytest.raises(gpu.RreaGpuError):
        ctx.population_split(0, 10 * n, 0.01)         # more clones than the tile can hold
    ctx.close()


def test_population_control_holds_an_avalanche_near_its_target(mods):
    """The resident loop with adaptive_resample_v1: the uniform-field case
    (2000 seeds, 1500 steps; unchecked it grows past 60,000 e-) with a
    20,000-macro target.  After every controlled step the live electrons stay
    at or below 1.25 x target, and the electron weight stays that of an
    uncontrolled run of the same seeds within 10 % (thinning keeps every
    weight's expectation)."""
    gpu, workloads, oracle = mods
    from conftest import TABLES
    from rrea_feedback_warpx_amrex_geant4_gb300 import avalanche
    runs = {}
    for target in (None, 20_000):
        ctx = avalanche.make_context("uniform_c0", 1 << 20, 5, tables=TABLES)
        run = avalanche.AvalancheRun(ctx, workloads.make_electrons("uniform_c0", 2000), population_target=target)
        res = run.run(1500, census_every=100)
        ctx.close()
        runs[target] = res
    free, held = runs[None], runs[20_000]
    assert free["history"][-1]["electron_count"] > 60_000
    assert held["population_thinned"] > 0
    for row in held["history"]:
        assert row["electron_count"] <= 25_000
    w_free = free["history"][-1]["electron_weight"]
    w_held = held["history"][-1]["electron_weight"]
    assert abs(w_held - w_free) <= 0.1 * w_free, (w_held, w_free)
