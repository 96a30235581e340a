"""The whole kinetic step through the drop-in C-ABI calls, in the overlay's
order (electron, photon and positron phases; DrainAndCommitSecondaries; the
Maxwell update from the step's net-chord current), for three steps in which
the device-resident field of one step drives the transport of the next: the
feedback loop of the overlay.

Both sides run in lockstep from identical inputs at every step: the oracle's
phase tiles (captured and photon-pushed as the overlay does), the oracle's
pending records with its drain survivors appended as new particles, and the
field the GPU left on the device (downloaded bit for bit for the oracle).

Tolerances as in the per-phase tests: each phase through the shared phase
comparison (discrete outcomes exact, FP64 state within 1e-12 but at most
0.1 % of the entries, within 1e-11); survivor keys
bit-exact; the net-chord current within 1e-12 of its largest entry (atomics
sum the signed index fluxes in nondeterministic order); the field
update within 1e-12 of each vector's largest entry given the GPU's current."""
import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu

CASE, N, DT_S, SUBSTEPS = "scaleup_c1", 4096, 5.0e-10, 2
ME_C2 = 510998.95
KEYS = ("species", "process", "root_species", "parent_index", "root_key", "lineage")


@pytest.fixture(scope="module")
def mods():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu, workloads
    from oracle import compare, oracle
    build.build()
    oracle.load_tables(TABLES)
    return gpu, workloads, oracle, compare


def _commit(workloads, tile, recs, photon):
    """Survivor records become particles of the tile (new ids after the
    tile's largest), their captured start equal to the current state."""
    if len(recs) == 0:
        return tile
    mag = recs["energy_eV"] if photon else workloads.proper_velocity(recs["energy_eV"])
    add = {"r": np.hypot(recs["x"], recs["y"]), "z": recs["z"], "theta": np.arctan2(recs["y"], recs["x"]),
           "ux": mag * recs["dir_x"], "uy": mag * recs["dir_y"], "uz": mag * recs["dir_z"], "w": recs["weight"],
           "id": np.abs(tile["id"]).max(initial=0) + 1 + np.arange(len(recs), dtype=np.int64),
           "cpu": np.zeros(len(recs), dtype=np.int32)}
    for k in ("r", "z", "theta", "ux", "uy", "uz"):
        add["prev_" + k] = add[k]
    return {k: np.ascontiguousarray(np.concatenate([tile[k], add[k]])) for k in tile}


def _parent_energy(workloads, species, tile):
    """Per-particle energy scale of the final-state arithmetic (eV); the
    electron phase is compared at the strict default, as in its own tests."""
    if species == "electron":
        return None
    if species == "photon":
        return np.sqrt(tile["ux"] ** 2 + tile["uy"] ** 2 + tile["uz"] ** 2)
    return workloads.kinetic_energy(tile["prev_ux"], tile["prev_uy"], tile["prev_uz"]) + 2.0 * ME_C2


def test_three_kinetic_steps_match_oracle(mods):
    gpu, workloads, oracle, compare = mods
    cfg = workloads.make_config(gpu, CASE)
    field = workloads.make_field(CASE)
    ctx = gpu.RreaGpuContext(cfg, 8 * N)
    ctx.load_tables(TABLES)
    ctx.set_field(**field)
    fld = {k: np.array(v, dtype=np.float64) for k, v in field.items()}
    dr, dz = (cfg.r_hi - cfg.r_lo) / cfg.nr, (cfg.z_hi - cfg.z_lo) / cfg.nz
    tiles = {"electron": workloads.make_electrons(CASE, N, seed=61),
             "photon": workloads.make_photons(CASE, N // 2, DT_S, seed=62, e_lo=5.0e4, e_hi=2.0e7),
             "positron": workloads.make_electrons(CASE, N // 16, seed=63)}
    survivors = 0
    for step in range(3):
        ctx.reset_current()
        results, pending = {}, []
        for species in ("electron", "photon", "positron"):
            # run_pair leaves the current alone: it accumulates over the phases
            g, o = compare.run_pair(ctx, cfg, fld, tiles[species], step, DT_S, species=species)
            e0 = _parent_energy(workloads, species, tiles[species])
            problems = compare.compare(cfg, g, o, max(cfg.r_hi, cfg.z_hi), parent_energy=e0)
            assert not problems, f"{species} step {step}: " + "; ".join(problems)
            results[species] = o[1]
            tiles[species] = o[0]
            pending.append(o[1]["secondaries"])
        pending = np.concatenate(pending)
        got = ctx.drain_secondaries(pending, step, DT_S)
        od = oracle.drain(cfg, fld, step, DT_S, pending)
        ref = od["survivors"]
        assert len(got) == len(ref), f"survivors step {step}"
        for key in KEYS:
            np.testing.assert_array_equal(got[key], ref[key], err_msg=f"survivor {key} step {step}")
        survivors += len(ref)
        # the step's net-chord current: phase chords and the newborns' residual legs
        rows = np.concatenate([oracle.segment_rows(r) for r in (results["electron"], results["positron"], od)])
        cur = oracle.deposit_segments(cfg, DT_S, rows)
        gi = ctx.current_index()
        for key in ("rho", "jr", "jz"):
            scale = max(np.abs(cur[key]).max(), 1e-300)
            np.testing.assert_allclose(gi[key], cur[key], rtol=0, atol=1e-12 * scale, err_msg=f"{key} step {step}")
        jr, jz = ctx.current()
        before = ctx.field()
        ctx.advance_field(DT_S, SUBSTEPS)
        after = ctx.field()
        expect = oracle.advance_maxwell(cfg.nr, cfg.nz, dr, dz, DT_S, SUBSTEPS, *before, jr.ravel(), jz.ravel())
        for name, g, o in zip(("er", "ez", "bt"), after, expect):
            scale = max(np.abs(o).max(), 1e-300)
            np.testing.assert_allclose(g, o, rtol=0, atol=1e-12 * scale, err_msg=f"{name} step {step}")
        # the device field (not uploaded again) drives the next step on both sides
        fld["er"], fld["ez"], fld["bt"] = (np.array(a, dtype=np.float64).ravel() for a in after)
        for species, code in (("electron", 0), ("positron", 1), ("photon", 2)):
            workloads.capture_prev(tiles[species])
            tiles[species] = _commit(workloads, tiles[species], ref[ref["species"] == code], species == "photon")
        workloads.push_photons(tiles["photon"], DT_S)
    assert survivors > 0, "no drain survivors: the workload does not exercise the commit"
    ctx.close()
