"""Transient FIFO of DrainAndCommitSecondaries on the GPU vs the oracle on the
same pending records, through the C-ABI entry points
rrea_gpu_drain_secondaries (host records) and rrea_gpu_drain_resident (the
queue filled by the resident phases).

The pending records are the oracle's own electron, photon and positron
phase secondaries of one step, concatenated in phase order, so both sides
start from bit-identical input.

Tolerances: survivor count, order and keys (species, process, root species,
parent index, root key, lineage) bit-exact; birth fraction exactly 1; FP64
payload within 1e-12 (positions with a 1e-12 x domain floor, energies
relative) but at most 0.1 % of the entries, within 1e-11; cell sources within
1.6e-11 and the net-chord current within 1e-12 of each grid's largest
entry (both summed with atomics in arbitrary order)."""
import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu

KEYS = ("species", "process", "root_species", "parent_index", "root_key", "lineage")


@pytest.fixture(scope="module")
def mods():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu, workloads
    from oracle import compare, oracle
    build.build()
    oracle.load_tables(TABLES)
    return gpu, workloads, oracle, compare


def _setup(gpu, workloads, case, capacity, periodic=False):
    cfg = workloads.make_config(gpu, case)
    cfg.periodic_z = 1 if periodic else 0
    ctx = gpu.RreaGpuContext(cfg, capacity)
    ctx.load_tables(TABLES)
    field = workloads.make_field(case)
    ctx.set_field(**field)
    return cfg, ctx, field


def _pending(workloads, oracle, cfg, field, case, n, step, dt_s):
    e = workloads.make_electrons(case, n, seed=3)
    oe = oracle.electron_step(cfg, field, step, dt_s, workloads.copy_tile(e))
    g = workloads.make_photons(case, n, dt_s, seed=4, e_lo=5.0e4, e_hi=1.0e8)
    og = oracle.photon_step(cfg, step, dt_s, workloads.copy_tile(g))
    p = workloads.make_electrons(case, n, seed=5)
    op = oracle.positron_step(cfg, field, step, dt_s, workloads.copy_tile(p))
    return np.concatenate([oe["secondaries"], og["secondaries"], op["secondaries"]])


def _compare_survivors(compare, cfg, got, ref):
    assert len(got) == len(ref), f"survivor count {len(got)} vs oracle {len(ref)}"
    for key in KEYS:
        bad = np.nonzero(got[key] != ref[key])[0]
        assert bad.size == 0, f"survivor {key} differs at {bad[:10].tolist()} ({bad.size})"
    assert (got["birth_fraction"] == 1.0).all()
    np.testing.assert_array_equal(got["weight"], ref["weight"])
    scale = max(cfg.r_hi, cfg.z_hi)
    for key, atol in (("x", compare.RTOL * scale), ("y", compare.RTOL * scale), ("z", compare.RTOL * scale),
                      ("dir_x", compare.RTOL), ("dir_y", compare.RTOL), ("dir_z", compare.RTOL),
                      ("energy_eV", compare.RTOL * np.abs(ref["energy_eV"]))):
        ok, n_over = compare.entries_ok(got[key], ref[key], atol)
        assert ok, f"survivor {key} differs for {n_over} (worst {compare._worst(got[key], ref[key], atol):.2e})"


def _compare_cells(compare, got, ref):
    for f in range(5):
        ok, n_over = compare.cells_ok(got[f], ref[f])
        assert ok, f"cell source field {f} differs in {n_over} cells"


def _compare_current(oracle, cfg, ctx, dt_s, o):
    ref = oracle.deposit_segments(cfg, dt_s, oracle.segment_rows(o))
    gi = ctx.current_index()
    for key in ("rho", "jr", "jz"):
        scale = max(np.abs(ref[key]).max(), 1e-300)
        np.testing.assert_allclose(gi[key], ref[key], rtol=0, atol=1e-12 * scale, err_msg=key)


@pytest.mark.parametrize("case,n,dt_s,capacity,periodic", [
    ("scaleup_c1", 1024, 1.0e-7, 4096, False),   # 30 m residual chords: Moller, brems, Compton, pair children
    ("uniform_c0", 1024, 3.0e-8, 4096, False),   # small domain: escapes through the faces
    ("uniform_c0", 1024, 3.0e-8, 257, False),    # FIFO advanced in 257-item chunks, buffers grown mid-drain
    ("uniform_c0", 512, 3.0e-8, 4096, True),     # periodic z: wrapped residual chords, no net-chord current
])
def test_drain_matches_oracle(mods, case, n, dt_s, capacity, periodic):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _setup(gpu, workloads, case, capacity, periodic)
    step = 3
    pending = _pending(workloads, oracle, cfg, field, case, n, step, dt_s)
    assert (pending["birth_fraction"] < 1.0).any()
    ctx.reset_sources()
    if not periodic:
        ctx.reset_current()
    got = ctx.drain_secondaries(pending, step, dt_s)
    items, n_surv = ctx.last_drain_stats()
    o = oracle.drain(cfg, field, step, dt_s, pending)
    assert items > len(pending), "no newborn children: the workload does not exercise the FIFO"
    assert n_surv == len(got)
    _compare_survivors(compare, cfg, got, o["survivors"])
    _compare_cells(compare, ctx.sources(), o["cells"])
    if not periodic:
        _compare_current(oracle, cfg, ctx, dt_s, o)
    ctx.close()


def test_drain_passes_settled_records_through(mods):
    """Records born at the end of the step (birth 1) are not transported:
    they survive unchanged, in FIFO order, ahead of any newborn children."""
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _setup(gpu, workloads, "uniform_c0", 1024)
    pending = _pending(workloads, oracle, cfg, field, "uniform_c0", 256, 0, 3.0e-8)
    pending["birth_fraction"][::2] = 1.0
    got = ctx.drain_secondaries(pending, 0, 3.0e-8)
    o = oracle.drain(cfg, field, 0, 3.0e-8, pending)
    _compare_survivors(compare, cfg, got, o["survivors"])
    # (root key, root species, lineage) names a record uniquely
    where = {(int(r["root_key"]), int(r["root_species"]), int(r["lineage"])): i for i, r in enumerate(got)}
    last = -1
    for rec in pending[::2]:
        i = where[(int(rec["root_key"]), int(rec["root_species"]), int(rec["lineage"]))]
        assert i > last, "settled records left FIFO order"
        last = i
        for key in KEYS + ("x", "y", "z", "dir_x", "dir_y", "dir_z", "energy_eV", "weight", "birth_fraction"):
            assert got[i][key] == rec[key], key
    ctx.close()


def test_drain_rejects_invalid_birth_payload(mods):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _setup(gpu, workloads, "uniform_c0", 64)
    pending = _pending(workloads, oracle, cfg, field, "uniform_c0", 64, 0, 3.0e-8)
    for field_name, value in (("weight", 0.0), ("birth_fraction", 1.5), ("species", 7), ("x", np.nan)):
        bad = pending.copy()
        bad[field_name][0] = value
        with pytest.raises(gpu.RreaGpuError) as err:
            ctx.drain_secondaries(bad, 0, 3.0e-8)
        assert err.value.status == 1  # RREA_GPU_ERR_ARGUMENT
        with pytest.raises(oracle.OracleFailure):
            oracle.drain(cfg, field, 0, 3.0e-8, bad)
    assert len(ctx.drain_secondaries(pending[:0], 0, 3.0e-8)) == 0
    ctx.close()


def test_resident_queue_drain_matches_oracle(mods):
    """The resident electron phase queues its ordered secondaries on the
    device; drain_resident consumes that queue."""
    gpu, workloads, oracle, compare = mods
    case, n, dt_s, step = "scaleup_c1", 2048, 1.0e-7, 2
    # 30 m chords make several secondaries per electron: room for 2 x 8192 + 4096
    cfg, ctx, field = _setup(gpu, workloads, case, 4 * n)
    arr = workloads.make_electrons(case, n, seed=9)
    o_phase = oracle.electron_step(cfg, field, step, dt_s, workloads.copy_tile(arr))
    ctx.stage_electrons(workloads.copy_tile(arr))
    n_sec = ctx.step_electrons_resident(step, dt_s)
    assert n_sec == len(o_phase["secondaries"]) and ctx.pending_secondaries() == n_sec
    ctx.reset_sources()
    ctx.reset_current()
    n_surv = ctx.drain_resident(step, dt_s)
    assert ctx.pending_secondaries() == 0
    got = ctx.fetch_survivors()
    assert len(got) == n_surv
    o = oracle.drain(cfg, field, step, dt_s, o_phase["secondaries"])
    _compare_survivors(compare, cfg, got, o["survivors"])
    _compare_cells(compare, ctx.sources(), o["cells"])
    ctx.close()
