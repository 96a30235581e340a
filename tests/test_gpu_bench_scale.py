"""One whole bench step at the benchmarked population, against the oracle.

The populations are bench.py's own (2^21 electrons from the scale-up seed
distribution, 2^20 photons, 2^17 positrons; 256 x 2048 cells over
200 m x 2 km; E_z = -500 kV/m; dt = 0.5 ns), and the step is the bench's
resident step: the three phases, the transient FIFO, the survivor commit,
the compaction of ended particles and the Maxwell update from the step's
net-chord current.  The oracle runs the same step on the same staged tiles.

Exact: tile sizes, ids and their order after commit and compaction (so
every disposition, secondary count and FIFO survivor agreed), weights.
FP64 state: within 1e-12 relative (positions: of the domain size) but at
most 0.1 % of the entries, within 1e-11 (oracle/compare.py).  Field after the update: within 1e-12 of each vector's largest
entry."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT, TABLES

pytestmark = pytest.mark.gpu

NAMES = {0: "electrons", 1: "positrons", 2: "photons"}


@pytest.fixture(scope="module")
def mods():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu, workloads
    from oracle import avalanche as oav, compare, oracle
    build.build()
    oracle.load_tables(TABLES)
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench
    return gpu, workloads, oracle, oav, compare, bench


def _fetch(ctx, workloads, species):
    n = ctx.resident_count(species)
    t = {k: np.ascontiguousarray(v[:n]) for k, v in workloads.make_electrons("uniform_c0", max(n, 1)).items()}
    getattr(ctx, "fetch_" + NAMES[species])(t)
    return t


def test_one_bench_step_matches_oracle(mods):
    gpu, workloads, oracle, oav, compare, bench = mods
    n = int(os.environ.get("RREA_BENCH_SCALE_POPULATION", 1 << 21))
    cfg = workloads.make_config(gpu, bench.CASE)
    field = workloads.make_field(bench.CASE)
    ctx = gpu.RreaGpuContext(cfg, n + n // 4)
    ctx.load_tables(TABLES)
    ctx.set_field(**field)
    ctx.set_launch(128, 16, diagnostics=False)
    e, g, p = bench.gpu_arm_populations(n)
    ctx.stage_electrons(e)
    ctx.stage_photons(g)
    ctx.stage_positrons(p)
    # GPU: the bench's resident step
    ctx.reset_current()
    ctx.step_electrons_resident(0, bench.DT_S)
    ctx.step_photons_resident(0, bench.DT_S)
    ctx.step_positrons_resident(0, bench.DT_S)
    ctx.drain_resident(0, bench.DT_S)
    ctx.commit_survivors_resident()
    for s in NAMES:
        ctx.compact_resident(s)
    ctx.advance_field(bench.DT_S, bench.FIELD_SUBSTEPS)
    got = {s: _fetch(ctx, workloads, s) for s in NAMES}
    field_after = ctx.field()
    ctx.close()
    # oracle: the same step from the same tiles
    ocfg = workloads.make_config(oracle, bench.CASE)
    run = oav.AvalancheRun(ocfg, field, e, photons=g, positrons=p, feedback=True,
                           field_substeps=bench.FIELD_SUBSTEPS)
    moved = run.advance(bench.DT_S)
    assert moved == n + len(g["id"]) + len(p["id"])
    scale = max(cfg.r_hi, cfg.z_hi)
    report = []
    for s in NAMES:
        want = run.tiles[s]
        have = got[s]
        assert len(have["id"]) == len(want["id"]), f"{NAMES[s]} tile size"
        np.testing.assert_array_equal(have["id"], want["id"], err_msg=f"{NAMES[s]} ids")
        np.testing.assert_array_equal(have["w"], want["w"], err_msg=f"{NAMES[s]} weights")
        umag = np.sqrt(want["ux"] ** 2 + want["uy"] ** 2 + want["uz"] ** 2)
        for f in ("r", "z", "ux", "uy", "uz"):
            atol = compare.RTOL * (scale if f in ("r", "z") else umag)
            ok, n_over = compare.entries_ok(have[f], want[f], atol)
            report.append(f"{NAMES[s]}.{f}: {n_over} of {len(want[f])} above 1e-12")
            assert ok, f"{NAMES[s]} {f}: {n_over} outside the tolerance"
    print("; ".join(report))
    for name, a, b in zip(("er", "ez", "bt"), field_after, (run.field["er"], run.field["ez"], run.field["bt"])):
        big = max(np.abs(b).max(), 1e-300)
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-12 * big, err_msg=name)
