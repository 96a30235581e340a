"""GPU positron phase vs the oracle on identical tiles, through the C-ABI
drop-in entry point rrea_gpu_apply_positrons.

Tolerances: dispositions, substep and hazard-draw counts, validity and
secondary keys bit-exact; FP64 state within 1e-12 relative (positions with
a 1e-12 x domain floor) but at most 0.1 % of the entries, within 1e-11;
secondary
energies and directions within 1e-12 of the parent's total energy scale (K + 2 m c^2: the in-flight annihilation
photon direction is a momentum difference at that scale); atomically
accumulated cell sources within 1.6e-11 of each grid's largest cell."""
import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu

ME_C2 = 510998.95


@pytest.fixture(scope="module")
def mods():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu, workloads
    from oracle import compare, oracle
    build.build()
    oracle.load_tables(TABLES)
    return gpu, workloads, oracle, compare


def _ctx(gpu, workloads, case, n):
    cfg = workloads.make_config(gpu, case)
    ctx = gpu.RreaGpuContext(cfg, n)
    ctx.load_tables(TABLES)
    field = workloads.make_field(case)
    ctx.set_field(**field)
    return cfg, ctx, field


def _positrons(workloads, case, n, seed, k_lo=None, k_hi=None):
    arr = workloads.make_electrons(case, n, seed=seed)
    if k_lo is not None:
        k = np.exp(np.random.default_rng(seed + 1).uniform(np.log(k_lo), np.log(k_hi), n))
        u = workloads.proper_velocity(k)
        norm = np.sqrt(arr["ux"] ** 2 + arr["uy"] ** 2 + arr["uz"] ** 2)
        for f in ("ux", "uy", "uz"):
            arr[f] *= u / norm
            arr["prev_" + f][:] = arr[f]
    return arr


def _total_energy(workloads, arr):
    return workloads.kinetic_energy(arr["prev_ux"], arr["prev_uy"], arr["prev_uz"]) + 2.0 * ME_C2


def _check(cfg, compare, g, o, e0):
    problems = compare.compare(cfg, g, o, max(cfg.r_hi, cfg.z_hi), parent_energy=e0)
    assert not problems, "; ".join(problems)


@pytest.mark.parametrize("case,n,steps,dt_s,k_lo,k_hi", [
    ("scaleup_c1", 2048, 2, 5.0e-10, None, None),      # the case's 1-20 MeV seed distribution
    ("uniform_c0", 512, 3, 5.0e-10, None, None),       # 7.2 MeV along +z
    ("scaleup_c1", 2048, 2, 2.0e-8, 1.2e4, 3.0e5),     # slow positrons: stops and at-rest annihilation
])
def test_positron_step_parity(mods, case, n, steps, dt_s, k_lo, k_hi):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, case, n)
    arr = _positrons(workloads, case, n, 7, k_lo, k_hi)
    for step in range(steps):
        e0 = _total_energy(workloads, arr)
        g, o = compare.run_pair(ctx, cfg, field, arr, step, dt_s, species="positron")
        _check(cfg, compare, g, o, e0)
        arr = o[0]
        workloads.capture_prev(arr)
    ctx.close()


def test_positron_processes_covered(mods):
    """Bhabha, brems and annihilation (in flight and at rest) all occur."""
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, "scaleup_c1", 8192)
    arr = _positrons(workloads, "scaleup_c1", 8192, 19, 1.2e4, 2.0e7)
    e0 = _total_energy(workloads, arr)
    g, o = compare.run_pair(ctx, cfg, field, arr, 1, 1.0e-8, species="positron")
    _check(cfg, compare, g, o, e0)
    procs = set(np.unique(g[1]["process"]).tolist())
    assert {3, 4, 9} <= procs, procs
    assert (g[1]["root_species"] == 1).all()
    assert (g[4] == 2).sum() > 100
    ctx.close()


def test_below_cutoff_positrons_annihilate_at_rest(mods):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, "uniform_c0", 32)
    arr = _positrons(workloads, "uniform_c0", 32, 3, 2.0e3, 9.0e3)
    arr["z"][:] = arr["prev_z"][:] = 100.0
    e0 = _total_energy(workloads, arr)
    g, o = compare.run_pair(ctx, cfg, field, arr, 0, 5.0e-10, species="positron")
    _check(cfg, compare, g, o, e0)
    assert (g[4] == 2).all()
    sec = g[1]
    assert len(sec) == 64 and (sec["species"] == 2).all() and (sec["process"] == 9).all()
    np.testing.assert_array_equal(sec["energy_eV"], np.full(64, ME_C2))
    assert g[5][1].sum() > 0.0  # the annihilated target electron leaves a positive ion
    ctx.close()


def test_resident_positrons_match_apply_mode(mods):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, "scaleup_c1", 4096)
    arr = _positrons(workloads, "scaleup_c1", 4096, 11)
    a = workloads.copy_tile(arr)
    n_apply = len(ctx.apply_positrons(a, 5, 5.0e-10))
    b = workloads.copy_tile(arr)
    ctx.stage_positrons(b)
    n_res = ctx.step_positrons_resident(5, 5.0e-10)
    ctx.fetch_positrons(b)
    assert n_apply == n_res
    for f in ("r", "z", "theta", "ux", "uy", "uz", "id"):
        np.testing.assert_array_equal(a[f], b[f])
    ctx.close()


def test_positron_escape_through_upper_face(mods):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, "uniform_c0", 32)
    arr = _positrons(workloads, "uniform_c0", 32, 3)
    arr["z"][:] = arr["prev_z"][:] = 500.0 - 0.01
    e0 = _total_energy(workloads, arr)
    g, o = compare.run_pair(ctx, cfg, field, arr, 0, 5.0e-10, species="positron")
    _check(cfg, compare, g, o, e0)
    assert (g[4] == 1).all()
    assert (g[0]["id"] < 0).all()
    ctx.close()
