"""GPU photon phase vs the oracle on identical photon tiles, through the
C-ABI drop-in entry point rrea_gpu_apply_photons.

Tolerances: dispositions, hazard-draw counts, validity and secondary keys
(species, process, parent, lineage, root key) bit-exact; FP64 state within
1e-12 relative (positions with a 1e-12 x domain floor) but at most 0.1 %
of the entries, within 1e-11; secondary energies
and directions within 1e-12 of the parent photon's energy scale (they are
differences of parent-scale quantities); atomically accumulated cell
sources within 1.6e-11 of each grid's largest cell."""
import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu


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


def _energy(arr):
    return np.sqrt(arr["ux"] ** 2 + arr["uy"] ** 2 + arr["uz"] ** 2)


def _check(cfg, compare, g, o, e0):
    problems = compare.compare(cfg, g, o, max(cfg.r_hi, cfg.z_hi), parent_energy=e0)
    assert not problems, "; ".join(problems)


@pytest.mark.parametrize("case,n,dt_s,e_lo,e_hi", [
    ("scaleup_c1", 4096, 2.0e-7, 5.0e4, 1.0e9),     # 60 m chords: Compton, pair, photoelectric
    ("uniform_c0", 1024, 5.0e-8, 5.0e4, 1.0e8),     # 15 m chords in the small domain
    ("scaleup_c1", 2048, 1.0e-6, 5.0e4, 2.0e5),     # low energies: photoelectric-rich
])
def test_photon_step_parity(mods, case, n, dt_s, e_lo, e_hi):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, case, n)
    arr = workloads.make_photons(case, n, dt_s, seed=17, e_lo=e_lo, e_hi=e_hi)
    for step in range(2):
        e0 = _energy(arr)
        g, o = compare.run_pair(ctx, cfg, field, arr, step, dt_s, species="photon")
        _check(cfg, compare, g, o, e0)
        assert (o[1]["events"][arr["id"] > 0] >= 1).all()
        arr = o[0]
        workloads.capture_prev(arr)
        workloads.push_photons(arr, dt_s)
    ctx.close()


def test_photon_processes_covered(mods):
    """One tile with enough path length exercises every photon channel."""
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, "scaleup_c1", 8192)
    arr = workloads.make_photons("scaleup_c1", 8192, 1.0e-6, seed=23, e_lo=5.0e4, e_hi=1.0e10)
    e0 = _energy(arr)
    g, o = compare.run_pair(ctx, cfg, field, arr, 3, 1.0e-6, species="photon")
    _check(cfg, compare, g, o, e0)
    procs = set(np.unique(g[1]["process"]).tolist())
    assert {5, 6, 7, 8} <= procs, procs          # Compton, photoelectric, pair nuclear, pair triplet
    assert (g[1]["root_species"] == 2).all()
    assert set(np.unique(g[1]["species"]).tolist()) <= {0, 1, 2}
    disp = set(np.unique(g[4]).tolist())
    assert {0, 1, 2} <= disp, disp
    ctx.close()


def test_resident_photons_match_apply_mode(mods):
    """The resident step pushes each photon itself; the apply step takes the
    host-pushed end point.  Same discrete history, same state to rounding."""
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, "scaleup_c1", 4096)
    dt = 2.0e-7
    arr = workloads.make_photons("scaleup_c1", 4096, dt, seed=29)
    a = workloads.copy_tile(arr)
    sec_a = ctx.apply_photons(a, 4, dt)
    _, ev_a, disp_a = ctx.diagnostics(4096)
    b = workloads.copy_tile(arr)
    for f in ("r", "z", "theta"):
        b[f][:] = b["prev_" + f]
    ctx.stage_photons(b)
    n_res = ctx.step_photons_resident(4, dt)
    _, ev_b, disp_b = ctx.diagnostics(4096)
    ctx.fetch_photons(b)
    assert n_res == len(sec_a)
    np.testing.assert_array_equal(disp_a, disp_b)
    np.testing.assert_array_equal(ev_a, ev_b)
    np.testing.assert_array_equal(a["id"], b["id"])
    alive = (a["id"] > 0)
    for f in ("r", "z"):
        np.testing.assert_allclose(b[f][alive], a[f][alive], rtol=1e-12, atol=1e-12 * cfg.z_hi)
    for f in ("ux", "uy", "uz"):
        np.testing.assert_allclose(b[f], a[f], rtol=1e-12, atol=1e-12 * _energy(arr).max())
    ctx.close()


def test_below_cutoff_and_zero_weight_photons(mods):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, "uniform_c0", 64)
    arr = workloads.make_photons("uniform_c0", 64, 5.0e-8, seed=5)
    for f in ("ux", "uy", "uz"):
        arr[f][:32] *= 2.0e4 / _energy(arr)[:32]          # 20 keV < photon cutoff
    arr["w"][40:48] = 0.0
    arr["id"][60:] *= -1
    e0 = _energy(arr)
    g, o = compare.run_pair(ctx, cfg, field, arr, 0, 5.0e-8, species="photon")
    _check(cfg, compare, g, o, e0)
    assert (g[4][:32] == 2).all() and (g[0]["id"][:32] < 0).all()
    assert (g[4][40:48] == 2).all()
    assert (g[4][60:] == -1).all()
    assert g[5][4].sum() > 0.0          # local deposits booked as energy loss
    ctx.close()


def test_photon_escape_through_upper_face(mods):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, "uniform_c0", 32)
    arr = workloads.make_photons("uniform_c0", 32, 1.0e-8, seed=9, e_lo=1.0e6, e_hi=2.0e6)
    e = _energy(arr)
    arr["ux"][:] = 0.0
    arr["uy"][:] = 0.0
    arr["uz"][:] = e
    arr["prev_z"][:] = 500.0 - 0.5
    workloads.push_photons(arr, 1.0e-8)
    g, o = compare.run_pair(ctx, cfg, field, arr, 0, 1.0e-8, species="photon")
    _check(cfg, compare, g, o, e)
    escaped = g[4] == 1
    assert escaped.sum() >= 30
    assert (g[0]["id"][escaped] < 0).all()
    ctx.close()


def test_photon_out_of_domain_fails_closed(mods):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, "uniform_c0", 8)
    arr = workloads.make_photons("uniform_c0", 8, 5.0e-8, seed=3)
    arr["prev_r"][2] = 80.0
    with pytest.raises(gpu.RreaGpuError) as e:
        ctx.apply_photons(arr, 0, 5.0e-8)
    assert e.value.status == 5
    with pytest.raises(oracle.OracleFailure):
        oracle.photon_step(cfg, 0, 5.0e-8, workloads.copy_tile(arr))
    ok = workloads.make_photons("uniform_c0", 8, 5.0e-8, seed=4)
    ctx.apply_photons(ok, 0, 5.0e-8)
    ctx.close()
