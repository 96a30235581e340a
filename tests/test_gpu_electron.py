"""GPU electron phase vs the oracle on identical inputs (tiles shaped like
the reference CPU case and the scale-up case), through the C-ABI drop-in
entry point.

Tolerances: dispositions, substep counts, hazard-draw counts, validity and
secondary keys bit-exact; FP64 state within 1e-12 relative (positions with
a 1e-12 x domain floor) but at most 0.1 % of the entries, within 1e-11;
atomically accumulated cell sources within 1.6e-11 of each grid's largest
cell."""
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


@pytest.mark.parametrize("case,n,steps", [("uniform_c0", 512, 3), ("scaleup_c1", 2048, 2)])
def test_electron_step_parity(mods, case, n, steps):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, case, n)
    arr = workloads.make_electrons(case, n, seed=7)
    scale = max(cfg.r_hi, cfg.z_hi)
    for step in range(steps):
        g, o = compare.run_pair(ctx, cfg, field, arr, step, 5.0e-10)
        problems = compare.compare(cfg, g, o, scale)
        assert not problems, f"step {step}: " + "; ".join(problems)
        # next step starts from the oracle's state (no error accumulation)
        arr = o[0]
        workloads.capture_prev(arr)
    ctx.close()


def test_resident_mode_matches_apply_mode(mods):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, "scaleup_c1", 4096)
    arr = workloads.make_electrons("scaleup_c1", 4096, seed=11)
    a = workloads.copy_tile(arr)
    n_apply = len(ctx.apply_electrons(a, 5, 5.0e-10))
    b = workloads.copy_tile(arr)
    ctx.stage_electrons(b)
    n_res = ctx.step_electrons_resident(5, 5.0e-10)
    ctx.fetch_electrons(b)
    assert n_apply == n_res
    for f in ("r", "z", "theta", "ux", "uy", "uz", "id"):
        np.testing.assert_array_equal(a[f], b[f])
    ctx.close()


def test_zero_weight_and_invalid_particles(mods):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, "uniform_c0", 64)
    arr = workloads.make_electrons("uniform_c0", 64, seed=3)
    arr["w"][::4] = 0.0
    arr["id"][1::8] *= -1
    g, o = compare.run_pair(ctx, cfg, field, arr, 0, 5.0e-10)
    assert not compare.compare(cfg, g, o, 500.0)
    assert (g[4][::4][arr["id"][::4] > 0] == 3).all()
    ctx.close()


def test_below_cutoff_electrons_demote(mods):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, "uniform_c0", 32)
    arr = workloads.make_electrons("uniform_c0", 32, seed=3)
    k = np.full(32, 5.0e3)
    u = workloads.proper_velocity(k)
    for f in ("uz", "prev_uz"):
        arr[f][:] = u
    arr["z"][:] = arr["prev_z"][:] = 100.0
    g, o = compare.run_pair(ctx, cfg, field, arr, 0, 5.0e-10)
    assert not compare.compare(cfg, g, o, 500.0)
    assert (g[4] == 2).all()
    cells = g[5]
    assert cells[0].sum() > 0.0  # low-energy electron sources were booked
    ctx.close()


def test_escape_through_upper_face(mods):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, "uniform_c0", 32)
    arr = workloads.make_electrons("uniform_c0", 32, seed=3)
    arr["z"][:] = arr["prev_z"][:] = 500.0 - 0.01
    g, o = compare.run_pair(ctx, cfg, field, arr, 0, 5.0e-10)
    assert not compare.compare(cfg, g, o, 500.0)
    assert (g[4] == 1).all()
    assert (g[0]["id"] < 0).all()
    ctx.close()


def test_out_of_domain_state_fails_closed(mods):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, "uniform_c0", 8)
    arr = workloads.make_electrons("uniform_c0", 8, seed=3)
    arr["prev_r"][3] = 60.0
    with pytest.raises(gpu.RreaGpuError) as e:
        ctx.apply_electrons(arr, 0, 5.0e-10)
    assert e.value.status == 5
    with pytest.raises(oracle.OracleFailure):
        oracle.electron_step(cfg, field, 0, 5.0e-10, workloads.copy_tile(arr))
    # the context stays usable after a failed step
    ok = workloads.make_electrons("uniform_c0", 8, seed=4)
    ctx.apply_electrons(ok, 0, 5.0e-10)
    ctx.close()


def test_count_live_matches_fetched_tile(mods):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, "uniform_c0", 2048)
    arr = workloads.make_electrons("uniform_c0", 2048, seed=9)
    arr["id"][::7] *= -1
    arr["z"][:100] = arr["prev_z"][:100] = 500.0 - 0.01   # these escape
    ctx.stage_electrons(arr)
    assert ctx.count_live(gpu.SPECIES_ELECTRON) == int((arr["id"] > 0).sum())
    ctx.step_electrons_resident(0, 5.0e-10)
    ctx.fetch_electrons(arr)
    assert ctx.count_live(gpu.SPECIES_ELECTRON) == int((arr["id"] > 0).sum())
    fits, projected = gpu.population_projection(ctx.count_live(gpu.SPECIES_ELECTRON), 0, 10, 2048)
    assert fits and projected == int((arr["id"] > 0).sum()) + 10
    ctx.close()


def test_table_driven_log_accuracy(mods):
    """The device's table-driven logarithm (Tang's method) against the
    correctly rounded host log: within 2 ulps over normal positive doubles
    from 1e-300 to 1e300, around 1, and at the table points; special inputs
    go to the CUDA log."""
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, "uniform_c0", 16)
    rng = np.random.default_rng(2)
    x = np.concatenate([
        10.0 ** rng.uniform(-300, 300, 400000),
        1.0 + rng.uniform(-1e-3, 1e-3, 200000),
        1.0 + rng.uniform(-1e-12, 1e-12, 50000),
        np.nextafter(1.0, 0.0) - np.arange(1000) * 2.0 ** -53,
        1.0 + np.arange(257) / 256.0,
        (1.0 + np.arange(257) / 256.0) * 2.0 ** rng.integers(-60, 60, 257),
        rng.uniform(1e3, 1e10, 200000),
        rng.uniform(0.0, 1.0, 200000),
    ])
    x = x[(x > 0.0) & np.isfinite(x) & (x >= np.finfo(np.float64).tiny)]
    fast, libm = ctx.selftest_math(0, x)
    ref = np.log(x.astype(np.longdouble))  # extended or quad precision

    def ulps(a):
        d = np.abs(a.astype(np.longdouble) - ref)
        return (d / np.spacing(np.abs(ref.astype(np.float64)))).astype(np.float64)

    assert ulps(fast).max() <= 2.0, ulps(fast).max()
    assert ulps(libm).max() <= 1.5
    special = np.array([0.0, -1.0, np.inf, np.nan, 5e-324, 1e-310])
    f2, l2 = ctx.selftest_math(0, special)
    np.testing.assert_array_equal(np.isnan(f2), np.isnan(l2))
    np.testing.assert_array_equal(f2[~np.isnan(f2)], l2[~np.isnan(l2)])
    ctx.close()


def test_table_driven_exp_accuracy(mods):
    """The device's table-driven exponential (Tang's method) against the
    correctly rounded host exp: within 2 ulps over |x| < 700, small
    arguments and the table points; larger and special arguments go to the
    CUDA exp."""
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, "uniform_c0", 16)
    rng = np.random.default_rng(3)
    ln2 = np.log(2.0)
    x = np.concatenate([
        rng.uniform(-699.0, 699.0, 400000),
        rng.uniform(-1e-3, 1e-3, 200000),
        rng.uniform(-1e-12, 1e-12, 50000),
        np.arange(-128 * 20, 128 * 20) * ln2 / 128.0,
        rng.uniform(-50.0, 5.0, 200000),
    ])
    fast, libm = ctx.selftest_math(1, x)
    ref = np.exp(x.astype(np.longdouble))

    def ulps(a):
        d = np.abs(a.astype(np.longdouble) - ref)
        return (d / np.spacing(np.abs(ref.astype(np.float64)))).astype(np.float64)

    assert ulps(fast).max() <= 2.0, ulps(fast).max()
    assert ulps(libm).max() <= 1.5
    special = np.array([700.0, -700.0, 710.0, -746.0, np.inf, -np.inf, np.nan])
    f2, l2 = ctx.selftest_math(1, special)
    np.testing.assert_array_equal(np.isnan(f2), np.isnan(l2))
    np.testing.assert_array_equal(f2[~np.isnan(f2)], l2[~np.isnan(l2)])
    ctx.close()


def test_chunked_drop_in_call_matches_resident_launch(mods):
    """A drop-in call on a tile of 2^18 or more particles uploads it in
    chunks whose kernels overlap the upload; its results equal one launch
    over the staged tile: the same state bit for bit, the same ordered
    secondaries and diagnostics."""
    gpu, workloads, oracle, compare = mods
    n = (1 << 18) + 4099
    cfg, ctx, field = _ctx(gpu, workloads, "scaleup_c1", n)
    arr = workloads.make_electrons("scaleup_c1", n, seed=21)
    arr["w"][::97] = 0.0
    arr["id"][5::113] *= -1
    a = workloads.copy_tile(arr)
    sec_a = ctx.apply_electrons(a, 4, 5.0e-10)
    diag_a = ctx.diagnostics(n)
    b = workloads.copy_tile(arr)
    ctx.stage_electrons(b)
    n_b = ctx.step_electrons_resident(4, 5.0e-10)
    diag_b = ctx.diagnostics(n)
    ctx.fetch_electrons(b)
    assert len(sec_a) == n_b > 0
    for f in ("r", "z", "theta", "ux", "uy", "uz", "id"):
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)
    for x, y in zip(diag_a, diag_b):
        np.testing.assert_array_equal(x, y)
    ctx.pending_secondaries(discard=True)
    ctx.close()


def test_chunked_drop_in_positrons_match_oracle(mods):
    """The chunked drop-in call of the positron phase (2^18 + 777 e+) against
    the oracle, parent indices of the secondaries included."""
    gpu, workloads, oracle, compare = mods
    n = (1 << 18) + 777
    cfg, ctx, field = _ctx(gpu, workloads, "scaleup_c1", n)
    arr = workloads.make_electrons("scaleup_c1", n, seed=31)
    g, o = compare.run_pair(ctx, cfg, field, arr, 2, 5.0e-10, species="positron")
    # annihilation photons share the parent's total energy (kinetic + 2 m c^2)
    e0 = workloads.kinetic_energy(arr["prev_ux"], arr["prev_uy"], arr["prev_uz"]) + 2.0 * 510998.95
    problems = compare.compare(cfg, g, o, max(cfg.r_hi, cfg.z_hi), parent_energy=e0)
    assert not problems, "; ".join(problems)
    assert len(o[1]["secondaries"]) > 0 and o[1]["secondaries"]["parent_index"].max() >= (1 << 18)
    ctx.close()
