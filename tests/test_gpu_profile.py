"""Transport through an altitude density profile
(rrea.air_density_model=altitude_profile): the GPU phases and the newborn
FIFO vs the oracle, both bound to the same profile through
rrea_gpu_set_density_profile / oracle.set_density_profile.

The profile is an exponential atmosphere with a +-20 % ripple on a 0.5 m
node spacing, so the midpoint ratio of every material piece differs from
its neighbours' and from the uniform ratio.  The oracle's profile
interpolation is pinned bit-exact to the reference's RreaAltitudeProfile
(tests/test_oracle_golden.py).

Tolerances as in the uniform-density phase tests: discrete outcomes
bit-exact, FP64 state within 1e-12 but at most 0.1 % of the entries, within
1e-11."""
import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu

ALT0 = 6000.0
REF = 1.20479  # the tables' reference density (kg/m^3)
KEYS = ("species", "process", "root_species", "parent_index", "root_key", "lineage")


def _profile(lo=5900.0, hi=8100.0):
    alt = np.arange(lo, hi + 0.25, 0.5)
    dens = 1.225 * np.exp(-alt / 7200.0) * (1.0 + 0.2 * np.sin(alt / 3.7))
    return alt, dens


@pytest.fixture(scope="module")
def mods():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu, workloads
    from oracle import compare, oracle
    build.build()
    oracle.load_tables(TABLES)
    yield gpu, workloads, oracle, compare
    oracle.set_density_profile()


def _setup(gpu, workloads, oracle, case, capacity, profile=None, periodic=False):
    cfg = workloads.make_config(gpu, case)
    cfg.periodic_z = 1 if periodic else 0
    ctx = gpu.RreaGpuContext(cfg, capacity)
    ctx.load_tables(TABLES)
    field = workloads.make_field(case)
    ctx.set_field(**field)
    alt, dens = profile if profile is not None else _profile()
    ctx.set_density_profile(alt, dens, ALT0, REF)
    oracle.set_density_profile(alt, dens, ALT0, REF)
    return cfg, ctx, field


def _check(compare, cfg, g, o, e0=None):
    problems = compare.compare(cfg, g, o, max(cfg.r_hi, cfg.z_hi), parent_energy=e0)
    assert not problems, "; ".join(problems)


@pytest.mark.parametrize("case,n,dt_s,periodic", [
    ("scaleup_c1", 2048, 5.0e-10, False),
    ("scaleup_c1", 1024, 1.0e-7, False),   # 30 m chords through the ripple
    ("uniform_c0", 1024, 3.0e-8, True),    # periodic z: wrapped pieces, each with its own midpoint
])
def test_electrons_through_profile_match_oracle(mods, case, n, dt_s, periodic):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _setup(gpu, workloads, oracle, case, 4 * n, periodic=periodic)
    arr = workloads.make_electrons(case, n, seed=71)
    g, o = compare.run_pair(ctx, cfg, field, arr, 1, dt_s)
    _check(compare, cfg, g, o)
    ctx.close()


def test_profile_changes_the_transport(mods):
    """The same tile with and without the profile gives different energy
    loss: the profile is really used."""
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _setup(gpu, workloads, oracle, "scaleup_c1", 4096)
    arr = workloads.make_electrons("scaleup_c1", 1024, seed=72)
    a = workloads.copy_tile(arr)
    ctx.apply_electrons(a, 0, 1.0e-7)
    ctx.set_density_profile()
    b = workloads.copy_tile(arr)
    ctx.apply_electrons(b, 0, 1.0e-7)
    alive = (a["id"] > 0) & (b["id"] > 0)
    ka = workloads.kinetic_energy(a["ux"], a["uy"], a["uz"])[alive]
    kb = workloads.kinetic_energy(b["ux"], b["uy"], b["uz"])[alive]
    assert np.mean(np.abs(ka - kb) > 1e-6 * kb) > 0.5
    ctx.close()


def test_photons_and_positrons_through_profile_match_oracle(mods):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _setup(gpu, workloads, oracle, "scaleup_c1", 8192)
    pho = workloads.make_photons("scaleup_c1", 2048, 1.0e-7, seed=73, e_lo=5.0e4, e_hi=1.0e8)
    e0 = np.sqrt(pho["ux"] ** 2 + pho["uy"] ** 2 + pho["uz"] ** 2)
    g, o = compare.run_pair(ctx, cfg, field, pho, 2, 1.0e-7, species="photon")
    _check(compare, cfg, g, o, e0)
    pos = workloads.make_electrons("scaleup_c1", 1024, seed=74)
    e0 = workloads.kinetic_energy(pos["prev_ux"], pos["prev_uy"], pos["prev_uz"]) + 2.0 * 510998.95
    g, o = compare.run_pair(ctx, cfg, field, pos, 2, 1.0e-7, species="positron")
    _check(compare, cfg, g, o, e0)
    ctx.close()


def test_drain_through_profile_matches_oracle(mods):
    gpu, workloads, oracle, compare = mods
    case, n, dt_s, step = "scaleup_c1", 1024, 1.0e-7, 3
    cfg, ctx, field = _setup(gpu, workloads, oracle, case, 8192)
    oe = oracle.electron_step(cfg, field, step, dt_s, workloads.make_electrons(case, n, seed=75))
    og = oracle.photon_step(cfg, step, dt_s, workloads.make_photons(case, n, dt_s, seed=76, e_lo=5.0e4, e_hi=1.0e8))
    pending = np.concatenate([oe["secondaries"], og["secondaries"]])
    got = ctx.drain_secondaries(pending, step, dt_s)
    ref = oracle.drain(cfg, field, step, dt_s, pending)["survivors"]
    assert ctx.last_drain_stats()[0] > len(pending)
    assert len(got) == len(ref)
    for key in KEYS:
        np.testing.assert_array_equal(got[key], ref[key], err_msg=key)
    scale = max(cfg.r_hi, cfg.z_hi)
    for key in ("x", "y", "z"):
        ok, n_over = compare.entries_ok(got[key], ref[key], compare.RTOL * scale)
        assert ok, f"survivor {key}: {n_over}"
    ok, n_over = compare.entries_ok(got["energy_eV"], ref["energy_eV"], compare.RTOL * np.abs(ref["energy_eV"]))
    assert ok, f"survivor energy: {n_over}"
    ctx.close()


def test_query_outside_profile_fails_the_step(mods):
    """Particles below the profile's lowest altitude: both sides fail with
    RREA_GPU_ERR_RANGE (the reference throws from Interpolate)."""
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _setup(gpu, workloads, oracle, "scaleup_c1", 4096, profile=_profile(6900.0, 7100.0))
    arr = workloads.make_electrons("scaleup_c1", 256, seed=77)  # z in [0, 10] m: altitude about 6 km
    with pytest.raises(gpu.RreaGpuError) as e:
        ctx.apply_electrons(workloads.copy_tile(arr), 0, 5.0e-10)
    assert e.value.status == 4
    with pytest.raises(oracle.OracleFailure) as e:
        oracle.electron_step(cfg, field, 0, 5.0e-10, workloads.copy_tile(arr))
    assert e.value.code == 4
    ctx.close()


def test_set_density_profile_validates(mods):
    gpu, workloads, oracle, compare = mods
    cfg = workloads.make_config(gpu, "scaleup_c1")
    ctx = gpu.RreaGpuContext(cfg, 16)
    alt, dens = _profile()
    for a, d, ref, code in ((alt[:1], dens[:1], REF, 1),               # fewer than two rows
                            (alt[::-1], dens, REF, 1),                 # not increasing
                            (alt, -dens, REF, 1),                      # non-positive density
                            (alt, dens, 0.0, 1),                       # no reference density
                            (alt + 5000.0, dens, REF, 4)):             # domain centre outside
        with pytest.raises(gpu.RreaGpuError) as e:
            ctx.set_density_profile(a, d, ALT0, ref)
        assert e.value.status == code
    ctx.set_density_profile(alt, dens, ALT0, REF)
    ctx.set_density_profile()
    ctx.close()
