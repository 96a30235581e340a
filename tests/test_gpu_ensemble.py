"""The batched ensemble (rrea_gpu_ensemble_*, ensemble.EnsembleRun) against
the same instances run one by one.

Instances: four uniform-field avalanches of the plain case's air, tables,
grid and 7.2 MeV seeds at 400, 550, 700 and 900 kV/m, 30-80 seeds, 25-60
steps of 0.5 ns; one of them under a 60-particle population target, so the
per-instance thinning runs.  Each instance alone is the same instance on a
context of its own (cpu = k).

  * every instance's tiles after 20 steps (all still running) are those of
    the instance alone, bit for bit: ids, cpu ordinals, positions, momenta,
    weights, in the same order;
  * each instance's census at its end (counts exactly, weight sums and
    spectra within 1e-12: the census sums with atomics) and its thinning
    totals match, the batched run thinning every instance in one plan per
    species (rrea_gpu_ensemble_population_thin_all) and the instance alone
    thinning its slice (rrea_gpu_ensemble_population_thin);
  * the autotuner's launch shapes and scheduling orders change no result."""
import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, ensemble, gpu, workloads
    build.build()
    return gpu, workloads, ensemble


def _instances(ensemble):
    I = ensemble.Instance
    return [I(4.0e5, 60, 40), I(5.5e5, 40, 25), I(7.0e5, 80, 60, target=60), I(9.0e5, 30, 50)]


def _tiles(run, gpu, workloads):
    ctx = run.ctx
    out = {}
    for sp, fetch in ((gpu.SPECIES_ELECTRON, ctx.fetch_electrons), (gpu.SPECIES_PHOTON, ctx.fetch_photons),
                      (gpu.SPECIES_POSITRON, ctx.fetch_positrons)):
        n = ctx.resident_count(sp)
        t = {k: np.ascontiguousarray(v[:n]) for k, v in workloads.make_electrons("uniform_c0", max(n, 1)).items()}
        fetch(t)
        out[sp] = t
    return out


def _instance_rows(tile, k):
    sel = (tile["cpu"] == k) & (tile["id"] > 0)
    return {key: v[sel] for key, v in tile.items()}


def test_instances_evolve_as_they_would_alone(mods):
    gpu, workloads, ensemble = mods
    inst = _instances(ensemble)
    batched = ensemble.EnsembleRun(inst, capacity=1 << 18, tables=TABLES)
    for _ in range(20):
        batched.advance()
    got = _tiles(batched, gpu, workloads)
    batched.close()
    for k in range(len(inst)):
        alone = ensemble.EnsembleRun(inst, capacity=1 << 18, only=[k], tables=TABLES)
        for _ in range(20):
            alone.advance()
        want = _tiles(alone, gpu, workloads)
        alone.close()
        for sp in got:
            a, b = _instance_rows(got[sp], k), _instance_rows(want[sp], k)
            assert len(a["id"]) == len(b["id"]), (k, sp)
            for key in a:
                np.testing.assert_array_equal(a[key], b[key], err_msg=f"instance {k} species {sp} {key}")
        assert len(_instance_rows(want[gpu.SPECIES_ELECTRON], k)["id"]) > inst[k].n_seeds // 2


def _compare(res_a, res_b):
    assert [r["instance"] for r in res_a] == [r["instance"] for r in res_b]
    for a, b in zip(res_a, res_b):
        for key in ("electron_count", "photon_count"):
            assert a[key] == b[key], (a["instance"], key)
        for key in ("multiplication", "electron_weight", "photon_weight", "positron_weight"):
            assert a[key] == pytest.approx(b[key], rel=1e-12, abs=1e-300), (a["instance"], key)
        for sp in ("electron", "photon"):
            np.testing.assert_allclose(a["spectra"][sp], b["spectra"][sp], rtol=1e-12, atol=0)


def test_census_at_each_end_matches_the_instances_alone(mods):
    gpu, workloads, ensemble = mods
    inst = _instances(ensemble)
    batched = ensemble.run_batched(inst, capacity=1 << 18, autotune=False, tables=TABLES)
    seq = ensemble.run_sequential(inst, capacity=1 << 18, tables=TABLES, one_pass=False)
    _compare(batched["results"], seq["results"])
    assert batched["thinned"] == seq["thinned"] > 0
    assert batched["steps"] == max(i.steps for i in inst)
    assert batched["particle_steps"] == seq["particle_steps"]


def test_one_pass_control_is_the_slice_control(mods):
    """Both control paths on the same batched state: tiles equal bit for bit
    after 30 steps with control every 5 steps."""
    gpu, workloads, ensemble = mods
    inst = _instances(ensemble)
    inst[0].target = 70
    tiles = []
    for one_pass in (True, False):
        run = ensemble.EnsembleRun(inst, capacity=1 << 18, tables=TABLES, control_every=5, one_pass=one_pass)
        for _ in range(30):
            run.advance()
        tiles.append((_tiles(run, gpu, workloads), run.thinned))
        run.close()
    (a, ta), (b, tb) = tiles
    assert ta == tb > 0
    for k in range(len(inst)):
        for sp in a:
            x, y = _instance_rows(a[sp], k), _instance_rows(b[sp], k)
            for key in x:
                np.testing.assert_array_equal(x[key], y[key], err_msg=f"instance {k} species {sp} {key}")


def test_autotune_changes_no_result(mods):
    gpu, workloads, ensemble = mods
    inst = _instances(ensemble)
    plain = ensemble.run_batched(inst, capacity=1 << 18, autotune=False, tables=TABLES)
    tuned = ensemble.run_batched(inst, capacity=1 << 18, autotune=True, tables=TABLES)
    _compare(plain["results"], tuned["results"])
    best, timings = tuned["autotune"]
    assert len(timings) >= 4 and best in [t[0] for t in timings]
