"""Whole avalanche runs of the plain uniform-field case through the resident
C-ABI (rrea_feedback_warpx_amrex_geant4_gb300.avalanche) against the
oracle's restatement of the same run (oracle/avalanche.py) and against the
Coleman-Dwyer avalanche length.

Case: the plain uniform-field case's physics (7.2 MeV seed electrons from
r = 0, z = 0 along -E; dry air at 1.225 kg/m^3; E_z = -400 kV/m; 10 keV
tracking cut; 32 x 256 cells over 50 m x 500 m; dt = 0.5 ns), with fewer
seeds and a shorter duration so that the oracle finishes in seconds.

  * same streams: one run with rng_seed 1 on both sides, census every 100
    steps.  Event choices are bit-exact per step, so the populations agree
    until a last-ulp difference flips one near-tie decision; the census
    counts must agree within 2 % at every row.
  * statistics: 8 GPU runs (rng_seed 11..18) against 8 oracle runs
    (rng_seed 1..8), all independent: the mean multiplication factor
    (electrons >= 1 MeV at the end over the seeds) within 3 sigma of the
    combined standard error, and a two-sample chi-squared test of the pooled
    final electron and photon spectra (bins with >= 10 entries on both
    sides) at p > 1e-3.
  * physics anchor: a 2000-seed run over 3000 steps; the e-folding length of
    the >= 1 MeV population within [0.8, 1.25] x the Coleman-Dwyer range
    7300 kV / (E - E_th n/n0), E_th = 276 or 284 kV/m at 1.293 kg/m^3
    (scripts/test_cd_science.py:341-382).
"""
import multiprocessing as mp
import os

import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu

CASE = "uniform_c0"
N_SEEDS, STEPS = 100, 1000
EVERY = 100


def _oracle_run(args):
    """One oracle run in a fresh (spawned) process."""
    rng_seed, n_seeds, steps, threads = args
    os.environ["OMP_NUM_THREADS"] = str(threads)
    from oracle import avalanche as oav, oracle
    from rrea_feedback_warpx_amrex_geant4_gb300 import avalanche as gav, workloads
    oracle.load_tables(TABLES)
    cfg = workloads.make_config(oracle, CASE, rng_seed=rng_seed)
    run = oav.AvalancheRun(cfg, workloads.make_field(CASE), workloads.make_electrons(CASE, n_seeds))
    res = run.run(steps, gav.DT_S, gav.SPECTRUM_EDGES_EV, gav.THRESHOLDS_EV, census_every=EVERY)
    return res


def _oracle_runs(seeds, n_seeds, steps):
    threads = max(1, (os.cpu_count() or 2) // len(seeds))
    with mp.get_context("spawn").Pool(len(seeds)) as pool:
        return pool.map(_oracle_run, [(s, n_seeds, steps, threads) for s in seeds])


@pytest.fixture(scope="module")
def mods():
    from rrea_feedback_warpx_amrex_geant4_gb300 import avalanche, build, gpu, workloads
    build.build()
    return gpu, workloads, avalanche


def _gpu_run(mods, rng_seed, n_seeds, steps, capacity=1 << 18, every=EVERY):
    gpu, workloads, avalanche = mods
    ctx = avalanche.make_context(CASE, capacity, rng_seed, tables=TABLES)
    try:
        return avalanche.AvalancheRun(ctx, workloads.make_electrons(CASE, n_seeds)).run(steps, census_every=every)
    finally:
        ctx.close()


def test_same_streams_track_the_oracle(mods):
    gpu_res = _gpu_run(mods, 1, N_SEEDS, 600)
    orc = _oracle_runs([1], N_SEEDS, 600)[0]
    assert len(gpu_res["history"]) == len(orc["history"])
    for g, o in zip(gpu_res["history"], orc["history"]):
        assert g["step"] == o["step"]
        for k in ("electron_count", "photon_count", "electron_ge_1MeV"):
            assert abs(g[k] - o[k]) <= 0.02 * max(o[k], 1), (g["step"], k, g[k], o[k])
    assert gpu_res["history"][-1]["electron_count"] > 2 * N_SEEDS, "the run did not avalanche"


def _chi2_two_sample(a, b, min_count=10):
    from scipy import stats
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    sel = (a >= min_count) & (b >= min_count)
    a, b = a[sel], b[sel]
    ka, kb = np.sqrt(b.sum() / a.sum()), np.sqrt(a.sum() / b.sum())
    chi2 = float(np.sum((ka * a - kb * b) ** 2 / (a + b)))
    dof = int(sel.sum()) - 1
    return chi2, dof, float(stats.chi2.sf(chi2, dof))


def test_multiplication_and_spectra_agree_statistically(mods):
    k = 8
    gpu_runs = [_gpu_run(mods, 11 + i, N_SEEDS, STEPS) for i in range(k)]
    orc_runs = _oracle_runs(list(range(1, k + 1)), N_SEEDS, STEPS)
    mg = np.array([r["multiplication"] for r in gpu_runs])
    mo = np.array([r["multiplication"] for r in orc_runs])
    se = np.sqrt(mg.var(ddof=1) / k + mo.var(ddof=1) / k)
    assert abs(mg.mean() - mo.mean()) <= 3.0 * se, (mg, mo)
    assert mg.mean() > 3.0, "the runs did not avalanche"
    for species in ("electron", "photon"):
        a = np.sum([r["spectra"][species] for r in gpu_runs], axis=0)
        b = np.sum([r["spectra"][species] for r in orc_runs], axis=0)
        chi2, dof, p = _chi2_two_sample(a, b)
        assert dof >= 10, (species, dof)
        assert p > 1.0e-3, (species, chi2, dof, p)


def test_avalanche_length_matches_coleman_dwyer(mods):
    gpu, workloads, avalanche = mods
    res = _gpu_run(mods, 1, 2000, 3000, capacity=1 << 23)
    lam = avalanche.avalanche_length_m(res["history"])
    lo = avalanche.coleman_dwyer_length_m(4.0e5, workloads.AIR_DENSITY, 276.0)
    hi = avalanche.coleman_dwyer_length_m(4.0e5, workloads.AIR_DENSITY, 284.0)
    assert 0.8 * lo <= lam <= 1.25 * hi, (lam, lo, hi)
