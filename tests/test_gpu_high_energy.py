"""Charged-particle parity on the elastic branches the production-energy
tests do not reach (apply_gs_elastic_scatter, O/RreaTransportStep.H:371-423;
SampleGsCosTheta, S/RreaInteractionTables.cpp:2504-2544):

  * Wentzel-VI: electrons and positrons of 100 MeV to 1 GeV, whose
    multiple-scattering angles come from the Wentzel-VI inverse CDF (E above
    the 100 MeV GS/Wentzel transition), over the scale-up grid at
    dt = 0.5 ns and 10 ns;
  * the isotropic branch (n >= 1e5 collisions in one substep): 1-20 MeV
    electrons over dt = 100 ns with the substep count capped at 1 and the
    strict subcycle guard off, so that one substep carries the whole path.

The oracle counts its elastic draws by branch; each case asserts its branch
was taken.  Tolerances as in the phase tests (oracle/compare.py)."""
import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu

CASE = "scaleup_c1"


@pytest.fixture(scope="module")
def mods():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu, workloads
    from oracle import compare, oracle
    build.build()
    oracle.load_tables(TABLES)
    return gpu, workloads, oracle, compare


def _tile(workloads, n, k_lo, k_hi, seed):
    arr = workloads.make_electrons(CASE, n, seed=seed)
    rng = np.random.default_rng(seed + 1)
    k = np.exp(rng.uniform(np.log(k_lo), np.log(k_hi), n))
    d = np.stack([arr["ux"], arr["uy"], arr["uz"]], 1)
    d /= np.linalg.norm(d, axis=1)[:, None]
    u = workloads.proper_velocity(k)
    for i, f in enumerate(("ux", "uy", "uz")):
        arr[f][:] = u * d[:, i]
    arr["z"][:] += 500.0
    workloads.capture_prev(arr)
    return arr, k


def _run(mods, cfg, arr, dt, species, parent_energy):
    gpu, workloads, oracle, compare = mods
    # room for the secondaries of long steps (about five per particle at 100 ns)
    ctx = gpu.RreaGpuContext(cfg, 8 * len(arr["id"]))
    ctx.load_tables(TABLES)
    field = workloads.make_field(CASE)
    ctx.set_field(**field)
    oracle.elastic_branches(reset=True)
    g, o = compare.run_pair(ctx, cfg, field, arr, 4, dt, species=species)
    branches = oracle.elastic_branches(reset=True)
    problems = compare.compare(cfg, g, o, max(cfg.r_hi, cfg.z_hi), parent_energy=parent_energy)
    ctx.close()
    return problems, branches, o


@pytest.mark.parametrize("species", ["electron", "positron"])
@pytest.mark.parametrize("dt", [5.0e-10, 1.0e-8])
def test_wentzel_vi_branch_parity(mods, species, dt):
    gpu, workloads, oracle, compare = mods
    cfg = workloads.make_config(gpu, CASE)
    arr, k = _tile(workloads, 2048, 1.0e8, 1.0e9, seed=61)
    problems, branches, o = _run(mods, cfg, arr, dt, species, k)
    assert branches["wentzel"] > 1000, branches
    assert len(o[1]["secondaries"]) > 0
    assert not problems, "; ".join(problems)


def test_isotropic_branch_parity(mods):
    gpu, workloads, oracle, compare = mods
    cfg = workloads.make_config(gpu, CASE, max_subcycles=1)
    cfg.strict_transport_guards = 0
    arr, k = _tile(workloads, 4096, 1.0e6, 2.0e7, seed=71)
    problems, branches, o = _run(mods, cfg, arr, 1.0e-7, "electron", k)
    assert branches["isotropic"] > 10, branches
    assert not problems, "; ".join(problems)
