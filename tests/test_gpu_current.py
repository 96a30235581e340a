"""Net-chord current (charge-conserving J deposition of the charged phases)
on the GPU vs the oracle's replay of the same step's segments, through the
C-ABI (rrea_gpu_download_current_index / rrea_gpu_download_current).

Tolerance: every padded grid within 1e-12 of its largest entry (the GPU sums
with atomics in arbitrary order, and the segment endpoints are the transport
results, equal to the oracle's within 1e-12 relative).  The continuity
identity drho + dt div J = 0 is checked on the GPU output alone, to 1e-12 of
the deposited charge."""
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


def _run(mods, case, n, species, arr, dt=5.0e-10, step=0):
    gpu, workloads, oracle, compare = mods
    cfg, ctx, field = _ctx(gpu, workloads, case, n)
    ctx.reset_current()
    g, o = compare.run_pair(ctx, cfg, field, arr, step, dt, species=species)
    gi = ctx.current_index()
    jr, jz = ctx.current()
    ref = oracle.deposit_segments(cfg, dt, oracle.segment_rows(o[1]))
    ctx.close()
    return cfg, g, o, gi, (jr, jz), ref


def _assert_grids(gi, phys, ref):
    for key in ("rho", "jr", "jz"):
        scale = max(np.abs(ref[key]).max(), 1e-300)
        np.testing.assert_allclose(gi[key], ref[key], rtol=0, atol=1e-12 * scale, err_msg=key)
    for got, key in zip(phys, ("jr_phys", "jz_phys")):
        scale = max(np.abs(ref[key]).max(), 1e-300)
        np.testing.assert_allclose(got, ref[key], rtol=0, atol=1e-12 * scale, err_msg=key)


@pytest.mark.parametrize("species", ["electron", "positron"])
def test_current_matches_oracle_scaleup(mods, species):
    gpu, workloads, oracle, compare = mods
    arr = workloads.make_electrons("scaleup_c1", 2048, seed=13)
    cfg, g, o, gi, phys, ref = _run(mods, "scaleup_c1", 2048, species, arr)
    assert np.abs(ref["jz"]).max() > 0.0
    _assert_grids(gi, phys, ref)


def test_current_with_escapes_and_demotions(mods):
    """Electrons at the upper z face escape (boundary-cloud closure); slow
    ones demote; the rest survive."""
    gpu, workloads, oracle, compare = mods
    arr = workloads.make_electrons("uniform_c0", 96, seed=5)
    arr["z"][:32] = arr["prev_z"][:32] = 500.0 - 0.01
    k = np.full(32, 5.0e3)
    for f in ("uz", "prev_uz"):
        arr[f][32:64] = workloads.proper_velocity(k)
    cfg, g, o, gi, phys, ref = _run(mods, "uniform_c0", 96, "electron", arr)
    assert (o[1]["disposition"][:32] == 1).all() and (o[1]["disposition"][32:64] == 2).all()
    assert np.abs(ref["rho"]).max() > 0.0  # the escape closure moves charge into the pad cells
    _assert_grids(gi, phys, ref)


def test_current_positron_annihilation(mods):
    gpu, workloads, oracle, compare = mods
    arr = workloads.make_electrons("scaleup_c1", 1024, seed=17)
    k = np.exp(np.random.default_rng(2).uniform(np.log(1.2e4), np.log(3.0e5), 1024))
    norm = np.sqrt(arr["ux"] ** 2 + arr["uy"] ** 2 + arr["uz"] ** 2)
    u = workloads.proper_velocity(k)
    for f in ("ux", "uy", "uz"):
        arr[f] *= u / norm
        arr["prev_" + f][:] = arr[f]
    cfg, g, o, gi, phys, ref = _run(mods, "scaleup_c1", 1024, "positron", arr, dt=2.0e-8)
    assert (o[1]["disposition"] == 2).sum() > 500
    _assert_grids(gi, phys, ref)


def test_continuity_identity_on_gpu_current(mods):
    """All electrons survive one step: the change of their CIC charge on the
    padded grid equals -dt times the index-space divergence of the GPU J."""
    gpu, workloads, oracle, compare = mods
    n, dt = 512, 5.0e-10
    arr = workloads.make_electrons("uniform_c0", n, seed=21)
    cfg, ctx, field = _ctx(gpu, workloads, "uniform_c0", n)
    ctx.reset_current()
    start = workloads.copy_tile(arr)
    ctx.apply_electrons(arr, 0, dt)
    _, _, disp = ctx.diagnostics(n)
    assert (disp == 0).all()
    gi = ctx.current_index()
    ctx.close()
    nr, nz, drr, dzz, z_lo = cfg.nr + 2, cfg.nz + 4, cfg.r_hi / cfg.nr, cfg.z_hi / cfg.nz, -2.0 * cfg.z_hi / cfg.nz
    rho = np.zeros((nz, nr))

    def cic(q, r, z):
        xr, xz = r / drr - 0.5, (z - z_lo) / dzz - 0.5
        i0, j0 = np.floor(xr).astype(int), np.floor(xz).astype(int)
        fr, fz = xr - i0, xz - j0
        for a, wr in ((0, 1 - fr), (1, fr)):
            for b, wz in ((0, 1 - fz), (1, fz)):
                i = i0 + a
                i = np.where(i < 0, -1 - i, i)
                np.add.at(rho, (j0 + b, i), q * wr * wz)

    w = arr["w"]
    cic(w, start["prev_r"], start["prev_z"])     # charge -w leaves the start ...
    cic(-w, arr["r"], arr["z"])                  # ... and arrives at the end
    div = (gi["jr"][:, 1:] - gi["jr"][:, :-1]) + (gi["jz"][1:, :] - gi["jz"][:-1, :])
    np.testing.assert_allclose(rho + dt * div, 0.0, atol=1e-12 * w.sum())
