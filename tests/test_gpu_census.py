"""rrea_gpu_census_resident (the device census of a resident tile) against
the oracle's numpy restatement on the same tiles.

Count, bin membership and threshold membership are exact (the kernel and the
restatement evaluate K with the same round-to-nearest operations); the FP64
sums, accumulated with atomics in nondeterministic order, agree within
1e-12 relative.  Energies are drawn log-uniform over the spectrum range and
beyond it, with some exactly on bin edges and thresholds; a tenth of the
particles are invalid (negative id) and must not count."""
import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    from rrea_feedback_warpx_amrex_geant4_gb300 import avalanche, build, gpu, workloads
    from oracle import avalanche as oav
    build.build()
    cfg = workloads.make_config(gpu, "uniform_c0")
    ctx = gpu.RreaGpuContext(cfg, 1 << 17)
    ctx.load_tables(TABLES)
    ctx.set_field(**workloads.make_field("uniform_c0"))
    yield gpu, workloads, avalanche, oav, ctx
    ctx.close()


def _tile(workloads, n, rng, photon, edges, thresholds):
    k = np.exp(rng.uniform(np.log(1.0e3), np.log(3.0e9), n))
    k[: len(edges)] = edges[: min(len(edges), n)]
    k[len(edges): len(edges) + len(thresholds)] = thresholds
    mu = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    s = np.sqrt(1.0 - mu * mu)
    d = np.stack([s * np.cos(phi), s * np.sin(phi), mu], axis=1)
    mag = k if photon else workloads.proper_velocity(k)
    t = workloads.make_electrons("uniform_c0", n)
    t["ux"][:], t["uy"][:], t["uz"][:] = mag * d[:, 0], mag * d[:, 1], mag * d[:, 2]
    t["w"][:] = rng.uniform(0.5, 2.0, n)
    t["id"][rng.uniform(size=n) < 0.1] *= -1
    for f in ("ux", "uy", "uz"):
        t["prev_" + f][:] = t[f]
    return t


@pytest.mark.parametrize("species", [0, 1, 2])
def test_census_matches_restatement(env, species):
    gpu, workloads, avalanche, oav, ctx = env
    rng = np.random.default_rng(17 + species)
    edges = avalanche.SPECTRUM_EDGES_EV
    thr = np.array([1.0e5, 1.0e6, 2.5e7])
    t = _tile(workloads, 50_000, rng, species == 2, edges, thr)
    getattr(ctx, ("stage_electrons", "stage_positrons", "stage_photons")[species])(t)
    g = ctx.census(species, edges, thr)
    o = oav.census(t, species, edges, thr)
    assert g["count"] == o["count"]
    assert g["max_weight"] == o["max_weight"]
    for key in ("sum_w", "sum_w2", "sum_wk", "under", "over"):
        assert g[key] == pytest.approx(o[key], rel=1e-12, abs=1e-300), key
    np.testing.assert_allclose(g["above"], o["above"], rtol=1e-12)
    np.testing.assert_allclose(g["hist"], o["hist"], rtol=1e-12, atol=0)
    # membership is exact: the same bins are empty on both sides
    np.testing.assert_array_equal(g["hist"] > 0, o["hist"] > 0)


def test_census_refuses_bad_edges(env):
    gpu, workloads, avalanche, oav, ctx = env
    with pytest.raises(gpu.RreaGpuError):
        ctx.census(0, [1.0, 1.0])
    with pytest.raises(gpu.RreaGpuError):
        ctx.census(0, np.logspace(0, 1, 1100))
    with pytest.raises(gpu.RreaGpuError):
        ctx.census(0, [1.0, 2.0], np.ones(17))


def test_particle_charge_matches_restatement(env):
    """rrea_gpu_deposit_charge_resident against the oracle's
    DepositChargeCIC restatement (itself pinned bit-exact to the reference
    header): electrons -w and positrons +w on the 32 x 256 grid, particles
    near the axis and at the domain's edges included, invalid ones skipped.
    Atomics: within 1e-12 of the grid's largest cell; total charge kept."""
    gpu, workloads, avalanche, oav, ctx = env
    from oracle import oracle
    cfg = ctx.config
    rng = np.random.default_rng(5)
    tiles = []
    for species, stage in ((0, ctx.stage_electrons), (1, ctx.stage_positrons)):
        n = 40_000
        t = workloads.make_electrons("uniform_c0", n)
        t["r"][:] = cfg.r_hi * rng.uniform(0.0, 1.0, n) ** 2          # crowded near the axis
        t["z"][:] = cfg.z_hi * rng.uniform(0.0, 1.0, n)
        t["w"][:] = rng.uniform(0.5, 3.0, n)
        t["id"][rng.uniform(size=n) < 0.05] *= -1
        for f in ("r", "z"):
            t["prev_" + f][:] = t[f]
        stage(t)
        tiles.append((species, t))
    got = ctx.deposit_charge().ravel()
    dr, dz = (cfg.r_hi - cfg.r_lo) / cfg.nr, (cfg.z_hi - cfg.z_lo) / cfg.nz
    want = np.zeros(cfg.nr * cfg.nz)
    for species, t in tiles:
        v = t["id"] > 0
        q = -1.0 if species == 0 else 1.0
        want += oracle.deposit_charge_cic(cfg.nr, cfg.nz, dr, dz, cfg.r_lo, cfg.z_lo, t["r"][v], t["z"][v],
                                          q * t["w"][v])
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 * np.abs(want).max())
    total = sum((-1.0 if s == 0 else 1.0) * t["w"][t["id"] > 0].sum() for s, t in tiles)
    assert abs(got.sum() - total) <= 1e-12 * sum(t["w"].sum() for _, t in tiles)
