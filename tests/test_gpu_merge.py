"""The weight-doubling merge above the cap (rrea_gpu_population_merge_resident),
a population policy of this library with no reference counterpart, against a
numpy restatement of its rule and against the properties it must keep.

Tile: 200,000 scale-up electrons (K log-uniform 1-20 MeV, random
directions) packed into r < 2 m, z < 4 m (a dozen cells of the 256 x 2048
grid) with weights uniform in [0.5, 2]; every tenth row invalid.  Target
150,000 live particles.

  * the merge equals the restatement bit for bit: groups, pairs, requested
    and merged counts, every weight and id of the tile;
  * the weight of every cell is kept (within 1e-13 of the cell's weight: one
    rounding of w_a + w_b per merged pair);
  * the weighted kinetic energy keeps its expectation: the change stays
    within 5 sigma of the merge's own variance, sum over merged pairs of
    p (1 - p) (W (K_a - K_b))^2 with p = w_a / W;
  * after compaction the tile holds live - merged particles, and a second
    merge at the same target does nothing;
  * the same call on the same tile gives the same tile."""
import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu

CASE = "scaleup_c1"
N = 200_000
TARGET = 150_000
STEP = 7
MEC2 = 510998.95
M64 = 0xFFFFFFFFFFFFFFFF


@pytest.fixture(scope="module")
def mods():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu, workloads
    build.build()
    return gpu, workloads


def _tile(workloads):
    t = workloads.make_electrons(CASE, N, seed=31)
    rng = np.random.default_rng(32)
    t["r"][:] = 2.0 * np.sqrt(rng.uniform(0.0, 1.0, N))
    t["z"][:] = rng.uniform(0.0, 4.0, N)
    t["w"][:] = rng.uniform(0.5, 2.0, N)
    t["id"][::10] *= -1
    for f in ("r", "z", "theta", "ux", "uy", "uz"):
        t["prev_" + f][:] = t[f]
    return t


def _context(gpu, workloads):
    cfg = workloads.make_config(gpu, CASE)
    ctx = gpu.RreaGpuContext(cfg, N)
    ctx.load_tables(TABLES)
    ctx.set_field(**workloads.make_field(CASE))
    return cfg, ctx


def _fetch(ctx, workloads, n):
    t = workloads.make_electrons(CASE, n)
    ctx.fetch_electrons(t)
    return t


def _splitmix(v):
    v = (v + 0x9E3779B97F4A7C15) & M64
    v = ((v ^ (v >> 30)) * 0xBF58476D1CE4E5B9) & M64
    v = ((v ^ (v >> 27)) * 0x94D049BB133111EB) & M64
    return v ^ (v >> 31)


def _restated(t, cfg, target, seed, species, step):
    """The merge rule restated (test oracle)."""
    w = t["w"].copy()
    ids = t["id"].copy()
    live = np.nonzero(ids > 0)[0]
    n = len(live)
    out = {"live": n, "groups": 0, "pairs": 0, "requested": 0, "merged": 0}
    pairs = []
    if n <= target or n < 2:
        return out, w, ids, pairs
    dr = (cfg.r_hi - cfg.r_lo) / cfg.nr
    dz = (cfg.z_hi - cfg.z_lo) / cfg.nz
    fr = (t["r"][live] - cfg.r_lo) / dr
    fz = (t["z"][live] - cfg.z_lo) / dz
    ir = np.minimum(np.where(fr >= 0, fr.astype(np.int64), 0), cfg.nr - 1).astype(np.uint64)
    iz = np.minimum(np.where(fz >= 0, fz.astype(np.int64), 0), cfg.nz - 1).astype(np.uint64)
    ux, uy, uz = t["ux"][live], t["uy"][live], t["uz"][live]
    u2 = (ux * ux + uy * uy) + uz * uz
    b = (u2.view(np.uint64) >> np.uint64(50)) & np.uint64(0x1FFF)
    neg = (uz.view(np.int64) < 0).astype(np.uint64)
    keys = (iz << np.uint64(34)) | (ir << np.uint64(14)) | (b << np.uint64(1)) | neg
    perm = np.argsort(keys, kind="stable")
    sk = keys[perm]
    heads = np.ones(n, dtype=bool)
    heads[1:] = sk[1:] != sk[:-1]
    start = np.maximum.accumulate(np.where(heads, np.arange(n), 0))
    rank = np.arange(n) - start
    pair = (rank % 2 == 0) & np.append(sk[1:] == sk[:-1], False)
    P = int(pair.sum())
    R = min(n - target, P)
    out.update(groups=int(heads.sum()), pairs=P, requested=R)
    merged = 0
    for j, i in enumerate(np.nonzero(pair)[0]):
        if (j + 1) * R // P == j * R // P:
            continue
        a, bb = live[perm[i]], live[perm[i + 1]]
        ka = abs(int(ids[a])) ^ (int(t["cpu"][a]) << 40)
        kb = abs(int(ids[bb])) ^ (int(t["cpu"][bb]) << 40)
        h = _splitmix(seed ^ 0x6D65726765 ^ (species << 56))
        h = _splitmix(h ^ step)
        h = _splitmix(h ^ ka)
        h = _splitmix(h ^ kb)
        u = (float(h >> 11) + 0.5) * 2.0 ** -53
        s = w[a] + w[bb]
        keep, drop = (a, bb) if u * s < w[a] else (bb, a)
        pairs.append((a, bb))
        w[keep] = s
        ids[drop] = -ids[drop]
        merged += 1
    out["merged"] = merged
    return out, w, ids, np.array(pairs, dtype=np.int64).reshape(-1, 2)


def _kinetic(t):
    u2 = t["ux"] ** 2 + t["uy"] ** 2 + t["uz"] ** 2
    g = np.sqrt(1.0 + u2 / 299792458.0 ** 2)
    return (g - 1.0) * MEC2


def _cells(cfg, t):
    ok = t["id"] > 0
    ir = np.minimum((t["r"][ok] / ((cfg.r_hi - cfg.r_lo) / cfg.nr)).astype(np.int64), cfg.nr - 1)
    iz = np.minimum((t["z"][ok] / ((cfg.z_hi - cfg.z_lo) / cfg.nz)).astype(np.int64), cfg.nz - 1)
    return np.bincount(iz * cfg.nr + ir, weights=t["w"][ok], minlength=cfg.nr * cfg.nz)


def test_merge_matches_restatement_and_keeps_cells(mods):
    gpu, workloads = mods
    cfg, ctx = _context(gpu, workloads)
    try:
        t = _tile(workloads)
        ctx.stage_electrons(workloads.copy_tile(t))
        st = ctx.population_merge(gpu.SPECIES_ELECTRON, TARGET, STEP)
        got = _fetch(ctx, workloads, N)
        want, w, ids, pairs = _restated(t, cfg, TARGET, cfg.rng_seed, gpu.SPECIES_ELECTRON, STEP)
        assert st == want, (st, want)
        assert st["merged"] == st["requested"] == (N - N // 10) - TARGET
        np.testing.assert_array_equal(got["id"], ids)
        np.testing.assert_array_equal(got["w"], w)
        before, after = _cells(cfg, t), _cells(cfg, got)
        np.testing.assert_allclose(after, before, rtol=1e-13, atol=0.0)
        # the weighted kinetic energy keeps its expectation: each merged pair
        # contributes W K_keep, of mean w_a K_a + w_b K_b and variance
        # p (1 - p) W^2 (K_a - K_b)^2
        k = _kinetic(t)
        e_before = float((t["w"][t["id"] > 0] * k[t["id"] > 0]).sum())
        e_after = float((got["w"][got["id"] > 0] * k[got["id"] > 0]).sum())
        a, b = pairs[:, 0], pairs[:, 1]
        wsum = t["w"][a] + t["w"][b]
        pa = t["w"][a] / wsum
        var = float((pa * (1.0 - pa) * (wsum * (k[a] - k[b])) ** 2).sum())
        assert var > 0.0
        assert abs(e_after - e_before) <= 5.0 * np.sqrt(var) + 1e-12 * e_before
    finally:
        ctx.close()


def test_merge_compacts_and_is_idempotent_and_repeatable(mods):
    gpu, workloads = mods
    tiles = []
    for _ in range(2):
        cfg, ctx = _context(gpu, workloads)
        try:
            t = _tile(workloads)
            ctx.stage_electrons(workloads.copy_tile(t))
            st = ctx.population_merge(gpu.SPECIES_ELECTRON, TARGET, STEP)
            tiles.append(_fetch(ctx, workloads, N))
            ctx.compact_resident(gpu.SPECIES_ELECTRON)
            assert ctx.resident_count(gpu.SPECIES_ELECTRON) == st["live"] - st["merged"] == TARGET
            again = ctx.population_merge(gpu.SPECIES_ELECTRON, TARGET, STEP + 1)
            assert again["live"] == TARGET and again["merged"] == 0
        finally:
            ctx.close()
    for key in ("w", "id", "r", "z", "ux"):
        np.testing.assert_array_equal(tiles[0][key], tiles[1][key], err_msg=key)
