"""The plane-crossing diagnostic on the device (rrea_gpu_set_planes,
rrea_gpu_plane_flux, rrea_gpu_restore_plane_flux) against the oracle's
restatement of defer_cd_electron_plane_crossings (O/RreaTransportStep.H:
249-332), whose enumeration and accumulator are pinned to the reference's
own I/RreaPlaneFlux.H by tests/test_oracle_plane_flux.py.

Case: 4096 scale-up electrons (1-20 MeV, r < 5 m, z in 0-10 m, a quarter of
them turned toward -z), planes every 5 cm over z in [-0.475, 10.475] m, one
electron phase of 2 ns and the drain of the same pending secondaries on both
sides (the newborn electron legs cross planes too).  No plane sits on the
absorbing face z = 0: there a segment that ends by escaping through the face
crosses the plane or not by the last ulp of its clipped end point, which the
device's Cartesian chord ends round differently from the x86-64 arithmetic
(9 of the 4096 electrons on a plane at z = 0).

  * the weighted counts (all, local runaway, >= 1 MeV, per direction) are
    sums of unit weights, exact in any order: equal, plane by plane, except
    where a crossing's selection sits within the transport's 1e-12 of a
    threshold (at most 2 entries of the 220 x 6, off by one);
  * the local runaways' w r and w r^2 sums within 1e-12 of each column's
    largest entry (atomics in arbitrary order) outside those planes;
  * the diagnostic changes no transport result (tiles bit-identical with
    and without planes);
  * strictly increasing finite planes only; restore refuses negative values."""
import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu

CASE = "scaleup_c1"
DT_S = 2.0e-9
PLANES = np.round(np.arange(-0.475, 10.475 + 1e-9, 0.05), 10)


@pytest.fixture(scope="module")
def mods():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu, workloads
    from oracle import oracle
    build.build()
    oracle.load_tables(TABLES)
    return gpu, workloads, oracle


def _electrons(workloads, n=4096):
    e = workloads.make_electrons(CASE, n, seed=21)
    flip = np.arange(n) % 4 == 0
    for f in ("uz", "prev_uz"):
        e[f][flip] *= -1.0
    return e


def _context(gpu, workloads, capacity=1 << 14):
    cfg = workloads.make_config(gpu, CASE)
    ctx = gpu.RreaGpuContext(cfg, capacity)
    ctx.load_tables(TABLES)
    field = workloads.make_field(CASE)
    ctx.set_field(**field)
    return cfg, ctx, field


def _compare(got, ref):
    counts_g, counts_r = got[:, :6], ref[:, :6]
    diff = np.abs(counts_g - counts_r)
    assert diff.max() <= 1.0 and (diff > 0).sum() <= 2, np.argwhere(diff > 0)[:10]
    clean = ~(diff > 0).any(axis=1)
    for c in range(6, 10):
        scale = max(np.abs(ref[:, c]).max(), 1e-300)
        np.testing.assert_allclose(got[clean, c], ref[clean, c], rtol=0, atol=1e-12 * scale, err_msg=f"column {c}")


def test_phase_and_drain_crossings_match_oracle(mods):
    gpu, workloads, oracle = mods
    cfg, ctx, field = _context(gpu, workloads)
    ctx.set_planes(PLANES)
    oracle.set_planes(PLANES)
    try:
        e = _electrons(workloads)
        ctx.apply_electrons(workloads.copy_tile(e), 5, DT_S)
        got_phase = ctx.plane_flux()
        o = oracle.electron_step(cfg, field, 5, DT_S, workloads.copy_tile(e))
        ref_phase = oracle.plane_flux()
        assert ref_phase[:, 0].sum() > 5000 and ref_phase[:, 1].sum() > 1000
        assert ref_phase[:, 2].sum() > 1000 and ref_phase[:, 4].sum() > 1000
        _compare(got_phase, ref_phase)

        pending = o["secondaries"]
        assert (pending["species"] == 0).sum() > 50
        ctx.restore_plane_flux(None)
        ctx.drain_secondaries(pending, 5, DT_S)
        got_drain = ctx.plane_flux()
        oracle.drain(cfg, field, 5, DT_S, pending)
        ref_drain = oracle.plane_flux()
        assert ref_drain[:, :2].sum() > 20
        _compare(got_drain, ref_drain)
    finally:
        oracle.set_planes([])
        ctx.close()


def test_planes_change_no_transport_result(mods):
    gpu, workloads, oracle = mods
    tiles = []
    for planes in (PLANES, ()):
        cfg, ctx, field = _context(gpu, workloads)
        ctx.set_planes(planes)
        t = workloads.copy_tile(_electrons(workloads))
        sec = ctx.apply_electrons(t, 5, DT_S)
        tiles.append((t, sec))
        ctx.close()
    (a, sa), (b, sb) = tiles
    for key in a:
        np.testing.assert_array_equal(a[key], b[key], err_msg=key)
    assert len(sa) == len(sb)


def test_plane_arguments_are_checked(mods):
    gpu, workloads, oracle = mods
    cfg, ctx, field = _context(gpu, workloads, capacity=1024)
    try:
        for bad in ([1.0, 1.0], [2.0, 1.0], [0.0, np.nan]):
            with pytest.raises(gpu.RreaGpuError):
                ctx.set_planes(bad)
        ctx.set_planes([1.0, 2.0])
        v = np.zeros(20)
        v[3] = -1.0
        with pytest.raises(gpu.RreaGpuError):
            ctx.restore_plane_flux(v)
        v[3] = 2.5
        ctx.restore_plane_flux(v)
        np.testing.assert_array_equal(ctx.plane_flux().ravel(), v)
    finally:
        ctx.close()
