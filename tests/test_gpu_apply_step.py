"""Apply in one call (rrea_gpu_apply_step: the electron, photon and positron
phases on host tiles and the transient FIFO of their secondaries on the
device) against the same step through the per-phase drop-in calls and
drain_secondaries over their concatenated secondaries.

Case: scale-up tiles of 4096 electrons, 2048 photons (50 keV-20 MeV) and
512 positrons, one 0.5 ns step.

  * tiles (every column, ids included) and survivors (every field, FIFO
    order) bit-identical: the same kernels see the same inputs and the FIFO
    holds the same items in the same order;
  * cell sources within 16e-12 of each grid's largest cell (FP64 atomics in
    arbitrary order), net-chord currents within 1e-12 of their largest face;
  * a NULL tile skips its species;
  * a survivor buffer too small is RREA_GPU_ERR_CAPACITY and leaves the
    caller's tiles and buffer untouched (fail closed)."""
import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu

CASE = "scaleup_c1"
DT = 5.0e-10
STEP = 3


@pytest.fixture(scope="module")
def mods():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu, workloads
    build.build()
    return gpu, workloads


def _context(gpu, workloads):
    cfg = workloads.make_config(gpu, CASE)
    ctx = gpu.RreaGpuContext(cfg, 1 << 14)
    ctx.load_tables(TABLES)
    ctx.set_field(**workloads.make_field(CASE))
    ctx.reset_sources()
    ctx.reset_current()
    return ctx


def _inputs(workloads):
    e = workloads.make_electrons(CASE, 4096, seed=51)
    g = workloads.make_photons(CASE, 2048, DT, seed=52, e_lo=5.0e4, e_hi=2.0e7)
    p = workloads.make_electrons(CASE, 512, seed=53)
    return e, g, p


def test_apply_step_equals_phase_calls(mods):
    gpu, workloads = mods
    e, g, p = _inputs(workloads)
    a = _context(gpu, workloads)
    b = _context(gpu, workloads)
    try:
        ea, ga, pa = (workloads.copy_tile(t) for t in (e, g, p))
        pending = np.concatenate([a.apply_electrons(ea, STEP, DT), a.apply_photons(ga, STEP, DT),
                                  a.apply_positrons(pa, STEP, DT)])
        surv_a = a.drain_secondaries(pending, STEP, DT)
        eb, gb, pb = (workloads.copy_tile(t) for t in (e, g, p))
        surv_b = b.apply_step(eb, gb, pb, STEP, DT)
        assert len(pending) > 100 and len(surv_a) > 50
        for name, x, y in (("electrons", ea, eb), ("photons", ga, gb), ("positrons", pa, pb)):
            for key in x:
                np.testing.assert_array_equal(x[key], y[key], err_msg=f"{name} {key}")
        assert surv_a.dtype == surv_b.dtype and len(surv_a) == len(surv_b)
        assert surv_a.tobytes() == surv_b.tobytes()
        ca, cb = a.sources(), b.sources()
        for k in range(ca.shape[0]):
            scale = max(np.abs(ca[k]).max(), 1e-300)
            np.testing.assert_allclose(cb[k], ca[k], rtol=0.0, atol=16e-12 * scale, err_msg=f"cell grid {k}")
        (jra, jza), (jrb, jzb) = a.current(), b.current()
        for x, y in ((jra, jrb), (jza, jzb)):
            scale = max(np.abs(x).max(), 1e-300)
            np.testing.assert_allclose(y, x, rtol=0.0, atol=1e-12 * scale)
    finally:
        a.close()
        b.close()


def test_apply_step_skips_null_tiles(mods):
    gpu, workloads = mods
    e, g, p = _inputs(workloads)
    a = _context(gpu, workloads)
    b = _context(gpu, workloads)
    try:
        ea = workloads.copy_tile(e)
        surv_a = a.drain_secondaries(a.apply_electrons(ea, STEP, DT), STEP, DT)
        eb = workloads.copy_tile(e)
        surv_b = b.apply_step(eb, None, None, STEP, DT)
        for key in ea:
            np.testing.assert_array_equal(ea[key], eb[key], err_msg=key)
        assert surv_a.tobytes() == surv_b.tobytes()
    finally:
        a.close()
        b.close()


def test_apply_step_fails_closed_on_a_short_survivor_buffer(mods):
    """A survivor buffer too small for the step's survivors is
    RREA_GPU_ERR_CAPACITY with the count reported, and the caller's tiles
    stay as they were (nothing is written back before every stage passed)."""
    import ctypes
    gpu, workloads = mods
    e, g, p = _inputs(workloads)
    ctx = _context(gpu, workloads)
    try:
        eb, gb, pb = (workloads.copy_tile(t) for t in (e, g, p))
        tiles = [gpu.tile_struct(t) for t in (eb, gb, pb)]
        buf = np.zeros(4, dtype=gpu.SECONDARY_DTYPE)
        n = ctypes.c_int64()
        st = ctx.lib.rrea_gpu_apply_step(ctx.handle, ctypes.byref(tiles[0]), ctypes.byref(tiles[1]),
                                         ctypes.byref(tiles[2]), STEP, 0.0, DT, ctypes.c_void_p(buf.ctypes.data), 4,
                                         ctypes.byref(n))
        assert st == 8  # RREA_GPU_ERR_CAPACITY
        assert n.value > 4
        for name, x, y in (("electrons", e, eb), ("photons", g, gb), ("positrons", p, pb)):
            for key in x:
                np.testing.assert_array_equal(x[key], y[key], err_msg=f"{name} {key}")
        assert not buf.tobytes().strip(b"\0")
    finally:
        ctx.close()
