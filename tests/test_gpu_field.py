"""Field update on the device (Maxwell TM-RZ leapfrog driven by the kinetic
net-chord current) vs the oracle's restatement, through the C-ABI
(rrea_gpu_advance_field / rrea_gpu_download_field).

The GPU's own current feeds both sides, so the comparison isolates the field
arithmetic: the GPU Er/Ez/Btheta must equal the oracle's within 1e-12 of each
vector's largest magnitude (operations and order are the same; the fields are
sums of differences of nearby values)."""
import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu, workloads
    from oracle import oracle
    build.build()
    oracle.load_tables(TABLES)
    return gpu, workloads, oracle


@pytest.mark.parametrize("case,n,substeps", [("uniform_c0", 4096, 2), ("scaleup_c1", 4096, 3)])
def test_field_step_matches_oracle(mods, case, n, substeps):
    gpu, workloads, oracle = mods
    cfg = workloads.make_config(gpu, case)
    ctx = gpu.RreaGpuContext(cfg, n)
    ctx.load_tables(TABLES)
    field = workloads.make_field(case)
    rng = np.random.default_rng(8)
    field["er"] = rng.normal(0.0, 2.0e3, field["er"].shape)
    field["ez"] = rng.normal(0.0, 2.0e3, field["ez"].shape)
    bt = rng.normal(0.0, 1.0e-5, field["bt"].shape).reshape(cfg.nz + 1, cfg.nr + 1)
    bt[:, 0] = 0.0
    field["bt"] = bt.ravel()
    er0 = field["er"].reshape(cfg.nz, cfg.nr + 1)
    er0[:, 0] = 0.0
    field["er"] = er0.ravel()
    ctx.set_field(**field)
    dt = 5.0e-10
    for step in range(3):
        ctx.reset_current()
        arr = workloads.make_electrons(case, n, seed=40 + step)
        ctx.apply_electrons(arr, step, dt)
        jr, jz = ctx.current()
        assert np.abs(jz).max() > 0.0
        before = ctx.field()
        ctx.advance_field(dt, substeps)
        after = ctx.field()
        ref = oracle.advance_maxwell(cfg.nr, cfg.nz, cfg.r_hi / cfg.nr, cfg.z_hi / cfg.nz, dt, substeps, *before,
                                     jr.ravel(), jz.ravel())
        for name, g, o in zip(("er", "ez", "bt"), after, ref):
            scale = max(np.abs(o).max(), 1e-300)
            np.testing.assert_allclose(g, o, rtol=0, atol=1e-12 * scale, err_msg=name)
    ctx.close()


def test_field_step_refuses_cfl_violation(mods):
    gpu, workloads, oracle = mods
    cfg = workloads.make_config(gpu, "uniform_c0")
    ctx = gpu.RreaGpuContext(cfg, 16)
    ctx.load_tables(TABLES)
    ctx.set_field(**workloads.make_field("uniform_c0"))
    with pytest.raises(gpu.RreaGpuError) as e:
        ctx.advance_field(1.0e-6, 1)
    assert e.value.status == 1
    ctx.advance_field(5.0e-10, 1)
    ctx.close()


def test_split_field_update_with_scaled_current(mods):
    """The sharded-run halves (rrea_gpu_current_device, then
    rrea_gpu_advance_field_from_current) on the device vectors viewed by torch:
    doubling the current in place, as an allreduce over two identical ranks
    would, gives the field of the doubled current."""
    import torch

    from rrea_feedback_warpx_amrex_geant4_gb300 import distributed

    gpu, workloads, oracle = mods
    case, n, substeps, dt = "uniform_c0", 4096, 2, 5.0e-10
    cfg = workloads.make_config(gpu, case)
    ctx = gpu.RreaGpuContext(cfg, n)
    ctx.load_tables(TABLES)
    ctx.set_field(**workloads.make_field(case))
    ctx.reset_current()
    ctx.apply_electrons(workloads.make_electrons(case, n, seed=5), 0, dt)
    jr, jz = ctx.current()
    (jr_ptr, n_jr), (jz_ptr, n_jz) = ctx.current_device()
    vr, vz = distributed.device_view(jr_ptr, n_jr), distributed.device_view(jz_ptr, n_jz)
    np.testing.assert_array_equal(vr.cpu().numpy(), jr.ravel())
    np.testing.assert_array_equal(vz.cpu().numpy(), jz.ravel())
    vr.mul_(2.0)
    vz.mul_(2.0)
    torch.cuda.synchronize()
    before = ctx.field()
    ctx.advance_field_from_current(dt, substeps)
    after = ctx.field()
    ref = oracle.advance_maxwell(cfg.nr, cfg.nz, cfg.r_hi / cfg.nr, cfg.z_hi / cfg.nz, dt, substeps, *before,
                                 2.0 * jr.ravel(), 2.0 * jz.ravel())
    for name, g, o in zip(("er", "ez", "bt"), after, ref):
        scale = max(np.abs(o).max(), 1e-300)
        np.testing.assert_allclose(g, o, rtol=0, atol=1e-12 * scale, err_msg=name)
    ctx.close()
