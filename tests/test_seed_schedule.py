"""Seed schedule input adapter (rrea_gpu_seed_schedule_*, host-only C-ABI
calls of the library, no GPU needed) against the reference's own
RreaSeedSchedule compiled by oracle/ref_golden.cpp on the same CSV
(tests/golden/ref_seed_schedule_input.csv): quoted and padded cells, blank
lines, optional macro_index and species_id columns, direction hints and
proper velocities, a case filter, one case that fails validation.

Exact equality: loading is parsing and sorting."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

CSV = os.path.join(GOLDEN, "ref_seed_schedule_input.csv")
BOUNDS = (1.0e4, 1.0e9, 0.0, 1000.0, 0.0, 8000.0)


@pytest.fixture(scope="module")
def gpu():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu as g
    build.build()
    return g


def test_load_matches_reference(gpu):
    ref = np.load(os.path.join(GOLDEN, "ref_seed_schedule_events.npy"))
    checks = np.load(os.path.join(GOLDEN, "ref_seed_schedule_checks.npy")).ravel()
    s = gpu.SeedSchedule(CSV, "C2")
    e = s.events()
    assert len(e) == len(ref)
    cols = ("macro_index", "species_id", "time_s", "x_m", "y_m", "z_m", "r_m", "kinetic_energy_eV", "ux", "uy", "uz",
            "weight")
    for i, c in enumerate(cols):
        np.testing.assert_array_equal(e[c].astype(np.float64), ref[:, i], err_msg=c)
    assert len(gpu.SeedSchedule(CSV, "")) == int(checks[0])
    s.validate(*BOUNDS)
    bad = gpu.SeedSchedule(CSV, "BAD")
    assert len(bad) == int(checks[2]) and checks[3] == 0.0
    with pytest.raises(gpu.RreaGpuError) as err:
        bad.validate(*BOUNDS)
    assert err.value.status == 1 and "r_m" in str(err.value)


def test_validation_bounds(gpu):
    s = gpu.SeedSchedule(CSV, "C2")
    with pytest.raises(gpu.RreaGpuError):
        s.validate(1.0e4, 1.0e9, 0.0, 500.0, 0.0, 8000.0)   # seeds beyond r = 500 m
    with pytest.raises(gpu.RreaGpuError):
        s.validate(2.0e6, 1.0e9, 0.0, 1000.0, 0.0, 8000.0)  # energies below 2 MeV
    with pytest.raises(gpu.RreaGpuError):
        s.validate(0.0, 1.0e9, 0.0, 1000.0, 0.0, 8000.0)    # invalid bounds


@pytest.mark.parametrize("text,needle", [
    ("case_id,time_s\nC2,0\n", "missing seed schedule column"),
    ("case_id,case_id\n", "duplicate seed schedule column"),
    ("case_id,time_s,x_m,y_m,z_m,r_m,kinetic_energy_eV,ux,uy,uz,weight_real_electrons\n"
     "C2,1e-9,0,0,1,0,1e6,0,0,-1,abc\n", "invalid numeric value"),
])
def test_malformed_schedules(gpu, tmp_path, text, needle):
    p = tmp_path / "seeds.csv"
    p.write_text(text)
    with pytest.raises(gpu.RreaGpuError) as err:
        gpu.SeedSchedule(p, "")
    assert needle in str(err.value)
    with pytest.raises(gpu.RreaGpuError):
        gpu.SeedSchedule(tmp_path / "missing.csv", "")


def test_host_calls_refuse_bad_arguments(gpu):
    """The host-only seed-schedule entry points return status codes for
    null handles and short buffers (no GPU involved)."""
    import ctypes

    lib = gpu.load_library()
    n = ctypes.c_int64()
    assert lib.rrea_gpu_seed_schedule_size(None, ctypes.byref(n)) == 1
    assert lib.rrea_gpu_seed_schedule_validate(None, 1.0e4, 1.0e9, 0.0, 1.0, 0.0, 1.0) == 1
    assert lib.rrea_gpu_seed_schedule_free(None) == 0
    out = ctypes.c_void_p()
    assert lib.rrea_gpu_seed_schedule_load(None, b"", ctypes.byref(out)) == 1
    s = gpu.SeedSchedule(CSV, "C2")
    buf = np.zeros(3, dtype=gpu.SEED_EVENT_DTYPE)
    assert lib.rrea_gpu_seed_schedule_events(s.handle, ctypes.c_void_p(buf.ctypes.data), 3, ctypes.byref(n)) == 8
    assert n.value == len(s)
