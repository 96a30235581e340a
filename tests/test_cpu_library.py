"""CPU-side checks of the shipped library: it builds for sm_103a, loads
without a GPU, and exports every entry point include/rrea_gpu.h declares.
No compute call is made here."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def gpu():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu
    build.build()
    return gpu


def declared_entry_points():
    text = open(os.path.join(ROOT, "include", "rrea_gpu.h")).read()
    return sorted(set(re.findall(r"\b(rrea_gpu_[a-z_]+)\s*\(", text)))


def test_header_declares_expected_symbols(gpu):
    assert set(declared_entry_points()) == set(gpu.EXPORTED_SYMBOLS)


def test_library_exports_every_declared_symbol(gpu):
    lib = ctypes.CDLL(gpu.LIB_PATH)
    for name in declared_entry_points():
        assert hasattr(lib, name), name


def test_default_config_matches_reference_defaults(gpu):
    cfg = gpu.default_config()
    # RreaParticleInteractionConfig defaults (RreaParticleInteraction.H:1576-1596)
    assert cfg.max_optical_depth_per_substep == 0.05
    assert cfg.max_subcycles == 256
    assert cfg.strict_transport_guards == 1
    assert cfg.max_gs_collisions_per_substep == 32.0
    assert cfg.gs_total_collision_cap == 1024.0
    assert cfg.max_field_impulse_fraction == 0.1
    assert cfg.field_impulse_floor_eV == 1.0e4
    assert cfg.density_ratio == 1.0


def test_missing_library_fails_loudly(tmp_path):
    from rrea_feedback_warpx_amrex_geant4_gb300 import gpu
    with pytest.raises(RuntimeError):
        gpu._lib_saved = gpu._lib
        try:
            gpu._lib = None
            gpu.load_library(str(tmp_path / "absent.so"))
        finally:
            gpu._lib = gpu._lib_saved


def test_structure_layouts_match_header(gpu):
    from oracle import oracle as o
    assert ctypes.sizeof(gpu.RreaGpuConfig) == ctypes.sizeof(o.RreaGpuConfig) == 136
    assert gpu.SECONDARY_DTYPE.itemsize == 4 * 4 + 8 * 3 + 8 * 9


def test_noalloc_source_calls_no_allocator():
    """The allocation-free ordering entry point keeps its scratch in a
    file-scope device array and never calls an allocating routine."""
    src = open(os.path.join(ROOT, "rrea_feedback_warpx_amrex_geant4_gb300", "csrc", "rrea_noalloc.cu")).read()
    code = "\n".join(line.split("//")[0] for line in src.splitlines())
    for banned in ("cudaMalloc", "cudaFree", "cudaHostAlloc", "cudaMallocAsync", "malloc(", "new ", "torch"):
        assert banned not in code, banned
    assert "static __device__ __align__(256)" in code
    assert "cudaGetSymbolAddress" in code



def test_population_projection_matches_reference_rule(gpu):
    """RreaStrictPopulationProjection (O/RreaParticleInteraction.H:1257-1275);
    host-only, no GPU call."""
    P = gpu.population_projection
    assert P(100, 10, 50, 140) == (True, 140)          # inclusive ceiling
    assert P(100, 10, 50, 140, True) == (False, 140)   # equality rejected
    assert P(100, 10, 51, 140) == (False, 141)
    assert P(5, 6, 0, 10)[0] is False                   # removals > current
    big = 2 ** 64 - 1
    assert P(big, 0, 1, big) == (False, big)            # saturates on overflow
    assert P(0, 0, 0, 0) == (True, 0)


def test_library_leaves_no_internal_symbol_undefined(gpu):
    """Every launcher and kernel the library calls is defined in it: an
    internal symbol left undefined would only surface when the library is
    loaded on the GPU machine."""
    import shutil
    import subprocess

    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm is not available")
    out = subprocess.run([nm, "-D", "--undefined-only", gpu.LIB_PATH], capture_output=True, text=True, check=True)
    internal = [line for line in out.stdout.splitlines() if "rrea" in line]
    assert not internal, internal


def test_one_call_apply_and_merge_refuse_bad_arguments(gpu):
    """rrea_gpu_apply_step and rrea_gpu_population_merge_resident check their
    arguments before any device work: a null context (or a negative survivor
    capacity) is RREA_GPU_ERR_ARGUMENT, on a box without a GPU too."""
    lib = gpu.load_library()
    n = ctypes.c_int64()
    stats = (ctypes.c_int64 * 5)()
    arg = 1  # RREA_GPU_ERR_ARGUMENT
    assert lib.rrea_gpu_apply_step(None, None, None, None, 0, 0.0, 5e-10, None, 0, ctypes.byref(n)) == arg
    assert lib.rrea_gpu_apply_step(None, None, None, None, 0, 0.0, 5e-10, None, -1, ctypes.byref(n)) == arg
    assert lib.rrea_gpu_population_merge_resident(None, 0, 10, 0, stats) == arg
    assert lib.rrea_gpu_population_merge_resident(None, 0, -1, 0, stats) == arg
