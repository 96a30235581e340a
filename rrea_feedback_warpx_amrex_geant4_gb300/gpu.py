"""Python host side of the GB300 kinetic step: a thin ctypes binding over the
C-ABI in include/rrea_gpu.h (lib/librrea_gpu.so).

The names mirror the reference overlay: ``RreaParticleInteraction.Apply``
runs the per-timestep transport of one electron tile the way
``rrea::warpx::RreaParticleInteraction::Apply`` does
(native_amrex_rrea/warpx_overlay/Source/Rrea/RreaParticleInteraction.H:1609-1623),
and every non-OK status raises, as the reference aborts.  There is no CPU
fallback: a missing library raises at load.
"""
import ctypes
import os

import numpy as np

from . import DEFAULT_TABLES, PACKAGE_DIR

# RREA_GPU_LIB selects a parity-study build of the library (see build.py)
LIB_PATH = os.environ.get("RREA_GPU_LIB") or os.path.join(PACKAGE_DIR, "lib", "librrea_gpu.so")

STATUS_NAMES = {
    0: "OK", 1: "ERR_ARGUMENT", 2: "ERR_TABLES", 3: "ERR_CUDA", 4: "ERR_RANGE", 5: "ERR_GEOMETRY",
    6: "ERR_RNG_OVERFLOW", 7: "ERR_GUARD", 8: "ERR_CAPACITY", 9: "ERR_INVALID_STATE", 10: "ERR_NOT_READY",
}

_D = ctypes.POINTER(ctypes.c_double)


class RreaGpuConfig(ctypes.Structure):
    """rrea_gpu_config (include/rrea_gpu.h)."""

    _fields_ = [
        ("r_lo", ctypes.c_double), ("r_hi", ctypes.c_double),
        ("z_lo", ctypes.c_double), ("z_hi", ctypes.c_double),
        ("nr", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("periodic_z", ctypes.c_int32), ("strict_transport_guards", ctypes.c_int32),
        ("density_ratio", ctypes.c_double),
        ("low_energy_cutoff_eV", ctypes.c_double), ("photon_cutoff_eV", ctypes.c_double),
        ("max_optical_depth_per_substep", ctypes.c_double), ("max_subcycles", ctypes.c_uint64),
        ("max_gs_collisions_per_substep", ctypes.c_double), ("gs_total_collision_cap", ctypes.c_double),
        ("max_field_impulse_fraction", ctypes.c_double), ("field_impulse_floor_eV", ctypes.c_double),
        ("rng_seed", ctypes.c_uint64),
        ("debug_disable_hard_moller", ctypes.c_int32), ("reserved0", ctypes.c_int32),
    ]


class RreaFluidConfig(ctypes.Structure):
    """Mirror of rrea_gpu_fluid_config (include/rrea_gpu.h)."""

    _fields_ = [(name, ctypes.c_double) for name in (
        "electron_mobility_m2_per_vs", "positive_ion_mobility_m2_per_vs", "negative_ion_mobility_m2_per_vs",
        "positive_ion_reduced_mobility_stp_m2_per_vs", "negative_ion_reduced_mobility_stp_m2_per_vs",
        "ion_mobility_density_ratio_floor", "ion_drift_cfl", "transport_density_ratio", "attachment_frequency_s",
        "electron_ion_recombination_coefficient_m3_per_s", "ion_ion_recombination_coefficient_m3_per_s",
        "detachment_frequency_s")] + [(name, ctypes.c_int32) for name in (
        "ion_drift_enable", "electron_drift_enable", "electron_mobility_model", "ion_mobility_model",
        "attachment_model", "material_min_substeps", "material_max_substeps", "reserved0")] + [
        (name, ctypes.c_double) for name in (
            "material_conduction_target", "material_conduction_guard", "material_diffusion_target",
            "material_diffusion_guard", "material_reaction_target", "material_reaction_guard")]


MOBILITY_ABSOLUTE, MOBILITY_EN_TABLE_FLUX, MOBILITY_REDUCED_STP = 0, 1, 2   # RREA_GPU_MOBILITY_*
ATTACHMENT_CONSTANT, ATTACHMENT_EN_TABLE = 0, 1                             # RREA_GPU_ATTACHMENT_*
FLUID_TRANSPORT_DIAG = ("max_face_conductivity", "max_diffusion_number", "unlimited_max_outgoing_cfl",
                        "min_outflow_scale", "limited_outflow_fraction", "limited_electron_number_fraction",
                        "max_outgoing_cfl", "max_drift_speed", "cfl_dt", "pos_center_r", "pos_center_z",
                        "neg_center_r", "neg_center_z", "density_ratio_at_pos_center")
FLUID_COUPLED_DIAG = ("substeps", "full_conduction", "full_diffusion", "full_reaction", "max_reaction_number",
                      "max_dt_sigma", "max_diffusion_number", "max_residual")
FLUID_REDUCED_COLUMNS = ("total_ne_low", "total_n_pos", "total_n_neg", "N_low_e_real", "N_pos_real", "N_neg_real",
                         "rho_fluid_C", "total_rho_fluid", "total_S_low_electron", "total_S_positive_ion",
                         "total_S_direct_negative_ion", "ionization_event_count", "total_energy_loss_ev_m3",
                         "max_ne_low", "max_sigma", "min_tau_m")
FLUID_CLOSURE_DIAG = ("min_en_td", "max_en_td", "held_below", "above_range", "invalid", "electron_count",
                      "held_below_electron_count", "electron_source_rate")


class RreaGpuTile(ctypes.Structure):
    """rrea_gpu_tile (include/rrea_gpu.h)."""

    _fields_ = [("n", ctypes.c_int64)] + [
        (name, _D) for name in ("r", "z", "theta", "ux", "uy", "uz", "w",
                                "prev_r", "prev_z", "prev_theta", "prev_ux", "prev_uy", "prev_uz")
    ] + [("id", ctypes.POINTER(ctypes.c_int64)), ("cpu", ctypes.POINTER(ctypes.c_int32))]


TILE_FIELDS = ("r", "z", "theta", "ux", "uy", "uz", "w",
               "prev_r", "prev_z", "prev_theta", "prev_ux", "prev_uy", "prev_uz")

SEED_EVENT_DTYPE = np.dtype([  # rrea_gpu_seed_event
    ("macro_index", "<i4"), ("species_id", "<i4"), ("time_s", "<f8"), ("x_m", "<f8"), ("y_m", "<f8"),
    ("z_m", "<f8"), ("r_m", "<f8"), ("kinetic_energy_eV", "<f8"), ("ux", "<f8"), ("uy", "<f8"), ("uz", "<f8"),
    ("weight", "<f8"),
])

SECONDARY_DTYPE = np.dtype([
    ("species", "<i4"), ("process", "<i4"), ("root_species", "<i4"), ("pad", "<i4"),
    ("parent_index", "<i8"), ("root_key", "<u8"), ("lineage", "<u8"),
    ("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("dir_x", "<f8"), ("dir_y", "<f8"), ("dir_z", "<f8"),
    ("weight", "<f8"), ("energy_eV", "<f8"), ("birth_fraction", "<f8"),
])

# Every entry point include/rrea_gpu.h declares.
EXPORTED_SYMBOLS = (
    "rrea_gpu_default_config", "rrea_gpu_create", "rrea_gpu_destroy", "rrea_gpu_load_tables",
    "rrea_gpu_set_field", "rrea_gpu_apply_electrons", "rrea_gpu_download_sources", "rrea_gpu_reset_sources",
    "rrea_gpu_download_diagnostics", "rrea_gpu_last_error", "rrea_gpu_stage_electrons",
    "rrea_gpu_step_electrons_resident", "rrea_gpu_fetch_electrons", "rrea_gpu_set_launch", "rrea_gpu_stream",
    "rrea_gpu_last_step_stats", "rrea_gpu_apply_photons", "rrea_gpu_stage_photons",
    "rrea_gpu_step_photons_resident", "rrea_gpu_fetch_photons", "rrea_gpu_order_secondaries_noalloc",
    "rrea_gpu_apply_positrons", "rrea_gpu_stage_positrons", "rrea_gpu_step_positrons_resident",
    "rrea_gpu_fetch_positrons", "rrea_gpu_reset_current", "rrea_gpu_download_current",
    "rrea_gpu_download_current_index", "rrea_gpu_advance_field", "rrea_gpu_download_field",
    "rrea_gpu_count_live", "rrea_gpu_population_projection", "rrea_gpu_drain_secondaries",
    "rrea_gpu_drain_resident", "rrea_gpu_fetch_survivors", "rrea_gpu_pending_secondaries",
    "rrea_gpu_last_drain_stats", "rrea_gpu_kernel_launches", "rrea_gpu_current_device",
    "rrea_gpu_advance_field_from_current", "rrea_gpu_selftest_math", "rrea_gpu_set_density_profile",
    "rrea_gpu_commit_survivors_resident", "rrea_gpu_compact_resident", "rrea_gpu_resident_count",
    "rrea_gpu_seed_schedule_load", "rrea_gpu_seed_schedule_free", "rrea_gpu_seed_schedule_size",
    "rrea_gpu_seed_schedule_events", "rrea_gpu_seed_schedule_validate", "rrea_gpu_seed_schedule_last_error",
    "rrea_gpu_inject_seeds_resident", "rrea_gpu_thin_cic_groups", "rrea_gpu_census_resident",
    "rrea_gpu_deposit_charge_resident", "rrea_gpu_population_thin_resident", "rrea_gpu_population_split_resident",
    "rrea_gpu_population_merge_resident", "rrea_gpu_apply_step",
    "rrea_gpu_default_fluid_config", "rrea_gpu_fluid_configure", "rrea_gpu_fluid_load_closure",
    "rrea_gpu_fluid_set_state", "rrea_gpu_fluid_get_state", "rrea_gpu_fluid_set_source_rates",
    "rrea_gpu_fluid_get_source_rates", "rrea_gpu_fluid_set_density_ratio", "rrea_gpu_fluid_set_closure_fields",
    "rrea_gpu_fluid_get_closure_fields", "rrea_gpu_fluid_take_sources", "rrea_gpu_fluid_react",
    "rrea_gpu_fluid_max_reaction_frequency", "rrea_gpu_fluid_conductivity", "rrea_gpu_fluid_charge_density",
    "rrea_gpu_fluid_evaluate_closure", "rrea_gpu_fluid_transport", "rrea_gpu_advance_field_coupled",
    "rrea_gpu_sources_device", "rrea_gpu_advance_field_coupled_from_current", "rrea_gpu_fluid_reductions",
    "rrea_gpu_set_schedule", "rrea_gpu_ensemble_configure", "rrea_gpu_ensemble_partition", "rrea_gpu_ensemble_retire",
    "rrea_gpu_ensemble_census", "rrea_gpu_ensemble_population_thin", "rrea_gpu_ensemble_population_thin_all",
    "rrea_gpu_default_adjoint_config", "rrea_gpu_adjoint_stage", "rrea_gpu_adjoint_forward",
    "rrea_gpu_adjoint_forward_frozen",
    "rrea_gpu_adjoint_backward", "rrea_gpu_adjoint_final_state", "rrea_gpu_set_planes", "rrea_gpu_plane_flux",
    "rrea_gpu_restore_plane_flux",
)
NOALLOC_MAX_PARENTS = 1 << 18  # RREA_GPU_NOALLOC_MAX_PARENTS
SPECIES_ELECTRON, SPECIES_POSITRON, SPECIES_PHOTON = 0, 1, 2  # RREA_SPECIES_*

_lib = None


class RreaGpuError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"rrea_gpu status {status} ({STATUS_NAMES.get(status, '?')}): {message}")
        self.status = status


def load_library(path=LIB_PATH):
    """Loads the in-tree CUDA library; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: run __graft_entry__.build() (no CPU fallback exists)")
    lib = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    lib.rrea_gpu_default_config.argtypes = [ctypes.POINTER(RreaGpuConfig)]
    lib.rrea_gpu_default_config.restype = None
    lib.rrea_gpu_create.argtypes = [ctypes.POINTER(RreaGpuConfig), ctypes.c_int64, ctypes.POINTER(vp)]
    lib.rrea_gpu_destroy.argtypes = [vp]
    lib.rrea_gpu_load_tables.argtypes = [vp, ctypes.c_char_p]
    lib.rrea_gpu_set_field.argtypes = [vp, _D, _D, _D, _D, _D]
    lib.rrea_gpu_set_density_profile.argtypes = [vp, _D, _D, ctypes.c_int64, ctypes.c_double, ctypes.c_double]
    lib.rrea_gpu_apply_electrons.argtypes = [vp, ctypes.POINTER(RreaGpuTile), ctypes.c_int32, ctypes.c_double,
                                             ctypes.c_double, vp, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]
    lib.rrea_gpu_apply_photons.argtypes = lib.rrea_gpu_apply_electrons.argtypes
    lib.rrea_gpu_apply_positrons.argtypes = lib.rrea_gpu_apply_electrons.argtypes
    lib.rrea_gpu_stage_positrons.argtypes = [vp, ctypes.POINTER(RreaGpuTile)]
    lib.rrea_gpu_step_positrons_resident.argtypes = [vp, ctypes.c_int32, ctypes.c_double,
                                                     ctypes.POINTER(ctypes.c_int64)]
    lib.rrea_gpu_fetch_positrons.argtypes = [vp, ctypes.POINTER(RreaGpuTile)]
    lib.rrea_gpu_stage_photons.argtypes = [vp, ctypes.POINTER(RreaGpuTile)]
    lib.rrea_gpu_step_photons_resident.argtypes = [vp, ctypes.c_int32, ctypes.c_double,
                                                   ctypes.POINTER(ctypes.c_int64)]
    lib.rrea_gpu_fetch_photons.argtypes = [vp, ctypes.POINTER(RreaGpuTile)]
    lib.rrea_gpu_order_secondaries_noalloc.argtypes = [vp, ctypes.c_int64, vp, ctypes.c_int64, vp, vp,
                                                       ctypes.c_char_p, ctypes.c_size_t]
    lib.rrea_gpu_advance_field.argtypes = [vp, ctypes.c_double, ctypes.c_int32]
    lib.rrea_gpu_count_live.argtypes = [vp, ctypes.c_int32, ctypes.POINTER(ctypes.c_int64)]
    lib.rrea_gpu_population_projection.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                                   ctypes.c_uint64, ctypes.c_int32, ctypes.POINTER(ctypes.c_uint64)]
    lib.rrea_gpu_download_field.argtypes = [vp, _D, _D, _D]
    _i64p = ctypes.POINTER(ctypes.c_int64)
    lib.rrea_gpu_drain_secondaries.argtypes = [vp, vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_double, vp,
                                               ctypes.c_int64, _i64p]
    lib.rrea_gpu_drain_resident.argtypes = [vp, ctypes.c_int32, ctypes.c_double, _i64p]
    lib.rrea_gpu_fetch_survivors.argtypes = [vp, vp, ctypes.c_int64, _i64p]
    lib.rrea_gpu_pending_secondaries.argtypes = [vp, _i64p, ctypes.c_int32]
    lib.rrea_gpu_commit_survivors_resident.argtypes = [vp, _i64p]
    lib.rrea_gpu_seed_schedule_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(vp)]
    lib.rrea_gpu_seed_schedule_free.argtypes = [vp]
    lib.rrea_gpu_seed_schedule_size.argtypes = [vp, _i64p]
    lib.rrea_gpu_seed_schedule_events.argtypes = [vp, vp, ctypes.c_int64, _i64p]
    lib.rrea_gpu_seed_schedule_validate.argtypes = [vp] + [ctypes.c_double] * 6
    lib.rrea_gpu_seed_schedule_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    lib.rrea_gpu_seed_schedule_last_error.restype = None
    lib.rrea_gpu_inject_seeds_resident.argtypes = [vp, vp, ctypes.c_double, ctypes.c_double, _i64p]
    lib.rrea_gpu_thin_cic_groups.argtypes = [vp, _D, _D, _D, _i64p, ctypes.c_int64, _i64p,
                                             ctypes.POINTER(ctypes.c_uint64), _i64p, _i64p,
                                             ctypes.POINTER(ctypes.c_int32), _i64p]
    lib.rrea_gpu_compact_resident.argtypes = [vp, ctypes.c_int32, _i64p]
    lib.rrea_gpu_deposit_charge_resident.argtypes = [vp, _D]
    lib.rrea_gpu_population_thin_resident.argtypes = [vp, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32,
                                                      ctypes.c_uint64, vp, ctypes.c_int64, _i64p]
    lib.rrea_gpu_population_split_resident.argtypes = [vp, ctypes.c_int32, ctypes.c_int64, ctypes.c_double, _i64p]
    lib.rrea_gpu_population_merge_resident.argtypes = [vp, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, _i64p]
    lib.rrea_gpu_apply_step.argtypes = [vp, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                        ctypes.c_double, ctypes.c_double, vp, ctypes.c_int64, _i64p]
    lib.rrea_gpu_census_resident.argtypes = [vp, ctypes.c_int32, _D, ctypes.c_int32, _D, ctypes.c_int32, _D]
    lib.rrea_gpu_resident_count.argtypes = [vp, ctypes.c_int32, _i64p]
    lib.rrea_gpu_last_drain_stats.argtypes = [vp, _i64p, _i64p]
    lib.rrea_gpu_kernel_launches.argtypes = [ctypes.POINTER(ctypes.c_uint64)]
    lib.rrea_gpu_current_device.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp)]
    lib.rrea_gpu_advance_field_from_current.argtypes = [vp, ctypes.c_double, ctypes.c_int32]
    lib.rrea_gpu_selftest_math.argtypes = [vp, ctypes.c_int32, _D, ctypes.c_int64, _D, _D]
    lib.rrea_gpu_reset_current.argtypes = [vp]
    lib.rrea_gpu_download_current.argtypes = [vp, _D, _D]
    lib.rrea_gpu_download_current_index.argtypes = [vp, _D, _D, _D]
    lib.rrea_gpu_download_sources.argtypes = [vp, _D]
    lib.rrea_gpu_reset_sources.argtypes = [vp]
    lib.rrea_gpu_download_diagnostics.argtypes = [vp, ctypes.c_int64, ctypes.POINTER(ctypes.c_uint64),
                                                  ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int32)]
    lib.rrea_gpu_last_error.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
    lib.rrea_gpu_last_error.restype = None
    lib.rrea_gpu_stage_electrons.argtypes = [vp, ctypes.POINTER(RreaGpuTile)]
    lib.rrea_gpu_step_electrons_resident.argtypes = [vp, ctypes.c_int32, ctypes.c_double,
                                                     ctypes.POINTER(ctypes.c_int64)]
    lib.rrea_gpu_fetch_electrons.argtypes = [vp, ctypes.POINTER(RreaGpuTile)]
    lib.rrea_gpu_set_launch.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]
    lib.rrea_gpu_stream.argtypes = [vp, ctypes.POINTER(vp)]
    lib.rrea_gpu_last_step_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                             ctypes.POINTER(ctypes.c_double)]
    _fc = ctypes.POINTER(RreaFluidConfig)
    lib.rrea_gpu_default_fluid_config.argtypes = [_fc]
    lib.rrea_gpu_default_fluid_config.restype = None
    lib.rrea_gpu_fluid_configure.argtypes = [vp, _fc]
    lib.rrea_gpu_fluid_load_closure.argtypes = [vp, ctypes.c_char_p]
    lib.rrea_gpu_fluid_set_state.argtypes = [vp, _D, _D, _D, _D]
    lib.rrea_gpu_fluid_get_state.argtypes = [vp, _D, _D, _D, _D, _D, _D]
    lib.rrea_gpu_fluid_set_source_rates.argtypes = [vp, _D, _D, _D]
    lib.rrea_gpu_fluid_get_source_rates.argtypes = [vp, _D, _D, _D]
    lib.rrea_gpu_fluid_set_density_ratio.argtypes = [vp, _D]
    lib.rrea_gpu_fluid_set_closure_fields.argtypes = [vp, _D, _D, _D]
    lib.rrea_gpu_fluid_get_closure_fields.argtypes = [vp, _D, _D, _D]
    lib.rrea_gpu_fluid_take_sources.argtypes = [vp, ctypes.c_double]
    lib.rrea_gpu_fluid_react.argtypes = [vp, ctypes.c_double, ctypes.c_int32, _D]
    lib.rrea_gpu_fluid_max_reaction_frequency.argtypes = [vp, _D]
    lib.rrea_gpu_fluid_conductivity.argtypes = [vp]
    lib.rrea_gpu_fluid_charge_density.argtypes = [vp]
    lib.rrea_gpu_fluid_evaluate_closure.argtypes = [vp, _D, _D, _D]
    lib.rrea_gpu_fluid_transport.argtypes = [vp, ctypes.c_double, _D, _D, _D, _D, _D]
    lib.rrea_gpu_advance_field_coupled.argtypes = [vp, ctypes.c_double, _D]
    lib.rrea_gpu_set_schedule.argtypes = [vp, ctypes.c_int32]
    lib.rrea_gpu_set_planes.argtypes = [vp, _D, ctypes.c_int32]
    lib.rrea_gpu_plane_flux.argtypes = [vp, _D]
    lib.rrea_gpu_restore_plane_flux.argtypes = [vp, _D]
    lib.rrea_gpu_sources_device.argtypes = [vp, ctypes.POINTER(vp)]
    lib.rrea_gpu_fluid_reductions.argtypes = [vp, ctypes.c_double, _D]
    lib.rrea_gpu_advance_field_coupled_from_current.argtypes = [vp, ctypes.c_double, _D]
    lib.rrea_gpu_ensemble_configure.argtypes = [vp, ctypes.c_int32, _D]
    lib.rrea_gpu_ensemble_partition.argtypes = [vp, ctypes.c_int32, _i64p]
    lib.rrea_gpu_ensemble_retire.argtypes = [vp, ctypes.c_int32]
    lib.rrea_gpu_ensemble_census.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, _D, ctypes.c_int32, _D,
                                             ctypes.c_int32, _D]
    lib.rrea_gpu_ensemble_population_thin.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int64,
                                                      ctypes.c_int32, ctypes.c_uint64, _i64p]
    lib.rrea_gpu_ensemble_population_thin_all.argtypes = [vp, ctypes.c_int32, _i64p, ctypes.c_int32,
                                                          ctypes.c_uint64, _i64p, _i64p]
    for name in EXPORTED_SYMBOLS:
        fn = getattr(lib, name)
        if fn.restype is not None and name not in ("rrea_gpu_default_config", "rrea_gpu_last_error",
                                                   "rrea_gpu_default_fluid_config",
                                                   "rrea_gpu_default_adjoint_config"):
            fn.restype = ctypes.c_int
    _lib = lib
    return lib


def kernel_launches():
    """Kernels the library has launched in this process."""
    n = ctypes.c_uint64()
    status = load_library().rrea_gpu_kernel_launches(ctypes.byref(n))
    if status != 0:
        raise RreaGpuError(status, "kernel launch count")
    return n.value


def default_config(**overrides):
    cfg = RreaGpuConfig()
    load_library().rrea_gpu_default_config(ctypes.byref(cfg))
    for k, v in overrides.items():
        setattr(cfg, k, v)
    return cfg


def default_fluid_config(**overrides):
    """rrea_gpu_default_fluid_config (the reference's LowEnergyFluidConfig and
    material substep defaults), then `overrides`."""
    cfg = RreaFluidConfig()
    load_library().rrea_gpu_default_fluid_config(ctypes.byref(cfg))
    for k, v in overrides.items():
        setattr(cfg, k, v)
    return cfg


def _opt(a, n=None):
    """A contiguous float64 copy of `a` (or None) and its pointer."""
    if a is None:
        return None, None
    arr = np.ascontiguousarray(np.ravel(a), dtype=np.float64).copy()
    if n is not None and arr.size != n:
        raise ValueError(f"expected {n} values, got {arr.size}")
    return arr, arr.ctypes.data_as(_D)


def tile_struct(arrays):
    """Builds an rrea_gpu_tile over a dict of contiguous numpy arrays."""
    t = RreaGpuTile()
    t.n = int(arrays["id"].shape[0])
    for name in TILE_FIELDS:
        a = arrays[name]
        assert a.dtype == np.float64 and a.flags.c_contiguous, name
        setattr(t, name, a.ctypes.data_as(_D))
    t.id = arrays["id"].ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    t.cpu = arrays["cpu"].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    return t


class SeedSchedule:
    """The seed schedule CSV adapter (RreaSeedSchedule): load, list, validate.
    Host-only; RreaGpuContext.inject_seeds appends its windows to the
    resident tiles."""

    def __init__(self, path, case_id=""):
        self.lib = load_library()
        h = ctypes.c_void_p()
        self._check(self.lib.rrea_gpu_seed_schedule_load(str(path).encode(), case_id.encode(), ctypes.byref(h)))
        self.handle = h

    def _check(self, status):
        if status != 0:
            buf = ctypes.create_string_buffer(1024)
            self.lib.rrea_gpu_seed_schedule_last_error(buf, 1024)
            raise RreaGpuError(status, buf.value.decode())

    def __len__(self):
        n = ctypes.c_int64()
        self._check(self.lib.rrea_gpu_seed_schedule_size(self.handle, ctypes.byref(n)))
        return n.value

    def events(self):
        out = np.zeros(len(self), dtype=SEED_EVENT_DTYPE)
        n = ctypes.c_int64()
        self._check(self.lib.rrea_gpu_seed_schedule_events(self.handle, ctypes.c_void_p(out.ctypes.data) if len(out)
                                                           else None, len(out), ctypes.byref(n)))
        return out

    def validate(self, electron_min_energy_eV, electron_max_energy_eV, radial_min_m, radial_max_m, axial_min_m,
                 axial_max_m):
        self._check(self.lib.rrea_gpu_seed_schedule_validate(self.handle, electron_min_energy_eV,
                                                             electron_max_energy_eV, radial_min_m, radial_max_m,
                                                             axial_min_m, axial_max_m))

    def close(self):
        if self.handle:
            self.lib.rrea_gpu_seed_schedule_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RreaGpuContext:
    """Owns one rrea_gpu_ctx (device arena, field, resident tile, buffers)."""

    def __init__(self, config, capacity):
        self.lib = load_library()
        self.config = config
        self.capacity = int(capacity)
        # the drop-in phases' secondaries land here (reused: its pages are
        # mapped once, not on every call); callers get a copy of the filled part
        self._sec_buf = None
        self._surv_buf = None
        handle = ctypes.c_void_p()
        self._check(self.lib.rrea_gpu_create(ctypes.byref(config), self.capacity, ctypes.byref(handle)), None)
        self.handle = handle

    def _check(self, status, handle="self"):
        if status != 0:
            msg = ""
            if handle is not None and getattr(self, "handle", None) is not None:
                buf = ctypes.create_string_buffer(2048)
                self.lib.rrea_gpu_last_error(self.handle, buf, 2048)
                msg = buf.value.decode(errors="replace")
            raise RreaGpuError(status, msg)

    def close(self):
        if getattr(self, "handle", None) is not None:
            self.lib.rrea_gpu_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load_tables(self, path=DEFAULT_TABLES):
        self._check(self.lib.rrea_gpu_load_tables(self.handle, path.encode()))

    def set_field(self, er, ez, bt, amb_er, amb_ez):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (er, ez, bt, amb_er, amb_ez)]
        self._check(self.lib.rrea_gpu_set_field(self.handle, *[a.ctypes.data_as(_D) for a in arrs]))

    PLANE_VALUES = ("all_tracked_up_weight", "all_tracked_down_weight", "local_runaway_up_weight",
                    "local_runaway_down_weight", "e_ge_1mev_up_weight", "e_ge_1mev_down_weight",
                    "local_runaway_up_r_weighted_m", "local_runaway_down_r_weighted_m",
                    "local_runaway_up_r2_weighted_m2", "local_runaway_down_r2_weighted_m2")

    def set_planes(self, plane_z_m=()):
        """Turns on the plane-crossing diagnostic at the given strictly
        increasing z (an empty list turns it off); accumulators start at 0."""
        z = np.ascontiguousarray(plane_z_m, dtype=np.float64)
        self._check(self.lib.rrea_gpu_set_planes(self.handle, z.ctypes.data_as(_D) if z.size else None, z.size))
        self.n_planes = int(z.size)

    def plane_flux(self):
        """The cumulative accumulators, (n_planes, 10) in PLANE_VALUES order."""
        out = np.zeros((getattr(self, "n_planes", 0), len(self.PLANE_VALUES)))
        if out.size:
            self._check(self.lib.rrea_gpu_plane_flux(self.handle, out.ctypes.data_as(_D)))
        return out

    def restore_plane_flux(self, values=None):
        if values is None:
            self._check(self.lib.rrea_gpu_restore_plane_flux(self.handle, None))
            return
        v = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        if v.size != getattr(self, "n_planes", 0) * len(self.PLANE_VALUES):
            raise ValueError("10 values per plane")
        self._check(self.lib.rrea_gpu_restore_plane_flux(self.handle, v.ctypes.data_as(_D)))

    def set_density_profile(self, altitude_m=None, density_kg_m3=None, altitude_msl_at_z0_m=0.0,
                            reference_density_kg_m3=0.0):
        """Binds the altitude density profile (rrea.air_density_model=
        altitude_profile): the transport density ratio at z is the profile
        density at altitude_msl_at_z0_m + z over reference_density_kg_m3.
        No arrays restores the configured uniform ratio."""
        if altitude_m is None:
            self._check(self.lib.rrea_gpu_set_density_profile(self.handle, None, None, 0, 0.0, 0.0))
            return
        alt = np.ascontiguousarray(altitude_m, dtype=np.float64)
        dens = np.ascontiguousarray(density_kg_m3, dtype=np.float64)
        if alt.shape != dens.shape:
            raise ValueError("altitude and density columns differ in length")
        self._check(self.lib.rrea_gpu_set_density_profile(self.handle, alt.ctypes.data_as(_D), dens.ctypes.data_as(_D),
                                                          alt.shape[0], altitude_msl_at_z0_m,
                                                          reference_density_kg_m3))

    def set_launch(self, threads_per_block=128, blocks_per_sm=16, diagnostics=True):
        self._check(self.lib.rrea_gpu_set_launch(self.handle, threads_per_block, blocks_per_sm, int(diagnostics)))

    def _apply(self, fn, arrays, step, dt_s, time_s, want_secondaries):
        t = tile_struct(arrays)
        n_sec = ctypes.c_int64()
        cap = 2 * self.capacity + 4096 if want_secondaries else 0
        ptr = None
        if want_secondaries:
            if self._sec_buf is None or len(self._sec_buf) < cap:
                self._sec_buf = np.empty(cap, dtype=SECONDARY_DTYPE)
            ptr = ctypes.c_void_p(self._sec_buf.ctypes.data)
        self._check(fn(self.handle, ctypes.byref(t), int(step), float(time_s), float(dt_s), ptr, cap,
                       ctypes.byref(n_sec)))
        return self._sec_buf[: n_sec.value].copy() if want_secondaries else n_sec.value

    def apply_electrons(self, arrays, step, dt_s, time_s=0.0, want_secondaries=True):
        """Drop-in electron phase on host arrays (modified in place).
        Returns the ordered secondaries as a structured array."""
        return self._apply(self.lib.rrea_gpu_apply_electrons, arrays, step, dt_s, time_s, want_secondaries)

    def apply_step(self, electrons, photons, positrons, step, dt_s, time_s=0.0):
        """Apply in one call: the three phases on host tiles (modified in
        place; None skips a species) and the transient FIFO of their
        secondaries on the device.  Returns the survivors in FIFO order."""
        tiles = [tile_struct(a) if a is not None else None for a in (electrons, photons, positrons)]
        refs = [ctypes.byref(t) if t is not None else None for t in tiles]
        cap = 2 * self.capacity + 4096
        if self._surv_buf is None or len(self._surv_buf) < cap:
            self._surv_buf = np.empty(cap, dtype=SECONDARY_DTYPE)
        n = ctypes.c_int64()
        self._check(self.lib.rrea_gpu_apply_step(self.handle, refs[0], refs[1], refs[2], int(step), float(time_s),
                                                 float(dt_s), ctypes.c_void_p(self._surv_buf.ctypes.data), cap,
                                                 ctypes.byref(n)))
        return self._surv_buf[: n.value].copy()

    def apply_positrons(self, arrays, step, dt_s, time_s=0.0, want_secondaries=True):
        """Drop-in positron phase on host arrays (modified in place)."""
        return self._apply(self.lib.rrea_gpu_apply_positrons, arrays, step, dt_s, time_s, want_secondaries)

    def stage_positrons(self, arrays):
        self._check(self.lib.rrea_gpu_stage_positrons(self.handle, ctypes.byref(tile_struct(arrays))))

    def step_positrons_resident(self, step, dt_s):
        n_sec = ctypes.c_int64()
        self._check(self.lib.rrea_gpu_step_positrons_resident(self.handle, int(step), float(dt_s),
                                                              ctypes.byref(n_sec)))
        return n_sec.value

    def fetch_positrons(self, arrays):
        self._check(self.lib.rrea_gpu_fetch_positrons(self.handle, ctypes.byref(tile_struct(arrays))))

    def apply_photons(self, arrays, step, dt_s, time_s=0.0, want_secondaries=True):
        """Drop-in photon phase on host arrays (modified in place): (r, theta,
        z) is the pushed end point, prev_* the start, u the momentum in eV."""
        return self._apply(self.lib.rrea_gpu_apply_photons, arrays, step, dt_s, time_s, want_secondaries)

    def stage_photons(self, arrays):
        self._check(self.lib.rrea_gpu_stage_photons(self.handle, ctypes.byref(tile_struct(arrays))))

    def step_photons_resident(self, step, dt_s):
        n_sec = ctypes.c_int64()
        self._check(self.lib.rrea_gpu_step_photons_resident(self.handle, int(step), float(dt_s),
                                                            ctypes.byref(n_sec)))
        return n_sec.value

    def fetch_photons(self, arrays):
        self._check(self.lib.rrea_gpu_fetch_photons(self.handle, ctypes.byref(tile_struct(arrays))))

    def stage_electrons(self, arrays):
        self._check(self.lib.rrea_gpu_stage_electrons(self.handle, ctypes.byref(tile_struct(arrays))))

    def step_electrons_resident(self, step, dt_s):
        n_sec = ctypes.c_int64()
        self._check(self.lib.rrea_gpu_step_electrons_resident(self.handle, int(step), float(dt_s),
                                                              ctypes.byref(n_sec)))
        return n_sec.value

    def fetch_electrons(self, arrays):
        self._check(self.lib.rrea_gpu_fetch_electrons(self.handle, ctypes.byref(tile_struct(arrays))))

    def sources(self):
        c = self.config
        out = np.zeros(5 * c.nr * c.nz)
        self._check(self.lib.rrea_gpu_download_sources(self.handle, out.ctypes.data_as(_D)))
        return out.reshape(5, c.nz, c.nr)

    def reset_sources(self):
        self._check(self.lib.rrea_gpu_reset_sources(self.handle))

    def drain_secondaries(self, pending, step, dt_s):
        """DrainAndCommitSecondaries' transient FIFO over host records (a
        SECONDARY_DTYPE array in phase order); returns the survivors in FIFO
        order.  Discards the resident queue."""
        pending = np.ascontiguousarray(pending, dtype=SECONDARY_DTYPE)
        n = ctypes.c_int64()
        self._check(self.lib.rrea_gpu_drain_secondaries(
            self.handle, ctypes.c_void_p(pending.ctypes.data) if len(pending) else None, len(pending), int(step),
            float(dt_s), None, 0, ctypes.byref(n)))
        return self.fetch_survivors(n.value)

    def drain_resident(self, step, dt_s):
        """Drains the queue the resident phases filled; returns the survivor count."""
        n = ctypes.c_int64()
        self._check(self.lib.rrea_gpu_drain_resident(self.handle, int(step), float(dt_s), ctypes.byref(n)))
        return n.value

    def fetch_survivors(self, n=None):
        if n is None:
            n = self.last_drain_stats()[1]
        out = np.zeros(int(n), dtype=SECONDARY_DTYPE)
        got = ctypes.c_int64()
        self._check(self.lib.rrea_gpu_fetch_survivors(self.handle, ctypes.c_void_p(out.ctypes.data) if n else None,
                                                      int(n), ctypes.byref(got)))
        return out[: got.value]

    def commit_survivors_resident(self):
        """Appends the last resident drain's survivors to the resident tiles;
        returns the counts committed per species (electron, positron, photon)."""
        out = np.zeros(3, dtype=np.int64)
        self._check(self.lib.rrea_gpu_commit_survivors_resident(
            self.handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        return out

    def compact_resident(self, species):
        """Drops the invalid particles of a resident tile (order kept); returns its new size."""
        n = ctypes.c_int64()
        self._check(self.lib.rrea_gpu_compact_resident(self.handle, species, ctypes.byref(n)))
        return n.value

    def inject_seeds(self, schedule, time_s, dt_s):
        """InjectScheduledSeeds on the resident tiles: the schedule's events in
        [time_s, time_s + dt_s); returns (electrons, positrons) added."""
        out = np.zeros(2, dtype=np.int64)
        self._check(self.lib.rrea_gpu_inject_seeds_resident(self.handle, schedule.handle, float(time_s), float(dt_s),
                                                            out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        return out

    def thin_cic_groups(self, fraction_r, fraction_z, weight, offsets, max_removals, keys):
        """Charge-exact thinning of CIC support groups (rows offsets[g] to
        offsets[g+1]); returns (weights, removed, draws, valid, capacity)."""
        fr = np.ascontiguousarray(fraction_r, dtype=np.float64)
        fz = np.ascontiguousarray(fraction_z, dtype=np.float64)
        w = np.array(weight, dtype=np.float64)
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        g = off.shape[0] - 1
        mx = np.ascontiguousarray(max_removals, dtype=np.int64)
        k = np.ascontiguousarray(keys, dtype=np.uint64)
        removed, draws, cap = (np.zeros(g, dtype=np.int64) for _ in range(3))
        valid = np.zeros(g, dtype=np.int32)
        i64 = ctypes.POINTER(ctypes.c_int64)
        self._check(self.lib.rrea_gpu_thin_cic_groups(
            self.handle, fr.ctypes.data_as(_D), fz.ctypes.data_as(_D), w.ctypes.data_as(_D), off.ctypes.data_as(i64),
            g, mx.ctypes.data_as(i64), k.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), removed.ctypes.data_as(i64),
            draws.ctypes.data_as(i64), valid.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), cap.ctypes.data_as(i64)))
        return w, removed, draws, valid, cap

    POPULATION_STATS = ("members", "live", "candidates", "supports", "capacity", "floor", "requested", "removed")

    def population_thin(self, species, target, step, salt=0, candidates=None):
        """Global CIC thinning plan of adaptive_resample_v1 over the resident
        tile of `species` and its candidates (the last drain's survivors, or
        a SECONDARY_DTYPE array updated in place); returns the plan's stats."""
        stats = np.zeros(8, dtype=np.int64)
        if candidates is None:
            ptr, n = None, 0
        else:
            assert candidates.dtype == SECONDARY_DTYPE and candidates.flags.c_contiguous
            ptr, n = ctypes.c_void_p(candidates.ctypes.data) if len(candidates) else None, len(candidates)
        self._check(self.lib.rrea_gpu_population_thin_resident(
            self.handle, int(species), int(target), int(step), int(salt), ptr, n,
            stats.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        return dict(zip(self.POPULATION_STATS, (int(v) for v in stats)))

    def population_split(self, species, target, split_min_weight):
        """Split refill of the resident tile; returns the clones added."""
        added = ctypes.c_int64()
        self._check(self.lib.rrea_gpu_population_split_resident(self.handle, int(species), int(target),
                                                                float(split_min_weight), ctypes.byref(added)))
        return added.value

    MERGE_STATS = ("live", "groups", "pairs", "requested", "merged")

    def population_merge(self, species, target, step):
        """Weight-doubling merge of the resident tile above `target` valid
        particles (merged particles are invalidated; compact_resident removes
        them); returns the MERGE_STATS as a dict."""
        stats = np.zeros(len(self.MERGE_STATS), dtype=np.int64)
        self._check(self.lib.rrea_gpu_population_merge_resident(
            self.handle, int(species), int(target), int(step), stats.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        return dict(zip(self.MERGE_STATS, (int(v) for v in stats)))

    def deposit_charge(self):
        """Cell-centred CIC charge of the resident electrons (-w) and
        positrons (+w), elementary charges per cell, shape (nz, nr)."""
        c = self.config
        out = np.zeros(c.nr * c.nz)
        self._check(self.lib.rrea_gpu_deposit_charge_resident(self.handle, out.ctypes.data_as(_D)))
        return out.reshape(c.nz, c.nr)

    def set_schedule(self, cost_order=True):
        self._check(self.lib.rrea_gpu_set_schedule(self.handle, int(bool(cost_order))))

    # ---- batched ensemble ----------------------------------------------------
    def ensemble_configure(self, ambient_ez):
        """Ensemble mode: instance k (a particle's cpu ordinal) moves in the
        uniform field E_z = ambient_ez[k]; call before staging."""
        ez = np.ascontiguousarray(ambient_ez, dtype=np.float64)
        self._check(self.lib.rrea_gpu_ensemble_configure(self.handle, ez.size, ez.ctypes.data_as(_D)))
        self.n_instances = int(ez.size)

    def ensemble_partition(self, species):
        """Stable partition of a species tile by instance; returns the slice sizes."""
        counts = np.zeros(self.n_instances, dtype=np.int64)
        self._check(self.lib.rrea_gpu_ensemble_partition(self.handle, int(species),
                                                         counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        return counts

    def ensemble_retire(self, instance):
        self._check(self.lib.rrea_gpu_ensemble_retire(self.handle, int(instance)))

    def ensemble_census(self, species, instance, edges_eV, thresholds_eV=()):
        edges = np.ascontiguousarray(edges_eV, dtype=np.float64)
        thr = np.ascontiguousarray(thresholds_eV, dtype=np.float64)
        out = np.zeros(7 + thr.size + edges.size - 1)
        self._check(self.lib.rrea_gpu_ensemble_census(self.handle, int(species), int(instance),
                                                      edges.ctypes.data_as(_D), edges.size,
                                                      thr.ctypes.data_as(_D) if thr.size else None, thr.size,
                                                      out.ctypes.data_as(_D)))
        return unpack_census(out, thr.size)

    def ensemble_population_thin(self, species, instance, target, step, salt=0):
        stats = np.zeros(8, dtype=np.int64)
        self._check(self.lib.rrea_gpu_ensemble_population_thin(self.handle, int(species), int(instance), int(target),
                                                               int(step), int(salt),
                                                               stats.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        return dict(zip(self.POPULATION_STATS, stats.tolist()))

    def ensemble_population_thin_all(self, species, targets, step, salt=0):
        """Population control of every instance in one pass (targets per
        instance, 0 = none); returns (removed per instance, total stats)."""
        t = np.ascontiguousarray(targets, dtype=np.int64)
        if t.size != self.n_instances:
            raise ValueError("one target per instance")
        removed = np.zeros(self.n_instances, dtype=np.int64)
        stats = np.zeros(8, dtype=np.int64)
        P = ctypes.POINTER(ctypes.c_int64)
        self._check(self.lib.rrea_gpu_ensemble_population_thin_all(self.handle, int(species), t.ctypes.data_as(P),
                                                                   int(step), int(salt), removed.ctypes.data_as(P),
                                                                   stats.ctypes.data_as(P)))
        return removed, dict(zip(self.POPULATION_STATS, stats.tolist()))

    # ---- low-energy carrier fluid ------------------------------------------
    def fluid_configure(self, fluid_config=None, **overrides):
        """Allocates (first call) and configures the carrier fluid."""
        cfg = fluid_config if fluid_config is not None else default_fluid_config()
        for k, v in overrides.items():
            setattr(cfg, k, v)
        self._check(self.lib.rrea_gpu_fluid_configure(self.handle, ctypes.byref(cfg)))
        self.fluid_config = cfg
        return cfg

    def fluid_load_closure(self, path):
        self._check(self.lib.rrea_gpu_fluid_load_closure(self.handle, str(path).encode()))

    def _cells(self):
        return self.config.nr * self.config.nz

    def fluid_set_state(self, n_pos=None, n_neg=None, n_e=None, rho=None):
        n = self._cells()
        keep = [_opt(a, n) for a in (n_pos, n_neg, n_e, rho)]
        self._check(self.lib.rrea_gpu_fluid_set_state(self.handle, *[p for _, p in keep]))

    def fluid_state(self):
        """Dict of n_pos, n_neg, n_e, rho, sigma, tau (cells i + nr*j)."""
        n = self._cells()
        out = {k: np.zeros(n) for k in ("n_pos", "n_neg", "n_e", "rho", "sigma", "tau")}
        self._check(self.lib.rrea_gpu_fluid_get_state(self.handle, *[out[k].ctypes.data_as(_D) for k in out]))
        return out

    def fluid_set_source_rates(self, s_e=None, s_pos=None, s_neg=None):
        n = self._cells()
        keep = [_opt(a, n) for a in (s_e, s_pos, s_neg)]
        self._check(self.lib.rrea_gpu_fluid_set_source_rates(self.handle, *[p for _, p in keep]))

    def fluid_source_rates(self):
        n = self._cells()
        out = {k: np.zeros(n) for k in ("s_e", "s_pos", "s_neg")}
        self._check(self.lib.rrea_gpu_fluid_get_source_rates(self.handle, *[out[k].ctypes.data_as(_D) for k in out]))
        return out

    def fluid_set_density_ratio(self, chi=None):
        arr, p = _opt(chi, self._cells())
        self._check(self.lib.rrea_gpu_fluid_set_density_ratio(self.handle, p))

    def fluid_set_closure_fields(self, mu=None, nu=None, diffusion=None):
        n = self._cells()
        keep = [_opt(mu, n), _opt(nu, n), _opt(diffusion, 3 * n)]
        self._check(self.lib.rrea_gpu_fluid_set_closure_fields(self.handle, *[p for _, p in keep]))

    def fluid_closure_fields(self):
        n = self._cells()
        mu, nu, d3 = np.zeros(n), np.zeros(n), np.zeros(3 * n)
        self._check(self.lib.rrea_gpu_fluid_get_closure_fields(self.handle, mu.ctypes.data_as(_D), nu.ctypes.data_as(_D),
                                                               d3.ctypes.data_as(_D)))
        return mu, nu, d3.reshape(3, n)

    def fluid_take_sources(self, dt_s):
        self._check(self.lib.rrea_gpu_fluid_take_sources(self.handle, dt_s))

    def fluid_react(self, dt_s, clear_sources=True):
        r = ctypes.c_double(0.0)
        self._check(self.lib.rrea_gpu_fluid_react(self.handle, dt_s, int(bool(clear_sources)), ctypes.byref(r)))
        return r.value

    def fluid_max_reaction_frequency(self):
        r = ctypes.c_double(0.0)
        self._check(self.lib.rrea_gpu_fluid_max_reaction_frequency(self.handle, ctypes.byref(r)))
        return r.value

    def fluid_conductivity(self):
        self._check(self.lib.rrea_gpu_fluid_conductivity(self.handle))

    def fluid_charge_density(self):
        self._check(self.lib.rrea_gpu_fluid_charge_density(self.handle))

    def fluid_evaluate_closure(self, er_cell=None, ez_cell=None):
        n = self._cells()
        a, pa = _opt(er_cell, n)
        b, pb = _opt(ez_cell, n)
        d = np.zeros(8)
        self._check(self.lib.rrea_gpu_fluid_evaluate_closure(self.handle, pa, pb, d.ctypes.data_as(_D)))
        return dict(zip(FLUID_CLOSURE_DIAG, d))

    def fluid_transport(self, dt_s, efr=None, efz=None):
        """One explicit carrier-transport update; returns (flux_r (3, faces),
        flux_z (3, faces), diagnostics dict)."""
        c = self.config
        nfr, nfz = (c.nr + 1) * c.nz, c.nr * (c.nz + 1)
        a, pa = _opt(efr, nfr)
        b, pb = _opt(efz, nfz)
        fr, fz, d = np.zeros(3 * nfr), np.zeros(3 * nfz), np.zeros(14)
        self._check(self.lib.rrea_gpu_fluid_transport(self.handle, dt_s, pa, pb, fr.ctypes.data_as(_D),
                                                      fz.ctypes.data_as(_D), d.ctypes.data_as(_D)))
        return fr.reshape(3, nfr), fz.reshape(3, nfz), dict(zip(FLUID_TRANSPORT_DIAG, d))

    def sources_device(self):
        """(device pointer, length) of the five cell-source grids."""
        p = ctypes.c_void_p()
        self._check(self.lib.rrea_gpu_sources_device(self.handle, ctypes.byref(p)))
        return p.value, 5 * self._cells()

    def advance_field_coupled_from_current(self, dt_s):
        d = np.zeros(8)
        self._check(self.lib.rrea_gpu_advance_field_coupled_from_current(self.handle, dt_s, d.ctypes.data_as(_D)))
        return dict(zip(FLUID_COUPLED_DIAG, d))

    def fluid_reductions(self, dt_s):
        """The reduced diagnostics' fluid and source totals (FLUID_REDUCED_COLUMNS)."""
        d = np.zeros(16)
        self._check(self.lib.rrea_gpu_fluid_reductions(self.handle, dt_s, d.ctypes.data_as(_D)))
        return dict(zip(FLUID_REDUCED_COLUMNS, d))

    def advance_field_coupled(self, dt_s):
        """The coupled fluid + Maxwell step; returns its diagnostics dict."""
        d = np.zeros(8)
        self._check(self.lib.rrea_gpu_advance_field_coupled(self.handle, dt_s, d.ctypes.data_as(_D)))
        return dict(zip(FLUID_COUPLED_DIAG, d))

    def census(self, species, edges_eV, thresholds_eV=()):
        """Census of a resident species tile (the reduced diagnostics'
        particle reductions and a weighted energy spectrum over the bins
        [edges[b], edges[b+1])); returns a dict of count, max_weight,
        sum_w, sum_w2, sum_wk, under, over, above (per threshold), hist."""
        edges = np.ascontiguousarray(edges_eV, dtype=np.float64)
        thr = np.ascontiguousarray(thresholds_eV, dtype=np.float64)
        out = np.zeros(7 + thr.size + edges.size - 1)
        self._check(self.lib.rrea_gpu_census_resident(self.handle, int(species), edges.ctypes.data_as(_D), edges.size,
                                                      thr.ctypes.data_as(_D) if thr.size else None, thr.size,
                                                      out.ctypes.data_as(_D)))
        return unpack_census(out, thr.size)

    def resident_count(self, species):
        n = ctypes.c_int64()
        self._check(self.lib.rrea_gpu_resident_count(self.handle, species, ctypes.byref(n)))
        return n.value

    def pending_secondaries(self, discard=False):
        n = ctypes.c_int64()
        self._check(self.lib.rrea_gpu_pending_secondaries(self.handle, ctypes.byref(n), int(bool(discard))))
        return n.value

    def last_drain_stats(self):
        items, surv = ctypes.c_int64(), ctypes.c_int64()
        self._check(self.lib.rrea_gpu_last_drain_stats(self.handle, ctypes.byref(items), ctypes.byref(surv)))
        return items.value, surv.value

    def selftest_math(self, which, x):
        """(table-driven, CUDA) log (which 0) or exp (which 1) of x on the device."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        fast, libm = np.zeros_like(x), np.zeros_like(x)
        self._check(self.lib.rrea_gpu_selftest_math(self.handle, int(which), x.ctypes.data_as(_D), x.size,
                                                    fast.ctypes.data_as(_D), libm.ctypes.data_as(_D)))
        return fast, libm

    def count_live(self, species):
        live = ctypes.c_int64()
        self._check(self.lib.rrea_gpu_count_live(self.handle, int(species), ctypes.byref(live)))
        return live.value

    def advance_field(self, dt_s, substeps=1):
        self._check(self.lib.rrea_gpu_advance_field(self.handle, float(dt_s), int(substeps)))

    def current_device(self):
        """Converts the step's current and returns the device addresses and
        lengths of the physical face currents: ((jr_ptr, n_jr), (jz_ptr, n_jz))."""
        jr, jz = ctypes.c_void_p(), ctypes.c_void_p()
        self._check(self.lib.rrea_gpu_current_device(self.handle, ctypes.byref(jr), ctypes.byref(jz)))
        c = self.config
        return (jr.value, (c.nr + 1) * c.nz), (jz.value, c.nr * (c.nz + 1))

    def advance_field_from_current(self, dt_s, substeps=1):
        self._check(self.lib.rrea_gpu_advance_field_from_current(self.handle, float(dt_s), int(substeps)))

    def field(self):
        """Scattered field vectors (er, ez, bt), flat, layouts as set_field."""
        c = self.config
        er = np.zeros((c.nr + 1) * c.nz)
        ez = np.zeros(c.nr * (c.nz + 1))
        bt = np.zeros((c.nr + 1) * (c.nz + 1))
        self._check(self.lib.rrea_gpu_download_field(self.handle, er.ctypes.data_as(_D), ez.ctypes.data_as(_D),
                                                     bt.ctypes.data_as(_D)))
        return er, ez, bt

    def reset_current(self):
        self._check(self.lib.rrea_gpu_reset_current(self.handle))

    def current(self):
        """Physical face current densities (Jr (nz, nr+1), Jz (nz+1, nr)) in A/m^2."""
        c = self.config
        jr = np.zeros((c.nz, c.nr + 1))
        jz = np.zeros((c.nz + 1, c.nr))
        self._check(self.lib.rrea_gpu_download_current(self.handle, jr.ctypes.data_as(_D), jz.ctypes.data_as(_D)))
        return jr, jz

    def current_index(self):
        """Padded index-space grids: rho (nz+4, nr+2), jr (nz+4, nr+3), jz (nz+5, nr+2)."""
        c = self.config
        rho = np.zeros((c.nz + 4, c.nr + 2))
        jr = np.zeros((c.nz + 4, c.nr + 3))
        jz = np.zeros((c.nz + 5, c.nr + 2))
        self._check(self.lib.rrea_gpu_download_current_index(self.handle, rho.ctypes.data_as(_D),
                                                             jr.ctypes.data_as(_D), jz.ctypes.data_as(_D)))
        return {"rho": rho, "jr": jr, "jz": jz}

    def diagnostics(self, n):
        sub = np.zeros(n, dtype=np.uint64)
        ev = np.zeros(n, dtype=np.uint64)
        disp = np.zeros(n, dtype=np.int32)
        self._check(self.lib.rrea_gpu_download_diagnostics(
            self.handle, n, sub.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
            ev.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), disp.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))))
        return sub, ev, disp

    def last_step_stats(self):
        """(particles transported, secondaries, transport-kernel ms) of the last step."""
        t, s, ms = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_double()
        self._check(self.lib.rrea_gpu_last_step_stats(self.handle, ctypes.byref(t), ctypes.byref(s), ctypes.byref(ms)))
        return t.value, s.value, ms.value

    def stream(self):
        s = ctypes.c_void_p()
        self._check(self.lib.rrea_gpu_stream(self.handle, ctypes.byref(s)))
        return s.value


def unpack_census(out, n_thresholds):
    """Named fields of an rrea_gpu_census_resident output vector."""
    return {"count": int(out[0]), "max_weight": float(out[1]), "sum_w": float(out[2]), "sum_w2": float(out[3]),
            "sum_wk": float(out[4]), "under": float(out[5]), "over": float(out[6]),
            "above": out[7:7 + n_thresholds].copy(), "hist": out[7 + n_thresholds:].copy()}


def population_projection(current, removals, insertions, ceiling, reject_equality=False):
    """RreaStrictPopulationProjection: (fits, projected)."""
    projected = ctypes.c_uint64()
    status = load_library().rrea_gpu_population_projection(int(current), int(removals), int(insertions), int(ceiling),
                                                           int(bool(reject_equality)), ctypes.byref(projected))
    return status == 0, projected.value


def order_secondaries_noalloc(d_counts, n_parents, d_unordered, n_secondaries, d_ordered, stream=None):
    """rrea_gpu_order_secondaries_noalloc on device addresses (ints);
    returns (status, message)."""
    buf = ctypes.create_string_buffer(512)
    st = load_library().rrea_gpu_order_secondaries_noalloc(
        ctypes.c_void_p(d_counts), int(n_parents), ctypes.c_void_p(d_unordered), int(n_secondaries),
        ctypes.c_void_p(d_ordered), ctypes.c_void_p(stream), buf, 512)
    return st, buf.value.decode(errors="replace")


class RreaParticleInteraction:
    """Host mirror of rrea::warpx::RreaParticleInteraction: construct with the
    transport configuration, then Apply(tile, step, time_s, dt_s) once per
    step.  Raises RreaGpuError where the reference calls amrex::Abort."""

    def __init__(self, config, capacity, tables=DEFAULT_TABLES, field=None):
        self.ctx = RreaGpuContext(config, capacity)
        self.ctx.load_tables(tables)
        if field is not None:
            self.ctx.set_field(**field)

    def SetField(self, er, ez, bt, amb_er, amb_ez):
        self.ctx.set_field(er, ez, bt, amb_er, amb_ez)

    def Apply(self, electrons, step, time_s, dt_s, photons=None, positrons=None):
        """Electron, photon and positron phases in the reference's order
        (RreaParticleInteraction.cpp:54-57).  Returns the ordered secondaries
        of each phase (None for a species not given)."""
        if not dt_s > 0.0:
            return None, None, None
        sec_e = self.ctx.apply_electrons(electrons, step, dt_s, time_s=time_s)
        sec_g = self.ctx.apply_photons(photons, step, dt_s, time_s=time_s) if photons is not None else None
        sec_p = self.ctx.apply_positrons(positrons, step, dt_s, time_s=time_s) if positrons is not None else None
        return sec_e, sec_g, sec_p

    def DrainAndCommitSecondaries(self, pending, step, dt_s):
        """The transient FIFO of RreaSecondaryCommit.cpp:331-474 over the
        secondaries Apply returned (concatenated in phase order); returns the
        survivors that the overlay inserts, in FIFO order."""
        return self.ctx.drain_secondaries(pending, step, dt_s)
