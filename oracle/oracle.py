"""ORACLE: test infrastructure only.

ctypes wrapper over oracle/liboracle.so, the CPU restatement of the
reference kinetic step.  Used by tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py to check and time the GPU path; the shipped GPU
library never loads it.
"""
import ctypes
import os

import numpy as np

from .build import build_oracle

HERE = os.path.dirname(os.path.abspath(__file__))

_lib = None


class RreaGpuConfig(ctypes.Structure):
    """Mirror of rrea_gpu_config (include/rrea_gpu.h)."""

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


class RreaGpuTile(ctypes.Structure):
    """Mirror of rrea_gpu_tile (include/rrea_gpu.h)."""

    _fields_ = [("n", ctypes.c_int64)] + [
        (name, ctypes.POINTER(ctypes.c_double))
        for name in ("r", "z", "theta", "ux", "uy", "uz", "w",
                     "prev_r", "prev_z", "prev_theta", "prev_ux", "prev_uy", "prev_uz")
    ] + [("id", ctypes.POINTER(ctypes.c_int64)), ("cpu", ctypes.POINTER(ctypes.c_int32))]


SECONDARY_DTYPE = np.dtype([
    ("species", "<i4"), ("process", "<i4"), ("root_species", "<i4"), ("pad", "<i4"),
    ("parent_index", "<i8"), ("root_key", "<u8"), ("lineage", "<u8"),
    ("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("dir_x", "<f8"), ("dir_y", "<f8"), ("dir_z", "<f8"),
    ("weight", "<f8"), ("energy_eV", "<f8"), ("birth_fraction", "<f8"),
])

TILE_FIELDS = ("r", "z", "theta", "ux", "uy", "uz", "w",
               "prev_r", "prev_z", "prev_theta", "prev_ux", "prev_uy", "prev_uz")


def lib():
    global _lib
    if _lib is None:
        path = build_oracle()
        _lib = ctypes.CDLL(path)
        d = ctypes.POINTER(ctypes.c_double)
        _lib.oracle_load_tables.argtypes = [ctypes.c_char_p]
        _lib.oracle_primitive.argtypes = [ctypes.c_int, d, ctypes.c_int64, d]
        _lib.oracle_rng.argtypes = [ctypes.POINTER(ctypes.c_uint64), ctypes.c_int64,
                                    ctypes.POINTER(ctypes.c_uint64), d]
        _lib.oracle_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
        _lib.oracle_electron_step.argtypes = [ctypes.POINTER(RreaGpuConfig), d, d, d, d, d, ctypes.c_int32,
                                              ctypes.c_double, ctypes.POINTER(RreaGpuTile)]
        _lib.oracle_positron_step.argtypes = _lib.oracle_electron_step.argtypes
        _lib.oracle_advance_maxwell.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                                ctypes.c_double, ctypes.c_int, d, d, d, d, d]
        _lib.oracle_drain.argtypes = [ctypes.POINTER(RreaGpuConfig), d, d, d, d, d, ctypes.c_int32, ctypes.c_double,
                                      ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]
        _lib.oracle_survivors.argtypes = [ctypes.c_void_p]
        _lib.oracle_deposit_segments.argtypes = [ctypes.POINTER(RreaGpuConfig), ctypes.c_double, d, ctypes.c_int64,
                                                 d, d, d, d, d]
        _lib.oracle_photon_step.argtypes = [ctypes.POINTER(RreaGpuConfig), ctypes.c_int32, ctypes.c_double,
                                            ctypes.POINTER(RreaGpuTile)]
        _lib.oracle_counts.argtypes = [ctypes.POINTER(ctypes.c_int64)] * 3
        _lib.oracle_elastic_branches.argtypes = [ctypes.POINTER(ctypes.c_uint64), ctypes.c_int]
        _lib.oracle_photon_flow.argtypes = [d, ctypes.c_int64, ctypes.POINTER(ctypes.c_int32)]
        _lib.oracle_interleave_trace.argtypes = [ctypes.c_int, ctypes.c_uint64, d, ctypes.c_int64,
                                                 ctypes.POINTER(ctypes.c_int64)]
        _lib.oracle_secondaries.argtypes = [ctypes.c_void_p]
        _lib.oracle_sources.argtypes = [d]
        _lib.oracle_segments.argtypes = [d]
        _lib.oracle_diagnostics.argtypes = [ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                                            ctypes.POINTER(ctypes.c_int32)]
        _lib.oracle_cell_sources.argtypes = [d]
        _lib.oracle_set_density_profile.argtypes = [d, d, ctypes.c_int64, ctypes.c_double, ctypes.c_double]
        _lib.oracle_density_query.argtypes = [ctypes.c_int, d, ctypes.c_int64, ctypes.c_double, d]
        _lib.oracle_set_planes.argtypes = [d, ctypes.c_int64]
        _lib.oracle_plane_flux.argtypes = [d]
        _lib.oracle_plane_enumerate.argtypes = [d, ctypes.c_int64, d, ctypes.c_int64, ctypes.c_int64, d,
                                                ctypes.POINTER(ctypes.c_int64)]
        _lib.oracle_plane_enumerate.restype = None
        _lib.oracle_plane_accumulate.argtypes = [d, ctypes.c_int64, ctypes.c_int64, d, ctypes.POINTER(ctypes.c_int32)]
        _lib.oracle_plane_accumulate.restype = None
    return _lib


class OracleFailure(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"oracle status {code}: {message}")
        self.code = code


def _check(rc):
    if rc != 0:
        buf = ctypes.create_string_buffer(1024)
        lib().oracle_last_error(buf, 1024)
        raise OracleFailure(rc, buf.value.decode())


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


_loaded_path = None


def load_tables(path):
    global _loaded_path
    if _loaded_path == path:
        return
    _check(lib().oracle_load_tables(path.encode()))
    _loaded_path = path


_planes = 0


def set_planes(plane_z_m=()):
    """The plane-crossing diagnostic's planes (empty: off)."""
    global _planes
    z = np.ascontiguousarray(plane_z_m, dtype=np.float64)
    _check(lib().oracle_set_planes(z.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), z.size))
    _planes = int(z.size)


def plane_flux():
    """The last step's (or drain's) crossings accumulated from zero: (n_planes, 10)."""
    out = np.zeros((_planes, 10))
    _check(lib().oracle_plane_flux(out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    return out


def plane_enumerate(segments, planes, cap=64):
    """RreaForEachNonperiodicPlaneCrossing over rows (z0, z1): a list of
    (plane, fraction, direction) arrays, None where the geometry is invalid."""
    seg = np.ascontiguousarray(segments, dtype=np.float64).reshape(-1, 2)
    pl = np.ascontiguousarray(planes, dtype=np.float64)
    out = np.zeros((len(seg), cap, 3))
    counts = np.zeros(len(seg), dtype=np.int64)
    lib().oracle_plane_enumerate(seg.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(seg), pl.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), pl.size, cap,
                                 out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    return [None if c < 0 else out[i, :c] for i, c in enumerate(counts)]


def plane_accumulate(rows, n_planes):
    """Crossing rows (plane, direction, weight, r, local, mev) added one by
    one (an invalid one is refused and changes nothing): (ok flags, bins)."""
    r = np.ascontiguousarray(rows, dtype=np.float64).reshape(-1, 6)
    out = np.zeros((n_planes, 10))
    ok = np.zeros(len(r), dtype=np.int32)
    lib().oracle_plane_accumulate(r.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(r), n_planes,
                                  out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                  ok.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    return ok, out


def set_density_profile(altitude_m=None, density_kg_m3=None, altitude_msl_at_z0_m=0.0,
                        reference_density_kg_m3=0.0):
    """Binds the altitude density profile (TransportDensityRatioAtZ with
    rrea.air_density_model=altitude_profile); no arrays unbinds it."""
    if altitude_m is None:
        alt = dens = np.zeros(0)
    else:
        alt = np.ascontiguousarray(altitude_m, dtype=np.float64)
        dens = np.ascontiguousarray(density_kg_m3, dtype=np.float64)
        if alt.shape != dens.shape:
            raise ValueError("altitude and density columns differ in length")
    _check(lib().oracle_set_density_profile(_dptr(alt), _dptr(dens), alt.shape[0], altitude_msl_at_z0_m,
                                            reference_density_kg_m3))


def profile_density(altitude_m):
    """The bound profile's density (kg/m^3) at each altitude."""
    a = np.ascontiguousarray(altitude_m, dtype=np.float64)
    out = np.zeros_like(a)
    _check(lib().oracle_density_query(0, _dptr(a), a.shape[0], 0.0, _dptr(out)))
    return out


def density_ratio_at_z(z_m, uniform_ratio):
    """TransportDensityRatioAtZ at each axial position."""
    z = np.ascontiguousarray(z_m, dtype=np.float64)
    out = np.zeros_like(z)
    _check(lib().oracle_density_query(1, _dptr(z), z.shape[0], uniform_ratio, _dptr(out)))
    return out


def interleave_trace(kind, seed):
    """Trace (records of code, a, b, c) of scripted scenario `seed` through
    the oracle's event (kind 0) or substep (kind 1) skeleton."""
    cap = 4096
    out = np.zeros((cap, 4))
    n = ctypes.c_int64()
    lib().oracle_interleave_trace(int(kind), int(seed), _dptr(out), cap, ctypes.byref(n))
    if n.value > cap:
        raise RuntimeError("scenario trace longer than its buffer")
    return out[: n.value]


def photon_flow_valid(rows):
    """The photon energy-flow ledger check on rows of (kind, weight,
    incident, x1, x2, x3, has_recoil, local); returns a bool per row."""
    rows = np.ascontiguousarray(rows, dtype=np.float64).reshape(-1, 8)
    ok = np.zeros(rows.shape[0], dtype=np.int32)
    lib().oracle_photon_flow(_dptr(rows), rows.shape[0], ok.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    return ok.astype(bool)


def elastic_branches(reset=True):
    """Elastic angle draws since the last reset, by branch: dict of gs,
    wentzel, isotropic, single."""
    out = np.zeros(4, dtype=np.uint64)
    lib().oracle_elastic_branches(out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), int(bool(reset)))
    return dict(zip(("gs", "wentzel", "isotropic", "single"), (int(v) for v in out)))


def primitive(which, inputs, out_cols):
    inputs = np.ascontiguousarray(inputs, dtype=np.float64)
    n = inputs.shape[0]
    out = np.zeros((n, out_cols), dtype=np.float64)
    _check(lib().oracle_primitive(which, _dptr(inputs), n, _dptr(out)))
    return out


def rng(keys):
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    n = keys.shape[0]
    counter = np.zeros(n, dtype=np.uint64)
    uniform = np.zeros(n, dtype=np.float64)
    lib().oracle_rng(keys.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), n,
                     counter.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), _dptr(uniform))
    return counter, uniform


def make_tile_struct(arrays):
    """arrays: dict of contiguous numpy arrays (TILE_FIELDS f8, id i8, cpu i4)."""
    t = RreaGpuTile()
    t.n = arrays["id"].shape[0]
    for name in TILE_FIELDS:
        setattr(t, name, _dptr(arrays[name]))
    t.id = arrays["id"].ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    t.cpu = arrays["cpu"].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    return t


def electron_step(cfg, field, step, dt_s, arrays):
    """Runs the oracle electron phase in place on `arrays` (numpy tile).
    Returns dict with secondaries, sources, segments, diagnostics, cells."""
    cfg = as_config(cfg)
    t = make_tile_struct(arrays)
    _check(lib().oracle_electron_step(ctypes.byref(cfg), _dptr(field["er"]), _dptr(field["ez"]),
                                      _dptr(field["bt"]), _dptr(field["amb_er"]), _dptr(field["amb_ez"]),
                                      step, dt_s, ctypes.byref(t)))
    return _collect(cfg, t)


def positron_step(cfg, field, step, dt_s, arrays):
    """Runs the oracle positron phase in place on `arrays` (numpy tile)."""
    cfg = as_config(cfg)
    t = make_tile_struct(arrays)
    _check(lib().oracle_positron_step(ctypes.byref(cfg), _dptr(field["er"]), _dptr(field["ez"]),
                                      _dptr(field["bt"]), _dptr(field["amb_er"]), _dptr(field["amb_ez"]),
                                      step, dt_s, ctypes.byref(t)))
    return _collect(cfg, t)


def netchord_shapes(cfg):
    """Shapes (rows, cols) of the padded rho/Jr/Jz and physical Jr/Jz grids."""
    nr, nz = cfg.nr + 2, cfg.nz + 4
    return {"rho": (nz, nr), "jr": (nz, nr + 1), "jz": (nz + 1, nr),
            "jr_phys": (cfg.nz, cfg.nr + 1), "jz_phys": (cfg.nz + 1, cfg.nr)}


def deposit_segments(cfg, dt_s, rows):
    """Net-chord current of segment rows (kind, a0..a6, faces) on cfg's padded
    grid; returns dict of rho, jr, jz (padded index space) and jr_phys, jz_phys."""
    cfg = as_config(cfg)
    rows = np.ascontiguousarray(rows, dtype=np.float64).reshape(-1, 9)
    shapes = netchord_shapes(cfg)
    out = {k: np.zeros(v) for k, v in shapes.items()}
    _check(lib().oracle_deposit_segments(ctypes.byref(cfg), dt_s, _dptr(rows), rows.shape[0], _dptr(out["rho"]),
                                         _dptr(out["jr"]), _dptr(out["jz"]), _dptr(out["jr_phys"]),
                                         _dptr(out["jz_phys"])))
    return out


def segment_rows(result):
    """Segment rows (kind, a0..a6, faces) from a step result's segments."""
    seg = result["segments"]
    rows = np.zeros((seg.shape[0], 9))
    rows[:, :8] = seg[:, :8]
    rows[:, 8] = seg[:, 9]
    return rows


def advance_maxwell(nr, nz, dr, dz, dt_s, substeps, er, ez, bt, jr, jz):
    """Maxwell TM-RZ field step (no fluid) on copies of er, ez, bt; returns them."""
    er, ez, bt = (np.array(a, dtype=np.float64).ravel().copy() for a in (er, ez, bt))
    jr, jz = (np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (jr, jz))
    _check(lib().oracle_advance_maxwell(nr, nz, dr, dz, dt_s, substeps, _dptr(er), _dptr(ez), _dptr(bt), _dptr(jr),
                                        _dptr(jz)))
    return er, ez, bt


def drain(cfg, field, step, dt_s, initial):
    """DrainAndCommitSecondaries over the structured array `initial`
    (SECONDARY_DTYPE, in the phases' order).  Returns dict with the final
    survivors (FIFO order), the newborns' sources, segments and cell grids."""
    cfg = as_config(cfg)
    initial = np.ascontiguousarray(initial, dtype=SECONDARY_DTYPE)
    n_surv = ctypes.c_int64()
    _check(lib().oracle_drain(ctypes.byref(cfg), _dptr(field["er"]), _dptr(field["ez"]), _dptr(field["bt"]),
                              _dptr(field["amb_er"]), _dptr(field["amb_ez"]), step, dt_s,
                              ctypes.c_void_p(initial.ctypes.data), initial.shape[0], ctypes.byref(n_surv)))
    surv = np.zeros(n_surv.value, dtype=SECONDARY_DTYPE)
    if n_surv.value:
        lib().oracle_survivors(ctypes.c_void_p(surv.ctypes.data))
    t = RreaGpuTile()
    t.n = 0
    res = _collect(cfg, t)
    res["survivors"] = surv
    return res


def photon_step(cfg, step, dt_s, arrays):
    """Runs the oracle photon phase in place on `arrays` (photon tile: prev_*
    is the captured start, r/theta/z the straight-push endpoint)."""
    cfg = as_config(cfg)
    t = make_tile_struct(arrays)
    _check(lib().oracle_photon_step(ctypes.byref(cfg), step, dt_s, ctypes.byref(t)))
    return _collect(cfg, t)


def _collect(cfg, t):
    n_sec, n_src, n_seg = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    lib().oracle_counts(ctypes.byref(n_sec), ctypes.byref(n_src), ctypes.byref(n_seg))
    sec = np.zeros(n_sec.value, dtype=SECONDARY_DTYPE)
    if n_sec.value:
        lib().oracle_secondaries(sec.ctypes.data)
    src = np.zeros((n_src.value, 7))
    if n_src.value:
        lib().oracle_sources(_dptr(src))
    seg = np.zeros((n_seg.value, 11))
    if n_seg.value:
        lib().oracle_segments(_dptr(seg))
    n = t.n
    sub = np.zeros(n, dtype=np.uint64)
    ev = np.zeros(n, dtype=np.uint64)
    disp = np.zeros(n, dtype=np.int32)
    lib().oracle_diagnostics(sub.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                             ev.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                             disp.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    cells = np.zeros(5 * cfg.nr * cfg.nz)
    lib().oracle_cell_sources(_dptr(cells))
    return {"secondaries": sec, "sources": src, "segments": seg, "subcycles": sub, "events": ev,
            "disposition": disp, "cells": cells.reshape(5, cfg.nz, cfg.nr)}


def deposit_charge_cic(nr, nz, dr, dz, r_lo, z_lo, r, z, qw):
    """Cell-centred CIC charge of point particles (DepositChargeCIC,
    I/RreaSegmentDepositionRZ.H:68-92): weights from the distance to the cell
    centres, the support folded evenly at the axis and clamped at the outer
    r and both z edges; deposits added in particle order.  Returns rho as a
    flat nr*nz array (index i + nr*j)."""
    r = np.asarray(r, dtype=np.float64)
    z = np.asarray(z, dtype=np.float64)
    qw = np.asarray(qw, dtype=np.float64)
    xr = (r - r_lo) / dr - 0.5
    xz = (z - z_lo) / dz - 0.5
    i0 = np.floor(xr).astype(np.int64)
    j0 = np.floor(xz).astype(np.int64)
    fr = xr - i0
    fz = xz - j0
    rho = np.zeros(nr * nz)
    idx, val = [], []
    for a in (0, 1):
        for b in (0, 1):
            i = i0 + a
            j = j0 + b
            i = np.where(i < 0, -1 - i, i)
            i = np.minimum(i, nr - 1)
            j = np.clip(j, 0, nz - 1)
            idx.append(i + nr * j)
            val.append(qw * (1.0 - fr if a == 0 else fr) * (1.0 - fz if b == 0 else fz))
    # the reference adds a particle's four corners before the next particle's
    order = np.stack(idx, axis=1).ravel()
    np.add.at(rho, order, np.stack(val, axis=1).ravel())
    return rho


def default_config(**overrides):
    """The library's default configuration (rrea_gpu_default_config, the
    reference defaults of RreaParticleInteraction.H:1576-1596 with a 1 keV
    tracking cut) built here without loading the GPU library, then
    `overrides`."""
    cfg = RreaGpuConfig(r_lo=0.0, r_hi=50.0, z_lo=0.0, z_hi=500.0, nr=32, nz=256, periodic_z=0,
                        strict_transport_guards=1, density_ratio=1.0, low_energy_cutoff_eV=1.0e3,
                        photon_cutoff_eV=5.0e4, max_optical_depth_per_substep=0.05, max_subcycles=256,
                        max_gs_collisions_per_substep=32.0, gs_total_collision_cap=1024.0,
                        max_field_impulse_fraction=0.1, field_impulse_floor_eV=1.0e4, rng_seed=0,
                        debug_disable_hard_moller=0, reserved0=0)
    for k, v in overrides.items():
        setattr(cfg, k, v)
    return cfg


def as_config(cfg):
    """Copies any rrea_gpu_config-layout ctypes structure into the oracle's."""
    return RreaGpuConfig.from_buffer_copy(bytes(cfg))


ME_C2_EV = 510998.95000   # I/RreaConstants.H:9
C_M_PER_S = 299792458.0   # I/RreaConstants.H:10


def commit_survivors(recs, species, first_id):
    """Particles the overlay creates from surviving FIFO records of one
    species (RreaWarpXCoupling::CommitLocalParticleBatch,
    O/RreaCouplingSources.cpp:240-330; the captured pre-push state of
    append_rrea_previous_position_attributes, :28-100): records with weight
    <= 0 (photons also with energy <= 0) are dropped; e-/e+ get the proper
    velocity of their kinetic energy (RreaElectronProperVelocityFromKineticEv,
    I/RreaSeedSchedule.H:31-43) along the direction, photons the momentum E
    along it; ids continue from first_id in FIFO order.  Returns a dict of
    columns r, z, theta, ux, uy, uz, w, id."""
    recs = recs[recs["species"] == species]
    keep = recs["weight"] > 0.0
    if species == 2:
        keep &= recs["energy_eV"] > 0.0
    r = recs[keep]
    d = np.stack([r["dir_x"], r["dir_y"], r["dir_z"]], axis=1)
    norm = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
    e = r["energy_eV"]
    u = d.copy()
    with np.errstate(divide="ignore", invalid="ignore"):
        if species == 2:
            scale = np.where(norm > 0.0, e / np.where(norm > 0.0, norm, 1.0), e)
            u = d * scale[:, None]
            u[:, 2] = np.where(norm > 0.0, d[:, 2] * scale, e)
        else:
            gamma = 1.0 + e / ME_C2_EV
            umag = C_M_PER_S * np.sqrt(np.maximum(gamma * gamma - 1.0, 0.0))
            pos = e > 0.0
            nz = norm > 0.0
            for k in range(3):
                scaled = np.where(nz, umag * d[:, k] / np.where(nz, norm, 1.0), umag if k == 2 else 0.0)
                u[:, k] = np.where(pos, scaled, d[:, k])
    return {"r": np.hypot(r["x"], r["y"]), "z": r["z"].copy(), "theta": np.arctan2(r["y"], r["x"]),
            "ux": u[:, 0], "uy": u[:, 1], "uz": u[:, 2], "w": r["weight"].copy(),
            "id": first_id + np.arange(len(r), dtype=np.int64)}

