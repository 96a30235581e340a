"""ORACLE: test infrastructure only.

ctypes front end of the carrier-fluid restatement (oracle/fluid.cpp): the
local chemistry, conductivity, charge reconstruction, closure cell fields
and explicit carrier transport of the reference's LowEnergyFluidState, on
numpy arrays (cells i + nr*j; faces species-major)."""
import ctypes

import numpy as np

from . import oracle as _o


class FluidConfig(ctypes.Structure):
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


MOBILITY_ABSOLUTE, MOBILITY_EN_TABLE_FLUX, MOBILITY_REDUCED_STP = 0, 1, 2
ATTACHMENT_CONSTANT, ATTACHMENT_EN_TABLE = 0, 1


def default_config(**overrides):
    """LowEnergyFluidConfig defaults (I/LowEnergyFluidState.H:80-124) and the
    material substep controls (I/RreaAmrexAdvance.H:51-58), then `overrides`."""
    c = FluidConfig(electron_mobility_m2_per_vs=0.1, positive_ion_mobility_m2_per_vs=2.0e-4,
                    negative_ion_mobility_m2_per_vs=2.0e-4, ion_drift_cfl=0.5, transport_density_ratio=1.0,
                    attachment_frequency_s=2.0e6, ion_drift_enable=0, electron_drift_enable=1,
                    material_min_substeps=2, material_max_substeps=64, material_conduction_target=0.08,
                    material_conduction_guard=0.1, material_diffusion_target=0.8, material_diffusion_guard=1.0,
                    material_reaction_target=0.08, material_reaction_guard=0.1)
    for k, v in overrides.items():
        setattr(c, k, v)
    return c


def as_config(cfg):
    return FluidConfig.from_buffer_copy(bytes(cfg))


_ready = False


def _lib():
    global _ready
    lib = _o.lib()
    if not _ready:
        d = ctypes.POINTER(ctypes.c_double)
        c = ctypes.POINTER(FluidConfig)
        i64, dbl, i32 = ctypes.c_int64, ctypes.c_double, ctypes.c_int
        lib.oracle_fluid_react.argtypes = [c, i64, dbl, d, d, d, d, d, d, d, d, i32, d]
        lib.oracle_fluid_max_reaction_frequency.argtypes = [c, i64, d, d, d, d, d]
        lib.oracle_fluid_conductivity.argtypes = [c, i64, d, d, d, d, d, d, d]
        lib.oracle_fluid_charge_density.argtypes = [i64, d, d, d, d]
        lib.oracle_fluid_load_closure.argtypes = [ctypes.c_char_p]
        lib.oracle_fluid_closure_fields.argtypes = [i32, i32, dbl, dbl, dbl, dbl, dbl, d, d, d, d, d, d, d, d, d]
        lib.oracle_fluid_transport.argtypes = [c, i32, i32, dbl, dbl, dbl, dbl, i32, dbl, d, d, d, d, d, d, d, d, d,
                                               d, d, d, d, d]
        lib.oracle_fluid_coupled_step.argtypes = [c, i32, i32, dbl, dbl, dbl, dbl] + [d] * 20
        _ready = True
    return lib


def _arr(a):
    return np.ascontiguousarray(a, dtype=np.float64).copy()


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def react(cfg, dt, ne, np_, nn, se, sp, sn, rho, nu=None, clear=True):
    """UpdateFromIonizationSource on copies; returns (state dict, residual)."""
    st = {k: _arr(v) for k, v in dict(ne=ne, np=np_, nn=nn, se=se, sp=sp, sn=sn, rho=rho).items()}
    nu_a = None if nu is None else _arr(nu)
    res = ctypes.c_double(0.0)
    _o._check(_lib().oracle_fluid_react(ctypes.byref(as_config(cfg)), len(st["ne"]), dt, _p(st["ne"]), _p(st["np"]),
                                        _p(st["nn"]), _p(st["se"]), _p(st["sp"]), _p(st["sn"]), _p(st["rho"]),
                                        _p(nu_a), int(bool(clear)), ctypes.byref(res)))
    return st, res.value


def max_reaction_frequency(cfg, ne, np_, nn, nu=None):
    out = ctypes.c_double(0.0)
    a = [_arr(x) for x in (ne, np_, nn)]
    nu_a = None if nu is None else _arr(nu)
    _o._check(_lib().oracle_fluid_max_reaction_frequency(ctypes.byref(as_config(cfg)), len(a[0]), *map(_p, a),
                                                         _p(nu_a), ctypes.byref(out)))
    return out.value


def conductivity(cfg, ne, np_, nn, chi=None, mu=None):
    a = [_arr(x) for x in (ne, np_, nn)]
    chi_a = None if chi is None else _arr(chi)
    mu_a = None if mu is None else _arr(mu)
    sigma, tau = np.zeros(len(a[0])), np.zeros(len(a[0]))
    _o._check(_lib().oracle_fluid_conductivity(ctypes.byref(as_config(cfg)), len(a[0]), *map(_p, a), _p(chi_a),
                                               _p(mu_a), _p(sigma), _p(tau)))
    return sigma, tau


def charge_density(ne, np_, nn):
    a = [_arr(x) for x in (ne, np_, nn)]
    rho = np.zeros(len(a[0]))
    _lib().oracle_fluid_charge_density(len(a[0]), *map(_p, a), _p(rho))
    return rho


_closure_path = None


def load_closure(path):
    global _closure_path
    if _closure_path != path:
        _o._check(_lib().oracle_fluid_load_closure(path.encode()))
        _closure_path = path


def closure_fields(nr, nz, r_lo, z_lo, dr, dz, er, ez, chi=None, ne=None, src=None, scalar_chi=1.0):
    """BuildElectronClosureCellFields; returns (mu, nu, diffusion (3, n), diag8)."""
    n = nr * nz
    a = [None if x is None else _arr(x) for x in (er, ez, chi, ne, src)]
    mu, nu, d3, diag = np.zeros(n), np.zeros(n), np.zeros(3 * n), np.zeros(8)
    _o._check(_lib().oracle_fluid_closure_fields(nr, nz, r_lo, z_lo, dr, dz, scalar_chi, *map(_p, a), _p(mu), _p(nu),
                                                 _p(d3), _p(diag)))
    return mu, nu, d3.reshape(3, n), diag


TRANSPORT_DIAG = ("max_face_conductivity", "max_diffusion_number", "unlimited_max_outgoing_cfl",
                  "min_outflow_scale", "limited_outflow_fraction", "limited_electron_number_fraction",
                  "max_outgoing_cfl", "max_drift_speed", "cfl_dt", "pos_center_r", "pos_center_z", "neg_center_r",
                  "neg_center_z", "density_ratio_at_pos_center")


def transport(cfg, grid, dt, n_pos, n_neg, n_e, rho, efr, efz, chi=None, mu=None, diffusion=None):
    """One explicit carrier-transport update on copies.  grid = (nr, nz, r_lo,
    z_lo, dr, dz, periodic_z).  Returns a dict with the new densities and
    charge, the limited and raw face fluxes (species-major) and the
    diagnostics."""
    nr, nz, r_lo, z_lo, dr, dz, per = grid
    st = [_arr(x) for x in (n_pos, n_neg, n_e, rho)]
    chi_a = None if chi is None else _arr(chi)
    mu_a = None if mu is None else _arr(mu)
    d_a = None if diffusion is None else _arr(np.ravel(diffusion))
    nfr, nfz = (nr + 1) * nz, nr * (nz + 1)
    fr, fz, rr, rz, diag = np.zeros(3 * nfr), np.zeros(3 * nfz), np.zeros(3 * nfr), np.zeros(3 * nfz), np.zeros(14)
    _o._check(_lib().oracle_fluid_transport(ctypes.byref(as_config(cfg)), nr, nz, r_lo, z_lo, dr, dz, int(per), dt,
                                            *map(_p, st), _p(chi_a), _p(mu_a), _p(d_a), _p(_arr(efr)), _p(_arr(efz)),
                                            _p(fr), _p(fz), _p(rr), _p(rz), _p(diag)))
    return dict(n_pos=st[0], n_neg=st[1], n_e=st[2], rho=st[3], flux_r=fr.reshape(3, nfr), flux_z=fz.reshape(3, nfz),
                raw_r=rr.reshape(3, nfr), raw_z=rz.reshape(3, nfz), diag=dict(zip(TRANSPORT_DIAG, diag)))


COUPLED_DIAG = ("substeps", "full_conduction", "full_diffusion", "full_reaction", "max_reaction_number",
                "max_dt_sigma", "max_diffusion_number", "max_residual")


def coupled_step(cfg, nr, nz, z_lo, dr, dz, dt, field, ambient, current, state, chi=None):
    """RreaAmrexAdvance::AdvanceOneStep with the fluid, on copies.
    field = (er, ez, bt) scattered; ambient = (amb_er, amb_ez); current =
    (jr, jz) physical kinetic face current; state = dict(ne, np, nn, rho, se,
    sp, sn).  Returns (field, state with sigma/mu/nu/diffusion, diag)."""
    n = nr * nz
    f = [_arr(x) for x in field]
    st = {k: _arr(state[k]) for k in ("ne", "np", "nn", "rho", "se", "sp", "sn")}
    mu, nu, d3, sigma, diag = np.zeros(n), np.zeros(n), np.zeros(3 * n), np.zeros(n), np.zeros(8)
    chi_a = None if chi is None else _arr(chi)
    _o._check(_lib().oracle_fluid_coupled_step(
        ctypes.byref(as_config(cfg)), nr, nz, z_lo, dr, dz, dt, *map(_p, f), _p(_arr(ambient[0])),
        _p(_arr(ambient[1])), _p(_arr(current[0])), _p(_arr(current[1])),
        *[_p(st[k]) for k in ("ne", "np", "nn", "rho", "se", "sp", "sn")], _p(chi_a), _p(mu), _p(nu), _p(d3),
        _p(sigma), _p(diag)))
    st.update(mu=mu, nu=nu, diffusion=d3.reshape(3, n), sigma=sigma)
    return tuple(f), st, dict(zip(COUPLED_DIAG, diag))
