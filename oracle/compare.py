"""ORACLE: test infrastructure only.

Parity comparison of one GPU species phase (electron, positron or photon) against the
oracle on the same input tile.  Discrete results (dispositions, substep and hazard-draw counts,
validity, secondary keys) must match exactly; FP64 state within 1e-12
relative (positions with a 1e-12 x domain-size floor), except at most
0.1 % of the entries (at least one), which stay within 1e-11: a particle
with tens of interleaved events accumulates the last-ulp differences of the
device's FMA contraction and log/exp against the x86-64 host arithmetic;
cell-source grids, which the GPU accumulates with atomics in
nondeterministic order, within 1.6e-11 of each grid's largest cell, except
at most 0.1 % of the nonzero cells (at least four: one deposit's CIC
stencil) within the bound that the position tolerance carries into a CIC
weight (1e-12 x domain / cell size of the grid's largest cell).
"""
import numpy as np

from . import oracle as _oracle
from rrea_feedback_warpx_amrex_geant4_gb300.workloads import copy_tile

RTOL = 1.0e-12
TAIL_FRACTION = 1.0e-3
TAIL_RTOL = 1.0e-11


def _close(a, b, rtol, atol):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b) <= atol + rtol * np.maximum(np.abs(a), np.abs(b))


def entries_ok(a, b, atol):
    """True when every entry is within RTOL (relative, with the absolute
    floor atol) but at most TAIL_FRACTION of them (at least one), which
    stay within TAIL_RTOL; returns (ok, n_over_rtol)."""
    strict = _close(a, b, RTOL, atol)
    loose = _close(a, b, TAIL_RTOL, np.asarray(atol, dtype=np.float64) * (TAIL_RTOL / RTOL))
    n_over = int((~strict).sum())
    allowed = max(1, int(TAIL_FRACTION * strict.size))
    return bool(loose.all() and n_over <= allowed), n_over


def cells_ok(g, o, spread=0.0):
    """Cell grid check: every cell within 16 RTOL of the grid's largest
    cell (a cell sums up to ~10^4 deposits in arbitrary order), except at
    most TAIL_FRACTION of the nonzero cells (at least four), which stay
    within `spread` of it (the position tolerance over the cell size: the
    CIC weights move that much when a deposit's position does).  Returns
    (ok, n_over)."""
    g = np.asarray(g, dtype=np.float64)
    o = np.asarray(o, dtype=np.float64)
    scale = max(np.abs(o).max(), 1e-300)
    strict = _close(g, o, 0.0, 16 * RTOL * scale)
    loose = _close(g, o, 0.0, max(16 * RTOL, spread) * scale)
    n_over = int((~strict).sum())
    nonzero = int(((g != 0.0) | (o != 0.0)).sum())
    allowed = max(4, int(TAIL_FRACTION * nonzero))
    return bool(loose.all() and n_over <= allowed), n_over


def _worst(a, b, atol):
    """Largest |a-b| / (atol + max|a|,|b|) over the compared entries."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.size == 0:
        return 0.0
    scale = np.asarray(atol, dtype=np.float64) / RTOL + np.maximum(np.abs(a), np.abs(b))
    return float(np.max(np.abs(a - b) / np.where(scale > 0, scale, 1.0)))


def run_pair(ctx, cfg, field, arr, step, dt_s, species="electron"):
    """Runs GPU (apply mode) and oracle on copies of `arr` for one species
    phase ("electron", "positron" or "photon"); returns both."""
    g_arr = copy_tile(arr)
    o_arr = copy_tile(arr)
    ctx.reset_sources()
    if species == "photon":
        g_sec = ctx.apply_photons(g_arr, step, dt_s)
    elif species == "positron":
        g_sec = ctx.apply_positrons(g_arr, step, dt_s)
    else:
        g_sec = ctx.apply_electrons(g_arr, step, dt_s)
    n = arr["id"].shape[0]
    g_sub, g_ev, g_disp = ctx.diagnostics(n)
    g_cells = ctx.sources()
    if species == "photon":
        o = _oracle.photon_step(cfg, step, dt_s, o_arr)
    elif species == "positron":
        o = _oracle.positron_step(cfg, field, step, dt_s, o_arr)
    else:
        o = _oracle.electron_step(cfg, field, step, dt_s, o_arr)
    return (g_arr, g_sec, g_sub, g_ev, g_disp, g_cells), (o_arr, o)


ME_C2 = 510998.95


def compare(cfg, gpu, orc, domain_scale, parent_energy=None):
    """Returns a list of mismatch descriptions (empty when parity holds).

    `parent_energy` (per input particle, eV) makes the secondary tolerances
    follow the conditioning of the final-state arithmetic: a secondary's
    energy and momentum are differences of parent-scale quantities (Compton
    recoil = E - E', recoil momentum = E d - E' d'), so one rounding of the
    parent-scale operands moves them by ~1e-16 x E_parent.  Energies then
    get an absolute floor of 1e-12 x E_parent and directions 1e-12 x
    E_parent / |p_secondary|."""
    g_arr, g_sec, g_sub, g_ev, g_disp, g_cells = gpu
    o_arr, o = orc
    problems = []
    if not np.array_equal(g_disp, o["disposition"]):
        bad = np.nonzero(g_disp != o["disposition"])[0]
        problems.append(f"disposition differs at {bad[:10].tolist()} ({len(bad)} particles)")
    if not np.array_equal(g_sub, o["subcycles"]):
        bad = np.nonzero(g_sub != o["subcycles"])[0]
        problems.append(f"subcycles differ at {bad[:10].tolist()} ({len(bad)})")
    if not np.array_equal(g_ev, o["events"]):
        bad = np.nonzero(g_ev != o["events"])[0]
        problems.append(f"hazard draws differ at {bad[:10].tolist()} ({len(bad)})")
    if not np.array_equal(g_arr["id"], o_arr["id"]):
        problems.append("validity (id sign) differs")
    alive = (o_arr["id"] > 0) & (o["disposition"] == 0)
    atol_pos = RTOL * domain_scale
    for name, atol in (("z", atol_pos), ("r", atol_pos)):
        ok, n_over = entries_ok(g_arr[name][alive], o_arr[name][alive], atol)
        if not ok:
            w = _worst(g_arr[name][alive], o_arr[name][alive], atol)
            problems.append(f"{name} differs for {n_over} survivors (worst {w:.2e})")
    gx, gy = g_arr["r"] * np.cos(g_arr["theta"]), g_arr["r"] * np.sin(g_arr["theta"])
    ox, oy = o_arr["r"] * np.cos(o_arr["theta"]), o_arr["r"] * np.sin(o_arr["theta"])
    for name, a, b in (("x", gx, ox), ("y", gy, oy)):
        ok, n_over = entries_ok(a[alive], b[alive], atol_pos * 4)
        if not ok:
            w = _worst(a[alive], b[alive], atol_pos * 4)
            problems.append(f"{name} differs for {n_over} survivors (worst {w:.2e})")
    umag = np.sqrt(o_arr["ux"] ** 2 + o_arr["uy"] ** 2 + o_arr["uz"] ** 2)
    moved = o["disposition"] <= 1
    moved &= o["disposition"] >= 0
    for name in ("ux", "uy", "uz"):
        ok, n_over = entries_ok(g_arr[name][moved], o_arr[name][moved], RTOL * umag[moved])
        if not ok:
            strict = _close(g_arr[name][moved], o_arr[name][moved], RTOL, RTOL * umag[moved])
            w = _worst(g_arr[name][moved], o_arr[name][moved], RTOL * umag[moved])
            idx = np.nonzero(moved)[0][~strict][:5].tolist()
            problems.append(f"{name} differs for {n_over} particles (worst {w:.2e} of |u|; at {idx}, "
                            f"substeps {o['subcycles'][idx].tolist()}, events {o['events'][idx].tolist()})")
    os_ = o["secondaries"]
    if len(g_sec) != len(os_):
        problems.append(f"secondary count {len(g_sec)} vs oracle {len(os_)}")
    else:
        for key in ("species", "process", "parent_index", "root_key", "lineage", "root_species"):
            if not np.array_equal(g_sec[key], os_[key]):
                problems.append(f"secondary {key} differs")
        atol_e = 0.0
        atol_dir = RTOL
        if parent_energy is not None and len(os_):
            ep = np.asarray(parent_energy, dtype=np.float64)[os_["parent_index"]]
            ek = os_["energy_eV"]
            p_sec = np.where(os_["species"] == 2, ek, np.sqrt(np.maximum(ek * (ek + 2.0 * ME_C2), 0.0)))
            atol_e = RTOL * ep
            atol_dir = np.maximum(RTOL, RTOL * ep / np.maximum(p_sec, 1.0))
        for key, atol in (("x", atol_pos), ("y", atol_pos), ("z", atol_pos), ("dir_x", atol_dir),
                          ("dir_y", atol_dir), ("dir_z", atol_dir), ("weight", 0.0), ("energy_eV", atol_e),
                          ("birth_fraction", RTOL)):
            ok, n_over = entries_ok(g_sec[key], os_[key], atol)
            if not ok:
                w = _worst(g_sec[key], os_[key], atol)
                problems.append(f"secondary {key} differs for {n_over} (worst {w:.2e})")
    cell = min((cfg.r_hi - cfg.r_lo) / cfg.nr, (cfg.z_hi - cfg.z_lo) / cfg.nz)
    spread = RTOL * domain_scale / cell
    for f in range(5):
        ok, n_over = cells_ok(g_cells[f], o["cells"][f], spread)
        if not ok:
            problems.append(f"cell source field {f} differs in {n_over} cells")
    return problems
