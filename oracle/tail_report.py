"""ORACLE: test infrastructure only.

Size of the FP64 parity tail of the GPU phases against the oracle: for each
case below, one phase on a seeded tile through the C-ABI and through the
oracle, then per compared quantity the largest relative difference and how
many particles exceed 1e-13, 1e-12 and 1e-10 (the measures behind
oracle/compare.py's rule).  Run it against each build variant of the
library to see which device arithmetic choice moves which results:

  RREA_FMAD=0   no FMA contraction (products and sums round as x86-64)
  RREA_LIBM=1   CUDA's log/exp in place of the table-driven ones

  python -m oracle.tail_report [--json out.json]

Discrete outcomes (dispositions, substeps, hazard draws, secondary keys)
must match exactly in every case; their mismatches are reported too.
"""
import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

CASES = [
    # (name, species, case, n, dt_s, k_lo_eV, k_hi_eV)
    ("e_scaleup_0.5ns", "electron", "scaleup_c1", 16384, 5.0e-10, None, None),
    ("e_uniform_c0_0.5ns", "electron", "uniform_c0", 8192, 5.0e-10, None, None),
    ("e_scaleup_10ns", "electron", "scaleup_c1", 8192, 1.0e-8, None, None),
    ("e_100MeV_1GeV_10ns", "electron", "scaleup_c1", 4096, 1.0e-8, 1.0e8, 1.0e9),
    ("p_scaleup_10ns", "positron", "scaleup_c1", 8192, 1.0e-8, None, None),
    ("g_scaleup_1us", "photon", "scaleup_c1", 16384, 1.0e-6, None, None),
]
ME_C2 = 510998.95


def _rel(a, b, scale):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    s = np.maximum(np.asarray(scale, dtype=np.float64), 1e-300)
    return np.abs(a - b) / s


def _stats(r):
    r = np.asarray(r)
    if r.size == 0:
        return {"n": 0, "max": 0.0, "gt_1e-13": 0, "gt_1e-12": 0, "gt_1e-10": 0}
    return {"n": int(r.size), "max": float(r.max()), "gt_1e-13": int((r > 1e-13).sum()),
            "gt_1e-12": int((r > 1e-12).sum()), "gt_1e-10": int((r > 1e-10).sum())}


def run_case(ctx, gpu, workloads, compare, oracle, name, species, case, n, dt_s, k_lo, k_hi):
    cfg = workloads.make_config(gpu, case)
    field = workloads.make_field(case)
    if species == "photon":
        arr = workloads.make_photons(case, n, dt_s, seed=4711, e_lo=5.0e4, e_hi=1.0e8)
    else:
        arr = workloads.make_electrons(case, n, seed=4711)
        if k_lo is not None:
            rng = np.random.default_rng(4712)
            k = np.exp(rng.uniform(np.log(k_lo), np.log(k_hi), n))
            d = np.stack([arr["ux"], arr["uy"], arr["uz"]], 1)
            d /= np.linalg.norm(d, axis=1)[:, None]
            u = workloads.proper_velocity(k)
            for i, f in enumerate(("ux", "uy", "uz")):
                arr[f][:] = u * d[:, i]
            workloads.capture_prev(arr)
    g, o = compare.run_pair(ctx, cfg, field, arr, 2, dt_s, species=species)
    g_arr, g_sec, g_sub, g_ev, g_disp, g_cells = g
    o_arr, orc = o
    out = {"case": name, "particles": n,
           "discrete_mismatches": int((g_disp != orc["disposition"]).sum() + (g_sub != orc["subcycles"]).sum()
                                      + (g_ev != orc["events"]).sum()),
           "secondaries": [int(len(g_sec)), int(len(orc["secondaries"]))]}
    alive = (o_arr["id"] > 0) & (orc["disposition"] == 0)
    scale_pos = max(cfg.r_hi, cfg.z_hi)
    for f in ("r", "z"):
        # positions relative to the domain size plus the coordinate (the
        # measure oracle/compare.py holds to 1e-12)
        out[f] = _stats(_rel(g_arr[f][alive], o_arr[f][alive], np.abs(o_arr[f][alive]) + scale_pos))
    moved = (orc["disposition"] >= 0) & (orc["disposition"] <= 1)
    umag = np.sqrt(o_arr["ux"] ** 2 + o_arr["uy"] ** 2 + o_arr["uz"] ** 2)
    for f in ("ux", "uy", "uz"):
        out[f] = _stats(_rel(g_arr[f][moved], o_arr[f][moved], umag[moved]))
    if len(g_sec) == len(orc["secondaries"]) and len(g_sec):
        os_ = orc["secondaries"]
        out["secondary_energy"] = _stats(_rel(g_sec["energy_eV"], os_["energy_eV"], np.abs(os_["energy_eV"])))
        out["secondary_dir_z"] = _stats(_rel(g_sec["dir_z"], os_["dir_z"], 1.0))
    scale = max(np.abs(orc["cells"]).max(), 1e-300)
    out["cells"] = _stats(np.abs(g_cells - orc["cells"]).ravel() / scale)
    return out


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--json", default=None)
    a = p.parse_args()
    import torch

    from oracle import compare, oracle
    from rrea_feedback_warpx_amrex_geant4_gb300 import DEFAULT_TABLES, build, gpu, workloads

    torch.cuda.set_device(0)
    build.build()
    oracle.load_tables(DEFAULT_TABLES)
    rows = []
    for name, species, case, n, dt_s, k_lo, k_hi in CASES:
        cfg = workloads.make_config(gpu, case)
        ctx = gpu.RreaGpuContext(cfg, n)
        ctx.load_tables(DEFAULT_TABLES)
        ctx.set_field(**workloads.make_field(case))
        rows.append(run_case(ctx, gpu, workloads, compare, oracle, name, species, case, n, dt_s, k_lo, k_hi))
        ctx.close()
    report = {"variant": {"RREA_FMAD": os.environ.get("RREA_FMAD", "1"), "RREA_LIBM": os.environ.get("RREA_LIBM", "0")},
              "library": gpu.LIB_PATH, "cases": rows}
    text = json.dumps(report)
    if a.json:
        with open(a.json, "w") as f:
            f.write(text)
    print(text)


if __name__ == "__main__":
    main()
