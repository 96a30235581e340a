"""DRAM traffic per particle-step of the electron transport kernel, the
counter behind the bench line's roofline.traffic.

  run     stages n electrons of the scale-up seed distribution (the bench's
          electron population: K log-uniform 1-20 MeV in the -E hemisphere,
          5 m x 10 m disk, E_z = -500 kV/m, 256 x 2048 cells) and runs
          `launches` resident electron phases of 0.5 ns.  Meant to run under
              ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum,
                  sm__pipe_fp64_cycles_active.avg.pct_of_peak_sustained_active
                  --print-units base --clock-control none
                  -k regex:electron_step_kernel -s 1 -c 1 --csv --log-file <csv>
          (a pass or two on this one launch of 1 M electrons).
  record  reads that CSV and writes profiles/electron_step_kernel_traffic.json:
          (read + write bytes) / n per particle-step (every staged electron is
          live in the captured launch), with the library's source digest, so
          the bench never applies a record to another kernel build.
"""
import argparse
import csv
import json
import os

from . import build, gpu, workloads
from .gpu import DEFAULT_TABLES

CASE = "scaleup_c1"
DT_S = 5.0e-10
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RECORD = os.path.join(ROOT, "profiles", "electron_step_kernel_traffic.json")
METRICS = ("dram__bytes_read.sum", "dram__bytes_write.sum", "gpu__time_duration.sum")
# recorded when the capture has it (the FP64 pipe is the kernel's real bound)
FP64_PIPE = "sm__pipe_fp64_cycles_active.avg.pct_of_peak_sustained_active"


def run(n, launches, threads=128, blocks_per_sm=16):
    cfg = workloads.make_config(gpu, CASE)
    ctx = gpu.RreaGpuContext(cfg, n)
    try:
        ctx.load_tables(DEFAULT_TABLES)
        ctx.set_field(**workloads.make_field(CASE))
        ctx.set_launch(threads, blocks_per_sm, diagnostics=False)
        ctx.stage_electrons(workloads.make_electrons(CASE, n))
        moved = []
        for step in range(launches):
            # the same staged tile every launch: restage between launches so
            # each one moves the n electrons of the draw
            if step:
                ctx.stage_electrons(workloads.make_electrons(CASE, n))
            ctx.reset_sources()
            ctx.step_electrons_resident(step, DT_S)
            moved.append(ctx.last_step_stats()[0])
        return moved
    finally:
        ctx.close()


def read_capture(path):
    """The captured launch's metrics (base units) from an ncu --csv log."""
    values = {}
    with open(path, newline="") as f:
        lines = [ln for ln in f if ln.startswith('"')]
    for row in csv.DictReader(lines):
        if "electron_step_kernel" not in row.get("Kernel Name", ""):
            continue
        name = row.get("Metric Name")
        if name in METRICS or name == FP64_PIPE:
            values[name] = float(row["Metric Value"].replace(",", ""))
    missing = [m for m in METRICS if m not in values]
    if missing:
        raise ValueError(f"{path}: no {', '.join(missing)} for electron_step_kernel")
    return values


def record(path, n, out=RECORD, command=""):
    v = read_capture(path)
    traffic = v["dram__bytes_read.sum"] + v["dram__bytes_write.sum"]
    rec = {"kernel": "electron_step_kernel", "source_digest": build.source_digest(),
           "electrons": n, "dram_bytes_read": v["dram__bytes_read.sum"],
           "dram_bytes_write": v["dram__bytes_write.sum"], "duration_ns": v["gpu__time_duration.sum"],
           "dram_bytes_per_particle_step": traffic / n,
           "fp64_pipe_pct": v.get(FP64_PIPE),
           "capture": f"one electron phase of {n} scale-up electrons under ncu, {command}".strip()}
    with open(out, "w") as f:
        json.dump(rec, f, indent=1)
        f.write("\n")
    return rec


def main():
    p = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    sub = p.add_subparsers(dest="cmd", required=True)
    r = sub.add_parser("run")
    r.add_argument("--electrons", type=int, default=1 << 20)
    r.add_argument("--launches", type=int, default=2)
    w = sub.add_parser("record")
    w.add_argument("--csv", required=True)
    w.add_argument("--electrons", type=int, default=1 << 20)
    w.add_argument("--out", default=RECORD)
    args = p.parse_args()
    if args.cmd == "run":
        print(json.dumps({"electrons": args.electrons, "moved": run(args.electrons, args.launches)}))
    else:
        print(json.dumps(record(args.csv, args.electrons, args.out)))


if __name__ == "__main__":
    main()
