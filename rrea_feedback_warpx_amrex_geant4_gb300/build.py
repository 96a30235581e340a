"""Builds the GB300 kinetic-step library in-tree:
rrea_feedback_warpx_amrex_geant4_gb300/lib/librrea_gpu.so (sm_103a only).

Parity-study and tuning variants (RREA_LIBM=1: CUDA's log/exp in place of
the table-driven ones; RREA_FMAD=0, below; RREA_DEFINES=NAME=VALUE,...:
compile-time settings such as RREA_NEWBORN_MIN_BLOCKS) build into the path
RREA_GPU_LIB names, with their own object directory, and the bindings load
from there when RREA_GPU_LIB is set; the default build is the product.

FP64 FMA contraction is on (--fmad=true): GB300's FP64 pipe issues a fused
multiply-add for the price of a multiply, a measured 9 % of the electron
kernel.  RREA_FMAD=0 builds with --fmad=false, whose products and sums round
like the reference's x86-64 host build (no FMA), to isolate last-ulp
differences when chasing a parity question.
"""
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.environ.get("RREA_GPU_LIB") or os.path.join(LIBDIR, "librrea_gpu.so")

SOURCES = [
    os.path.join(CSRC, "rrea_capi.cu"),
    os.path.join(CSRC, "rrea_kernels.cu"),
    os.path.join(CSRC, "rrea_photon_kernels.cu"),
    os.path.join(CSRC, "rrea_positron_kernels.cu"),
    os.path.join(CSRC, "rrea_noalloc.cu"),
    os.path.join(CSRC, "rrea_commit.cu"),
    os.path.join(CSRC, "rrea_resample.cu"),
    os.path.join(CSRC, "rrea_newborn.cu"),
    os.path.join(CSRC, "rrea_deposit.cu"),
    os.path.join(CSRC, "rrea_field.cu"),
    os.path.join(CSRC, "rrea_census.cu"),
    os.path.join(CSRC, "rrea_population.cu"),
    os.path.join(CSRC, "rrea_fluid.cu"),
    os.path.join(CSRC, "rrea_ensemble.cu"),
    os.path.join(CSRC, "rrea_adjoint.cu"),
    os.path.join(CSRC, "host", "table_set.cpp"),
    os.path.join(CSRC, "host", "seed_schedule.cpp"),
    os.path.join(CSRC, "host", "closure_table.cpp"),
]
# Sources compiled without FMA contraction whatever the variant: the carrier
# fluid rounds every product and sum like the reference's host build.
NO_FMAD = ("rrea_fluid.cu",)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _deps():
    out = []
    for d, _, files in os.walk(CSRC):
        out += [os.path.join(d, f) for f in files if f.endswith((".cu", ".cuh", ".h", ".hpp", ".cpp"))]
    out.append(os.path.join(ROOT, "include", "rrea_gpu.h"))
    return out


# the sources that define the charged and photon transport kernels
KERNEL_SOURCES = ("rrea_kernels.cu", "rrea_kernels.h", "rrea_photon_kernels.cu", "rrea_positron_kernels.cu")


def source_digest():
    """SHA-256 (first 16 hex digits) over the sources that define the
    transport kernels (the device headers and their translation units) and
    the build flag that changes their code: the identity of a kernel build,
    so a counter measured on one build is never applied to another."""
    import hashlib

    files = [os.path.join(CSRC, f) for f in KERNEL_SOURCES]
    dev = os.path.join(CSRC, "device")
    files += [os.path.join(dev, f) for f in os.listdir(dev)]
    h = hashlib.sha256()
    for path in sorted(files):
        h.update(os.path.relpath(path, ROOT).encode())
        with open(path, "rb") as f:
            h.update(f.read())
    h.update(("fmad=" + os.environ.get("RREA_FMAD", "1")).encode())
    h.update(("libm=" + os.environ.get("RREA_LIBM", "0")).encode())
    h.update(("defines=" + os.environ.get("RREA_DEFINES", "")).encode())
    return h.hexdigest()[:16]


def build(force=False, verbose=False):
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in _deps()):
            return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    defines = [d for d in os.environ.get("RREA_DEFINES", "").split(",") if d]
    variant = f"fmad{os.environ.get('RREA_FMAD', '1')}_libm{os.environ.get('RREA_LIBM', '0')}"
    if defines:
        variant += "_" + "_".join(d.replace("=", "") for d in defines)
    objdir = os.path.join(PKG, "_build" if variant == "fmad1_libm0" else "_build_" + variant)
    os.makedirs(objdir, exist_ok=True)
    nvcc = _nvcc()
    fmad = "false" if os.environ.get("RREA_FMAD", "1") == "0" else "true"
    common = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I", CSRC, "-I", os.path.join(ROOT, "include")] + ARCH
    if os.environ.get("RREA_LIBM", "0") == "1":
        common += ["-DRREA_CUDA_LIBM"]
    common += ["-D" + d for d in defines]
    if verbose:
        common += ["-Xptxas", "-v"]
    objs = []
    procs = []
    for src in SOURCES:
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        cmd = [nvcc, "-c", src, "-o", obj] + common
        cmd += ["--fmad=false" if os.path.basename(src) in NO_FMAD else f"--fmad={fmad}"]
        if src.endswith(".cpp"):
            cmd = [nvcc, "-x", "cu", "-c", src, "-o", obj] + common
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), cmd))
        objs.append(obj)
    failed = False
    for p, cmd in procs:
        out, _ = p.communicate()
        if out and (verbose or p.returncode):
            sys.stdout.write(out.decode(errors="replace"))
        if p.returncode != 0:
            failed = True
    if failed:
        raise RuntimeError("nvcc compilation failed")
    tmp = LIB + ".tmp"
    subprocess.check_call([nvcc, "-shared", "-o", tmp] + objs + ARCH + ["-lz", "-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose="-v" in sys.argv))
