"""ORACLE build (test infrastructure only): compiles the CPU restatement into
oracle/liboracle.so with g++.  Contraction of a*b+c into FMA is disabled so
the restatement rounds like the reference's x86-64 build on any host."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "liboracle.so")
SOURCES = [
    os.path.join(HERE, "oracle_core.cpp"),
    os.path.join(HERE, "oracle_api.cpp"),
    os.path.join(HERE, "fluid.cpp"),
    os.path.join(ROOT, "rrea_feedback_warpx_amrex_geant4_gb300", "csrc", "host", "closure_table.cpp"),
    os.path.join(ROOT, "rrea_feedback_warpx_amrex_geant4_gb300", "csrc", "host", "table_set.cpp"),
]


def build_oracle(force=False):
    deps = SOURCES + [os.path.join(HERE, "oracle_core.hpp"), os.path.join(HERE, "interleave.hpp"),
                          os.path.join(HERE, "interleave_scenarios.hpp"), os.path.join(HERE, "fluid.hpp")]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB
    cmd = ["g++", "-std=c++17", "-O3", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
           "-I", ROOT] + SOURCES + ["-lz", "-o", LIB + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def reference_dir():
    """The reference checkout: $RREA_REFERENCE_DIR, else a `reference`
    directory beside the repository."""
    return os.environ.get("RREA_REFERENCE_DIR") or os.path.join(os.path.dirname(ROOT), "reference")


def build_reference_golden(reference=None):
    """Builds oracle/_ref/ref_golden from the reference's own sources when the
    reference checkout is present (never on the GPU host)."""
    reference = reference or reference_dir()
    if not os.path.isdir(os.path.join(reference, "native_amrex_rrea")):
        return None
    subprocess.check_call(["make", "-s", "-f", os.path.join("oracle", "Makefile.ref"), f"REF={reference}",
                           "oracle/_ref/ref_golden", "oracle/_ref/ref_golden_fluid"], cwd=ROOT)
    return os.path.join(HERE, "_ref", "ref_golden")


if __name__ == "__main__":
    print(build_oracle(force=True))
