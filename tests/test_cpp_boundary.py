"""The C-ABI boundary from C and C++ (the overlay's host language).

tests/cpp/overlay_host.cpp is a C++17 host shaped like the overlay's GB300
Apply body (SoA host tiles, rrea_gpu_apply_electrons, abort on a non-OK
status); tests/cpp/header_c11.c compiles the header as C11.  The CPU tests
build both with the system compilers against include/rrea_gpu.h and the
library, and check every structure offset the C++ compiler assigns against
the ctypes binding the other tests use.  The GPU test runs one electron
phase through the C++ host and through ctypes on the same input: the
outputs must be byte-identical (same library, same inputs)."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, TABLES

CPP = os.path.join(ROOT, "tests", "cpp")
INCLUDE = os.path.join(ROOT, "include")


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu
    if shutil.which("g++") is None or shutil.which("gcc") is None:
        pytest.skip("no C/C++ compiler")
    lib = build.build()
    out = tmp_path_factory.mktemp("cpp")
    exe = str(out / "overlay_host")
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", INCLUDE,
                    os.path.join(CPP, "overlay_host.cpp"), "-L", libdir, "-lrrea_gpu", f"-Wl,-rpath,{libdir}",
                    "-o", exe], check=True, capture_output=True, text=True)
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", INCLUDE, "-c",
                    os.path.join(CPP, "header_c11.c"), "-o", str(out / "header_c11.o")], check=True,
                   capture_output=True, text=True)
    return exe, gpu


def _layout(exe):
    out = subprocess.run([exe, "layout"], check=True, capture_output=True, text=True).stdout
    return {k: int(v) for k, v in (line.split() for line in out.splitlines())}


def test_cpp_struct_offsets_match_ctypes(host):
    exe, gpu = host
    lay = _layout(exe)
    for name, cls in (("rrea_gpu_config", gpu.RreaGpuConfig), ("rrea_gpu_tile", gpu.RreaGpuTile)):
        assert lay[name] == ctypes.sizeof(cls), name
        for field, _ in cls._fields_:
            assert lay[f"{name}.{field}"] == getattr(cls, field).offset, (name, field)
    for name, dt in (("rrea_gpu_secondary", gpu.SECONDARY_DTYPE), ("rrea_gpu_seed_event", gpu.SEED_EVENT_DTYPE)):
        assert lay[name] == dt.itemsize, name
        for field in dt.names:
            assert lay[f"{name}.{field}"] == dt.fields[field][1], (name, field)


def test_cpp_host_rejects_bad_usage(host):
    exe, _ = host
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 1 and "usage" in r.stderr


@pytest.mark.gpu
def test_cpp_host_apply_matches_ctypes(host, tmp_path):
    exe, gpu = host
    from rrea_feedback_warpx_amrex_geant4_gb300 import workloads
    n, step, dt = 2048, 3, 5.0e-10
    cfg = workloads.make_config(gpu, "scaleup_c1")
    tile = workloads.make_electrons("scaleup_c1", n, seed=515)
    cols = gpu.TILE_FIELDS
    with open(tmp_path / "in.bin", "wb") as f:
        f.write(bytes(cfg))
        f.write(np.int64(step).tobytes() + np.float64(dt).tobytes() + np.int64(n).tobytes())
        for c in cols:
            f.write(tile[c].tobytes())
        f.write(tile["id"].tobytes() + tile["cpu"].tobytes())
    r = subprocess.run([exe, "apply", TABLES, str(tmp_path / "in.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = (tmp_path / "out.bin").read_bytes()
    # the same phase through ctypes
    ctx = gpu.RreaGpuContext(cfg, n)
    ctx.load_tables(TABLES)
    ctx.set_field(**workloads.make_field("scaleup_c1"))
    ref = workloads.copy_tile(tile)
    sec = ctx.apply_electrons(ref, step, dt)
    ctx.close()
    off = 0
    for c in cols:
        got = np.frombuffer(raw, dtype=np.float64, count=n, offset=off)
        off += 8 * n
        np.testing.assert_array_equal(got, ref[c], err_msg=c)
    np.testing.assert_array_equal(np.frombuffer(raw, dtype=np.int64, count=n, offset=off), ref["id"])
    off += 8 * n
    n_sec = int(np.frombuffer(raw, dtype=np.int64, count=1, offset=off)[0])
    off += 8
    assert n_sec == len(sec) > 0
    assert raw[off:off + n_sec * gpu.SECONDARY_DTYPE.itemsize] == sec.tobytes()
