"""Charge-exact CIC thinning on the GPU (rrea_gpu_thin_cic_groups) against
the reference's own RreaThinCicWeights / RreaCicResampleRemovalCapacity
compiled by oracle/ref_golden.cpp (tests/golden/ref_cic_thin_*.npy): 400
seeded support groups of 2 to 12 particles, with repeated support points,
fractions on the cell faces, zero weights and partial removal budgets.

Tolerances: removed, draws, validity and capacity exact; which particles
end at weight 0 exact; surviving weights within 4 ulps (the reference works
in x86 extended precision, the GPU in double-double)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, TABLES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu, workloads
    build.build()
    c = gpu.RreaGpuContext(workloads.make_config(gpu, "uniform_c0"), 16)
    c.load_tables(TABLES)
    yield gpu, c
    c.close()


def _golden():
    parts = np.load(os.path.join(GOLDEN, "ref_cic_thin_particles.npy"))
    groups = np.load(os.path.join(GOLDEN, "ref_cic_thin_groups.npy"))
    n = groups[:, 0].astype(np.int64)
    offsets = np.concatenate([[0], np.cumsum(n)])
    keys = (groups[:, 2].astype(np.uint64) << np.uint64(32)) | groups[:, 3].astype(np.uint64)
    return parts, groups, offsets, keys


def test_thinning_matches_reference(ctx):
    gpu, c = ctx
    parts, groups, offsets, keys = _golden()
    w, removed, draws, valid, cap = c.thin_cic_groups(parts[:, 1], parts[:, 2], parts[:, 3], offsets,
                                                       groups[:, 1].astype(np.int64), keys)
    np.testing.assert_array_equal(valid, groups[:, 6].astype(np.int32))
    np.testing.assert_array_equal(cap, groups[:, 7].astype(np.int64))
    np.testing.assert_array_equal(removed, groups[:, 4].astype(np.int64))
    np.testing.assert_array_equal(draws, groups[:, 5].astype(np.int64))
    ref = parts[:, 4]
    np.testing.assert_array_equal(w == 0.0, ref == 0.0)
    live = ref > 0.0
    assert np.all(np.abs(w[live] - ref[live]) <= 4.0 * np.spacing(ref[live]))
    assert removed.sum() > 0


def test_thinning_conserves_the_cell_charges(ctx):
    """Every group's four CIC cell charges survive the thinning to
    round-off (the reference's own verifier tolerance)."""
    gpu, c = ctx
    parts, groups, offsets, keys = _golden()
    fr, fz, w0 = parts[:, 1], parts[:, 2], parts[:, 3]
    w, removed, *_ = c.thin_cic_groups(fr, fz, w0, offsets, groups[:, 1].astype(np.int64), keys)
    cols = np.stack([(1 - fr) * (1 - fz), fr * (1 - fz), (1 - fr) * fz, fr * fz], axis=1)
    gid = np.repeat(np.arange(len(groups)), np.diff(offsets))
    before = np.zeros((len(groups), 4))
    after = np.zeros((len(groups), 4))
    np.add.at(before, gid, cols * w0[:, None])
    np.add.at(after, gid, cols * w[:, None])
    tol = 512 * np.finfo(float).eps * np.diff(offsets)[:, None] * np.maximum(1.0, np.abs(before))
    assert np.all(np.abs(after - before) <= tol)


def test_thinning_refuses_oversized_groups(ctx):
    gpu, c = ctx
    n = 65
    with pytest.raises(gpu.RreaGpuError) as e:
        c.thin_cic_groups(np.full(n, 0.5), np.full(n, 0.5), np.ones(n), [0, n], [1], [1])
    assert e.value.status == 1
