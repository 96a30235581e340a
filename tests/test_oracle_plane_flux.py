"""The plane-crossing diagnostic's restatement (oracle ForEachPlaneCrossing
and AccumulatePlaneCrossings) against the reference's own
RreaForEachNonperiodicPlaneCrossing and RreaPlaneFluxAccumulator
(I/RreaPlaneFlux.H), compiled into oracle/_ref/ref_golden:

  * 600 seeded segments over 8 planes (ends on planes, reversals, zero
    length, non-finite ends): the same planes, fractions and directions in
    the same order, bit for bit, and the same refusals;
  * 400 crossings added one by one (two invalid): the same refusals and the
    same 80 flattened accumulators, bit for bit."""
import os

import numpy as np

from conftest import GOLDEN


def _load(name):
    return np.load(os.path.join(GOLDEN, name + ".npy"))


def test_crossing_enumeration_matches_reference():
    from oracle import oracle
    segs = _load("ref_plane_segments")
    rows = _load("ref_plane_crossings")
    planes = _load("ref_plane_planes").ravel()
    got = oracle.plane_enumerate(segs[:, :2], planes)
    assert len(got) == len(segs)
    for i, (z0, z1, count) in enumerate(segs):
        if count < 0:
            assert got[i] is None, i
            continue
        want = rows[rows[:, 0] == i][:, 1:]
        assert got[i] is not None and len(got[i]) == int(count), i
        np.testing.assert_array_equal(got[i], want, err_msg=f"segment {i}")
    assert (segs[:, 2] > 1).sum() > 50          # multi-plane segments
    assert (segs[:, 2] < 0).sum() > 0           # refused geometry


def test_accumulator_matches_reference():
    from oracle import oracle
    batch = _load("ref_plane_batch")
    ok, bins = oracle.plane_accumulate(batch, len(_load("ref_plane_planes").ravel()))
    np.testing.assert_array_equal(ok, _load("ref_plane_batch_ok").ravel().astype(np.int32))
    np.testing.assert_array_equal(bins.ravel(), _load("ref_plane_flux").ravel())
    assert (ok == 0).sum() == 2
