"""The oracle's charged-loop skeletons (oracle/interleave.hpp, which its
electron, positron and newborn loops run through) against the reference's
own templates RreaRunChargedEventInterleave and
RreaRunChargedSubstepInterleave (O/RreaChargedInterleave.H:546-732).

tests/golden/ref_interleave_*.npy hold the traces the reference templates
produce when oracle/_ref/ref_golden drives them with the scripted policies
of oracle/interleave_scenarios.hpp: every policy call with its arguments
(frozen energies, segment ends, ordinals, gate queries, event fractions,
stops), aborts, and the final energy, ordinal and event counts.  The first
eight event scenarios are the fixtures of the reference's own smoke
(refreeze at the survivor energy, loss to the exact sampled depth, null event
on a drag-closed channel, consumed parent, cutoff stop) plus an ordinal-cap
abort, an invalid revalidation and a three-channel pick; the rest are
seeded random scripts.  The oracle's traces must be bit-identical."""
import os

import numpy as np
import pytest

from conftest import GOLDEN


def _golden(name):
    return np.load(os.path.join(GOLDEN, name))


@pytest.mark.parametrize("kind,name", [(0, "ref_interleave_events.npy"), (1, "ref_interleave_substeps.npy")])
def test_skeleton_traces_match_reference(oracle_mod, kind, name):
    ref = _golden(name)
    seeds = np.unique(ref[:, 0]).astype(np.int64)
    assert len(seeds) >= 300
    for seed in seeds:
        want = ref[ref[:, 0] == seed][:, 1:]
        got = oracle_mod.interleave_trace(kind, int(seed))
        assert got.shape == want.shape, f"scenario {seed}: {got.shape} records vs {want.shape}"
        np.testing.assert_array_equal(got, want, err_msg=f"scenario {seed}")


def test_event_scenarios_cover_every_path():
    ref = _golden("ref_interleave_events.npy")
    codes = ref[:, 1].astype(int)
    for code, what in ((5, "mid-chord stop"), (8, "final state"), (9, "abort"), (7, "gate query")):
        assert (codes == code).sum() >= 10, what
    # null events: a closed gate at the event followed by an open one at the frozen energy
    gates = ref[codes == 7]
    assert ((gates[:, 4] == 0.0)).sum() >= 10
    # the smoke's refreeze fixture: the second iteration freezes 7.75e5 eV
    s0 = ref[(ref[:, 0] == 0) & (codes == 1)]
    assert s0[1, 2] == 7.75e5


def test_substep_scenarios_cover_every_exit():
    ref = _golden("ref_interleave_substeps.npy")
    ends = ref[ref[:, 1] == 17]
    assert (ends[:, 3] == 1.0).sum() >= 20, "sticky exits"
    assert (ends[:, 3] == 0.0).sum() >= 20, "runs that stay in the domain"
    assert len(np.unique(ends[:, 2])) >= 4, "varied committed-substep counts"
