"""The plane CSV writer's host logic (avalanche.PlaneFluxCsv), no GPU:
RreaPlaneFluxState's cadence (I/RreaPlaneFlux.H:339-413: due at or past the
next multiple of the interval within 32 ulps, a duplicate refused, a forced
write before the boundary keeps the schedule, a late write skips the missed
boundaries) and the core field mean of MaybeWriteCdPlaneFlux
(O/RreaCouplingPlaneWriter.cpp:50-125) on a uniform and a linear field."""
import types

import numpy as np
import pytest


def _writer(tmp_path, ambient, planes=(1.0, 2.5), interval=1.0e-7, core=3.0):
    from rrea_feedback_warpx_amrex_geant4_gb300 import avalanche
    return avalanche.PlaneFluxCsv(str(tmp_path / "p.csv"), planes, interval, core, ambient)


def _cfg(nr=4, nz=8):
    return types.SimpleNamespace(nr=nr, nz=nz, r_lo=0.0, r_hi=8.0, z_lo=0.0, z_hi=4.0)


def test_cadence(tmp_path):
    w = _writer(tmp_path, np.zeros(4 * 9))
    assert not w.due(0, 0.5e-7)
    assert w.due(1, 1.0e-7 - 1e-22)            # within the roundoff tolerance
    w.mark_written(1, 1.0e-7 - 1e-22)
    assert w.next_time_s == pytest.approx(2.0e-7)
    assert not w.due(1, 1.0e-7 - 1e-22)        # duplicate
    assert w.due(2, 1.5e-7, force=True)
    w.mark_written(2, 1.5e-7)                  # forced before the boundary: schedule kept
    assert w.next_time_s == pytest.approx(2.0e-7)
    w.mark_written(3, 4.2e-7)                  # late: past the missed boundaries
    assert w.next_time_s == pytest.approx(5.0e-7)
    assert w.writes == 3
    with pytest.raises(ValueError):
        _writer(tmp_path, np.zeros(36), planes=(2.0, 1.0))


def test_core_means(tmp_path):
    cfg = _cfg()
    amb = np.full(4 * 9, -4.0e5)
    w = _writer(tmp_path, amb)
    means = w.core_means(cfg, np.zeros(4 * 9))
    for total, ambient in means:
        assert total == pytest.approx(-4.0e5, rel=1e-15) and ambient == pytest.approx(-4.0e5, rel=1e-15)
    # scattered E_z linear in z: the cell-centre rows bracket the plane
    zf = np.arange(9) * 0.5
    scattered = np.repeat(100.0 * zf, 4)
    means = w.core_means(cfg, scattered)
    for (total, ambient), z in zip(means, (1.0, 2.5)):
        assert total - ambient == pytest.approx(100.0 * z, rel=1e-12)
