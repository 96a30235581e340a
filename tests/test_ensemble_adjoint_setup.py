"""Host-side setup of the batched and adjoint configurations (no GPU):
the batched ensemble's instances (E_z evenly spaced 300-1000 kV/m, seed
counts log-uniform 1e3-1e5, durations mapped linearly in 1/(E - 280 kV/m)
onto 0.5-4 us) and the adjoint's field profile (256 nodes over 0-500 m,
450 kV/m plus a seeded Gaussian-correlated perturbation of 20 kV/m with a
20 m correlation length)."""
import numpy as np


def test_batched_instances():
    from rrea_feedback_warpx_amrex_geant4_gb300 import ensemble
    inst = ensemble.batched_instances(64)
    e = np.array([i.field_v_per_m for i in inst])
    np.testing.assert_allclose(np.diff(e), (1.0e6 - 3.0e5) / 63)
    seeds = np.array([i.n_seeds for i in inst])
    assert seeds.min() >= 1000 and seeds.max() <= 100_000
    steps = np.array([i.steps for i in inst])
    assert steps.max() == 8000 and steps.min() == 1000          # 4 us and 0.5 us at 0.5 ns
    assert np.all(np.diff(steps) <= 0)                          # shorter runs in stronger fields
    assert ensemble.batched_instances(64, seed=7)[5].n_seeds == inst[5].n_seeds


def test_ensemble_seed_tile_marks_instances():
    from rrea_feedback_warpx_amrex_geant4_gb300 import ensemble
    inst = [ensemble.Instance(4e5, 3, 10), ensemble.Instance(5e5, 2, 10), ensemble.Instance(6e5, 4, 10)]
    t = ensemble.seed_tile(inst)
    np.testing.assert_array_equal(t["cpu"], [0, 0, 0, 1, 1, 2, 2, 2, 2])
    np.testing.assert_array_equal(t["id"], [1, 2, 3, 1, 2, 1, 2, 3, 4])
    only = ensemble.seed_tile(inst, only=[1])
    np.testing.assert_array_equal(only["cpu"], [1, 1])


def test_adjoint_field_profile():
    from rrea_feedback_warpx_amrex_geant4_gb300 import adjoint
    e = adjoint.adjoint_field_profile()
    assert e.shape == (256,)
    assert np.all(e < 0)                                        # along -z
    dev = -e - 4.5e5
    assert 5e3 < dev.std() < 4e4
    # neighbouring nodes (1.96 m apart) are strongly correlated at 20 m
    assert np.corrcoef(dev[:-1], dev[1:])[0, 1] > 0.9
    np.testing.assert_array_equal(adjoint.adjoint_field_profile(), e)   # seeded
