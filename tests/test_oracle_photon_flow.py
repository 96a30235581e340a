"""The photon energy-flow ledger check (DrainAndCommitSecondaries'
transaction validation, O/RreaSecondaryCommit.cpp:55-160, with the splits
of O/RreaParticleInteraction.H:1015-1090) that the oracle and the device
phases run at every Compton, photoelectric and pair interaction.  Mistakes
are planted in the check's inputs on the CPU: a payload whose parts miss the
incident energy by more than 64 eps of it, a negative or non-finite part, a
pair whose booked local flow is not what its energies leave."""
import numpy as np

ME = 510998.95


def _row(kind, w, inc, x1, x2, x3=0.0, recoil=False, local=0.0):
    return [kind, w, inc, x1, x2, x3, 1.0 if recoil else 0.0, local]


def test_consistent_interactions_pass(oracle_mod):
    inc = 3.7e6
    rows = [
        _row(0, 1.0, inc, 1.2e6, inc - 1.2e6),                  # Compton
        _row(1, 2.0, 8.0e4, 8.0e4 - 87.0, 87.0),                # photoelectric
        _row(2, 1.0, inc, 1.0e6, 0.9e6, local=inc - 2 * ME - 1.9e6),            # nuclear pair
        _row(2, 1.0, inc, 1.0e6, 0.9e6, 0.4e6, True, inc - 2 * ME - 2.3e6),     # triplet
        _row(2, 1.0, 2 * ME + 10.0, 5.0, 5.0, local=0.0),        # at threshold
    ]
    assert oracle_mod.photon_flow_valid(rows).all()


def test_planted_mistakes_fail(oracle_mod):
    inc = 3.7e6
    tol = 64 * np.finfo(float).eps * inc
    rows = [
        _row(0, 1.0, inc, 1.2e6, inc - 1.2e6 + 4 * tol),        # parts exceed the incident energy
        _row(0, 1.0, inc, -1.0, inc + 1.0),                      # negative recoil
        _row(0, 0.0, inc, 1.2e6, inc - 1.2e6),                   # zero weight
        _row(1, 1.0, 8.0e4, np.nan, 87.0),                       # non-finite photoelectron
        _row(1, 1.0, 8.0e4, 8.0e4, 87.0),                        # binding counted twice
        _row(2, 1.0, inc, 1.0e6, 0.9e6, local=inc - 2 * ME - 1.9e6 + 4 * tol),   # local off
        _row(2, 1.0, inc, 1.0e6, 0.9e6, 0.4e6, True, inc - 2 * ME - 1.9e6),      # recoil left out
        _row(2, 1.0, inc, 1.0e6, 0.9e6, local=-5.0e3),           # negative local below a positive split
    ]
    ok = oracle_mod.photon_flow_valid(rows)
    assert not ok.any(), ok
