"""The oracle's restatement of the particle charge deposit (DepositChargeCIC,
I/RreaSegmentDepositionRZ.H:68-92, the convention of the overlay's
DepositParticleChargeToRreaGrid, O/RreaWarpXCoupling.cpp:376-389) against
the reference header compiled into oracle/_ref/ref_golden: 3000 charges of
both signs, some within half a cell of the axis (folded), some beyond the
outer radius and the z edges (clamped).  Bit-exact: the same products,
added in the same order."""
import os

import numpy as np

from conftest import GOLDEN


def test_cic_charge_matches_reference(oracle_mod):
    grid = np.load(os.path.join(GOLDEN, "ref_cic_charge_grid.npy"))[0]
    parts = np.load(os.path.join(GOLDEN, "ref_cic_charge_particles.npy"))
    rho = np.load(os.path.join(GOLDEN, "ref_cic_charge_rho.npy"))[:, 0]
    nr, nz, dr, dz, r_lo, z_lo = int(grid[0]), int(grid[1]), grid[2], grid[3], grid[4], grid[5]
    got = oracle_mod.deposit_charge_cic(nr, nz, dr, dz, r_lo, z_lo, parts[:, 0], parts[:, 1], parts[:, 2])
    np.testing.assert_array_equal(got, rho)
    assert abs(got.sum() - parts[:, 2].sum()) <= 1e-12 * np.abs(parts[:, 2]).sum()  # charge kept
