"""Pins the oracle restatement to the reference's own compiled primitives
(tests/golden/ref_*.npy, written by oracle/ref_golden.cpp from the
reference sources).  Bit-exact for integer and index work; FP64 outputs must
match exactly (the restatement performs the same operations in the same
order with the same libm)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

PINS = [  # S/RreaRngEndpointSmoke.cpp kGoldenPins
    ((0x0, 0x0, 0x0, 0x0, 0x0), 0x3db5adc86dfdd12d, float.fromhex("0x1.edad6e436feecp-3")),
    ((0x1, 0x2, 0x3, 0x4, 0x5), 0x5d3617c86eb12224, float.fromhex("0x1.74d85f21bac4ap-2")),
    ((0xdeadbeef, 0x2bdc545d6b4b87, 0x2a, 0x7, 0x33), 0xeb74a9e550130b92, float.fromhex("0x1.d6e953caa0261p-1")),
    ((0x7ea, 0x1, 0x186a0, 0x3, 0x63), 0xaceff5afeec79e3c, float.fromhex("0x1.59dfeb5fdd8f3p-1")),
    ((0xffffffffffffffff,) * 5, 0xb22a341e3093f92f, float.fromhex("0x1.6454683c6127fp-1")),
    ((0x75bcd15, 0x3ade68b1, 0x37, 0x0, 0x6b), 0x9633b556ab3a3a1f, float.fromhex("0x1.2c676aad56747p-1")),
]


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npy"))


def test_rng_reference_pins(oracle_mod):
    keys = np.array([p[0] for p in PINS], dtype=np.uint64)
    counter, uniform = oracle_mod.rng(keys)
    assert [int(c) for c in counter] == [p[1] for p in PINS]
    assert list(uniform) == [p[2] for p in PINS]


def test_rng_fixture(oracle_mod):
    g = load("ref_rng")
    counter, uniform = oracle_mod.rng(g[:, :5])
    np.testing.assert_array_equal(counter, g[:, 5])
    np.testing.assert_array_equal(uniform.view(np.uint64), g[:, 6])


@pytest.mark.parametrize("name,which,nin,nout", [
    ("ref_interp", 1, 2, 1),
    ("ref_electron_accessors", 2, 2, 10),
    ("ref_gs_angle", 3, 4, 1),
    ("ref_single_elastic", 4, 3, 1),
    ("ref_moller_energy", 5, 2, 1),
    ("ref_brems_energy", 6, 2, 1),
    ("ref_brems_angle", 7, 2, 1),
    ("ref_half_kick", 8, 13, 4),
    ("ref_cone", 9, 5, 3),
    ("ref_moller_dirs", 10, 6, 6),
    ("ref_photon_recoil", 11, 8, 3),
    ("ref_poisson", 12, 2, 1),
    ("ref_hazard", 13, 6, 5),
    ("ref_drag_plan", 14, 10, 9),
    ("ref_positron_accessors", 22, 2, 5),
    ("ref_bhabha_energy", 23, 2, 1),
    ("ref_positron_brems_energy", 24, 2, 1),
    ("ref_photon_channel", 16, 2, 1),
    ("ref_klein_nishina", 17, 3, 3),
    ("ref_photoelectric", 18, 2, 2),
    ("ref_pair", 20, 5, 14),
    ("ref_annihilation", 21, 3, 6),
])
def test_primitive_matches_reference(oracle_mod, name, which, nin, nout):
    g = load(name)
    out = oracle_mod.primitive(which, g[:, :nin], nout)
    np.testing.assert_array_equal(out, g[:, nin:nin + nout])


def test_chord_matches_reference(oracle_mod):
    g = load("ref_chord")
    out = oracle_mod.primitive(15, g[:, :9], 17)
    ref = g[:, 9:26]
    np.testing.assert_array_equal(out[:, 0], ref[:, 0])
    valid = ref[:, 0] == 1.0
    np.testing.assert_array_equal(out[valid], ref[valid])


def test_photoelectron_cos_matches_reference(oracle_mod):
    """Sauter-Gavrila inversion (S/RreaInteractionTables.cpp SamplePhotoelectronCosTheta)
    runs in long double in the reference; the restatement follows it in long
    double too, so agreement is to a few ulps of the FP64 result."""
    g = load("ref_photoelectron_cos")
    out = oracle_mod.primitive(19, g[:, :2], 1)[:, 0]
    np.testing.assert_allclose(out, g[:, 2], rtol=0, atol=4e-16)


def test_netchord_deposition_matches_reference(oracle_mod):
    """Net-chord Umeda deposition and escape boundary closure
    (I/RreaSegmentDepositionRZ.H) on the coupling's padded grid: 8 x 12
    physical cells of 0.75 m x 1.25 m with two pad cells."""
    cfg = oracle_mod.RreaGpuConfig()
    cfg.r_lo, cfg.r_hi, cfg.z_lo, cfg.z_hi, cfg.nr, cfg.nz = 0.0, 6.0, 0.0, 15.0, 8, 12
    segs = load("ref_netchord_segments")
    assert (segs[:, 0] == 1).sum() > 50
    out = oracle_mod.deposit_segments(cfg, 3.7e-10, segs)
    for key in ("rho", "jr", "jz", "jr_phys", "jz_phys"):
        np.testing.assert_array_equal(out[key].ravel(), load("ref_netchord_" + key)[:, 0])


def test_netchord_continuity_identity(oracle_mod):
    """Cellwise RZ continuity on the padded index grid: the CIC charge change
    of a segment equals minus its index-space current divergence times dt."""
    cfg = oracle_mod.RreaGpuConfig()
    cfg.r_lo, cfg.r_hi, cfg.z_lo, cfg.z_hi, cfg.nr, cfg.nz = 0.0, 6.0, 0.0, 15.0, 8, 12
    rng = np.random.default_rng(3)
    dt = 1.0e-9
    for _ in range(50):
        r0, z0 = rng.uniform(0.0, 5.5), rng.uniform(1.0, 14.0)
        r1, z1 = abs(r0 + rng.uniform(-1.5, 1.5)), z0 + rng.uniform(-1.5, 1.5)
        q = rng.uniform(-2.0, 2.0)
        # an escape row with zero charge deposits nothing; use CIC through two segments of opposite sign
        rows = np.array([[0, r0, z0, r1, z1, q, 0, 0, 0]])
        out = oracle_mod.deposit_segments(cfg, dt, rows)
        rho = np.zeros((16, 10))
        for (r, z, s) in ((r0, z0, -q), (r1, z1, q)):
            xr, xz = r / 0.75 - 0.5, (z + 2.5) / 1.25 - 0.5
            i0, j0 = int(np.floor(xr)), int(np.floor(xz))
            fr, fz = xr - i0, xz - j0
            for a, wr in ((0, 1 - fr), (1, fr)):
                for b, wz in ((0, 1 - fz), (1, fz)):
                    i, j = i0 + a, j0 + b
                    if i < 0:
                        i = -1 - i
                    rho[j, i] += s * wr * wz
        div = (out["jr"][:, 1:] - out["jr"][:, :-1]) + (out["jz"][1:, :] - out["jz"][:-1, :])
        np.testing.assert_allclose(rho + dt * div, 0.0, atol=1e-13 * abs(q))


def test_maxwell_step_matches_reference(oracle_mod):
    """Maxwell TM-RZ leapfrog (I/RreaMaxwellTMRZ.H) over four outer steps of
    three material substeps with a fixed face current, 12 x 20 cells."""
    nr, nz, dr, dz = 12, 20, 0.75, 1.25
    init = load("ref_maxwell_init")[:, 0]
    ner, nez, nbt = (nr + 1) * nz, nr * (nz + 1), (nr + 1) * (nz + 1)
    er, ez, bt = init[:ner], init[ner:ner + nez], init[ner + nez:ner + nez + nbt]
    jr, jz = init[ner + nez + nbt:2 * ner + nez + nbt], init[2 * ner + nez + nbt:]
    dt = load("ref_maxwell_dt")[0, 0]
    for _ in range(4):
        er, ez, bt = oracle_mod.advance_maxwell(nr, nz, dr, dz, dt, 3, er, ez, bt, jr, jz)
    np.testing.assert_array_equal(np.concatenate([er, ez, bt]), load("ref_maxwell_out")[:, 0])


def test_altitude_profile_matches_reference(oracle_mod):
    """RreaAltitudeProfile::LoadCsv + Interpolate (S/RreaAltitudeProfile.cpp)
    on a synthetic exponential atmosphere: nodes, midpoints, both ends and
    random altitudes, bit-exact; the transport ratio is the density over the
    tables' reference density at altitude_msl_at_z0 + z."""
    nodes = load("ref_altitude_profile_nodes")
    rows = load("ref_altitude_profile")
    oracle_mod.set_density_profile(nodes[:, 0], nodes[:, 1], 6000.0, 1.20479)
    try:
        got = oracle_mod.profile_density(rows[:, 0])
        np.testing.assert_array_equal(got, rows[:, 1])
        ratio = oracle_mod.density_ratio_at_z(rows[:, 0] - 6000.0, 0.5)
        np.testing.assert_array_equal(ratio, rows[:, 1] / 1.20479)
        for bad in (5999.0, 14000.5, np.nan):
            with pytest.raises(oracle_mod.OracleFailure) as e:
                oracle_mod.profile_density(np.array([bad]))
            assert e.value.code == 4  # RREA_GPU_ERR_RANGE
    finally:
        oracle_mod.set_density_profile()
    np.testing.assert_array_equal(oracle_mod.density_ratio_at_z(np.array([0.0, 1.0e3]), 0.5), [0.5, 0.5])


@pytest.mark.parametrize("alt,dens", [
    ([0.0], [1.0]),                      # fewer than two rows
    ([0.0, 0.0], [1.0, 1.0]),            # not strictly increasing
    ([0.0, 1.0], [1.0, 0.0]),            # non-positive density
    ([0.0, 1.0], [1.0, np.nan]),         # non-finite
])
def test_altitude_profile_rejects_invalid_tables(oracle_mod, alt, dens):
    with pytest.raises(oracle_mod.OracleFailure) as e:
        oracle_mod.set_density_profile(np.array(alt), np.array(dens), 0.0, 1.2)
    assert e.value.code == 1  # RREA_GPU_ERR_ARGUMENT
