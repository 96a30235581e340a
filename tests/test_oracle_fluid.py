"""The oracle's carrier-fluid restatement (oracle/fluid.cpp) against golden
vectors from the reference's own fluid sources (oracle/ref_golden_fluid.cpp
drives S/LowEnergyFluidState.cpp, S/LowEnergyFluidFaceTransport.cpp and the
closure loader of S/RreaInteractionTables.cpp, compiled against a
single-box AMReX stand-in).

Both sides are the same IEEE double arithmetic in the same operand order
with the same libm on this host, so everything is bit-exact: the chemistry
(attachment, detachment, both pair-loss channels, the conservative charge,
the residual and the stiffness bound), the 64-eps neutrality rule, the
closure cell fields and their range counts, and the explicit transport
(raw and limited face fluxes, new densities and charge, every diagnostic)
for absolute, density-scaled and table mobilities, with and without a
periodic z."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

CLOSURE = os.path.join(ROOT, "data", "closure", "dry_air_swarm_hybrid_v3.csv")


@pytest.fixture(scope="module")
def fl():
    from oracle import fluid
    fluid.load_closure(CLOSURE)
    return fluid


def _g(name):
    return np.load(os.path.join(GOLDEN, f"ref_fluid_{name}.npy"))


def test_reaction_matches_reference(fl):
    setup, inp, out = _g("reaction_setup"), _g("reaction_in"), _g("reaction_out")
    for c, row in enumerate(setup):
        nr, nz, dt, att, a_ei, a_ii, det, table, clear, max_rate, residual = row
        cfg = fl.default_config(attachment_frequency_s=att, electron_ion_recombination_coefficient_m3_per_s=a_ei,
                                ion_ion_recombination_coefficient_m3_per_s=a_ii, detachment_frequency_s=det,
                                attachment_model=int(table))
        ne, np_, nn, se, sp, sn, rho, nu = inp[8 * c: 8 * c + 8]
        nu_arg = nu if table else None
        assert fl.max_reaction_frequency(cfg, ne, np_, nn, nu_arg) == max_rate
        st, res = fl.react(cfg, dt, ne, np_, nn, se, sp, sn, rho, nu_arg, clear=bool(clear))
        assert res == residual
        want = out[8 * c: 8 * c + 8]
        for k, name in enumerate(("ne", "np", "nn", "rho", "se", "sp", "sn")):
            np.testing.assert_array_equal(st[name], want[k], err_msg=f"case {c} {name}")
        np.testing.assert_array_equal(fl.charge_density(st["ne"], st["np"], st["nn"]), want[7])


def test_neutral_cells_reconstruct_zero_charge(fl):
    ne, np_, nn = _g("neutral_in")
    want = _g("neutral_out")[0]
    got = fl.charge_density(ne, np_, nn)
    np.testing.assert_array_equal(got, want)
    assert (want == 0.0).sum() > 5 and (want != 0.0).sum() > 5


def test_closure_cell_fields_match_reference(fl):
    er, ez, chi, ne, src = _g("closure_in")
    want = _g("closure_out")
    diag = _g("closure_diag")[0]
    nr, nz, r_lo, z_lo, dr, dz = diag[:6]
    mu, nu, d3, got_diag = fl.closure_fields(int(nr), int(nz), r_lo, z_lo, dr, dz, er, ez, chi, ne, src)
    np.testing.assert_array_equal(mu, want[0])
    np.testing.assert_array_equal(nu, want[1])
    np.testing.assert_array_equal(d3, want[2:5])
    # min/max E/N, held-below, above-range and invalid counts, electron count,
    # held-below electron count, source rate
    np.testing.assert_array_equal(got_diag[[0, 1, 2, 3, 4]], diag[[6, 7, 8, 9, 10]])
    np.testing.assert_allclose(got_diag[[5, 6, 7]], diag[[11, 12, 13]], rtol=1e-15)
    assert diag[8] > 0 and diag[9] > 0          # some cells held below, some above range


def transport_case(fl, k):
    row = _g("transport_setup")[k]
    nr, nz = int(row[0]), int(row[1])
    r_lo, z_lo, dr, dz = row[2:6]
    per, ions, reduced, table, dens_field = (bool(x) for x in row[6:11])
    dt = row[11]
    cfg = fl.default_config(ion_drift_enable=int(ions), electron_drift_enable=1,
                            positive_ion_mobility_m2_per_vs=row[12], negative_ion_mobility_m2_per_vs=row[13],
                            electron_mobility_m2_per_vs=row[14], ion_drift_cfl=row[18], transport_density_ratio=row[19])
    if reduced:
        cfg.ion_mobility_model = fl.MOBILITY_REDUCED_STP
        cfg.positive_ion_reduced_mobility_stp_m2_per_vs = row[15]
        cfg.negative_ion_reduced_mobility_stp_m2_per_vs = row[16]
        cfg.ion_mobility_density_ratio_floor = row[17]
    if table:
        cfg.electron_mobility_model = fl.MOBILITY_EN_TABLE_FLUX
    n, nfr, nfz = nr * nz, (nr + 1) * nz, nr * (nz + 1)
    inp = _g(f"transport_in_{k}")[:, 0]
    parts = np.split(inp, np.cumsum([n, n, n, n, n, n, 3 * n, nfr]))
    ne, np_, nn, rho, chi, mu, d3, efr, efz = parts
    out = _g(f"transport_out_{k}")[:, 0]
    o = np.split(out, np.cumsum([n, n, 3 * nfr, 3 * nfz, 3 * nfr, 3 * nfz, n, n, n]))
    want = dict(sigma=o[0], tau=o[1], raw_r=o[2].reshape(3, nfr), raw_z=o[3].reshape(3, nfz),
                flux_r=o[4].reshape(3, nfr), flux_z=o[5].reshape(3, nfz), n_pos=o[6], n_neg=o[7], n_e=o[8], rho=o[9])
    setup = dict(cfg=cfg, grid=(nr, nz, r_lo, z_lo, dr, dz, per), dt=dt, state=(np_, nn, ne, rho),
                 chi=chi if dens_field else None, mu=mu if table else None,
                 diffusion=d3.reshape(3, n) if table else None, efr=efr, efz=efz)
    return setup, want, row[20:]


@pytest.mark.parametrize("k", range(6))
def test_transport_matches_reference(fl, k):
    s, want, diag = transport_case(fl, k)
    sigma, tau = fl.conductivity(s["cfg"], s["state"][2], s["state"][0], s["state"][1], s["chi"], s["mu"])
    np.testing.assert_array_equal(sigma, want["sigma"])
    np.testing.assert_array_equal(tau, want["tau"])
    got = fl.transport(s["cfg"], s["grid"], s["dt"], *s["state"], s["efr"], s["efz"], s["chi"], s["mu"],
                       s["diffusion"])
    for key in ("raw_r", "raw_z", "flux_r", "flux_z", "n_pos", "n_neg", "n_e", "rho"):
        np.testing.assert_array_equal(got[key], want[key], err_msg=key)
    names = ("max_face_conductivity", "max_diffusion_number", "unlimited_max_outgoing_cfl", "min_outflow_scale",
             "limited_outflow_fraction", "limited_electron_number_fraction", "max_outgoing_cfl", "max_drift_speed",
             "cfl_dt", "pos_center_r", "pos_center_z", "neg_center_r", "neg_center_z", "density_ratio_at_pos_center")
    for name, value in zip(names, diag):
        assert got["diag"][name] == value, name


def test_limiter_engages_in_the_golden_cases(fl):
    """The fixtures exercise the positivity limiter (a scale below 1) and the
    table-mobility diffusion term."""
    rows = _g("transport_setup")
    assert rows[:, 23].min() < 1.0            # min outflow scale
    assert rows[:, 21].max() > 0.0            # diffusion number of the table cases


def test_transport_refuses_a_bad_cfl(fl):
    from oracle.oracle import OracleFailure
    s, _, _ = transport_case(fl, 0)
    cfg = fl.as_config(s["cfg"])
    cfg.ion_drift_cfl = 1.5
    with pytest.raises(OracleFailure):
        fl.transport(cfg, s["grid"], s["dt"], *s["state"], s["efr"], s["efz"])
