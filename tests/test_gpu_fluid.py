"""The carrier fluid on the device (rrea_gpu_fluid_*, rrea_gpu_advance_field_coupled)
against the reference's own fluid sources (the ref_fluid_* golden vectors
from S/LowEnergyFluidState.cpp and S/LowEnergyFluidFaceTransport.cpp) and
against the oracle's restatement of the coupled fluid/Maxwell step.

The fluid kernels are compiled without FMA contraction, so every product and
sum rounds as in the reference; what differs is the device's exp/expm1/log/
hypot against glibc's (within an ulp or two).  Hence:
  * explicit transport (no libm on the flux path): face fluxes, densities,
    fluid charge, conductivity bit-exact; diagnostics built from atomic sums
    within 1e-12;
  * the 64-eps neutral-charge rule: bit-exact;
  * chemistry (exp/expm1 in the attachment, detachment and pair-loss
    solutions): every density within 1e-12 of its cell's carrier scale
    (old densities plus the step's sources), the charge within 1e-12 of
    qe x that scale, the residual <= 512 eps like the reference's gate;
  * closure cell fields (log/exp interpolation): within 1e-13 relative,
    range counts exact;
  * the coupled step: field vectors within 1e-12 of each vector's largest
    entry, carrier densities within 1e-12 relative (of the grid's largest
    density), the same substep count."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, TABLES

pytestmark = pytest.mark.gpu

CLOSURE = os.path.join(ROOT, "data", "closure", "dry_air_swarm_hybrid_v3.csv")
QE = 1.602176634e-19


@pytest.fixture(scope="module")
def mods():
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu, workloads
    from oracle import fluid as ofl
    build.build()
    ofl.load_closure(CLOSURE)
    return gpu, workloads, ofl


def _g(name):
    return np.load(os.path.join(GOLDEN, f"ref_fluid_{name}.npy"))


def _ctx(gpu, nr, nz, r_lo, z_lo, dr, dz, periodic=False):
    cfg = gpu.default_config(r_lo=r_lo, r_hi=r_lo + nr * dr, z_lo=z_lo, z_hi=z_lo + nz * dz, nr=nr, nz=nz,
                             periodic_z=int(periodic))
    return gpu.RreaGpuContext(cfg, 1024)


def test_reaction_matches_reference(mods):
    gpu, workloads, ofl = mods
    setup, inp, out = _g("reaction_setup"), _g("reaction_in"), _g("reaction_out")
    worst = 0.0
    for c, row in enumerate(setup):
        nr, nz, dt, att, a_ei, a_ii, det, table, clear, max_rate, residual = row
        ctx = _ctx(gpu, int(nr), int(nz), 0.0, 0.0, 1.5, 2.0)
        ctx.fluid_configure(attachment_frequency_s=att, electron_ion_recombination_coefficient_m3_per_s=a_ei,
                            ion_ion_recombination_coefficient_m3_per_s=a_ii, detachment_frequency_s=det,
                            attachment_model=int(table))
        ne, np_, nn, se, sp, sn, rho, nu = inp[8 * c: 8 * c + 8]
        ctx.fluid_set_state(n_pos=np_, n_neg=nn, n_e=ne, rho=rho)
        ctx.fluid_set_source_rates(se, sp, sn)
        if table:
            ctx.fluid_set_closure_fields(nu=nu)
        assert ctx.fluid_max_reaction_frequency() == pytest.approx(max_rate, rel=1e-15)
        res = ctx.fluid_react(dt, clear_sources=bool(clear))
        assert res <= 512 * np.finfo(float).eps
        st = ctx.fluid_state()
        src = ctx.fluid_source_rates()
        want = out[8 * c: 8 * c + 8]
        scale = (np.maximum(ne, 0) + np.maximum(np_, 0) + np.maximum(nn, 0)
                 + (np.maximum(se, 0) + np.maximum(sp, 0) + np.maximum(sn, 0)) * dt)
        for got, ref in ((st["n_e"], want[0]), (st["n_pos"], want[1]), (st["n_neg"], want[2])):
            err = np.abs(got - ref)
            assert np.all(err <= 1e-12 * scale), (c, float((err / np.maximum(scale, 1e-300)).max()))
            worst = max(worst, float((err / np.maximum(scale, 1e-300)).max()))
        np.testing.assert_allclose(st["rho"], want[3], rtol=0, atol=1e-12 * QE * scale.max())
        for k, name in enumerate(("s_e", "s_pos", "s_neg")):
            np.testing.assert_array_equal(src[name], want[4 + k])
        ctx.fluid_charge_density()
        np.testing.assert_allclose(ctx.fluid_state()["rho"], want[7], rtol=0, atol=1e-12 * QE * scale.max())
        ctx.close()
    print(f"worst chemistry difference: {worst:.2e} of the cell's carrier scale")


def test_neutral_charge_rule_is_exact(mods):
    gpu, workloads, ofl = mods
    ne, np_, nn = _g("neutral_in")
    ctx = _ctx(gpu, 6, 5, 0.0, 0.0, 1.0, 1.0)
    ctx.fluid_configure()
    ctx.fluid_set_state(n_pos=np_, n_neg=nn, n_e=ne)
    ctx.fluid_charge_density()
    np.testing.assert_array_equal(ctx.fluid_state()["rho"], _g("neutral_out")[0])
    ctx.close()


def test_closure_fields_match_reference(mods):
    gpu, workloads, ofl = mods
    er, ez, chi, ne, src = _g("closure_in")
    want = _g("closure_out")
    diag = _g("closure_diag")[0]
    nr, nz, r_lo, z_lo, dr, dz = diag[:6]
    ctx = _ctx(gpu, int(nr), int(nz), r_lo, z_lo, dr, dz)
    ctx.fluid_configure(electron_mobility_model=gpu.MOBILITY_EN_TABLE_FLUX, attachment_model=gpu.ATTACHMENT_EN_TABLE)
    ctx.fluid_load_closure(CLOSURE)
    ctx.fluid_set_density_ratio(chi)
    ctx.fluid_set_state(n_e=ne)
    ctx.fluid_set_source_rates(s_e=src)
    d = ctx.fluid_evaluate_closure(er, ez)
    mu, nu, d3 = ctx.fluid_closure_fields()
    np.testing.assert_allclose(mu, want[0], rtol=1e-13, atol=0)
    np.testing.assert_allclose(nu, want[1], rtol=1e-13, atol=0)
    np.testing.assert_allclose(d3, want[2:5], rtol=1e-13, atol=1e-13 * np.abs(want[2:5]).max())
    assert (d["held_below"], d["above_range"], d["invalid"]) == (diag[8], diag[9], diag[10])
    assert d["min_en_td"] == pytest.approx(diag[6], rel=1e-15)
    assert d["max_en_td"] == pytest.approx(diag[7], rel=1e-15)
    for key, ref in (("electron_count", diag[11]), ("held_below_electron_count", diag[12]),
                     ("electron_source_rate", diag[13])):
        assert d[key] == pytest.approx(ref, rel=1e-12), key
    ctx.close()


@pytest.mark.parametrize("k", range(6))
def test_transport_matches_reference(mods, k):
    gpu, workloads, ofl = mods
    from test_oracle_fluid import transport_case
    s, want, diag = transport_case(ofl, k)
    nr, nz, r_lo, z_lo, dr, dz, per = s["grid"]
    ctx = _ctx(gpu, nr, nz, r_lo, z_lo, dr, dz, per)
    cfg = gpu.RreaFluidConfig.from_buffer_copy(bytes(s["cfg"]))
    ctx.fluid_configure(cfg)
    np_, nn, ne, rho = s["state"]
    ctx.fluid_set_state(n_pos=np_, n_neg=nn, n_e=ne, rho=rho)
    ctx.fluid_set_density_ratio(s["chi"])
    if s["mu"] is not None:
        ctx.fluid_set_closure_fields(mu=s["mu"], diffusion=s["diffusion"])
    ctx.fluid_conductivity()
    st = ctx.fluid_state()
    np.testing.assert_array_equal(st["sigma"], want["sigma"])
    np.testing.assert_array_equal(st["tau"], want["tau"])
    fr, fz, d = ctx.fluid_transport(s["dt"], s["efr"], s["efz"])
    np.testing.assert_array_equal(fr, want["flux_r"])
    np.testing.assert_array_equal(fz, want["flux_z"])
    st = ctx.fluid_state()
    for key in ("n_pos", "n_neg", "n_e", "rho"):
        np.testing.assert_array_equal(st[key], want[key], err_msg=key)
    names = gpu.FLUID_TRANSPORT_DIAG
    exact = ("max_face_conductivity", "unlimited_max_outgoing_cfl", "min_outflow_scale", "max_outgoing_cfl",
             "max_drift_speed", "cfl_dt")
    for name, value in zip(names, diag):
        if name in exact:
            assert d[name] == value, name
        else:
            assert d[name] == pytest.approx(value, rel=1e-12, abs=1e-300), name
    ctx.close()


def test_transport_fails_closed_on_a_negative_density(mods):
    gpu, workloads, ofl = mods
    from test_oracle_fluid import transport_case
    s, want, diag = transport_case(ofl, 0)
    nr, nz, r_lo, z_lo, dr, dz, per = s["grid"]
    ctx = _ctx(gpu, nr, nz, r_lo, z_lo, dr, dz, per)
    ctx.fluid_configure(gpu.RreaFluidConfig.from_buffer_copy(bytes(s["cfg"])))
    np_, nn, ne, rho = (np.array(a) for a in s["state"])
    ne[:] = 0.0            # no inflow can lift the planted negative density
    ne[3] = -5.0
    ctx.fluid_set_state(n_pos=np_, n_neg=nn, n_e=ne, rho=rho)
    with pytest.raises(gpu.RreaGpuError) as e:
        ctx.fluid_transport(s["dt"], s["efr"], s["efz"])
    assert "negative density" in str(e.value)
    ctx.close()


def _coupled_setup(gpu, workloads, ofl, table, dense, seed):
    """A 24 x 40 grid over 48 m x 400 m, E_z = -400 kV/m ambient plus a
    seeded scattered field, carriers near the axis (a dense blob when
    asked, which raises the conduction stiffness and the substep count) and
    ionization sources."""
    rng = np.random.default_rng(seed)
    nr, nz, dr, dz = 24, 40, 2.0, 10.0
    n = nr * nz
    cfg = gpu.default_config(r_hi=nr * dr, z_lo=0.0, z_hi=nz * dz, nr=nr, nz=nz)
    field = dict(er=rng.normal(0, 2e3, (nr + 1) * nz), ez=rng.normal(0, 2e3, nr * (nz + 1)),
                 bt=rng.normal(0, 1e-6, (nr + 1) * (nz + 1)), amb_er=np.zeros((nr + 1) * nz),
                 amb_ez=np.full(nr * (nz + 1), -4.0e5))
    field["er"].reshape(nz, nr + 1)[:, 0] = 0.0
    i = np.arange(n) % nr
    j = np.arange(n) // nr
    blob = np.exp(-((i * dr) / 10.0) ** 2 - ((j * dz - 200.0) / 60.0) ** 2)
    peak = 3.0e17 if dense else 1.0e12
    state = dict(ne=peak * blob * rng.uniform(0.5, 1.5, n), np=peak * blob * rng.uniform(0.5, 1.5, n),
                 nn=0.3 * peak * blob * rng.uniform(0.5, 1.5, n), rho=np.zeros(n),
                 se=1.0e20 * blob * rng.uniform(0, 1, n), sp=1.0e20 * blob * rng.uniform(0, 1, n),
                 sn=1.0e18 * blob * rng.uniform(0, 1, n))
    state["rho"] = QE * (state["np"] - state["nn"] - state["ne"])
    fcfg = ofl.default_config(ion_drift_enable=1, transport_density_ratio=0.948,
                              electron_ion_recombination_coefficient_m3_per_s=2.0e-13,
                              ion_ion_recombination_coefficient_m3_per_s=2.0e-12)
    if table:
        fcfg.electron_mobility_model = ofl.MOBILITY_EN_TABLE_FLUX
        fcfg.attachment_model = ofl.ATTACHMENT_EN_TABLE
    return cfg, field, state, fcfg, (nr, nz, dr, dz)


@pytest.mark.parametrize("table,dense", [(False, False), (False, True), (True, False), (True, True)])
def test_coupled_step_matches_oracle(mods, table, dense):
    gpu, workloads, ofl = mods
    cfg, field, state, fcfg, (nr, nz, dr, dz) = _coupled_setup(gpu, workloads, ofl, table, dense, 11)
    ctx = gpu.RreaGpuContext(cfg, 1024)
    ctx.set_field(**field)
    ctx.fluid_configure(gpu.RreaFluidConfig.from_buffer_copy(bytes(fcfg)))
    if table:
        ctx.fluid_load_closure(CLOSURE)
    ctx.fluid_set_state(n_pos=state["np"], n_neg=state["nn"], n_e=state["ne"], rho=state["rho"])
    ctx.fluid_set_source_rates(state["se"], state["sp"], state["sn"])
    ctx.reset_current()
    dt = 5.0e-10
    zeros_r, zeros_z = np.zeros((nr + 1) * nz), np.zeros(nr * (nz + 1))
    f = (field["er"], field["ez"], field["bt"])
    st = dict(state)
    for step in range(3):
        gd = ctx.advance_field_coupled(dt)
        f, st, od = ofl.coupled_step(fcfg, nr, nz, 0.0, dr, dz, dt, f, (field["amb_er"], field["amb_ez"]),
                                     (zeros_r, zeros_z), st)
        assert gd["substeps"] == od["substeps"], (step, gd, od)
        got = ctx.field()
        for name, g, o in zip(("er", "ez", "bt"), got, f):
            np.testing.assert_allclose(g, o, rtol=0, atol=1e-12 * np.abs(o).max(), err_msg=f"{name} step {step}")
        gs = ctx.fluid_state()
        for key, okey in (("n_e", "ne"), ("n_pos", "np"), ("n_neg", "nn")):
            np.testing.assert_allclose(gs[key], st[okey], rtol=1e-12, atol=1e-12 * st[okey].max(),
                                       err_msg=f"{key} step {step}")
        np.testing.assert_allclose(gs["rho"], st["rho"], rtol=0, atol=1e-12 * QE * st["ne"].max())
        np.testing.assert_allclose(gs["sigma"], st["sigma"], rtol=1e-12, atol=1e-12 * st["sigma"].max())
        f = got   # both sides continue from the GPU's field
        st = dict(ne=gs["n_e"], np=gs["n_pos"], nn=gs["n_neg"], rho=gs["rho"], se=st["se"], sp=st["sp"], sn=st["sn"])
    if dense:
        assert gd["substeps"] > 2
    ctx.close()


def test_sources_from_the_kinetic_step(mods):
    """rrea_gpu_fluid_take_sources: the electron phase's cell sources 0..2
    normalised by cell volume and dt, and one coupled step driven by that
    step's kinetic net-chord current, against the oracle fed the same
    current and sources."""
    gpu, workloads, ofl = mods
    case = "scaleup_c1"
    cfg = workloads.make_config(gpu, case)
    ctx = gpu.RreaGpuContext(cfg, 1 << 15)
    ctx.load_tables(TABLES)
    field = workloads.make_field(case)
    ctx.set_field(**field)
    fcfg = ofl.default_config(ion_drift_enable=1, transport_density_ratio=0.948)
    ctx.fluid_configure(gpu.RreaFluidConfig.from_buffer_copy(bytes(fcfg)))
    arr = workloads.make_electrons(case, 4096, seed=3)
    ctx.stage_electrons(arr)
    ctx.reset_sources()
    ctx.reset_current()
    dt = 5.0e-10
    ctx.step_electrons_resident(1, dt)
    cells = ctx.sources().reshape(5, -1)
    ctx.fluid_take_sources(dt)
    src = ctx.fluid_source_rates()
    nr, nz = cfg.nr, cfg.nz
    dr, dz = (cfg.r_hi - cfg.r_lo) / nr, (cfg.z_hi - cfg.z_lo) / nz
    r_in = cfg.r_lo + (np.arange(nr * nz) % nr) * dr
    vol = np.pi * ((r_in + dr) ** 2 - r_in ** 2) * dz
    for k, name in enumerate(("s_e", "s_pos", "s_neg")):
        np.testing.assert_allclose(src[name], cells[k] / (vol * dt), rtol=1e-15, atol=0)
    assert src["s_e"].sum() > 0
    jr, jz = ctx.current()
    before = ctx.field()
    n = nr * nz
    state = dict(ne=np.zeros(n), np=np.zeros(n), nn=np.zeros(n), rho=np.zeros(n), se=src["s_e"], sp=src["s_pos"],
                 sn=src["s_neg"])
    gd = ctx.advance_field_coupled(dt)
    f, st, od = ofl.coupled_step(fcfg, nr, nz, cfg.z_lo, dr, dz, dt, before, (field["amb_er"], field["amb_ez"]),
                                 (jr.ravel(), jz.ravel()), state)
    assert gd["substeps"] == od["substeps"]
    for name, g, o in zip(("er", "ez", "bt"), ctx.field(), f):
        np.testing.assert_allclose(g, o, rtol=0, atol=1e-12 * np.abs(o).max(), err_msg=name)
    gs = ctx.fluid_state()
    for key, okey in (("n_e", "ne"), ("n_pos", "np"), ("n_neg", "nn")):
        np.testing.assert_allclose(gs[key], st[okey], rtol=1e-12, atol=1e-12 * max(st[okey].max(), 1e-300), err_msg=key)
    assert gs["n_pos"].sum() > 0
    after = ctx.fluid_source_rates()
    assert not any(v.any() for v in after.values())   # the step clears the source rates
    # the reduced diagnostics' fluid and source totals
    red = ctx.fluid_reductions(dt)
    want = {"total_ne_low": gs["n_e"].sum(), "total_n_pos": gs["n_pos"].sum(), "total_n_neg": gs["n_neg"].sum(),
            "N_low_e_real": (gs["n_e"] * vol).sum(), "N_pos_real": (gs["n_pos"] * vol).sum(),
            "N_neg_real": (gs["n_neg"] * vol).sum(), "rho_fluid_C": (gs["rho"] * vol).sum(),
            "total_rho_fluid": gs["rho"].sum(), "total_S_low_electron": (cells[0] / (vol * dt)).sum(),
            "total_S_positive_ion": (cells[1] / (vol * dt)).sum(),
            "total_S_direct_negative_ion": (cells[2] / (vol * dt)).sum(),
            "ionization_event_count": (cells[3] / vol).sum(), "total_energy_loss_ev_m3": (cells[4] / vol).sum(),
            "max_ne_low": gs["n_e"].max(), "max_sigma": gs["sigma"].max(), "min_tau_m": gs["tau"].min()}
    for key, value in want.items():
        assert red[key] == pytest.approx(value, rel=1e-12, abs=1e-300), key
    ctx.close()
