"""The oracle's transient FIFO (DrainAndCommitSecondaries,
RreaSecondaryCommit.cpp:331-515) on the CPU: its structural invariants and
its payload checks.  The GPU FIFO is compared against it in
test_gpu_newborn.py."""
import numpy as np
import pytest

from conftest import TABLES


@pytest.fixture(scope="module")
def mods():
    from rrea_feedback_warpx_amrex_geant4_gb300 import workloads
    from oracle import oracle
    from oracle.build import build_oracle
    build_oracle()
    oracle.load_tables(TABLES)
    return workloads, oracle


class _ConfigFactory:
    """make_config sets every field it needs; the rest stay zero, as in
    rrea_gpu_default_config."""

    @staticmethod
    def default_config(**overrides):
        from oracle import oracle
        cfg = oracle.RreaGpuConfig()
        for k, v in overrides.items():
            setattr(cfg, k, v)
        return cfg


def _config(case):
    from rrea_feedback_warpx_amrex_geant4_gb300 import workloads
    return workloads.make_config(_ConfigFactory, case)


def _pending(workloads, oracle, cfg, field, case, n, step, dt_s):
    e = workloads.make_electrons(case, n, seed=3)
    oe = oracle.electron_step(cfg, field, step, dt_s, workloads.copy_tile(e))
    g = workloads.make_photons(case, n, dt_s, seed=4, e_lo=5.0e4, e_hi=1.0e8)
    og = oracle.photon_step(cfg, step, dt_s, workloads.copy_tile(g))
    return np.concatenate([oe["secondaries"], og["secondaries"]])


def test_fifo_invariants(mods):
    workloads, oracle = mods
    case, dt_s = "uniform_c0", 3.0e-8
    cfg = _config(case)
    field = workloads.make_field(case)
    pending = _pending(workloads, oracle, cfg, field, case, 256, 1, dt_s)
    o = oracle.drain(cfg, field, 1, dt_s, pending)
    surv = o["survivors"]
    assert len(surv) > 0
    assert (surv["birth_fraction"] == 1.0).all()
    keys = set(zip(surv["root_key"].tolist(), surv["root_species"].tolist(), surv["lineage"].tolist()))
    assert len(keys) == len(surv), "a (root, lineage) pair names two survivors"
    r = np.hypot(surv["x"], surv["y"])
    assert ((r >= cfg.r_lo) & (r < cfg.r_hi) & (surv["z"] >= cfg.z_lo) & (surv["z"] < cfg.z_hi)).all()
    charged = surv["species"] != 2
    assert (surv["energy_eV"][charged] >= cfg.low_energy_cutoff_eV).all()
    # children inherit their root from the pending record that started the chain
    roots = set(zip(pending["root_key"].tolist(), pending["root_species"].tolist()))
    assert set(zip(surv["root_key"].tolist(), surv["root_species"].tolist())) <= roots
    # lineages continue above every pending lineage of the same root
    top = {}
    for rec in pending:
        k = (int(rec["root_key"]), int(rec["root_species"]))
        top[k] = max(top.get(k, 0), int(rec["lineage"]))
    pend_keys = set(zip(pending["root_key"].tolist(), pending["root_species"].tolist(), pending["lineage"].tolist()))
    for rec in surv:
        k3 = (int(rec["root_key"]), int(rec["root_species"]), int(rec["lineage"]))
        if k3 not in pend_keys:
            assert k3[2] > top[k3[:2]]
    # deterministic
    o2 = oracle.drain(cfg, field, 1, dt_s, pending)
    for key in surv.dtype.names:
        np.testing.assert_array_equal(o2["survivors"][key], surv[key])


def test_fifo_rejects_invalid_birth_payload(mods):
    workloads, oracle = mods
    case = "uniform_c0"
    cfg = _config(case)
    field = workloads.make_field(case)
    pending = _pending(workloads, oracle, cfg, field, case, 64, 0, 3.0e-8)
    for name, value in (("weight", -1.0), ("birth_fraction", -0.5), ("root_species", 3), ("lineage", 1 << 14)):
        bad = pending.copy()
        bad[name][0] = value
        with pytest.raises(oracle.OracleFailure) as err:
            oracle.drain(cfg, field, 0, 3.0e-8, bad)
        assert err.value.code == 1
    assert len(oracle.drain(cfg, field, 0, 3.0e-8, pending[:0])["survivors"]) == 0


def test_commit_restatement_follows_the_overlay_rules():
    """oracle.commit_survivors (the checker of the resident commit) follows
    CommitLocalParticleBatch's rules (O/RreaCouplingSources.cpp:240-330):
    weight <= 0 dropped, photons with E <= 0 dropped, e-/e+ proper velocity
    along the direction, a zero direction giving (0, 0, u), photon momentum
    E along the direction, ids in FIFO order."""
    from oracle import oracle

    recs = np.zeros(6, dtype=oracle.SECONDARY_DTYPE)
    recs["species"] = [0, 0, 0, 2, 2, 1]
    recs["weight"] = [1.0, 0.0, 2.0, 3.0, 4.0, 5.0]
    recs["energy_eV"] = [1.0e6, 1.0e6, 2.0e6, 5.0e5, 0.0, 3.0e6]
    recs["x"], recs["y"], recs["z"] = [3.0, 1, 0, 1, 1, -2.0], [4.0, 1, 2.0, 1, 1, 0.0], [5.0, 1, 6, 7, 8, 9]
    recs["dir_x"], recs["dir_y"], recs["dir_z"] = [0.0, 1, 0, 0.6, 1, 0], [0.0, 0, 0, 0.8, 0, 0], [0.0, 0, 2.0, 0, 0, -1.0]
    e = oracle.commit_survivors(recs, 0, 100)
    np.testing.assert_array_equal(e["id"], [100, 101])
    np.testing.assert_array_equal(e["w"], [1.0, 2.0])
    np.testing.assert_allclose(e["r"], [5.0, 2.0])
    np.testing.assert_allclose(e["theta"], [np.arctan2(4.0, 3.0), np.pi / 2])
    u1 = oracle.C_M_PER_S * np.sqrt((1.0 + 1.0e6 / oracle.ME_C2_EV) ** 2 - 1.0)
    u2 = oracle.C_M_PER_S * np.sqrt((1.0 + 2.0e6 / oracle.ME_C2_EV) ** 2 - 1.0)
    np.testing.assert_allclose(np.stack([e["ux"], e["uy"], e["uz"]], axis=1), [[0.0, 0.0, u1], [0.0, 0.0, u2]])
    g = oracle.commit_survivors(recs, 2, 7)
    np.testing.assert_array_equal(g["id"], [7])
    np.testing.assert_allclose([g["ux"][0], g["uy"][0], g["uz"][0]], [3.0e5, 4.0e5, 0.0])
    p = oracle.commit_survivors(recs, 1, 1)
    np.testing.assert_allclose(p["theta"], [np.pi])
    assert p["uz"][0] < 0.0 and p["ux"][0] == 0.0
