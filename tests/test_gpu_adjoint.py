"""The pathwise adjoint of the charged push (rrea_gpu_adjoint_*,
adjoint.PushAdjoint and its torch.autograd.Function) against central finite
differences with common random numbers, and its forward against a numpy
restatement of the same model.

Problem: 3000 electrons of 0.3-20 MeV (a tenth of them against the field,
so some stop at the cutoff) in the adjoint configuration's field
profile (256 nodes over 0-500 m, 450 kV/m plus a correlated 20 kV/m
perturbation), 96 steps of 0.5 ns in 2 substeps, checkpoints every 32 steps;
the runaway threshold at 8 MeV (50 keV wide) and the crossing plane at 12 m
(1 m wide), where both loss terms move.

  * gradient: within 1e-5 relative of central differences (h = 0.01 V/m,
    common random numbers, every particle ending where it ended in the
    unperturbed run: the frozen topology the adjoint differentiates) on
    every node the particles reach with a gradient above 1e-3 of the
    largest, and exactly zero on the nodes none reaches.  The step is small
    because the loss is only piecewise smooth: the stopping powers are
    log-log between table nodes, and the slow particles near the lower
    nodes cross table nodes under a 1 V/m step, which moves that difference
    quotient by up to 3e-4 (2.5e-5 at 0.02 V/m; at 0.01 V/m one-sided
    quotients from either side agree to 3e-6).  The loss is summed in a
    fixed order with compensation, so the quotient carries only the two
    losses' final roundings (about 1e-11 here);
  * the frozen forward at the unperturbed nodes is the plain forward;
  * forward: final K and z within 1e-11 relative of the numpy restatement
    (the device's exp/log/sin/cos against numpy's);
  * autograd: torch's backward through the Function returns the adjoint;
  * cost: the reverse pass (recomputation included) within 3x the forward."""
import time

import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def problem():
    import torch
    from rrea_feedback_warpx_amrex_geant4_gb300 import adjoint, build
    build.build()
    rng = np.random.default_rng(3)
    n = 3000
    k = np.exp(rng.uniform(np.log(3.0e5), np.log(2.0e7), n))
    mu = rng.uniform(0.6, 1.0, n)
    mu[::10] *= -1.0
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    s = np.sqrt(1.0 - mu * mu)
    seeds = dict(z=rng.uniform(0.0, 5.0, n), dir=np.stack([s * np.cos(phi), s * np.sin(phi), mu], 1), k=k,
                 w=rng.uniform(0.5, 2.0, n), id=np.arange(1, n + 1, dtype=np.uint64))
    cfg = adjoint.default_config(steps=96, substeps=2, checkpoint_every=32, k_threshold_eV=8.0e6,
                                 z_plane_m=12.0, density_ratio=1.225 / 1.20479)
    prob = adjoint.PushAdjoint(cfg, seeds, tables=TABLES)
    e = torch.tensor(adjoint.adjoint_field_profile(), dtype=torch.float64, device="cuda")
    yield adjoint, prob, e, seeds, cfg
    prob.close()


def test_gradient_matches_central_differences(problem):
    adjoint, prob, e, seeds, cfg = problem
    prob.forward(e)
    g = prob.backward(e).cpu().numpy()
    big = np.abs(g).max()
    assert big > 0
    reached = np.nonzero(np.abs(g) > 1e-3 * big)[0]
    assert len(reached) >= 5
    fd = adjoint.central_differences(prob, e, reached.tolist(), h=0.01)
    np.testing.assert_allclose(g[reached], fd, rtol=1e-5, atol=1e-7 * big)
    far = np.arange(40, 256)        # beyond 80 m: no particle gets there in 48 ns
    assert np.all(g[far] == 0.0)


def test_frozen_forward_replays_the_recorded_run(problem):
    adjoint, prob, e, seeds, cfg = problem
    plain = prob.forward(e)
    state = prob.final_state()
    assert prob.forward(e, frozen=True) == plain
    np.testing.assert_array_equal(prob.final_state(), state)


def test_forward_matches_restatement(problem):
    adjoint, prob, e, seeds, cfg = problem
    from oracle import oracle
    oracle.load_tables(TABLES)
    prob.forward(e)
    got = prob.final_state()
    want = _numpy_forward(oracle, cfg, e.cpu().numpy(), seeds, n=400)
    np.testing.assert_array_equal(got[5, :400], want[5])          # same stops
    np.testing.assert_allclose(got[4, :400], want[4], rtol=1e-11)
    np.testing.assert_allclose(got[0, :400], want[0], rtol=1e-11, atol=1e-11)
    assert (got[5] == 0).sum() > 0                                   # some particles stopped


def test_autograd_function_and_cost(problem):
    import torch
    adjoint, prob, e, seeds, cfg = problem
    fn = adjoint.field_loss_function()
    x = e.clone().requires_grad_(True)
    loss = fn.apply(prob, x)
    loss.backward()
    prob.forward(e)
    want = prob.backward(e)
    torch.testing.assert_close(x.grad, want, rtol=1e-14, atol=0.0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(3):
        prob.forward(e)
    t_fwd = (time.perf_counter() - t0) / 3
    t0 = time.perf_counter()
    for _ in range(3):
        prob.backward(e)
    t_bwd = (time.perf_counter() - t0) / 3
    print(f"forward {1e3 * t_fwd:.2f} ms, reverse {1e3 * t_bwd:.2f} ms ({t_bwd / t_fwd:.2f}x)")
    assert t_bwd <= 3.0 * t_fwd


# ---- numpy restatement of the differentiated model (test oracle) ------------
KC = 299792458.0
MEC2 = 510998.95
GL_A = 0.5 - 0.5 / np.sqrt(3.0)
GL_B = 0.5 + 0.5 / np.sqrt(3.0)


def _splitmix(v):
    v = (v + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    v = ((v ^ (v >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    v = ((v ^ (v >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    return v ^ (v >> np.uint64(31))


def _rotation(seed, ids, step, sub, rms):
    with np.errstate(over="ignore"):
        inner = _splitmix((ids * np.uint64(0x9E3779B97F4A7C15) + np.uint64(0x5EED)) & np.uint64(0xFFFFFFFFFFFFFFFF))
        key = _splitmix(np.uint64(seed) ^ inner) ^ np.uint64(step << 20) ^ np.uint64(sub)
        u = [((_splitmix((key * np.uint64(4) + np.uint64(k)) & np.uint64(0xFFFFFFFFFFFFFFFF)) >> np.uint64(11))
              .astype(np.float64) + 0.5) * 2.0 ** -53 for k in range(4)]
    mu = 2.0 * u[0] - 1.0
    phi = 2.0 * np.pi * u[1]
    st = np.sqrt(np.maximum(0.0, 1.0 - mu * mu))
    n = np.stack([st * np.cos(phi), st * np.sin(phi), mu], 1)
    th = rms * np.sqrt(-2.0 * np.log(u[2])) * np.cos(2.0 * np.pi * u[3])
    return n, np.cos(th), np.sin(th)


def _numpy_forward(oracle, cfg, e, seeds, n):
    z = seeds["z"][:n].copy()
    d = seeds["dir"][:n] / np.linalg.norm(seeds["dir"][:n], axis=1)[:, None]
    k = seeds["k"][:n].copy()
    ids = seeds["id"][:n].astype(np.uint64)
    alive = np.ones(n, dtype=bool)
    dz_node = (cfg.z_hi - cfg.z_lo) / (cfg.n_nodes - 1)
    h = cfg.dt_s / cfg.substeps

    def field(zq):
        x = (zq - cfg.z_lo) / dz_node
        k0 = np.clip(np.floor(x), 0, cfg.n_nodes - 2).astype(int)
        f = x - k0
        v = (1.0 - f) * e[k0] + f * e[k0 + 1]
        return np.where(x > 0, np.where(x < cfg.n_nodes - 1, v, e[-1]), e[0])

    def drag(kk):
        rows = np.stack([np.zeros_like(kk), kk], 1)
        col = oracle.primitive(1, rows, 1)[:, 0]
        rows[:, 0] = 1.0
        soft = oracle.primitive(1, rows, 1)[:, 0]
        return cfg.density_ratio * (col + soft)

    def umag(kk):
        g = 1.0 + kk / MEC2
        return KC * np.sqrt(g * g - 1.0)

    for t in range(cfg.steps):
        for q in range(cfg.substeps):
            a = alive.copy()
            if not a.any():
                break
            g = 1.0 + k[a] / MEC2
            L = KC * np.sqrt(1.0 - 1.0 / (g * g)) * h
            za, zb = z[a] + GL_A * L * d[a, 2], z[a] + GL_B * L * d[a, 2]
            eavg = 0.5 * (field(za) + field(zb))
            w = -1.0 * d[a, 2] * L * eavg
            s = -1.0 * (KC * KC / MEC2) * 0.5 * h
            m = umag(k[a])[:, None] * d[a]
            m[:, 2] += s * eavg
            d1 = m / np.linalg.norm(m, axis=1)[:, None]
            k1 = k[a] + 0.5 * w
            z1 = z[a] + L * d[a, 2]
            loss = drag(k1) * L
            stop = ~(k1 - loss > cfg.cutoff_eV)
            k2 = np.where(stop, cfg.cutoff_eV, k1 - loss)
            m2 = umag(k2)[:, None] * d1
            m2[:, 2] += s * eavg
            d2 = m2 / np.linalg.norm(m2, axis=1)[:, None]
            k3 = k2 + 0.5 * w
            nrm, c, sn = _rotation(cfg.rng_seed, ids[a], t, q, cfg.scatter_rms_rad)
            nv = (nrm * d2).sum(1)
            cr = np.cross(nrm, d2)
            d3 = d2 * c[:, None] + cr * sn[:, None] + nrm * (nv * (1.0 - c))[:, None]
            idx = np.nonzero(a)[0]
            z[idx] = z1
            new_k = np.where(stop, cfg.cutoff_eV, k3)
            new_d = np.where(stop[:, None], d[a], d3)
            k[idx] = new_k
            d[idx] = new_d
            alive[idx] = ~stop & (k3 > cfg.cutoff_eV)
    return np.stack([z, d[:, 0], d[:, 1], d[:, 2], k, alive.astype(float)])
