"""Pathwise gradients of the charged push with respect to an axial field
profile (rrea_gpu_adjoint_*): a torch.autograd.Function whose forward and
backward are the library's hand-written device kernels, with checkpoints
every 32 steps.

The differentiated model and its loss are those of include/rrea_gpu.h's
adjoint section: the continuous part of the charged substep (chord, field
work, half kicks, table drag) with every discrete outcome frozen (one
counter-RNG rotation per particle and substep for the elastic deflection,
the cutoff stop at the same substep), and the loss

    sum_i w_i [ sig((K_i(T) - K_th) / tau_K)
                - lambda (sig((z_i(T) - z_p) / tau_z) - sig((z_i(0) - z_p) / tau_z)) ]

(a smoothed runaway count plus the smoothed net charge that crossed the
plane z_p, which is the time integral of J_z through it).

`adjoint_field_profile` draws the adjoint configuration's field: E_z on
256 nodes over 0-500 m, 450 kV/m plus a Gaussian-correlated perturbation
(sigma 20 kV/m, correlation length 20 m), seeded, pointing along -z."""
import ctypes

import numpy as np

from . import gpu, workloads
from .gpu import DEFAULT_TABLES


class AdjointConfig(ctypes.Structure):
    """Mirror of rrea_gpu_adjoint_config (include/rrea_gpu.h)."""

    _fields_ = [("z_lo", ctypes.c_double), ("z_hi", ctypes.c_double), ("n_nodes", ctypes.c_int32),
                ("steps", ctypes.c_int32), ("substeps", ctypes.c_int32), ("checkpoint_every", ctypes.c_int32)] + [
        (name, ctypes.c_double) for name in (
            "dt_s", "density_ratio", "cutoff_eV", "scatter_rms_rad", "k_threshold_eV", "k_width_eV", "z_plane_m",
            "z_width_m", "plane_weight")] + [("rng_seed", ctypes.c_uint64)]


_bound = False


def _lib():
    global _bound
    lib = gpu.load_library()
    if not _bound:
        vp, d = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)
        lib.rrea_gpu_default_adjoint_config.argtypes = [ctypes.POINTER(AdjointConfig)]
        lib.rrea_gpu_default_adjoint_config.restype = None
        lib.rrea_gpu_adjoint_stage.argtypes = [vp, ctypes.POINTER(AdjointConfig), ctypes.c_int64, d, d, d, d,
                                               ctypes.POINTER(ctypes.c_uint64)]
        lib.rrea_gpu_adjoint_forward.argtypes = [vp, vp, d]
        lib.rrea_gpu_adjoint_forward_frozen.argtypes = [vp, vp, d]
        lib.rrea_gpu_adjoint_backward.argtypes = [vp, vp, vp]
        lib.rrea_gpu_adjoint_final_state.argtypes = [vp, d]
        for name in ("rrea_gpu_adjoint_stage", "rrea_gpu_adjoint_forward", "rrea_gpu_adjoint_forward_frozen",
                     "rrea_gpu_adjoint_backward", "rrea_gpu_adjoint_final_state"):
            getattr(lib, name).restype = ctypes.c_int
        _bound = True
    return lib


def default_config(**overrides):
    c = AdjointConfig()
    _lib().rrea_gpu_default_adjoint_config(ctypes.byref(c))
    for k, v in overrides.items():
        setattr(c, k, v)
    return c


def adjoint_field_profile(n_nodes=256, z_hi=500.0, base=4.5e5, sigma=2.0e4, length=20.0, seed=4):
    """E_z on the nodes: -(base + a seeded Gaussian-correlated perturbation)."""
    z = np.linspace(0.0, z_hi, n_nodes)
    cov = sigma * sigma * np.exp(-0.5 * ((z[:, None] - z[None, :]) / length) ** 2)
    rng = np.random.default_rng(seed)
    chol = np.linalg.cholesky(cov + 1e-9 * sigma * sigma * np.eye(n_nodes))
    return -(base + chol @ rng.standard_normal(n_nodes))


def adjoint_seeds(n, seed=11):
    """The plain case's seeds (7.2 MeV along +z from the origin)."""
    t = workloads.make_electrons("uniform_c0", n, seed=seed)
    k = np.full(n, 7.2e6)
    d = np.stack([t["ux"], t["uy"], t["uz"]], 1)
    return dict(z=t["z"].copy(), dir=d / np.linalg.norm(d, axis=1)[:, None], k=k, w=t["w"].copy(),
                id=np.abs(t["id"]).astype(np.uint64))


class PushAdjoint:
    """One staged adjoint problem on a context."""

    def __init__(self, config, seeds, ctx=None, tables=DEFAULT_TABLES):
        self.lib = _lib()
        self.own = ctx is None
        if ctx is None:
            ctx = gpu.RreaGpuContext(workloads.make_config(gpu, "uniform_c0"), 1024)
            ctx.load_tables(tables)
        self.ctx = ctx
        self.config = config
        n = len(seeds["k"])
        z = np.ascontiguousarray(seeds["z"], dtype=np.float64)
        d = np.ascontiguousarray(seeds["dir"], dtype=np.float64).reshape(-1)
        k = np.ascontiguousarray(seeds["k"], dtype=np.float64)
        w = np.ascontiguousarray(seeds["w"], dtype=np.float64)
        ids = np.ascontiguousarray(seeds["id"], dtype=np.uint64)
        D = ctypes.POINTER(ctypes.c_double)
        self.ctx._check(self.lib.rrea_gpu_adjoint_stage(self.ctx.handle, ctypes.byref(config), n, z.ctypes.data_as(D),
                                                        d.ctypes.data_as(D), k.ctypes.data_as(D),
                                                        w.ctypes.data_as(D),
                                                        ids.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))))
        self.n = n

    def close(self):
        if self.own:
            self.ctx.close()

    def forward(self, e_nodes, frozen=False):
        """Loss for a CUDA float64 tensor of node values.  frozen=True ends
        every particle where the last plain forward ended it (the topology
        the adjoint differentiates); a plain forward records the ends."""
        import torch
        torch.cuda.synchronize()
        loss = ctypes.c_double()
        fn = self.lib.rrea_gpu_adjoint_forward_frozen if frozen else self.lib.rrea_gpu_adjoint_forward
        self.ctx._check(fn(self.ctx.handle, ctypes.c_void_p(e_nodes.data_ptr()), ctypes.byref(loss)))
        return loss.value

    def backward(self, e_nodes):
        """d loss / d nodes (CUDA float64 tensor) for the last forward's nodes."""
        import torch
        grad = torch.empty_like(e_nodes)
        torch.cuda.synchronize()
        self.ctx._check(self.lib.rrea_gpu_adjoint_backward(self.ctx.handle, ctypes.c_void_p(e_nodes.data_ptr()),
                                                           ctypes.c_void_p(grad.data_ptr())))
        return grad

    def final_state(self):
        out = np.zeros(6 * self.n)
        self.ctx._check(self.lib.rrea_gpu_adjoint_final_state(self.ctx.handle,
                                                              out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out.reshape(6, self.n)


def field_loss_function():
    """The torch.autograd.Function over a PushAdjoint: apply(problem, nodes)."""
    import torch

    class FieldProfileLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, problem, e_nodes):
            e = e_nodes.detach().contiguous()
            ctx.problem = problem
            ctx.save_for_backward(e)
            return torch.tensor(problem.forward(e), dtype=torch.float64, device=e.device)

        @staticmethod
        def backward(ctx, grad_out):
            (e,) = ctx.saved_tensors
            ctx.problem.forward(e)   # the reverse pass follows the forward of these nodes
            return None, grad_out * ctx.problem.backward(e)

    return FieldProfileLoss


def central_differences(problem, e_nodes, nodes, h=1.0):
    """Central finite differences of the loss at the listed nodes with the
    same streams (common random numbers) and the topology frozen at the
    nodes' run (every particle ends where it ended there), step h [V/m]."""
    out = []
    problem.forward(e_nodes)          # records the ends
    for k in nodes:
        e = e_nodes.clone()
        e[k] += h
        up = problem.forward(e, frozen=True)
        e[k] -= 2.0 * h
        down = problem.forward(e, frozen=True)
        out.append((up - down) / (2.0 * h))
        del e
    problem.forward(e_nodes)
    return np.array(out)


def measure(n=1_000_000, repeats=2, **overrides):
    """Seconds per gradient of the adjoint configuration (the perturbed
    field profile and the 7.2 MeV seeds, the default adjoint config: 2000
    steps of 0.5 ns in 4 substeps, checkpoints every 32 steps): one recording
    forward plus the reverse pass, timed after one untimed gradient; returns
    a dict."""
    import time

    import torch

    cfg = default_config(**overrides)
    prob = PushAdjoint(cfg, adjoint_seeds(n))
    try:
        e = torch.tensor(adjoint_field_profile(n_nodes=cfg.n_nodes, z_hi=cfg.z_hi), dtype=torch.float64, device="cuda")
        prob.forward(e)
        prob.backward(e)
        torch.cuda.synchronize()
        t_f = t_b = 0.0
        for _ in range(repeats):
            t0 = time.perf_counter()
            loss = prob.forward(e)
            t1 = time.perf_counter()
            g = prob.backward(e)
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            t_f += t1 - t0
            t_b += t2 - t1
        t_f /= repeats
        t_b /= repeats
        return {"electrons": n, "steps": cfg.steps, "substeps": cfg.substeps, "checkpoint_every": cfg.checkpoint_every,
                "nodes": cfg.n_nodes, "loss": loss, "grad_norm": float(torch.linalg.vector_norm(g)),
                "forward_s": t_f, "reverse_s": t_b, "s_per_grad": t_f + t_b, "reverse_over_forward": t_b / t_f,
                "particle_substeps_per_s_forward": n * cfg.steps * cfg.substeps / t_f}
    finally:
        prob.close()


if __name__ == "__main__":
    import argparse
    import json

    p = argparse.ArgumentParser(description="seconds per gradient of the adjoint configuration")
    p.add_argument("--electrons", type=int, default=1_000_000)
    p.add_argument("--steps", type=int, default=2000)
    p.add_argument("--repeats", type=int, default=2)
    a = p.parse_args()
    print(json.dumps(measure(a.electrons, a.repeats, steps=a.steps)))
