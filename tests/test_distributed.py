"""The cross-rank pieces of a sharded kinetic step, on two gloo ranks on the
CPU: the face-current allreduce before the replicated Maxwell update
(RreaWarpXCoupling.cpp:715-717, RreaAmrexAdvance.cpp:870-871) and the
max-over-ranks step timing.  Each rank deposits half of the reference's
golden net-chord segments with the oracle; the summed current must equal
the current of all segments deposited on one rank (to 1e-12 of its largest
entry: the sum order differs), and both ranks must end the Maxwell update
with bit-identical fields."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import GOLDEN, ROOT

DT = 3.7e-10
NR, NZ, DR, DZ = 8, 12, 0.75, 1.25


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _config(oracle):
    cfg = oracle.RreaGpuConfig()
    cfg.r_lo, cfg.r_hi, cfg.z_lo, cfg.z_hi, cfg.nr, cfg.nz = 0.0, NR * DR, 0.0, NZ * DZ, NR, NZ
    return cfg


def _worker(rank, world, port, outdir):
    import sys
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle
        from rrea_feedback_warpx_amrex_geant4_gb300 import distributed

        cfg = _config(oracle)
        rows = np.load(os.path.join(GOLDEN, "ref_netchord_segments.npy"))
        mine = oracle.deposit_segments(cfg, DT, rows[rank::world])
        jr = torch.from_numpy(mine["jr_phys"].ravel().copy())
        jz = torch.from_numpy(mine["jz_phys"].ravel().copy())
        distributed.allreduce_current(jr, jz, dist)
        # replicated Maxwell update from a common initial field
        rng = np.random.default_rng(11)
        er = rng.normal(size=(NR + 1) * NZ)
        ez = rng.normal(size=NR * (NZ + 1))
        bt = np.zeros((NR + 1) * (NZ + 1))
        er, ez, bt = oracle.advance_maxwell(NR, NZ, DR, DZ, DT, 2, er, ez, bt, jr.numpy(), jz.numpy())
        t_max, units = distributed.reduce_step_time(10.0 + rank, 100 * (rank + 1), dist, "cpu")
        np.savez(os.path.join(outdir, f"rank{rank}.npz"), jr=jr.numpy(), jz=jz.numpy(), er=er, ez=ez, bt=bt,
                 t_max=t_max, units=units)
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_current_allreduce_and_replicated_field(tmp_path, oracle_mod):
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [np.load(tmp_path / f"rank{r}.npz") for r in range(world)]
    cfg = _config(oracle_mod)
    rows = np.load(os.path.join(GOLDEN, "ref_netchord_segments.npy"))
    full = oracle_mod.deposit_segments(cfg, DT, rows)
    for key, ref in (("jr", full["jr_phys"].ravel()), ("jz", full["jz_phys"].ravel())):
        scale = max(np.abs(ref).max(), 1e-300)
        assert scale > 0.0
        for r in res:
            np.testing.assert_allclose(r[key], ref, rtol=0, atol=1e-12 * scale, err_msg=key)
    for key in ("jr", "jz", "er", "ez", "bt"):
        np.testing.assert_array_equal(res[0][key], res[1][key], err_msg=key)
    for r in res:
        assert float(r["t_max"]) == 11.0 and float(r["units"]) == 300.0
