"""Rank-level pieces of a sharded kinetic step.

Particles shard across ranks with no exchange inside the transport.  Two
things cross ranks per step: the face current, summed before the replicated
Maxwell update (RreaWarpXCoupling.cpp:715-717, RreaAmrexAdvance.cpp:870-871),
and the step's timing and work counts.  `dist` is torch.distributed after
init_process_group (NCCL on GPUs, gloo on the CPU)."""
import torch


class _DeviceVector:
    """A CUDA array interface over a float64 device vector owned by the
    library, so torch can view it without a copy."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (int(n),), "typestr": "<f8", "data": (int(ptr), False),
                                         "version": 3}


def device_view(ptr, n):
    """float64 tensor aliasing n doubles of device memory at ptr."""
    return torch.as_tensor(_DeviceVector(ptr, n), device="cuda")


def allreduce_current(jr, jz, dist):
    """Sums the face-current vectors of every rank in place.  On the GPU the
    sums are complete on return: the library's own stream does not wait on
    torch's streams."""
    dist.all_reduce(jr, op=dist.ReduceOp.SUM)
    dist.all_reduce(jz, op=dist.ReduceOp.SUM)
    if jr.is_cuda:
        torch.cuda.synchronize()


def exchange_current_and_advance(ctx, dist, dt_s, substeps):
    """The field update of a sharded step: convert this rank's current, sum
    it across ranks on the device, and run Maxwell on the sum."""
    (jr_ptr, n_jr), (jz_ptr, n_jz) = ctx.current_device()
    if dist is not None:
        allreduce_current(device_view(jr_ptr, n_jr), device_view(jz_ptr, n_jz), dist)
    ctx.advance_field_from_current(dt_s, substeps)


def exchange_and_advance_coupled(ctx, dist, dt_s):
    """The coupled fluid/Maxwell update of a sharded step: sum this rank's
    kinetic face current and cell sources across ranks on the device,
    normalise the sources into the fluid's rates, and run the replicated
    coupled step (every rank computes the same fluid and field)."""
    (jr_ptr, n_jr), (jz_ptr, n_jz) = ctx.current_device()
    if dist is not None:
        allreduce_current(device_view(jr_ptr, n_jr), device_view(jz_ptr, n_jz), dist)
        cells_ptr, n_cells = ctx.sources_device()
        cells = device_view(cells_ptr, n_cells)
        dist.all_reduce(cells, op=dist.ReduceOp.SUM)
        torch.cuda.synchronize()
    ctx.fluid_take_sources(dt_s)
    return ctx.advance_field_coupled_from_current(dt_s)


def reduce_step_time(total_ms, units, dist, device):
    """(max over ranks of the timed milliseconds, sum of the work units)."""
    t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t[0]), float(u[0])
