"""Ray-pair sharding of the formal solve over processes, one GPU per process.

Ray pairs are independent within a formal solve: rank k of W solves the contiguous
block of ray pairs ``ray_shard(hnrays, k, W)`` for every point and frequency, and one
FP64 sum-allreduce of the packed partial sums [J (P x F) | ALO diagonal (P x L)]
gives every rank the full J and ALO diagonal.  This is the reference's
multi-process formal solve (Solver::solve_feautrier_order_2 over ray pairs,
src/solver/solver.tpp:476, then Radiation::MPI_reduce_J, radiation.cpp:76-86, and
Lambda::MPI_gather, lambda.tpp:121-206) with the ray pairs split across ranks and
one collective instead of an MPI allreduce plus a gather.  The statistical
equilibrium is per point and cheap, so every rank runs it on the reduced totals
(replicated) and the populations stay identical on all ranks without a second
exchange.

The process group is torch.distributed's (NCCL between GPUs; gloo runs the same
host logic on CPU tensors)."""
import ctypes as C

import numpy as np
import torch
import torch.distributed as dist

from . import _abi


def ray_shard(hnrays, rank, world_size):
    """Contiguous, balanced block [begin, end) of the ray pairs for one rank (sizes
    differ by at most one; empty when world_size > hnrays and rank >= hnrays)."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError(f"rank {rank} outside a world of {world_size}")
    return (rank * hnrays) // world_size, ((rank + 1) * hnrays) // world_size


def _rank_world(group):
    if dist.is_available() and dist.is_initialized():
        return dist.get_rank(group), dist.get_world_size(group)
    return 0, 1


def sharded_formal_solve(partial, hnrays, P, F, L, device, group=None):
    """Run ``partial(rr_begin, rr_end, J, lam)`` on this rank's ray pairs and sum over
    the ranks.  ``partial`` writes the partial J [P][F] and ALO diagonal [P][L] into
    the given float64 tensors (views of one packed buffer on ``device``); a rank with
    no ray pairs contributes zeros.  Returns (J, lam) views of the reduced buffer."""
    rank, world = _rank_world(group)
    begin, end = ray_shard(hnrays, rank, world)
    buf = torch.zeros(P * F + P * L, dtype=torch.float64, device=device)
    J = buf[:P * F].view(P, F)
    lam = buf[P * F:].view(P, L)
    if end > begin:
        partial(begin, end, J, lam)
    if world > 1:
        dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    return J, lam


def formal_solve_fo2(dev, precision="split", group=None):
    """Sharded compute_radiation_field_feautrier_order_2 of a DeviceModel on this
    rank's GPU: J [P][F] and ALO diagonal [P][L] (torch CUDA tensors, identical on
    every rank after the allreduce)."""
    return formal_solve_fo2_handle(dev.h, dev.P, dev.F, dev.L, dev.R, precision, group)


def formal_solve_fo2_handle(handle, P, F, L, R, precision="split", group=None):
    """formal_solve_fo2 for a raw MgrModel handle (e.g. core.Model.upload()) of a
    model with P points, F frequencies, L lines and R ray pairs."""
    lib = _abi.load()
    device = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.ExternalStream(lib.mgr_model_stream(handle))
    prec = _abi.PRECISION[precision]

    def partial(b, e, J, lam):
        # the packed buffer was zeroed on torch's stream: order the solve after it
        stream.wait_stream(torch.cuda.current_stream())
        _abi._check(lib.mgr_formal_solve_fo2_rays_device(handle, prec, b, e, C.c_void_p(J.data_ptr()),
                                                         C.c_void_p(lam.data_ptr())))
        torch.cuda.current_stream().wait_stream(stream)

    return sharded_formal_solve(partial, R, P, F, L, device, group)


class _DeviceArray:
    """A raw device pointer as a torch-importable array (__cuda_array_interface__)."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (int(n),), "typestr": "<f8", "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def _allreduce_on_stream(group):
    """mgr_reduce_fn body: sum J and the ALO diagonal over the ranks, in place, ordered
    on the model's stream."""

    def reduce(J_ptr, nJ, lam_ptr, nlam, stream_ptr):
        stream = torch.cuda.ExternalStream(stream_ptr)
        with torch.cuda.stream(stream):
            for ptr, n in ((J_ptr, nJ), (lam_ptr, nlam)):
                t = torch.as_tensor(_DeviceArray(ptr, n), device="cuda")
                dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)

    return reduce


def compute_level_populations(dev, precision="split", use_ng=True, max_it=100, group=None, **params):
    """ALI loop with the formal solves sharded over ray pairs: every iteration solves
    this rank's ray pairs, sums J and the ALO diagonal over the ranks on the model's
    stream, then runs Jeff, the rate equations and the convergence test on the totals
    (replicated on every rank).  Needs world_size <= hnrays."""
    rank, world = _rank_world(group)
    if world == 1:
        return dev.compute_level_populations(precision, use_ng=use_ng, max_it=max_it, **params)
    begin, end = ray_shard(dev.R, rank, world)
    if end <= begin:
        raise ValueError(f"{world} ranks for {dev.R} ray pairs: every rank needs at least one ray pair")
    dev.set_ray_shard(begin, end, _allreduce_on_stream(group))
    try:
        return dev.compute_level_populations(precision, use_ng=use_ng, max_it=max_it, **params)
    finally:
        dev.set_ray_shard(0, dev.R)


def reduce_partials_host(J, lam, group=None):
    """Sum host (numpy) partial J / ALO diagonal arrays over the ranks in place
    (for callers of the host-buffer entry point mgr_formal_solve_fo2_rays)."""
    rank, world = _rank_world(group)
    if world == 1:
        return J, lam
    P, F = J.shape
    L = lam.shape[1]
    buf = torch.from_numpy(np.concatenate([J.ravel(), lam.ravel()]))
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    out = buf.numpy()
    J[...] = out[:P * F].reshape(P, F)
    lam[...] = out[P * F:].reshape(P, L)
    return J, lam


__all__ = ["ray_shard", "sharded_formal_solve", "formal_solve_fo2", "formal_solve_fo2_handle",
           "compute_level_populations", "reduce_partials_host"]
