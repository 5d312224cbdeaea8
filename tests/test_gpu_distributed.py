"""The sharded formal solve on one GPU: partial ray-pair solves through the C ABI add
up to the full solve, and the ALI loop with a ray-pair shard reproduces the
unsharded populations.  A second rank is emulated in the same process by a second
model that solves the other ray pairs inside the reduce callback (sequential work,
no kernel waits on another), and the NCCL path runs as a one-rank process group."""
import os
import socket

import numpy as np
import pytest

import helpers as H
from magritte_gb300 import _abi, distributed
from magritte_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def _rel(x, ref, floor=1e-300):
    return float(np.max(np.abs(x - ref) / np.maximum(np.abs(ref), floor)))


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_partial_rays_sum_to_full(gpu_lib, precision):
    a = H.setup(S.grid_sphere(n=16, nside=1, nquads=7))
    dev = _abi.DeviceModel(a)
    try:
        full = dev.formal_solve_fo2(precision)
        R = dev.R
        for k in (1, R // 2, R - 1):
            lo = dev.formal_solve_fo2_rays(0, k, precision)
            hi = dev.formal_solve_fo2_rays(k, R, precision)
            assert _rel(lo["J"] + hi["J"], full["J"]) < 1e-13
            assert _rel(lo["lambda_diag"] + hi["lambda_diag"], full["lambda_diag"]) < 1e-13
        with pytest.raises(_abi.MgrError):
            dev.formal_solve_fo2_rays(2, 2, precision)
        with pytest.raises(_abi.MgrError):
            dev.formal_solve_fo2_rays(0, R + 1, precision)
    finally:
        dev.close()


def test_distributed_formal_solve_one_rank(gpu_lib):
    """distributed.formal_solve_fo2 without a process group: the whole range on this
    GPU, through the device-pointer partial entry point and torch tensors."""
    import torch

    a = H.setup(S.grid_cube(n=10, nquads=5))
    dev = _abi.DeviceModel(a)
    try:
        full = dev.formal_solve_fo2("fp64")
        J, lam = distributed.formal_solve_fo2(dev, "fp64")
        torch.cuda.synchronize()
        assert _rel(J.cpu().numpy(), full["J"]) < 1e-13
        assert _rel(lam.cpu().numpy(), full["lambda_diag"]) < 1e-13
    finally:
        dev.close()


def _device(raw, a):
    dev = _abi.DeviceModel(a)
    dev.set_species(raw.linedata, raw.abundance, a["populations"])
    return dev


def test_sharded_ali_matches_unsharded(gpu_lib):
    """Rank 0 solves ray pairs [0, R/2) in its ALI loop; its reduce callback adds the
    partial sums of [R/2, R) that a second model (the emulated rank 1) solves with the
    same line data.  Populations after the loop match the unsharded loop."""
    import torch

    raw = S.grid_cube(n=10, nquads=11)
    a = H.setup(raw)
    ref_dev = _device(raw, a)
    try:
        ref = ref_dev.compute_level_populations("fp64", use_ng=True, max_it=12)
        ref_pop = ref_dev.populations(0)
    finally:
        ref_dev.close()
    dev, other = _device(raw, a), _abi.DeviceModel(a)
    R = dev.R
    tot = raw.abundance[:, raw.linedata[0].num][:, None]
    calls = []

    def reduce(J_ptr, nJ, lam_ptr, nlam, stream_ptr):
        s = torch.cuda.ExternalStream(stream_ptr)
        s.synchronize()
        # the line data and interpolation criterion (opacity / population_tot) the
        # shard's solve used
        em, op = dev.line_data()
        other.set_line_data(emissivity=em, opacity=op, interp_criterion=op / tot)
        part = other.formal_solve_fo2_rays(R // 2, R, "fp64")
        with torch.cuda.stream(s):
            J = torch.as_tensor(distributed._DeviceArray(J_ptr, nJ), device="cuda")
            lam = torch.as_tensor(distributed._DeviceArray(lam_ptr, nlam), device="cuda")
            J += torch.from_numpy(part["J"].ravel()).to("cuda", non_blocking=False)
            lam += torch.from_numpy(part["lambda_diag"].ravel()).to("cuda", non_blocking=False)
        calls.append(1)

    try:
        dev.set_ray_shard(0, R // 2, reduce)
        got = dev.compute_level_populations("fp64", use_ng=True, max_it=12)
        assert got["iterations"] == ref["iterations"]
        assert len(calls) >= got["iterations"] - 2  # one per normal (non-Ng) iteration
        assert _rel(dev.populations(0), ref_pop, 1e-10 * tot) < 1e-9
        # restore the unsharded loop
        dev.set_ray_shard(0, R)
        with pytest.raises(_abi.MgrError):
            dev.set_ray_shard(0, R // 2)  # a partial range needs a reduce function
    finally:
        dev.close()
        other.close()


def test_sharded_ali_reduce_error_is_reported(gpu_lib):
    raw = S.grid_cube(n=8, nquads=5)
    a = H.setup(raw)
    dev = _device(raw, a)

    def reduce(*args):
        raise RuntimeError("rank lost")

    try:
        dev.set_ray_shard(0, 1, reduce)
        with pytest.raises(_abi.MgrError) as e:
            dev.compute_level_populations("fp64", use_ng=False, max_it=3)
        assert "reduce function failed" in str(e.value)
        assert isinstance(e.value.__cause__, RuntimeError)
    finally:
        dev.close()


def test_nccl_one_rank_group_sharded_ali(gpu_lib):
    """The NCCL reduce of distributed.compute_level_populations on a one-rank group
    (the allreduce is the identity): same populations as the plain loop, with the
    collective enqueued on the model's stream through the callback."""
    import torch
    import torch.distributed as dist

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    store = dist.TCPStore("127.0.0.1", port, 1, True)
    dist.init_process_group("nccl", store=store, rank=0, world_size=1)
    try:
        raw = S.grid_cube(n=8, nquads=5)
        a = H.setup(raw)
        ref_dev = _device(raw, a)
        try:
            ref_dev.compute_level_populations("fp64", use_ng=True, max_it=8)
            ref_pop = ref_dev.populations(0)
        finally:
            ref_dev.close()
        dev = _device(raw, a)
        try:
            dev.set_ray_shard(0, dev.R, distributed._allreduce_on_stream(None))
            dev.compute_level_populations("fp64", use_ng=True, max_it=8)
            torch.cuda.synchronize()
            assert _rel(dev.populations(0), ref_pop, 1e-300) < 1e-13
            J, lam = distributed.formal_solve_fo2(dev, "fp64")
            full = dev.formal_solve_fo2("fp64")
            assert _rel(J.cpu().numpy(), full["J"]) < 1e-13
        finally:
            dev.close()
    finally:
        dist.destroy_process_group()
