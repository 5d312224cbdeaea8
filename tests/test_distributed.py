"""Ray-pair sharding over processes (magritte_gb300.distributed) on CPU: gloo ranks
(world_size 2 and 3) each run the formal-solve kernel's lane code (libmgr_emu.so) on
their block of ray pairs and sum the partial J / ALO diagonal with one allreduce;
the totals match the unsharded solve up to the order of the additions and the
oracle to the kernel's own bar."""
import ctypes as C
import os
import socket
import tempfile

import numpy as np
import pytest
import torch.multiprocessing as mp

import helpers as H
import oracle as O
from magritte_gb300 import _abi, build, distributed
from magritte_gb300 import synthetic as S


def test_ray_shard_blocks_cover_every_ray_pair_once():
    for R in (1, 5, 6, 24, 37):
        for W in (1, 2, 3, 4, 7, 8, 40):
            blocks = [distributed.ray_shard(R, k, W) for k in range(W)]
            assert blocks[0][0] == 0 and blocks[-1][1] == R
            for (b0, e0), (b1, e1) in zip(blocks, blocks[1:]):
                assert e0 == b1
            sizes = [e - b for b, e in blocks]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        distributed.ray_shard(6, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _emu(path):
    lib = C.CDLL(path)
    f = lib.mgr_emu_formal_solve_fo2_rays
    f.argtypes = [C.POINTER(_abi.MgrModelDesc), C.c_int, C.c_uint32, C.c_uint32, C.POINTER(C.c_double),
                  C.POINTER(C.c_double)]
    f.restype = C.c_int
    return lib


def _rank_main(rank, world, port, emu_path, out_dir, precision):
    import torch
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        a = H.setup(S.grid_sphere(n=12, nside=1, nquads=5))
        desc, keep = _abi.make_desc(a)
        lib = _emu(emu_path)
        prec = _abi.PRECISION[precision]

        def partial(b, e, J, lam):
            Jn, ln = np.zeros(tuple(J.shape)), np.zeros(tuple(lam.shape))
            rc = lib.mgr_emu_formal_solve_fo2_rays(C.byref(desc), prec, b, e,
                                                   Jn.ctypes.data_as(C.POINTER(C.c_double)),
                                                   ln.ctypes.data_as(C.POINTER(C.c_double)))
            assert rc == 0
            J.copy_(torch.from_numpy(Jn))
            lam.copy_(torch.from_numpy(ln))

        J, lam = distributed.sharded_formal_solve(partial, a["hnrays"], a["npoints"], a["nfreqs"], a["nlines"],
                                                  "cpu")
        # host-buffer partials summed by reduce_partials_host give the same totals
        b, e = distributed.ray_shard(a["hnrays"], rank, world)
        Jh, lh = np.zeros((a["npoints"], a["nfreqs"])), np.zeros((a["npoints"], a["nlines"]))
        if e > b:
            assert lib.mgr_emu_formal_solve_fo2_rays(C.byref(desc), prec, b, e,
                                                     Jh.ctypes.data_as(C.POINTER(C.c_double)),
                                                     lh.ctypes.data_as(C.POINTER(C.c_double))) == 0
        distributed.reduce_partials_host(Jh, lh)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), J=J.numpy(), lam=lam.numpy(), Jh=Jh, lh=lh,
                 shard=np.array([b, e]))
    finally:
        dist.destroy_process_group()


@pytest.fixture(scope="module")
def emu_path():
    return build.build_emu()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_solve_gloo_matches_unsharded(emu_path, world):
    a = H.setup(S.grid_sphere(n=12, nside=1, nquads=5))
    desc, keep = _abi.make_desc(a)
    lib = _emu(emu_path)
    lib.mgr_emu_formal_solve_fo2.argtypes = [C.POINTER(_abi.MgrModelDesc), C.c_int, C.POINTER(C.c_double),
                                             C.POINTER(C.c_double)]
    J0, l0 = np.zeros((a["npoints"], a["nfreqs"])), np.zeros((a["npoints"], a["nlines"]))
    assert lib.mgr_emu_formal_solve_fo2(C.byref(desc), 0, J0.ctypes.data_as(C.POINTER(C.c_double)),
                                        l0.ctypes.data_as(C.POINTER(C.c_double))) == 0
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_rank_main, args=(world, _free_port(), emu_path, d, "fp64"), nprocs=world, join=True,
                           start_method="spawn")
        res = [dict(np.load(os.path.join(d, f"rank{k}.npz"))) for k in range(world)]
    shards = [tuple(r["shard"]) for r in res]
    assert shards[0][0] == 0 and shards[-1][1] == a["hnrays"]
    for r in res:
        # identical on every rank, equal to the unsharded sums up to addition order
        np.testing.assert_array_equal(r["J"], res[0]["J"])
        assert H.max_rel(r["J"], J0) < 1e-13
        assert H.max_rel(r["lam"], l0) < 1e-13
        np.testing.assert_allclose(r["Jh"], r["J"], rtol=1e-15, atol=0)
        np.testing.assert_allclose(r["lh"], r["lam"], rtol=1e-15, atol=0)
    O.set_erf_mode(1)
    try:
        ref = O.Oracle(a).formal_solve_fo2()
    finally:
        O.set_erf_mode(0)
    has = ref["lambda_has"].astype(bool)
    assert H.max_rel(res[0]["J"], ref["J"]) < 1e-12
    assert H.max_rel(res[0]["lam"][has], ref["lambda_diag"][has]) < 1e-12


def test_partial_range_partitions_sum(emu_path):
    """Partial sums over [0, k) and [k, R) add up to the full solve for every split
    point k, in both precision modes; empty or out-of-range ranges are rejected."""
    a = H.setup(S.grid_cube(n=8, nquads=5))
    desc, keep = _abi.make_desc(a)
    lib = _emu(emu_path)
    lib.mgr_emu_formal_solve_fo2.argtypes = [C.POINTER(_abi.MgrModelDesc), C.c_int, C.POINTER(C.c_double),
                                             C.POINTER(C.c_double)]
    ptr = lambda x: x.ctypes.data_as(C.POINTER(C.c_double))
    P, F, L, R = a["npoints"], a["nfreqs"], a["nlines"], a["hnrays"]
    for prec in (0, 1):
        J0, l0 = np.zeros((P, F)), np.zeros((P, L))
        assert lib.mgr_emu_formal_solve_fo2(C.byref(desc), prec, ptr(J0), ptr(l0)) == 0
        for k in (1, R // 2, R - 1):
            Ja, la, Jb, lb = np.zeros((P, F)), np.zeros((P, L)), np.zeros((P, F)), np.zeros((P, L))
            assert lib.mgr_emu_formal_solve_fo2_rays(C.byref(desc), prec, 0, k, ptr(Ja), ptr(la)) == 0
            assert lib.mgr_emu_formal_solve_fo2_rays(C.byref(desc), prec, k, R, ptr(Jb), ptr(lb)) == 0
            assert H.max_rel(Ja + Jb, J0) < 1e-13
            assert H.max_rel(la + lb, l0) < 1e-13
    J, lam = np.zeros((P, F)), np.zeros((P, L))
    assert lib.mgr_emu_formal_solve_fo2_rays(C.byref(desc), 0, 3, 3, ptr(J), ptr(lam)) != 0
