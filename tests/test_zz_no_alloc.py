"""mgr_formal_solve_fo2_device_noalloc against mgr_formal_solve_fo2_device.

Both entry points run the same two kernels on the same origins; only the staging
buffer differs (a fixed device array instead of model-owned scratch), so J, u and the
ALO diagonal must agree bit for bit, on two calls in a row.  Further cases:

  * a model whose staging needs many passes through the fixed array (the 32^3 sphere
    cutout: about 0.8 GB of per-ray results against the 64 MiB array);
  * a model whose single origin needs more than the array holds, which the entry
    point must reject with MGR_ERR_CAPACITY before launching anything;
  * the device's free memory is the same before and after calls (nothing allocated);
  * a model with an imaging spectral discretisation is refused, as the ordinary entry
    point refuses it;
  * compute_Jeff after a call reads that call's J and ALO diagonal.

The file name sorts last so that the test also runs after every other GPU test in one
session."""
import ctypes as C

import numpy as np
import pytest

import helpers as H
from magritte_gb300 import _abi
from magritte_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

STAGE_BYTES = 64 << 20  # the entry point's fixed staging array


@pytest.fixture(scope="module")
def cube(gpu_lib):
    a = H.setup(S.grid_cube())  # 20^3 points, 6 ray pairs, 11 frequencies
    dev = _abi.DeviceModel(a)
    yield dev
    dev.close()


@pytest.fixture(scope="module")
def sphere32(gpu_lib):
    raw = S.grid_sphere(n=32)  # 32^3 cutout, 24 ray pairs, 4 lines x 31 quadrature points
    a = H.setup(raw)
    dev = _abi.DeviceModel(a)
    dev.set_species(raw.linedata, raw.abundance, a["populations"])
    yield dev
    dev.close()


def _solve(lib, fn, dev, precision, want_u, want_lam):
    import torch

    P, F, L, R = dev.P, dev.F, dev.L, dev.R
    J = torch.full((P, F), float("nan"), dtype=torch.float64, device="cuda")
    u = torch.full((R, P, F), float("nan"), dtype=torch.float64, device="cuda") if want_u else None
    lam = torch.full((P, L), float("nan"), dtype=torch.float64, device="cuda") if want_lam else None
    torch.cuda.synchronize()
    ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None
    rc = fn(dev.h, _abi.PRECISION[precision], ptr(J), ptr(u), ptr(lam))
    assert rc == 0, lib.mgr_last_error().decode()
    assert lib.mgr_sync(dev.h) == 0, lib.mgr_last_error().decode()
    out = [J.cpu().numpy()]
    out.append(u.cpu().numpy() if u is not None else None)
    out.append(lam.cpu().numpy() if lam is not None else None)
    return out


def _assert_same(ref, got):
    for r, g in zip(ref, got):
        if r is None:
            assert g is None
        else:
            np.testing.assert_array_equal(g, r)


@pytest.mark.parametrize("precision", ["fp64", "split"])
@pytest.mark.parametrize("want_u,want_lam", [(False, True), (True, True), (False, False)])
def test_noalloc_matches_scratch_entry_point(gpu_lib, cube, precision, want_u, want_lam):
    pytest.importorskip("torch")
    lib = gpu_lib
    ref = _solve(lib, lib.mgr_formal_solve_fo2_device, cube, precision, want_u, want_lam)
    assert np.isfinite(ref[0]).all()
    for _ in range(2):  # two calls in a row reuse the same staging area
        got = _solve(lib, lib.mgr_formal_solve_fo2_device_noalloc, cube, precision, want_u, want_lam)
        _assert_same(ref, got)


@pytest.mark.parametrize("precision", ["split", "fp64"])
def test_noalloc_many_passes_through_the_array(gpu_lib, sphere32, precision):
    """Staging of u and L_diag for all origins is far larger than the fixed array, so
    the call runs many chunks of origins; the results are still bit-identical."""
    pytest.importorskip("torch")
    lib, dev = gpu_lib, sphere32
    per_origin = dev.R * dev.F * 8 * 2
    assert dev.P * per_origin > 8 * STAGE_BYTES  # at least eight passes
    ref = _solve(lib, lib.mgr_formal_solve_fo2_device, dev, precision, False, True)
    for _ in range(2):
        got = _solve(lib, lib.mgr_formal_solve_fo2_device_noalloc, dev, precision, False, True)
        _assert_same(ref, got)


def test_noalloc_allocates_nothing(gpu_lib, sphere32):
    """Free device memory (cudaMemGetInfo) and torch's reserved memory are unchanged by
    calls after the first one, which may load the kernels' module."""
    torch = pytest.importorskip("torch")
    lib, dev = gpu_lib, sphere32
    P, F, L = dev.P, dev.F, dev.L
    J = torch.empty((P, F), dtype=torch.float64, device="cuda")
    lam = torch.empty((P, L), dtype=torch.float64, device="cuda")
    call = lambda: lib.mgr_formal_solve_fo2_device_noalloc(dev.h, _abi.PRECISION["split"], C.c_void_p(J.data_ptr()),
                                                          None, C.c_void_p(lam.data_ptr()))
    assert call() == 0, lib.mgr_last_error().decode()
    assert lib.mgr_sync(dev.h) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    reserved0 = torch.cuda.memory_reserved()
    for _ in range(3):
        assert call() == 0, lib.mgr_last_error().decode()
    assert lib.mgr_sync(dev.h) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_reserved() == reserved0


def test_noalloc_rejects_origin_larger_than_array(gpu_lib):
    """6144 ray pairs x 700 frequencies x 8 B x 2 staged arrays = 68.8 MB for one origin,
    above the 64 MiB array: MGR_ERR_CAPACITY.  With u given only L_diag is staged
    (34.4 MB per origin), which fits: the call then runs one origin per pass."""
    torch = pytest.importorskip("torch")
    lib = gpu_lib
    raw = S.grid_sphere(n=6, nside=32, nquads=175)  # 56 points, 12288 rays, 4 lines x 175
    dev = _abi.DeviceModel(H.setup(raw))
    try:
        assert dev.R * dev.F * 8 * 2 > STAGE_BYTES
        J = torch.empty((dev.P, dev.F), dtype=torch.float64, device="cuda")
        lam = torch.empty((dev.P, dev.L), dtype=torch.float64, device="cuda")
        rc = lib.mgr_formal_solve_fo2_device_noalloc(dev.h, _abi.PRECISION["split"], C.c_void_p(J.data_ptr()), None,
                                                     C.c_void_p(lam.data_ptr()))
        assert rc == _abi.MGR_ERR_CAPACITY
        assert b"bytes of staging" in lib.mgr_last_error()
        u = torch.empty((dev.R, dev.P, dev.F), dtype=torch.float64, device="cuda")
        rc = lib.mgr_formal_solve_fo2_device_noalloc(dev.h, _abi.PRECISION["split"], C.c_void_p(J.data_ptr()),
                                                     C.c_void_p(u.data_ptr()), C.c_void_p(lam.data_ptr()))
        assert rc == 0, lib.mgr_last_error().decode()
        assert lib.mgr_sync(dev.h) == 0, lib.mgr_last_error().decode()
    finally:
        dev.close()


def test_noalloc_refuses_imaging_discretisation(gpu_lib):
    """A model whose frequencies are an imaging discretisation has no line map for the
    ALO: both formal-solve entry points return MGR_ERR_UNSUPPORTED."""
    torch = pytest.importorskip("torch")
    lib = gpu_lib
    raw = S.grid_cube(n=6)
    f0 = raw.linedata[0].frequency[0]
    dev = _abi.DeviceModel(H.setup(raw, image_freqs=(f0 * (1 - 1e-5), f0 * (1 + 1e-5), 9)))
    try:
        J = torch.empty((dev.P, dev.F), dtype=torch.float64, device="cuda")
        lam = torch.empty((dev.P, dev.L), dtype=torch.float64, device="cuda")
        for fn in (lib.mgr_formal_solve_fo2_device, lib.mgr_formal_solve_fo2_device_noalloc):
            rc = fn(dev.h, _abi.PRECISION["fp64"], C.c_void_p(J.data_ptr()), None, C.c_void_p(lam.data_ptr()))
            assert rc == _abi.MGR_ERR_UNSUPPORTED
        assert lib.mgr_sync(dev.h) == 0
    finally:
        dev.close()


def test_jeff_after_noalloc_solve(gpu_lib, sphere32):
    """mgr_compute_jeff reads the J and ALO buffers of the latest formal solve: after a
    no-alloc call they are that call's, and Jeff equals Jeff after the ordinary call."""
    torch = pytest.importorskip("torch")
    lib, dev = gpu_lib, sphere32
    P, F, L = dev.P, dev.F, dev.L
    outs = []
    for fn in (lib.mgr_formal_solve_fo2_device, lib.mgr_formal_solve_fo2_device_noalloc):
        J = torch.empty((P, F), dtype=torch.float64, device="cuda")
        lam = torch.empty((P, L), dtype=torch.float64, device="cuda")
        rc = fn(dev.h, _abi.PRECISION["split"], C.c_void_p(J.data_ptr()), None, C.c_void_p(lam.data_ptr()))
        assert rc == 0, lib.mgr_last_error().decode()
        assert lib.mgr_sync(dev.h) == 0
        outs.append((dev.compute_jeff(0), J, lam))  # keep J / lam alive until Jeff ran
    for k in ("Jlin", "Jeff", "Jdif"):
        np.testing.assert_array_equal(outs[1][0][k], outs[0][0][k])
