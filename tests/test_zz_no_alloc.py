"""mgr_formal_solve_fo2_device_noalloc against mgr_formal_solve_fo2_device.

Both entry points run the same two kernels on the same origins; only the staging
buffer differs (a fixed device array instead of model-owned scratch), so J, u and the
ALO diagonal must agree bit for bit, on two calls in a row.  The file name sorts last
so that the test also runs after every other GPU test in one session."""
import ctypes as C

import numpy as np
import pytest

import helpers as H
from magritte_gb300 import _abi
from magritte_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cube(gpu_lib):
    a = H.setup(S.grid_cube())  # 20^3 points, 6 ray pairs, 11 frequencies
    dev = _abi.DeviceModel(a)
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


@pytest.mark.parametrize("precision", ["fp64", "split"])
@pytest.mark.parametrize("want_u,want_lam", [(False, True), (True, True), (False, False)])
def test_noalloc_matches_scratch_entry_point(gpu_lib, cube, precision, want_u, want_lam):
    pytest.importorskip("torch")
    lib = gpu_lib
    ref = _solve(lib, lib.mgr_formal_solve_fo2_device, cube, precision, want_u, want_lam)
    assert np.isfinite(ref[0]).all()
    for _ in range(2):  # two calls in a row reuse the same staging area
        got = _solve(lib, lib.mgr_formal_solve_fo2_device_noalloc, cube, precision, want_u, want_lam)
        for r, g in zip(ref, got):
            if r is None:
                assert g is None
            else:
                np.testing.assert_array_equal(g, r)

