"""Failure detection of the formal-solve path, exercised without any GPU fault.

The kernels never trap: an anomaly sets a bit of the model's device status word
(trace left the point cloud on an interior point, a count beyond the sized capacity, a
non-finite intensity), and the host returns it as MGR_ERR_TRACE / MGR_ERR_CAPACITY /
MGR_ERR_NONFINITE from the blocking entry points or mgr_sync.  The reference only
prints in these cases (src/solver/solver.tpp:97).  Each failure is made on the host:
  * a NaN emissivity at one point -> MGR_ERR_NONFINITE from the solve;
  * an interior point whose neighbour list is empty -> MGR_ERR_TRACE (the sizing pass of
    the model upload already walks into it);
  * an interpolation criterion jumping by 1e60 between two neighbours, whose
    interpolation count overflows the per-edge table -> MGR_ERR_CAPACITY from mgr_sync;
  * a half-ray capacity below the longest half ray -> MGR_ERR_CAPACITY, on the CPU
    emulation of the kernel (the GPU sizes its ray buffers from the model, so this case
    cannot be forced there).
After each failure the same process solves a healthy model and gets the healthy
result: the CUDA context stays usable."""
import ctypes as C

import numpy as np
import pytest

import helpers as H
from magritte_gb300 import _abi, build
from magritte_gb300 import synthetic as S


def _cube(n=8):
    return H.setup(S.grid_cube(n=n, nquads=5))


def _interior(a, n):
    # grid point (2, 2, 2) of an n^3 cube, numbered x-major like grid_neighbors
    return (2 * n + 2) * n + 2


# ---- CPU: the emulated kernel's capacity status ----------------------------------


def test_emulated_capacity_overflow():
    lib = C.CDLL(build.build_emu())
    lib.mgr_emu_formal_solve_fo2.argtypes = [C.POINTER(_abi.MgrModelDesc), C.c_int, C.POINTER(C.c_double),
                                             C.POINTER(C.c_double)]
    lib.mgr_emu_formal_solve_fo2.restype = C.c_int
    lib.mgr_emu_set_half_capacity.argtypes = [C.c_uint32]
    lib.mgr_emu_set_half_capacity.restype = None
    a = _cube()
    desc, keep = _abi.make_desc(a)
    P, F, L = a["npoints"], a["nfreqs"], a["nlines"]
    J, lam = np.zeros((P, F)), np.zeros((P, L))
    args = (C.byref(desc), _abi.PRECISION["fp64"], J.ctypes.data_as(C.POINTER(C.c_double)),
            lam.ctypes.data_as(C.POINTER(C.c_double)))
    try:
        lib.mgr_emu_set_half_capacity(3)  # the cube's half rays have up to 7 steps
        assert lib.mgr_emu_formal_solve_fo2(*args) == _abi.MGR_ERR_CAPACITY
    finally:
        lib.mgr_emu_set_half_capacity(0)
    assert lib.mgr_emu_formal_solve_fo2(*args) == _abi.MGR_OK
    assert np.isfinite(J).all()


# ---- GPU: status words through the C ABI ------------------------------------------


@pytest.mark.gpu
def test_nan_emissivity_reports_nonfinite(gpu_lib):
    a = _cube()
    dev = _abi.DeviceModel(a)
    try:
        good = dev.formal_solve_fo2("fp64")["J"]
        em = a["emissivity"].copy()
        em[_interior(a, 8)] = np.nan
        dev.set_line_data(emissivity=em)
        with pytest.raises(_abi.MgrError) as err:
            dev.formal_solve_fo2("fp64")
        assert err.value.code == _abi.MGR_ERR_NONFINITE
        assert gpu_lib.mgr_sync(dev.h) == _abi.MGR_OK  # the status word was consumed
        dev.set_line_data(emissivity=a["emissivity"])
        np.testing.assert_array_equal(dev.formal_solve_fo2("fp64")["J"], good)
    finally:
        dev.close()


@pytest.mark.gpu
def test_interior_point_without_neighbours_reports_trace(gpu_lib):
    n = 8
    a = _cube(n)
    p = _interior(a, n)
    assert a["point2boundary"][p] == a["npoints"]  # interior
    nn = a["n_neighbors"].copy()
    cum = np.concatenate([[0], np.cumsum(nn)[:-1]]).astype(np.uint32)
    keep = np.ones(len(a["neighbors"]), bool)
    keep[cum[p]:cum[p] + nn[p]] = False
    bad = dict(a)
    bad["neighbors"] = a["neighbors"][keep]
    nn[p] = 0
    bad["n_neighbors"] = nn
    bad["cum_n_neighbors"] = np.concatenate([[0], np.cumsum(nn)[:-1]]).astype(np.uint32)
    with pytest.raises(_abi.MgrError) as err:
        _abi.DeviceModel(bad)
    assert err.value.code == _abi.MGR_ERR_TRACE
    assert b"interior point" in gpu_lib.mgr_last_error()
    # the context is still usable
    dev = _abi.DeviceModel(a)
    try:
        assert np.isfinite(dev.formal_solve_fo2("fp64")["J"]).all()
    finally:
        dev.close()


@pytest.mark.gpu
def test_interpolation_count_overflow_reports_capacity(gpu_lib):
    a = _cube()
    dev = _abi.DeviceModel(a)
    try:
        good = dev.formal_solve_fo2("fp64")["J"]
        crit = a["interp_criterion"].copy()
        crit[_interior(a, 8)] *= 1.0e60  # log ratio beyond FP32: an unbounded count
        dev.set_line_data(interp_criterion=crit)
        assert gpu_lib.mgr_sync(dev.h) == _abi.MGR_ERR_CAPACITY
        assert b"capacity" in gpu_lib.mgr_last_error() or b"longer" in gpu_lib.mgr_last_error()
        dev.set_line_data(interp_criterion=a["interp_criterion"])
        assert gpu_lib.mgr_sync(dev.h) == _abi.MGR_OK
        np.testing.assert_array_equal(dev.formal_solve_fo2("fp64")["J"], good)
    finally:
        dev.close()
