"""The trace's FP32 next-point filter (trace_half, warp_next_point_f32) against the
exact FP64 walk on the CPU.

libmgr_emu.so restates the filtered walk with the kernel's own float arithmetic
(filt_cand / filt_ahead, explicit fmaf: the device computes the same floats), so its
decisions are the device's.  Over every origin and every ray of Cartesian cubes, sphere
cutouts (the benchmarked family), Delaunay point clouds (the non-LTE family) and
adaptive rays, the filtered walk must give the exact walk's point sequences, edges
and dZ bit for bit; the share of steps the filter leaves to the exact argmin is
reported (near ties, undecided ahead/behind neighbours)."""
import ctypes as C

import numpy as np
import pytest

import helpers as H
from magritte_gb300 import _abi, build
from magritte_gb300 import synthetic as S


@pytest.fixture(scope="module")
def emu():
    lib = C.CDLL(build.build_emu())
    u64p = C.POINTER(C.c_uint64)
    lib.mgr_emu_trace_filter_check.argtypes = [C.POINTER(_abi.MgrModelDesc), u64p, u64p, u64p, u64p]
    lib.mgr_emu_trace_filter_check.restype = C.c_int
    return lib


def _lattice_rays(raw):
    """The 13 lattice directions of the 26-neighbour grid and their antipodes as rays:
    every step has neighbours placed symmetrically about the ray, so the reference's
    argmin is decided by FP64 rounding between exact ties, which the filter must leave
    to the exact argmin."""
    import dataclasses
    dirs = []
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dz in (-1, 0, 1):
                v = (dx, dy, dz)
                if v != (0, 0, 0) and v > (0, 0, 0):
                    dirs.append(np.array(v, float) / np.linalg.norm(v))
    d = np.array(dirs + [-x for x in dirs])
    return dataclasses.replace(raw, ray_direction=d, ray_weight=np.full(len(d), 1.0 / len(d)))


MODELS = {
    "cube12": lambda: S.grid_cube(n=12, nquads=3),
    "cube10_lattice_rays": lambda: _lattice_rays(S.grid_cube(n=10, nquads=3)),
    "delaunay_nside4": lambda: S.nlte_sphere(npoints=2000, nside=4, nlev=2, nquads=3),
    "cube10_nside2": lambda: S.grid_cube(n=10, nside=2, nquads=3, seed=3),
    "sphere20_nside2": lambda: S.grid_sphere(n=20, nside=2, nquads=3, nlev=2),
    "delaunay_sphere": lambda: S.nlte_sphere(npoints=3000, nside=2, nlev=2, nquads=3),
    "cube8_adaptive": lambda: S.with_adaptive_rays(S.grid_cube(n=8, nquads=3)),
}


@pytest.mark.parametrize("name", sorted(MODELS))
def test_filtered_walk_is_the_exact_walk(emu, name):
    a = H.setup(MODELS[name]())
    desc, keep = _abi.make_desc(a)
    rays, steps, exact, bad = (C.c_uint64() for _ in range(4))
    assert emu.mgr_emu_trace_filter_check(C.byref(desc), C.byref(rays), C.byref(steps), C.byref(exact),
                                          C.byref(bad)) == 0
    assert rays.value == a["npoints"] * a["nrays"]
    assert steps.value > rays.value
    print(f"{name}: {rays.value} rays, {steps.value} steps, exact argmin on {exact.value} "
          f"({exact.value / steps.value:.2%})")
    assert bad.value == 0
