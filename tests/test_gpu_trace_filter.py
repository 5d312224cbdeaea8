"""The trace's FP32 next-point filter on the GPU: mgr_trace_self_check walks every half
ray (every origin, every ray) with the exact FP64 argmin and with the filter and
counts the rays whose point sequences, edges or dZ bits differ: none may.  Models: the
20^3 cube of the plain FP64 configuration, a cube traced along its own lattice
directions (exact ties at every step), a sphere cutout of the benchmarked family at
nside 2, the Delaunay non-LTE family at nside 2 and 4, adaptive rays."""
import ctypes as C

import pytest

import helpers as H
from magritte_gb300 import _abi
from magritte_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

def _lattice_rays(raw):
    """The 13 lattice directions of the 26-neighbour grid and their antipodes as rays
    (exact ties between neighbours placed symmetrically about every ray)."""
    import dataclasses

    import numpy as np
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
    "cube20": lambda: S.grid_cube(n=20, nquads=3),
    "cube16_lattice_rays": lambda: _lattice_rays(S.grid_cube(n=16, nquads=3)),
    "delaunay5k_nside4": lambda: S.nlte_sphere(npoints=5000, nside=4, nlev=2, nquads=3),
    "sphere32_nside2": lambda: S.grid_sphere(n=32, nside=2, nquads=3, nlev=2),
    "delaunay20k_nside2": lambda: S.nlte_sphere(npoints=20_000, nside=2, nlev=2, nquads=3),
    "cube12_adaptive": lambda: S.with_adaptive_rays(S.grid_cube(n=12, nquads=3)),
}


@pytest.mark.parametrize("name", sorted(MODELS))
def test_filtered_trace_equals_exact_trace(gpu_lib, name):
    a = H.setup(MODELS[name]())
    dev = _abi.DeviceModel(a)
    try:
        rays, steps, bad = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _abi._check(_abi.load().mgr_trace_self_check(dev.h, C.byref(rays), C.byref(steps), C.byref(bad)))
        assert rays.value == a["npoints"] * a["nrays"]
        assert steps.value > rays.value
        assert bad.value == 0
    finally:
        dev.close()
