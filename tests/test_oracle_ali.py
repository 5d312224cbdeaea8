"""Pins the oracle's ALI level-population loop.

* van Zadelhoff et al. (2002) problem 1a/1b in the 3D HEALPix-shell form of the
  reference's tests/benchmarks/numeric/vanZadelhoff_1_3D_healpix.py: the fractional
  level populations must agree with the RATRAN results the reference ships
  (tests/benchmarks/numeric/Ratran_results/vanZadelhoff_1{a,b}.out) within the
  reference test's own bound, 0.2 relative (vanZadelhoff_1_3D_healpix.py:173).
  The RATRAN files are read from the reference tree when it is present.  The model
  uses 14 shells instead of 20 and 30 ALI iterations to keep the CPU suite short.
* Statistical equilibrium in the collision-dominated limit reproduces LTE.
* compute_Jeff's line integral and ALO correction (model.cpp:514-545)."""
import os

import numpy as np
import pytest

import oracle as O
from magritte_gb300 import synthetic as S

RATRAN = "/root/reference/tests/benchmarks/numeric/Ratran_results/vanZadelhoff_1{}.out"


@pytest.fixture(scope="module", autouse=True)
def built():
    O.build()


@pytest.mark.parametrize("kind", ["a", "b"])
def test_van_zadelhoff_1_against_ratran(kind):
    path = RATRAN.format(kind)
    if not os.path.exists(path):
        pytest.skip("reference RATRAN results not available here")
    from scipy.interpolate import interp1d

    raw = S.van_zadelhoff_1(kind, nshells=14)
    a = O.reference_setup(raw)
    r = O.AliOracle(raw, a).run(use_ng=True, max_it=30)
    pops = r["populations"][0]
    abun = raw.abundance[:, 0]
    rs = np.linalg.norm(raw.position, axis=1)
    cols = np.loadtxt(path, skiprows=14, unpack=True)
    ra, rb, lp0, lp1 = cols[1], cols[2], cols[9], cols[10]
    i0 = interp1d(0.5 * (ra + rb), lp0, fill_value="extrapolate")
    i1 = interp1d(0.5 * (ra + rb), lp1, fill_value="extrapolate")
    rel = lambda x, y: 2.0 * (x - y) / (x + y)  # magritte/tools.py:69-73
    e0 = np.abs(rel(pops[:, 0] / abun, i0(rs)))
    e1 = np.abs(rel(pops[:, 1] / abun, i1(rs)))
    assert e0[1:].max() < 0.2 and e1[1:].max() < 0.2, (e0[1:].max(), e1[1:].max())


def test_statistical_equilibrium_collision_limit_is_lte():
    """With a collision partner density far above the critical density the rate
    equations give Boltzmann populations (detailed balance of Cd/Ce, tabulated at
    20 K, so the model is isothermal at 20 K)."""
    raw = S.grid_cube(n=4, nquads=5)
    raw.temperature[:] = 20.0
    ld = raw.linedata[0]
    raw.abundance[:, ld.colpar[0].num_col_partner] *= 1.0e12
    a = O.reference_setup(raw)
    ali = O.AliOracle(raw, a)
    P = raw.npoints
    Jeff = np.zeros((P, ld.nrad))
    Ls = np.zeros((P, ld.nrad))
    pop = ali.stateq(0, Jeff, Ls, a["populations"][0])
    np.testing.assert_allclose(pop, a["populations"][0], rtol=1e-8)


def test_jeff_is_weighted_line_integral_minus_alo_part():
    raw = S.grid_cube(n=4, nquads=5)
    a = O.reference_setup(raw)
    ali = O.AliOracle(raw, a)
    res = ali.orc.formal_solve_fo2()
    pops = a["populations"]
    out = ali.compute_jeff(res["J"], res["lambda_diag"], pops)
    ld = raw.linedata[0]
    w = raw.quad_weights[0]
    Jlin = res["J"].reshape(raw.npoints, ld.nrad, raw.nquads) @ w
    np.testing.assert_allclose(out["Jlin"][0], Jlin, rtol=1e-14)
    HH_OVER_FOUR_PI = 6.62607004e-34 / (4.0 * np.pi)
    diff = res["lambda_diag"] * pops[0][:, ld.irad]
    np.testing.assert_allclose(out["Jeff"][0], Jlin - HH_OVER_FOUR_PI * diff, rtol=1e-12)
