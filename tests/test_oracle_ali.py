"""Pins the oracle's ALI level-population loop.

* van Zadelhoff et al. (2002) problem 1a in the 1D spherically symmetric form of the
  reference's tests/benchmarks/numeric/vanZadelhoff_1_1D.py (250 shells, 200 rays,
  nquads 11, Ng acceleration, at most 100 iterations): the fractional level populations
  agree with the RATRAN results the reference ships
  (tests/benchmarks/numeric/Ratran_results/vanZadelhoff_1a.out, committed as
  tests/golden/ratran_vanZadelhoff_1a.npz) within the reference test's own bounds,
  0.12 and 0.13 relative (vanZadelhoff_1_1D.py:160), skipping the inner boundary.
* Statistical equilibrium in the collision-dominated limit reproduces LTE.
* compute_Jeff's line integral and ALO correction (model.cpp:514-545)."""
import os

import numpy as np
import pytest

import oracle as O
from magritte_gb300 import synthetic as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module", autouse=True)
def built():
    O.build()


def ratran_errors(raw, pops, kind):
    """Relative errors of the fractional populations against RATRAN at each shell
    (vanZadelhoff_1_1D.py:113-123)."""
    from scipy.interpolate import interp1d

    g = np.load(os.path.join(GOLDEN, f"ratran_vanZadelhoff_1{kind}.npz"))
    mid = 0.5 * (g["ra"] + g["rb"])
    i0 = interp1d(mid, g["lp0"], fill_value="extrapolate")
    i1 = interp1d(mid, g["lp1"], fill_value="extrapolate")
    abun = raw.abundance[:, 0]
    rs = np.linalg.norm(raw.position, axis=1)
    rel = lambda x, y: 2.0 * (x - y) / (x + y)  # magritte/tools.py:69-73
    return np.abs(rel(pops[:, 0] / abun, i0(rs))), np.abs(rel(pops[:, 1] / abun, i1(rs)))


def van_zadelhoff_1_1d(kind="a"):
    """vanZadelhoff_1_1D.py:20-85: the density-distribution shells at 250 points with
    200 rays and nquads 11."""
    return S.density_distribution_1d(kind, npoints=250, nrays=200, nquads=11)


def test_van_zadelhoff_1a_1d_against_ratran():
    raw = van_zadelhoff_1_1d("a")
    a = O.reference_setup(raw)
    r = O.AliOracle(raw, a).run(use_ng=True, max_it=100)
    e0, e1 = ratran_errors(raw, r["populations"][0], "a")
    assert e0[1:].max() < 0.12 and e1[1:].max() < 0.13, (e0[1:].max(), e1[1:].max())


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


def test_global_rate_system_with_diagonal_alo_is_the_block_solve():
    """With n_off_diag = 0 the reference's global rate system (one sparse system over all
    points, lineProducingSpecies.tpp:377-581) is block diagonal: the oracle's global
    assembly and dense solve give the per-point block solve's populations."""
    raw = S.grid_cube(n=6, nquads=5)
    import helpers as H

    block = O.AliOracle(raw, H.setup(raw)).run(use_ng=True, max_it=6, Ng_acceleration_mem_limit=4)
    glob = O.AliOracle(raw, H.setup(raw)).run(use_ng=True, max_it=6, Ng_acceleration_mem_limit=4, global_stateq=1)
    assert glob["iterations"] == block["iterations"]
    np.testing.assert_allclose(glob["populations"][0], block["populations"][0], rtol=1e-12)


@pytest.mark.parametrize("n_off_diag", [1, 2])
def test_non_local_alo_changes_the_path_not_the_fixed_point(n_off_diag):
    """The band elements of the ALO (n_off_diag > 0) change the first iterations'
    populations (by ~1e-4 here) but not the converged ones (the ALO terms cancel at the
    fixed point of the iteration)."""
    raw = S.grid_cube(n=6, nquads=5)
    import helpers as H

    one_b = O.AliOracle(raw, H.setup(raw)).run(use_ng=False, max_it=1)
    one_k = O.AliOracle(raw, H.setup(raw)).run(use_ng=False, max_it=1, n_off_diag=n_off_diag)
    d1 = np.max(np.abs(one_k["populations"][0] / one_b["populations"][0] - 1.0))
    assert d1 > 1e-5
    conv_b = O.AliOracle(raw, H.setup(raw)).run(use_ng=False, max_it=30, pop_prec=1e-10)
    conv_k = O.AliOracle(raw, H.setup(raw)).run(use_ng=False, max_it=30, pop_prec=1e-10, n_off_diag=n_off_diag)
    np.testing.assert_allclose(conv_k["populations"][0], conv_b["populations"][0], rtol=1e-9)
