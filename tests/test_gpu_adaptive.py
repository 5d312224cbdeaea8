"""Adaptive (per-point) ray directions on the GPU (Rays::use_adaptive_directions,
rays.cpp:5-146): each origin traces, shifts and weights its own rays.

* J, u and the ALO diagonal of the Feautrier solve (FP64 and split precision), the
  short-characteristics J (far wings on the scale of the line peak, as in
  test_gpu_sc0.py), and the anisotropic J2 elements within 1e-5 of the oracle.
* set_column along each point's own rays bit-exact.
* The drop-in path: core.Model with an [npoints * nrays] direction array."""
import numpy as np
import pytest

import helpers as H
import oracle as O
from magritte_gb300 import _abi
from magritte_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _oracle_with_correctly_rounded_erf():
    O.set_erf_mode(1)
    yield
    O.set_erf_mode(0)


@pytest.fixture(scope="module")
def adaptive(gpu_lib):
    raw = S.with_adaptive_rays(S.grid_sphere(n=14, nside=1, nquads=7), seed=4)
    a = H.setup(raw)
    dev = _abi.DeviceModel(a)
    yield raw, a, O.Oracle(a), dev
    dev.close()


def test_adaptive_formal_solves_match_oracle(adaptive):
    raw, a, orc, dev = adaptive
    ref = orc.formal_solve_fo2(want_u=True)
    has = ref["lambda_has"].astype(bool)
    for precision in ("fp64", "split"):
        g = dev.formal_solve_fo2(precision, want_u=True)
        for k in ("J", "u"):
            assert H.max_rel(g[k], ref[k]) < 1e-5, (precision, k)
        assert H.max_rel(g["lambda_diag"][has], ref["lambda_diag"][has]) < 1e-5, precision
    # short characteristics: far-wing values on the scale of the point's line peak, as in
    # test_gpu_sc0.py (its update amplifies single-ulp libm differences where dtau is small)
    J0, J0_ref = dev.formal_solve_sc0("fp64")["J"], orc.formal_solve_sc0()["J"]
    floor = 1e-2 * np.abs(J0_ref).max(axis=-1, keepdims=True)
    assert np.max(np.abs(J0 - J0_ref) / np.maximum(np.abs(J0_ref), floor)) < 1e-5
    an = dev.formal_solve_fo2_anis("fp64")
    an_ref = orc.formal_solve_fo2_anis()
    scale = np.abs(an_ref["J"]).max()
    for k in an_ref:
        assert np.abs(an[k] - an_ref[k]).max() <= 1e-5 * scale, k


def test_adaptive_column_bit_exact(adaptive):
    raw, a, orc, dev = adaptive
    rho = np.random.default_rng(3).uniform(1.0, 10.0, a["npoints"])
    np.testing.assert_array_equal(dev.set_column(rho), orc.set_column(rho))


def test_core_model_adaptive_rays(gpu_lib):
    from magritte_gb300 import loader

    raw = S.with_adaptive_rays(S.grid_cube(n=10, nquads=5), seed=1)
    ref = O.Oracle(H.setup(raw)).formal_solve_fo2()
    model = loader.to_core(raw, precision="fp64")
    model.compute_spectral_discretisation()
    model.compute_inverse_line_widths()
    model.compute_LTE_level_populations()
    model.compute_radiation_field_feautrier_order_2()
    assert model.geometry.rays.use_adaptive_directions
    assert H.max_rel(np.array(model.radiation.J), ref["J"]) < 1e-5
