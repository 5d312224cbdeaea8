"""GPU imagers (compute_image, compute_image_new) against the oracle, through the C
ABI: images within 1e-5 relative in FP64 mode and in split precision; image-plane
coordinates exact.  The new imager also meets the reference's analytic benchmark
bound (constant velocity gradient, 1.5e-3; see test_oracle_images.py)."""
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


@pytest.mark.parametrize("approx", ["CloseLines", "None"])
@pytest.mark.parametrize("rr", [0, 9])
def test_old_imager_matches_oracle(gpu_lib, approx, rr):
    raw = S.grid_sphere(n=16, nside=1, nquads=7)
    a = H.setup(raw, approx=approx)
    ref = O.Oracle(a).image_fo2(rr)
    dev = _abi.DeviceModel(a)
    try:
        for precision in ("fp64", "split"):
            g = dev.image(rr, precision)
            assert H.max_rel(g["I"], ref) < 1e-5, precision
        d = raw.ray_direction[rr]
        den = np.sqrt(d[0] ** 2 + d[1] ** 2)
        ix, iy = d[1] / den, -d[0] / den
        x = raw.position
        np.testing.assert_array_equal(g["ImX"], ix * x[:, 0] + iy * x[:, 1])
    finally:
        dev.close()


def test_new_imager_matches_oracle(gpu_lib):
    raw = S.velocity_gradient_shells(nshells=10)
    fcen = raw.linedata[0].frequency[0]
    dd = 1.0e4 / 2.99792458e8
    a = H.setup(raw, max_width_fraction=0.5, image_freqs=(fcen - fcen * dd, fcen + fcen * dd, 10))
    d = raw.ray_direction[raw.nrays // 2 - 1]
    ref = O.Oracle(a).image_new(d, 50, 50)
    dev = _abi.DeviceModel(a)
    try:
        for precision in ("fp64", "split"):
            g = dev.image_new(d, 50, 50, precision)
            np.testing.assert_array_equal(g["ImX"], ref["ImX"])
            np.testing.assert_array_equal(g["ImY"], ref["ImY"])
            assert H.max_rel(g["I"], ref["I"]) < 1e-5, precision
        # an oblique direction through the same model
        d2 = np.array([0.3, -0.5, 0.81])
        ref2 = O.Oracle(a).image_new(d2, 24, 20)
        g2 = dev.image_new(d2, 24, 20, "fp64")
        assert H.max_rel(g2["I"], ref2["I"]) < 1e-5
    finally:
        dev.close()


def test_core_model_compute_image_new(gpu_lib):
    """The drop-in API on the imaging benchmark: core.Model.compute_image_new(ray_nr,
    nx, ny) after the imaging spectral discretisation, against the oracle."""
    from magritte_gb300 import loader

    raw = S.velocity_gradient_shells(nshells=10)
    fcen = raw.linedata[0].frequency[0]
    dd = 1.0e4 / 2.99792458e8
    a = H.setup(raw, max_width_fraction=0.5, image_freqs=(fcen - fcen * dd, fcen + fcen * dd, 10))
    ray_nr = raw.nrays // 2 - 1
    ref = O.Oracle(a).image_new(raw.ray_direction[ray_nr], 50, 50)
    model = loader.to_core(raw, precision="fp64")
    model.parameters.max_width_fraction = 0.5
    model.compute_spectral_discretisation(fcen - fcen * dd, fcen + fcen * dd)
    model.compute_inverse_line_widths()
    model.compute_LTE_level_populations()
    model.compute_image_new(ray_nr, 50, 50)
    im = model.images[-1]
    assert H.max_rel(np.array(im.I).reshape(2500, -1), ref["I"]) < 1e-5
    np.testing.assert_array_equal(np.array(im.ImX), ref["ImX"])
    model.compute_image(ray_nr)
    assert np.isfinite(np.array(model.images[-1].I)).all()


@pytest.mark.parametrize("approx", ["CloseLines", "None"])
def test_optical_depth_images_match_oracle(gpu_lib, approx):
    """compute_image_optical_depth(_new): the imagers' rays, optical depth summed over
    the pairs; 1e-5 of the oracle in FP64 and split precision."""
    raw = S.grid_sphere(n=16, nside=1, nquads=7)
    a = H.setup(raw, approx=approx)
    orc = O.Oracle(a)
    ref_old = orc.image_optical_depth(3)
    d = np.array([0.3, -0.5, 0.81])
    ref_new = orc.image_optical_depth_new(d, 24, 20)
    dev = _abi.DeviceModel(a)
    try:
        for precision in ("fp64", "split"):
            g = dev.image_optical_depth(3, precision)
            assert H.max_rel(g["I"], ref_old, floor=1e-12 * np.abs(ref_old).max()) < 1e-5, precision
            g2 = dev.image_optical_depth_new(d, 24, 20, precision)
            np.testing.assert_array_equal(g2["ImX"], ref_new["ImX"])
            assert H.max_rel(g2["I"], ref_new["I"], floor=1e-12 * np.abs(ref_new["I"]).max()) < 1e-5, precision
    finally:
        dev.close()


def test_core_model_optical_depth_images(gpu_lib):
    from magritte_gb300 import loader

    raw = S.grid_cube(n=10, nquads=5)
    a = H.setup(raw)
    ref = O.Oracle(a).image_optical_depth(1)
    model = loader.to_core(raw, precision="fp64")
    model.compute_spectral_discretisation()
    model.compute_inverse_line_widths()
    model.compute_LTE_level_populations()
    model.compute_image_optical_depth(1)
    model.compute_image_optical_depth_new(1, 16, 16)
    assert [im.imageType for im in model.images] == [1, 1]
    assert H.max_rel(np.array(model.images[0].I), ref, floor=1e-12 * np.abs(ref).max()) < 1e-5
    assert np.array(model.images[1].I).shape == (256, raw.nquads)


@pytest.mark.parametrize("approx", ["CloseLines", "None"])
def test_image_for_point_matches_oracle(gpu_lib, approx):
    """compute_image_for_point (solver.tpp:629-653, :2582-2715): the rows S_ray,
    dtau_ray, u_ray of interior and boundary points' rays, FP64 and split precision,
    within the imagers' 1e-5 (split: above 1e-10 of the largest entry, and 1e-4 for the
    per-pair S and dtau, whose FP32 wing profiles round); the row count (traced points
    plus interpolation points) exact."""
    raw = S.grid_sphere(n=16, nside=1, nquads=7)
    a = H.setup(raw, approx=approx)
    orc = O.Oracle(a)
    b0 = int(np.nonzero(np.asarray(a["point2boundary"]) != a["npoints"])[0][0])
    dev = _abi.DeviceModel(a)
    try:
        for rr, p in ((0, a["npoints"] // 2), (9, 123), (5, b0)):
            ref = orc.image_for_point(rr, p)
            for precision in ("fp64", "split"):
                g = dev.image_for_point(rr, p, precision)
                assert g["u_ray"].shape == ref["u_ray"].shape, (rr, p)
                for k in ("S_ray", "dtau_ray", "u_ray"):
                    # split precision's single-precision sources underflow far in the line wings
                    floor = 1e-300 if precision == "fp64" else 1e-10 * np.abs(ref[k]).max()
                    kt = 1e-5 if (precision == "fp64" or k == "u_ray") else 1e-4
                    assert H.max_rel(g[k], ref[k], floor=floor) < kt, (rr, p, precision, k)
    finally:
        dev.close()


def test_set_column_matches_oracle_bit_exact(gpu_lib):
    """set_column (solver.tpp:2953-2991): the same walk and the same FP64 roundings, so
    every column equals the oracle's bit for bit."""
    raw = S.grid_sphere(n=16, nside=1, nquads=7)
    a = H.setup(raw)
    rho = np.random.default_rng(2).uniform(1e6, 1e8, a["npoints"])
    ref = O.Oracle(a).set_column(rho)
    dev = _abi.DeviceModel(a)
    try:
        np.testing.assert_array_equal(dev.set_column(rho), ref)
    finally:
        dev.close()


def test_core_model_image_for_point_and_column(gpu_lib):
    """The drop-in calls: core.Model.compute_image_for_point fills S_ray / dtau_ray /
    u_ray, set_column fills column from density."""
    from magritte_gb300 import loader

    raw = H.all_constant_model()
    model = loader.to_core(raw, precision="fp64")
    model.compute_spectral_discretisation()
    model.compute_inverse_line_widths()
    model.compute_LTE_level_populations()
    model.compute_image_for_point(0, 17)
    u = np.array(model.u_ray)[:, 0]
    if raw.ray_direction[0][0] > 0:
        u = u[::-1]
    assert np.max(np.abs(H.relative_error(H.all_constant_solution(raw), u))) < 1.7e-4
    assert np.array(model.S_ray).shape == np.array(model.dtau_ray).shape == (raw.npoints, 1)
    model.density.set(np.ones(raw.npoints))
    model.set_column()
    col = np.array(model.column)
    x = raw.position[:, 0]
    for r in range(raw.nrays):
        expect = (x[-1] - x) if raw.ray_direction[r][0] > 0 else (x - x[0])
        np.testing.assert_allclose(col[r], expect, rtol=1e-14, atol=1e-3)
