"""Pins the oracle's imagers.

* New imager: the reference's constant-velocity-gradient 3D benchmark
  (tests/benchmarks/analytic/constant_velocity_gradient_3D_new_imager.py): a
  50 x 50 image along ray hnrays-1 of the HEALPix-shell model with radial velocity
  gradient must agree with the analytic intensity within the benchmark's own bound,
  1.5e-3 relative (:247).  The analytic solution restates the benchmark's formula
  and the magritte/tools.py helpers it calls (:69-227).
(The reference pins its old imager only in 1D, spherically symmetric benchmarks,
which are outside this library's scope.)"""
import numpy as np
import pytest
from scipy.special import erf

import helpers as H
import oracle as O
from magritte_gb300 import synthetic as S

C_LIGHT, HH, KB, AMU, T_CMB = 2.99792458e8, 6.62607004e-34, 1.38064852e-23, 1.66053904e-27, 2.72548


@pytest.fixture(scope="module", autouse=True)
def built():
    O.build()


def _planck(T, nu):
    return 2.0 * HH / C_LIGHT**2 * nu**3 / np.expm1(HH * nu / (KB * T))


def test_new_imager_constant_velocity_gradient_3d():
    nshells, dx, dv, temp, nTT = 10, 1.0e4, 2.5e2 / C_LIGHT, 45.0, 1.0e8
    raw = S.velocity_gradient_shells(nshells=nshells)
    ld = raw.linedata[0]
    fcen = ld.frequency[0]
    dd = 1.0e4 / C_LIGHT
    a = O.reference_setup(raw, max_width_fraction=0.5, image_freqs=(fcen - fcen * dd, fcen + fcen * dd, 10))
    ray_nr = raw.nrays // 2 - 1
    img = O.Oracle(a).image_new(raw.ray_direction[ray_nr], 50, 50)
    im, imx, imy = img["I"], img["ImX"], img["ImY"]
    nu = a["nu"][0]
    rs = np.sqrt(imx**2 + imy**2)

    L, vmax = dx * nshells, dv * nshells
    pop = ld.weight * np.exp(-ld.energy / (KB * temp))
    pop = pop / pop.sum() * nTT
    i, j = ld.irad[0], ld.jrad[0]
    eta = HH * fcen / (4.0 * np.pi) * ld.A[0] * pop[i]
    chi = HH * fcen / (4.0 * np.pi) * (ld.Ba[0] * pop[j] - ld.Bs[0] * pop[i])
    src = eta / chi
    dnu = fcen * np.sqrt(2.0 * KB * temp / (AMU * C_LIGHT**2) * ld.inverse_mass + 0.0)
    r_in = np.linalg.norm(raw.position[0])
    r_out = np.linalg.norm(raw.position[-1])

    def z_max(r, theta):
        if r >= r_out:
            return 0.0
        if theta < np.arcsin(r_in / r):
            return r * np.cos(theta) - np.sqrt(r_in**2 - (r * np.sin(theta)) ** 2)
        return r * np.cos(theta) + np.sqrt(L**2 - (r * np.sin(theta)) ** 2)

    def tau(f, r, theta):
        l = float(z_max(r, theta))
        arg = float((f - fcen) / dnu)
        fct = float(vmax * f / dnu)
        up = chi * L / (fct * dnu) * 0.5 * (erf(arg) - erf(arg - fct * l / L))
        down = chi * L / (-fct * dnu) * 0.5 * (erf(arg) - erf(arg + fct * l / L))
        return up + down

    def I_im(f, r):
        f = f + vmax / C_LIGHT * fcen
        return src + (_planck(T_CMB, f) - src) * np.exp(-tau(f, r, 0.5 * np.pi))

    im_a = np.array([[I_im(f, r) for f in nu] for r in rs])
    err = np.abs(2.0 * (im - im_a) / (im + im_a))[:-1]
    assert np.isfinite(im).all()
    assert err.max() < 1.5e-3, err.max()


def test_optical_depth_image_all_constant_known_answer():
    """Optical-depth images (Solver::image_optical_depth, solver.tpp:655-684, 2718-2760)
    of the all-constant single ray: along the ray the optical depth is chi times the
    ray's length, for every model point (each point's ray spans the whole line)."""
    raw = H.all_constant_model()
    a = H.setup(raw)
    tau = O.Oracle(a).image_optical_depth(0)
    ld = raw.linedata[0]
    temp, nTT = raw.temperature[0], raw.abundance[0, 0]
    frq = ld.frequency[0]
    pop = ld.weight * np.exp(-ld.energy / (H.KB * temp))
    pop = pop / pop.sum() * nTT
    width = frq * np.sqrt(2.0 * H.KB * temp / (H.AMU * H.CC**2) * ld.inverse_mass + raw.vturb2[0])
    phi = 1.0 / (width * np.sqrt(np.pi))
    op = H.HH * frq / (4.0 * np.pi) * (ld.Ba[0] * pop[0] - ld.Bs[0] * pop[1])
    length = raw.position[-1, 0] - raw.position[0, 0]
    expect = (op * phi + a["min_opacity"]) * length
    assert np.max(np.abs(tau - expect) / expect) < 1e-5


def test_optical_depth_new_image_sums_the_imager_pairs():
    """The new optical-depth imager traces the same pixel rays as the new imager: a
    model without emission still has a positive optical depth where a pixel ray
    crosses the model and zero where it only touches a boundary point."""
    raw = S.velocity_gradient_shells(nshells=6)
    fcen = raw.linedata[0].frequency[0]
    dd = 1.0e4 / 2.99792458e8
    a = H.setup(raw, max_width_fraction=0.5, image_freqs=(fcen - fcen * dd, fcen + fcen * dd, 9))
    d = raw.ray_direction[raw.nrays // 2 - 1]
    orc = O.Oracle(a)
    t = orc.image_optical_depth_new(d, 20, 20)
    img = orc.image_new(d, 20, 20)
    np.testing.assert_array_equal(t["ImX"], img["ImX"])
    assert np.all(t["I"] >= 0.0)
    assert (t["I"] > 0.0).any()


def test_image_for_point_all_constant_known_answer(built):
    """image_feautrier_order_2_for_point (solver.tpp:629-653, :2582-2715) on the
    all-constant single ray (all_constant_single_ray.py:121-131): the ray through any
    point is the whole line, so u_ray holds the analytic u at every point (the
    reference's formal-solve bound 1.7e-4), S_ray the constant source em/op and dtau_ray
    chi dx."""
    raw = H.all_constant_model()
    a = H.setup(raw)
    orc = O.Oracle(a)
    u_ref = H.all_constant_solution(raw)
    x = raw.position[:, 0]
    for p in (0, 17, raw.npoints - 1):
        r = orc.image_for_point(0, p)
        assert r["u_ray"].shape == (raw.npoints, a["nfreqs"])
        u = r["u_ray"][:, 0]
        # rows run from the far end of ray 0's backward half to the far end of its antipode
        if raw.ray_direction[0][0] > 0:
            u = u[::-1]
        assert np.max(np.abs(H.relative_error(u_ref, u))) < 1.7e-4
        S_row = r["S_ray"][:, 0]
        assert np.max(np.abs(S_row / S_row[0] - 1.0)) < 1e-6
        dt = r["dtau_ray"][1:, 0]
        assert r["dtau_ray"][0, 0] == 0.0 and np.max(np.abs(dt / dt[0] - 1.0)) < 1e-5
    # the old imager's pixel is 2 u[last] - I_bdy of the same elimination
    img = orc.image_fo2(0)
    r = orc.image_for_point(0, 17)
    ibdy = 2.0 * r["u_ray"][-1] - img[17]
    assert np.all(ibdy > 0) and np.max(np.abs(ibdy / ibdy[0] - 1.0)) < 1e-3


def test_set_column_known_answers(built):
    """set_column / get_column (solver.tpp:2953-2991): on the single ray a unit density
    gives each point's distance to the line's end in the ray's direction; a linear
    density profile is integrated exactly by the trapezoid rule; columns are linear in
    the density."""
    raw = H.all_constant_model()
    a = H.setup(raw)
    orc = O.Oracle(a)
    x = raw.position[:, 0]
    P = raw.npoints
    col = orc.set_column(np.ones(P))
    for r in range(raw.nrays):
        if raw.ray_direction[r][0] > 0:
            np.testing.assert_allclose(col[r], x[-1] - x, rtol=1e-14, atol=1e-3)
        else:
            np.testing.assert_allclose(col[r], x - x[0], rtol=1e-14, atol=1e-3)
    rho = 1.0 + x / x[-1]
    colr = orc.set_column(rho)
    r_plus = [r for r in range(raw.nrays) if raw.ray_direction[r][0] > 0][0]
    exact = (x[-1] - x) + (x[-1] ** 2 - x ** 2) / (2.0 * x[-1])
    np.testing.assert_allclose(colr[r_plus], exact, rtol=1e-12, atol=1e-3)
    # linearity on a 3D model
    a3 = H.setup(S.grid_sphere(n=10, nside=1, nquads=5))
    o3 = O.Oracle(a3)
    rng = np.random.default_rng(5)
    r1, r2 = rng.uniform(1, 2, a3["npoints"]), rng.uniform(1, 2, a3["npoints"])
    c1, c2, c12 = o3.set_column(r1), o3.set_column(r2), o3.set_column(2.0 * r1 + 3.0 * r2)
    np.testing.assert_allclose(c12, 2.0 * c1 + 3.0 * c2, rtol=1e-12, atol=0)


@pytest.mark.parametrize("mwf, bound", [(0.5, 1.6e-5), (0.35, 1.2e-5), (0.10, 3.3e-7)])
def test_new_imager_constant_velocity_gradient_1d(mwf, bound):
    """tests/benchmarks/analytic/constant_velocity_gradient_1D_new_imager.py:86-165, 220-226:
    the projection-plane imager on the 1D spherically symmetric velocity gradient (50
    shells, 4 rays, image along ray hnrays-1 = +y, 50 x 50 pixels, 10 frequencies over
    +-10 km/s): max relative error against the closed form below the reference's bound
    for each max_width_fraction setting (all pixels but the last)."""
    raw = S.velocity_gradient_1d(npoints=50, nrays=4, nquads=10)
    fcen = raw.linedata[0].frequency[0]
    dd = 1.0e4 / H.CC
    a = H.setup(raw, max_width_fraction=mwf, image_freqs=(fcen - fcen * dd, fcen + fcen * dd, 10))
    d = raw.ray_direction[raw.nrays // 2 - 1]
    r = O.Oracle(a).image_new(d, 50, 50)
    ana = H.velocity_gradient_1d_image_solution(raw, a["nu"][0], r["ImX"], r["ImY"])
    assert np.max(np.abs(H.relative_error(r["I"], ana))[:-1]) < bound
