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
