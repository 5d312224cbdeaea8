"""Shared helpers for the test-suite: the reference's analytic benchmark solutions
(restated from magritte/tools.py:69-257 and the benchmark scripts) and model
builders that run the oracle's set-up."""
import numpy as np

from magritte_gb300 import synthetic as S
import oracle as O

KB, HH, CC, AMU = S.KB, S.HH, S.CC, S.AMU


def relative_error(a, b):
    """magritte/tools.py:69-73."""
    return 2.0 * (a - b) / (a + b)


def planck(T, nu):
    return 2.0 * HH / CC**2 * nu**3 / np.expm1(HH * nu / (KB * T))


def all_constant_model():
    """tests/benchmarks/analytic/all_constant_single_ray.py:17-67."""
    return S.single_ray_1d(npoints=50, dx=1.0e12, nTT=1.0e3, nH2=1.0e12, temp=4.5, turb=0.0, dv=0.0, nquads=1)


def all_constant_solution(raw):
    """all_constant_single_ray.py:121-131: u = (I_0 + I_1)/2 with I = S + (I_bdy - S) e^{-chi x}."""
    ld = raw.linedata[0]
    temp, nTT = raw.temperature[0], raw.abundance[0, 0]
    frq = ld.frequency[0]
    pop = ld.weight * np.exp(-ld.energy / (KB * temp))
    pop = pop / pop.sum() * nTT
    width = frq * np.sqrt(2.0 * KB * temp / (AMU * CC**2) * ld.inverse_mass + raw.vturb2[0])
    phi = 1.0 / (width * np.sqrt(np.pi))
    em = HH * frq / (4.0 * np.pi) * ld.A[0] * pop[1]
    op = HH * frq / (4.0 * np.pi) * (ld.Ba[0] * pop[0] - ld.Bs[0] * pop[1])
    chi = op * phi
    src = em / op
    bdy = planck(S.T_CMB, frq)
    x = raw.position[:, 0]
    I0 = src + (bdy - src) * np.exp(-chi * x)
    I1 = src + (bdy - src) * np.exp(-chi * (x[-1] - x))
    return 0.5 * (I0 + I1)


def all_constant_intensities(raw):
    """all_constant_single_ray.py:121-136: the two directions' intensities I_0, I_1."""
    u = all_constant_solution(raw)
    ld = raw.linedata[0]
    temp, nTT = raw.temperature[0], raw.abundance[0, 0]
    frq = ld.frequency[0]
    pop = ld.weight * np.exp(-ld.energy / (KB * temp))
    pop = pop / pop.sum() * nTT
    width = frq * np.sqrt(2.0 * KB * temp / (AMU * CC**2) * ld.inverse_mass + raw.vturb2[0])
    phi = 1.0 / (width * np.sqrt(np.pi))
    em = HH * frq / (4.0 * np.pi) * ld.A[0] * pop[1]
    op = HH * frq / (4.0 * np.pi) * (ld.Ba[0] * pop[0] - ld.Bs[0] * pop[1])
    chi = op * phi
    src = em / op
    bdy = planck(S.T_CMB, frq)
    x = raw.position[:, 0]
    return src + (bdy - src) * np.exp(-chi * x), src + (bdy - src) * np.exp(-chi * (x[-1] - x))


def all_zero_model():
    """tests/benchmarks/analytic/all_zero_single_ray.py:20-78 (velocity 0 up to the
    middle point, then rising by 150 m/s per point)."""
    raw = S.single_ray_1d(npoints=50, dx=1.0e12, nTT=0.0, nH2=0.0, temp=4.5, turb=0.0, nquads=1)
    dv = 150.0 / CC
    raw.velocity[:, 0] = [0.0 if i <= 25 else (i - 25) * dv for i in range(50)]
    return raw


def all_zero_solution(raw):
    """all_zero_single_ray.py:136-152: boundary intensities Doppler shifted to each point."""
    frq = raw.linedata[0].frequency[0]
    v = raw.velocity[:, 0]
    return 0.5 * (planck(S.T_CMB, frq * (1 - v)) + planck(S.T_CMB, frq * (1 + v)))


def setup(raw, **kw):
    return O.reference_setup(raw, **kw)


def max_rel(a, b, floor=0.0):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.maximum(np.abs(b), floor)
    return float(np.max(np.abs(a - b) / np.where(den > 0, den, 1.0)))


def _line_constants(ld, temp, nTT, vturb2):
    """LTE populations scaled by nTT and the first line's opacity, source and width
    (magritte/tools.py:76-230)."""
    pop = ld.weight * np.exp(-ld.energy / (KB * temp))
    pop = pop / pop.sum() * nTT
    i, j = ld.irad[0], ld.jrad[0]
    frq = ld.frequency[0]
    em = HH * frq / (4.0 * np.pi) * ld.A[0] * pop[i]
    op = HH * frq / (4.0 * np.pi) * (ld.Ba[0] * pop[j] - ld.Bs[0] * pop[i])
    dnu = frq * np.sqrt(2.0 * KB * temp / (AMU * CC**2) * ld.inverse_mass + vturb2)
    return frq, op, em / op, dnu


def density_distribution_1d_solution(raw, nu, angles, kind="a"):
    """u [angle][point][freq] of tests/benchmarks/analytic/density_distribution_1D.py:126-178:
    optical depths of the r^-2 opacity along a ray at angle theta from the radial
    direction, to the inner core (theta < asin(r_in/r)) or to the outer edge."""
    r_in, r_out, nH2_in = 1.0e13, 7.8e16, 2.0e13
    X_mol = {"a": 1.0e-8, "b": 1.0e-6}[kind]
    ld = raw.linedata[0]
    frq, chi, src, dnu = _line_constants(ld, 20.0, X_mol * nH2_in, (150.0 / CC) ** 2)
    rs = raw.position[:, 0]

    def phi(f):
        x = (f - frq) / dnu
        return np.exp(-x**2) / (np.sqrt(np.pi) * dnu)

    def tau(f, r, theta):
        pref = chi * phi(f) * r_in**2
        if theta == 0.0:
            return pref * (1.0 / r_in - 1.0 / r)
        if theta == np.pi:
            return pref * (1.0 / r - 1.0 / r_out)
        if theta < np.arcsin(r_in / r):
            closest = r * np.sin(theta)
            in_vertical = np.sqrt(r_in**2 - closest**2)
            out_vertical = np.sqrt(r**2 - closest**2)
            return pref * (np.arctan(out_vertical / closest) - np.arctan(in_vertical / closest)) / closest
        factor = np.arccos(r * np.sin(theta) / r_out) + 0.5 * np.pi - theta
        return pref / (r * np.sin(theta)) * factor

    def I_(f, r, theta):
        return src + (planck(S.T_CMB, f) - src) * np.exp(-tau(f, r, theta))

    return np.array([[[0.5 * (I_(f, r, a) + I_(f, r, np.pi + a)) for f in nu] for r in rs] for a in angles])


def velocity_gradient_1d_solution(raw, nu, angles):
    """u [angle][point][freq] of tests/benchmarks/analytic/constant_velocity_gradient_1D.py:127-187:
    the erf optical depth of a linear velocity field along the ray to the inner or outer
    boundary, with the boundary's CMB seen at its Doppler-shifted frequency."""
    from scipy.special import erf

    npoints = raw.npoints
    dx, dv = 1.0e4, 2.5e2 / CC
    L, vmax = dx * npoints, dv * npoints
    ld = raw.linedata[0]
    frq, chi, src, dnu = _line_constants(ld, 45.0, 1.0e8, 0.0)
    rs = raw.position[:, 0]
    r_in, r_out = rs[0], rs[-1]

    def v_(r):
        return dv * (1 + (r - r_in) / dx)

    def bdy(f, r, theta):
        r_shift = np.cos(theta) * v_(r)
        if theta < np.arcsin(r_in / r):
            edge = np.sqrt(1 - ((r / r_in) * np.abs(np.sin(theta))) ** 2) * v_(r_in)
        else:
            edge = np.sqrt(1 - ((r / r_out) * np.abs(np.sin(theta))) ** 2) * v_(r_out)
        return planck(S.T_CMB, f * (1.0 + (edge - r_shift)))

    def z_max(r, theta):
        if theta < np.arcsin(r_in / r):
            return r * np.cos(theta) - np.sqrt(r_in**2 - (r * np.sin(theta)) ** 2)
        return r * np.cos(theta) + np.sqrt(L**2 - (r * np.sin(theta)) ** 2)

    def tau(f, r, theta):
        l = float(z_max(r, theta))
        arg = float((f - frq) / dnu)
        fct = float(vmax * f / dnu)
        return chi * L / (fct * dnu) * 0.5 * (erf(-arg) + erf(fct * l / L + arg))

    def I_(f, r, theta):
        return src + (bdy(f, r, theta) - src) * np.exp(-tau(f, r, theta))

    return np.array([[[0.5 * (I_(f, r, a) + I_(f, r, np.pi + a)) for f in nu] for r in rs] for a in angles])


def ray_angles(raw):
    """The first hnrays rays' angles arctan2(y, x), as the 1D benchmarks take them."""
    d = raw.ray_direction[: raw.nrays // 2]
    return np.arctan2(d[:, 1], d[:, 0])


def velocity_gradient_1d_image_solution(raw, nu, imx, imy):
    """I [pixel][freq] of tests/benchmarks/analytic/constant_velocity_gradient_1D_new_imager.py:117-165:
    the image along +y of the 1D velocity gradient, at impact parameter r = |(x, y)|, the
    frequency measured from the outer edge's Doppler shift."""
    from scipy.special import erf

    npoints = raw.npoints
    dx, dv = 1.0e4, 2.5e2 / CC
    L, vmax = dx * npoints, dv * npoints
    ld = raw.linedata[0]
    frq, chi, src, dnu = _line_constants(ld, 45.0, 1.0e8, 0.0)
    r_in, r_out = raw.position[0, 0], raw.position[-1, 0]

    def z_max(r, theta):
        if r >= r_out:
            return 0.0
        if theta < np.arcsin(r_in / r):
            return r * np.cos(theta) - np.sqrt(r_in**2 - (r * np.sin(theta)) ** 2)
        return r * np.cos(theta) + np.sqrt(L**2 - (r * np.sin(theta)) ** 2)

    def tau(f, r, theta):
        l = float(z_max(r, theta))
        arg = float((f - frq) / dnu)
        fct = float(vmax * f / dnu)
        up = chi * L / (fct * dnu) * 0.5 * (erf(arg) - erf(arg - fct * l / L))
        down = chi * L / (-fct * dnu) * 0.5 * (erf(arg) - erf(arg + fct * l / L))
        return up + down

    def I_im(f, r):
        f = f + vmax / CC * frq
        return src + (planck(S.T_CMB, f) - src) * np.exp(-tau(f, r, 0.5 * np.pi))

    rs = np.sqrt(imx**2 + imy**2)
    return np.array([[I_im(f, r) for f in nu] for r in rs])


def band_alo_error(alo_off, alo_nr, lam, ref):
    """Largest difference between the non-local ALO of a banded solve in the library's
    layout (alo_off / alo_nr [P][L][hnrays][2K] and the diagonal lam [P][L]) and the
    oracle's Lambda lists (``Oracle.formal_solve_fo2_alo``: per (point, line) the
    elements merged by point, Lambda::add_element), relative to the largest element of
    each list.  Elements are compared per (point, line, element point) after summing
    the library's slots that name the same point."""
    P, L = lam.shape
    worst = 0.0
    for p in range(P):
        for l in range(L):
            mine = {p: lam[p, l]}
            for v, q in zip(alo_off[p, l].ravel(), alo_nr[p, l].ravel()):
                if v != 0.0:
                    mine[int(q)] = mine.get(int(q), 0.0) + v
            n = int(ref["alo_n"][p, l])
            theirs = {int(ref["alo_nr"][p, l, i]): ref["alo_ls"][p, l, i] for i in range(n)}
            scale = max([abs(v) for v in theirs.values()] + [1e-300])
            for q in set(mine) | set(theirs):
                worst = max(worst, abs(mine.get(q, 0.0) - theirs.get(q, 0.0)) / scale)
    return worst
