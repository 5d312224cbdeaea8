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
