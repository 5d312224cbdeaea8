"""The differentiable formal solve's lane code (libmgr_emu.so: solve_lane_s and
solve_lane_s_adj compiled for the host) on CPU.

Forward: the smooth J (FP64 pow / exp / expm1 / erf in place of the reference's
single-precision calls) against the oracle's formal solve in its smooth mode.
Backward: the hand-written adjoint of loss = sum(w * J) against FP64 central finite
differences (Richardson-extrapolated) of the oracle's smooth J, for emissivity,
opacity, inverse width (total derivatives: the line source em / op moves with em and
op), velocity and the frequencies nu, at sampled entries with the largest and at
random non-zero derivatives.  Bar: 1e-4 relative."""
import ctypes as C

import numpy as np
import pytest

import helpers as H
import oracle as O
from magritte_gb300 import _abi, build
from magritte_gb300 import synthetic as S

_f64p = C.POINTER(C.c_double)


def _p(x):
    return x.ctypes.data_as(_f64p)


@pytest.fixture(scope="module")
def emu():
    lib = C.CDLL(build.build_emu())
    lib.mgr_emu_fo2_smooth.argtypes = [C.POINTER(_abi.MgrModelDesc), _f64p]
    lib.mgr_emu_fo2_smooth.restype = C.c_int
    lib.mgr_emu_fo2_adjoint.argtypes = [C.POINTER(_abi.MgrModelDesc)] + [_f64p] * 7
    lib.mgr_emu_fo2_adjoint.restype = C.c_int
    return lib


@pytest.fixture(scope="module", autouse=True)
def _smooth_oracle():
    O.set_smooth(1)
    yield
    O.set_smooth(0)


def sphere_model(approx="CloseLines"):
    # 10^3 cutout: rays of uneven length, 4 lines with Doppler-shifted overlaps
    return H.setup(S.grid_sphere(n=10, nside=1, nquads=5), approx=approx)


def cube_model(approx="CloseLines"):
    # random velocities: many large-shift (line-integrated) pairs
    return H.setup(S.grid_cube(n=6, nquads=7), approx=approx)


MODELS = {"sphere": sphere_model, "cube": cube_model}


def emu_J(emu, a):
    desc, keep = _abi.make_desc(a)
    J = np.zeros((a["npoints"], a["nfreqs"]))
    assert emu.mgr_emu_fo2_smooth(C.byref(desc), _p(J)) == 0
    return J


def emu_adjoint(emu, a, gJ):
    desc, keep = _abi.make_desc(a)
    P, L, F = a["npoints"], a["nlines"], a["nfreqs"]
    g = {k: np.zeros((P, L)) for k in ("em", "op", "iw", "Sp")}
    g["vel"] = np.zeros((P, 3))
    g["nu"] = np.zeros((P, F))
    gJ = np.ascontiguousarray(gJ, np.float64)
    assert emu.mgr_emu_fo2_adjoint(C.byref(desc), _p(gJ), _p(g["em"]), _p(g["op"]), _p(g["iw"]), _p(g["Sp"]),
                                   _p(g["vel"]), _p(g["nu"])) == 0
    return g


def oracle_loss(a, w):
    return float(np.sum(w * O.Oracle(a).formal_solve_fo2()["J"]))


@pytest.mark.parametrize("model", sorted(MODELS))
@pytest.mark.parametrize("approx", ["CloseLines", "None"])
def test_smooth_forward_matches_smooth_oracle(emu, model, approx):
    a = MODELS[model](approx)
    ref = O.Oracle(a).formal_solve_fo2()["J"]
    got = emu_J(emu, a)
    assert H.max_rel(got, ref) < 1e-10


def _sample(gtot, rng, k_top=5, k_rand=5):
    flat = np.abs(gtot).ravel()
    # entries within 1e-2 of the largest: below that the differences of a loss summed
    # over every origin cannot resolve 1e-4 in double precision
    nz = np.nonzero(flat > 1e-2 * flat.max())[0]
    top = nz[np.argsort(flat[nz])[-k_top:]]
    rnd = rng.choice(nz, size=min(k_rand, len(nz)), replace=False)
    return np.unique(np.concatenate([top, rnd]))


@pytest.mark.parametrize("model", sorted(MODELS))
def test_adjoint_matches_oracle_finite_differences(emu, model):
    a = MODELS[model]("CloseLines")
    rng = np.random.default_rng(11)
    w = rng.normal(size=(a["npoints"], a["nfreqs"]))
    g = emu_adjoint(emu, a, w)
    em, op = a["emissivity"], a["opacity"]
    total = {"emissivity": g["em"] + g["Sp"] / op, "opacity": g["op"] - g["Sp"] * em / op ** 2,
             "inverse_width": g["iw"], "velocity": g["vel"], "nu": g["nu"]}
    checked, skipped = 0, 0
    for key, gt in total.items():
        for idx in _sample(gt, rng):
            arr = a[key]
            flat = arr.reshape(-1)
            x0 = flat[idx]
            if key == "velocity":
                h = 1e-4 * np.abs(arr).max()
            elif key == "nu":
                # a step of 1e-3 of the local line width
                p = idx // a["nfreqs"]
                h = 1e-3 / a["inverse_width"][p].max()
            else:
                h = 1e-3 * abs(x0)

            def central(step):
                flat[idx] = x0 + step
                lp = oracle_loss(a, w)
                flat[idx] = x0 - step
                lm = oracle_loss(a, w)
                flat[idx] = x0
                return (lp - lm) / (2 * step)

            c1, c2 = central(h), central(h / 2)
            if abs(c1 - c2) > 1e-2 * abs(c2) + 1e-6 * np.abs(gt).max():
                # the steps disagree: the perturbation crossed a branch of the held
                # structure (large-shift test, line bracket); not a derivative check
                skipped += 1
                continue
            fd = (4.0 * c2 - c1) / 3.0
            an = gt.reshape(-1)[idx]
            assert abs(an - fd) <= 1e-4 * abs(fd) + 1e-7 * np.abs(gt).max(), (key, idx, an, fd)
            checked += 1
    assert checked >= 30 and skipped <= 5, (checked, skipped)
