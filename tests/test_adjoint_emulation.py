"""The differentiable new imager's lane code (libmgr_emu.so: image_lane_s and
image_lane_adj compiled for the host) on CPU.

Forward: the smooth image (FP64 pow / exp / expm1 / erf in place of the reference's
single-precision calls) against the oracle's new imager in its smooth mode.
Backward: the hand-written adjoint against FP64 central finite differences
(Richardson-extrapolated) of the oracle's smooth image, for emissivity, opacity, inverse width (total derivatives:
the line source em / op moves with em and op) and velocity, at sampled points with
the largest and at random non-zero derivatives.  Bar: 1e-4 relative."""
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
    lib.mgr_emu_image_new_smooth.argtypes = [C.POINTER(_abi.MgrModelDesc), _f64p, C.c_uint32, C.c_uint32, _f64p]
    lib.mgr_emu_image_new_smooth.restype = C.c_int
    lib.mgr_emu_image_new_adjoint.argtypes = [C.POINTER(_abi.MgrModelDesc), _f64p, C.c_uint32, C.c_uint32, _f64p,
                                              _f64p, _f64p, _f64p, _f64p, _f64p]
    lib.mgr_emu_image_new_adjoint.restype = C.c_int
    return lib


@pytest.fixture(scope="module", autouse=True)
def _smooth_oracle():
    O.set_smooth(1)
    yield
    O.set_smooth(0)


def shells_model(approx="CloseLines"):
    raw = S.velocity_gradient_shells(nshells=6)
    fcen = raw.linedata[0].frequency[0]
    dd = 1.0e4 / 2.99792458e8
    return H.setup(raw, approx=approx, max_width_fraction=0.5,
                   image_freqs=(fcen - fcen * dd, fcen + fcen * dd, 9))


def sphere_model(approx="CloseLines"):
    raw = S.grid_sphere(n=12, nside=1, nquads=5)
    lines = raw.linedata[0].frequency
    f0 = lines[1]
    dd = 8.0e3 / 2.99792458e8
    return H.setup(raw, approx=approx, image_freqs=(f0 * (1 - dd), f0 * (1 + dd), 7))


MODELS = {"shells": shells_model, "sphere": sphere_model}
DIRS = {"axis": np.array([0.0, 0.0, 1.0]), "oblique": np.array([0.3, -0.5, 0.81])}


def emu_image(emu, a, d, nx, ny):
    desc, keep = _abi.make_desc(a)
    I = np.zeros((nx * ny, a["nfreqs"]))
    dd = np.ascontiguousarray(d, np.float64)
    assert emu.mgr_emu_image_new_smooth(C.byref(desc), _p(dd), nx, ny, _p(I)) == 0
    return I


def emu_adjoint(emu, a, d, nx, ny, gI):
    desc, keep = _abi.make_desc(a)
    P, L = a["npoints"], a["nlines"]
    g = {k: np.zeros((P, L)) for k in ("em", "op", "iw", "Sp")}
    g["vel"] = np.zeros((P, 3))
    dd = np.ascontiguousarray(d, np.float64)
    gI = np.ascontiguousarray(gI, np.float64)
    assert emu.mgr_emu_image_new_adjoint(C.byref(desc), _p(dd), nx, ny, _p(gI), _p(g["em"]), _p(g["op"]),
                                         _p(g["iw"]), _p(g["Sp"]), _p(g["vel"])) == 0
    return g


def oracle_loss(a, d, nx, ny, w):
    return float(np.sum(w * O.Oracle(a).image_new(d, nx, ny)["I"]))


@pytest.mark.parametrize("model", sorted(MODELS))
@pytest.mark.parametrize("direction", sorted(DIRS))
@pytest.mark.parametrize("approx", ["CloseLines", "None"])
def test_smooth_forward_matches_smooth_oracle(emu, model, direction, approx):
    a = MODELS[model](approx)
    d = DIRS[direction]
    ref = O.Oracle(a).image_new(d, 12, 10)["I"]
    got = emu_image(emu, a, d, 12, 10)
    assert H.max_rel(got, ref, floor=1e-12 * np.abs(ref).max()) < 1e-10


def _sample(gtot, rng, k_top=6, k_rand=6):
    flat = np.abs(gtot).ravel()
    # entries within 1e-2 of the largest: below that, the differences of a loss summed
    # over the whole image cannot resolve 1e-4 in double precision
    nz = np.nonzero(flat > 1e-2 * flat.max())[0]
    top = nz[np.argsort(flat[nz])[-k_top:]]
    rnd = rng.choice(nz, size=min(k_rand, len(nz)), replace=False)
    return np.unique(np.concatenate([top, rnd]))


@pytest.mark.parametrize("model", sorted(MODELS))
@pytest.mark.parametrize("direction", sorted(DIRS))
def test_adjoint_matches_oracle_finite_differences(emu, model, direction):
    a = MODELS[model]("CloseLines")
    d = DIRS[direction]
    nx, ny = 10, 8
    rng = np.random.default_rng(7)
    w = rng.normal(size=(nx * ny, a["nfreqs"]))
    g = emu_adjoint(emu, a, d, nx, ny, w)
    em, op = a["emissivity"], a["opacity"]
    total = {"emissivity": g["em"] + g["Sp"] / op, "opacity": g["op"] - g["Sp"] * em / op ** 2,
             "inverse_width": g["iw"], "velocity": g["vel"]}
    checked = 0
    for key, gt in total.items():
        for idx in _sample(gt, rng):
            arr = a[key]
            flat = arr.reshape(-1)
            x0 = flat[idx]
            # Richardson-extrapolated central differences (steps h and h/2, error
            # O(h^4)): steps large enough that the loss's rounding stays far below
            # the differences, 1e-3 relative for the line data and 1e-4 of the
            # largest speed for velocities
            h = 1e-3 * abs(x0) if key != "velocity" else 1e-4 * np.abs(arr).max()

            def central(step):
                flat[idx] = x0 + step
                lp = oracle_loss(a, d, nx, ny, w)
                flat[idx] = x0 - step
                lm = oracle_loss(a, d, nx, ny, w)
                flat[idx] = x0
                return (lp - lm) / (2 * step)

            fd = (4.0 * central(h / 2) - central(h)) / 3.0
            an = gt.reshape(-1)[idx]
            # 1e-4 relative, above the differences' own noise floor (1e-7 of the largest)
            assert abs(an - fd) <= 1e-4 * abs(fd) + 1e-7 * np.abs(gt).max(), (key, idx, an, fd)
            checked += 1
    assert checked >= 20
