"""The formal-solve kernel's per-lane code, compiled for the host, against the oracle.

libmgr_emu.so runs the same solve_lane/lambda_element source the GPU kernel runs
(with a sequential trace), so these CPU tests check the kernel's arithmetic,
branch structure and two-sided elimination without a GPU.  In FP64 mode the only
differences to the oracle are the order of the elimination (machine precision);
split precision stays within the 1e-5 bar."""
import ctypes as C

import numpy as np
import pytest

import helpers as H
import oracle as O
from magritte_gb300 import _abi, build
from magritte_gb300 import synthetic as S


@pytest.fixture(scope="module", autouse=True)
def _oracle_with_correctly_rounded_erf():
    O.set_erf_mode(1)
    yield
    O.set_erf_mode(0)


@pytest.fixture(scope="module")
def emu():
    lib = C.CDLL(build.build_emu())
    lib.mgr_emu_formal_solve_fo2.argtypes = [C.POINTER(_abi.MgrModelDesc), C.c_int, C.POINTER(C.c_double),
                                             C.POINTER(C.c_double)]
    lib.mgr_emu_formal_solve_fo2.restype = C.c_int
    return lib


def run(emu, a, precision):
    desc, keep = _abi.make_desc(a)
    J = np.zeros((a["npoints"], a["nfreqs"]))
    lam = np.zeros((a["npoints"], a["nlines"]))
    rc = emu.mgr_emu_formal_solve_fo2(C.byref(desc), _abi.PRECISION[precision],
                                      J.ctypes.data_as(C.POINTER(C.c_double)),
                                      lam.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 0
    return J, lam


MODELS = {
    "cube10": lambda: S.grid_cube(n=10, nquads=5),
    "cube12_seed3": lambda: S.grid_cube(n=12, nquads=7, seed=3),
    "sphere14": lambda: S.grid_sphere(n=14, nside=1, nquads=5),
    "sphere16": lambda: S.grid_sphere(n=16, nside=1, nquads=7),
    "all_constant": H.all_constant_model,
    "all_zero": H.all_zero_model,
    # 1D spherical symmetry (shell walk, Z-dependent shifts)
    "sph_density": lambda: S.density_distribution_1d("a", npoints=60, nrays=20, nquads=11),
    "sph_velocity": lambda: S.velocity_gradient_1d(npoints=40, nrays=20, nquads=21),
    # adaptive (per-point) ray directions and weights
    "cube10_adaptive": lambda: S.with_adaptive_rays(S.grid_cube(n=10, nquads=5)),
}


@pytest.mark.parametrize("name", sorted(MODELS))
@pytest.mark.parametrize("approx", ["CloseLines", "None", "OneLine"])
def test_emulated_kernel_matches_oracle(emu, name, approx):
    raw = MODELS[name]()
    a = H.setup(raw, approx=approx)
    ref = O.Oracle(a).formal_solve_fo2()
    has = ref["lambda_has"].astype(bool)
    J64, lam64 = run(emu, a, "fp64")
    assert H.max_rel(J64, ref["J"]) < 1e-12
    assert H.max_rel(lam64[has], ref["lambda_diag"][has]) < 1e-12
    J32, lam32 = run(emu, a, "split")
    assert H.max_rel(J32, ref["J"]) < 1e-5
    assert H.max_rel(lam32[has], ref["lambda_diag"][has]) < 1e-5


def run_sc0(emu, a, precision):
    desc, keep = _abi.make_desc(a)
    J = np.zeros((a["npoints"], a["nfreqs"]))
    lam = np.zeros((a["npoints"], a["nlines"]))
    emu.mgr_emu_formal_solve_sc0.argtypes = emu.mgr_emu_formal_solve_fo2.argtypes
    emu.mgr_emu_formal_solve_sc0.restype = C.c_int
    rc = emu.mgr_emu_formal_solve_sc0(C.byref(desc), _abi.PRECISION[precision],
                                      J.ctypes.data_as(C.POINTER(C.c_double)),
                                      lam.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 0
    return J, lam


@pytest.mark.parametrize("name", sorted(MODELS))
@pytest.mark.parametrize("approx", ["CloseLines", "OneLine"])
def test_emulated_shortchar_matches_oracle(emu, name, approx):
    """solve_lane_sc0 (the short-characteristics kernel's lane code) against the
    oracle's solve_shortchar_order_0."""
    raw = MODELS[name]()
    a = H.setup(raw, approx=approx)
    ref = O.Oracle(a).formal_solve_sc0()
    has = ref["lambda_has"].astype(bool)
    J64, lam64 = run_sc0(emu, a, "fp64")
    assert H.max_rel(J64, ref["J"]) < 1e-12
    assert H.max_rel(lam64[has], ref["lambda_diag"][has]) < 1e-12
    # Split precision: the short-characteristics update
    #   I = e^-dtau I + expm1(-dtau)/dtau (S_c - S_n (1 + dtau)) + S_c - S_n
    # cancels (S_c - S_n) terms for small dtau, so input roundings are amplified by
    # ~|S_c - S_n| / (dtau S): with the reference's single-precision expm1f the update
    # itself carries ~1e-4 relative noise, and split precision (FP32 sources, 1e-7)
    # lands within it.  The bar is 5e-4 here (1e-5 for Feautrier).
    J32, lam32 = run_sc0(emu, a, "split")
    assert H.max_rel(J32, ref["J"]) < 5e-4
    if name not in ("all_zero", "sph_velocity"):
        # all_zero has dtau = min_dtau everywhere and the 1D velocity gradient is
        # optically thin per step (dtau ~ 1e-4): there the reference's factor + 1 =
        # expm1f(-dtau)/dtau + 1 is single-precision rounding noise of ~ 1e-7 / dtau
        # (solver.tpp:1631-1637); their FP64 ALO above matches to 1e-12
        assert H.max_rel(lam32[has], ref["lambda_diag"][has]) < 5e-4


@pytest.mark.parametrize("name", ["cube10", "sphere14", "sphere16", "sph_velocity"])
@pytest.mark.parametrize("approx", ["CloseLines", "None"])
@pytest.mark.parametrize("rr", [0, 7])
def test_emulated_old_imager_matches_oracle(emu, name, approx, rr):
    """image_lane (the imager kernels' lane code) over rest-frame traces against the
    oracle's image_feautrier_order_2."""
    raw = MODELS[name]()
    a = H.setup(raw, approx=approx)
    rr = rr % a["nrays"]
    ref = O.Oracle(a).image_fo2(rr)
    desc, keep = _abi.make_desc(a)
    emu.mgr_emu_image.argtypes = [C.POINTER(_abi.MgrModelDesc), C.c_int, C.c_uint32, C.POINTER(C.c_double)]
    emu.mgr_emu_image.restype = C.c_int
    for precision, tol in (("fp64", 1e-12), ("split", 1e-5)):
        I = np.zeros((a["npoints"], a["nfreqs"]))
        assert emu.mgr_emu_image(C.byref(desc), _abi.PRECISION[precision], rr,
                                 I.ctypes.data_as(C.POINTER(C.c_double))) == 0
        assert H.max_rel(I, ref) < tol, precision


@pytest.mark.parametrize("name", ["cube10", "sphere14", "all_constant", "all_zero"])
@pytest.mark.parametrize("approx", ["CloseLines", "None"])
def test_emulated_uv_matches_oracle(emu, name, approx):
    """solve_lane<..., UV> (the uv kernel's lane code) against the oracle's
    solve_feautrier_order_2_uv.  u to 1e-12.  v is the finite-difference derivative
    -(c_- u[c-1] + c_+ u[c+1] + c_0 u[c]) with |c| ~ 1/dtau; the neighbour values come
    from the two sweeps here and from the back substitution in the reference, so the
    two agree to 1e-9 of u plus the rounding of u amplified by the coefficients
    (which dominates on optically thin pairs, where the reference's own v is noise)."""
    raw = MODELS[name]()
    a = H.setup(raw, approx=approx)
    ref = O.Oracle(a).formal_solve_fo2_uv()
    desc, keep = _abi.make_desc(a)
    p = C.POINTER(C.c_double)
    emu.mgr_emu_formal_solve_fo2_uv.argtypes = [C.POINTER(_abi.MgrModelDesc), C.c_int, p, p, p, p]
    for precision, tol_u, tol_v in (("fp64", 1e-12, 1e-9), ("split", 1e-5, 1e-5)):
        u, v, dtm, dtp = (np.zeros_like(ref["u"]) for _ in range(4))
        assert emu.mgr_emu_formal_solve_fo2_uv(C.byref(desc), _abi.PRECISION[precision],
                                               *[x.ctypes.data_as(p) for x in (u, v, dtm, dtp)]) == 0
        assert H.max_rel(u, ref["u"]) < tol_u, precision
        both = (dtm > 0) & (dtp > 0)
        cm = np.where(both, dtp / np.where(both, dtm * dtm + dtm * dtp, 1.0), 0.0)
        cp = np.where(both, dtm / np.where(both, dtm * dtp + dtp * dtp, 1.0), 0.0)
        noise = 64 * np.finfo(float).eps * np.abs(ref["u"]) * (cm + cp + np.abs(cm - cp))
        bound = (tol_v if precision == "split" else 1e-9) * np.abs(ref["u"]) + noise
        assert np.all(np.abs(v - ref["v"]) <= bound), precision


@pytest.mark.parametrize("name", ["cube10", "sphere14", "all_constant", "sph_velocity"])
@pytest.mark.parametrize("approx", ["CloseLines", "None"])
def test_emulated_image_for_point_matches_oracle(emu, name, approx):
    """image_lane with its per-row outputs (the image_for_point kernel's lane code) against
    the oracle's image_feautrier_order_2_for_point: row count exact, S_ray / dtau_ray /
    u_ray to 1e-12 in FP64; in split precision u_ray to 1e-5 and S_ray / dtau_ray to
    1e-4 (above 1e-10 of the largest entry: single-precision sources underflow far in
    the line wings)."""
    raw = MODELS[name]()
    a = H.setup(raw, approx=approx)
    orc = O.Oracle(a)
    p64 = C.POINTER(C.c_double)
    emu.mgr_emu_image_for_point.argtypes = [C.POINTER(_abi.MgrModelDesc), C.c_int, C.c_uint32, C.c_uint32,
                                            C.POINTER(C.c_uint32), p64, p64, p64, C.c_uint32]
    emu.mgr_emu_image_for_point.restype = C.c_int
    desc, keep = _abi.make_desc(a)
    P = a["npoints"]
    bnd = np.nonzero(np.asarray(a["point2boundary"]) != P)[0]
    for rr, p in ((0, P // 2), (1 % a["nrays"], P // 3), (0, int(bnd[0]))):
        ref = orc.image_for_point(rr, p)
        n = ref["u_ray"].shape[0]
        for precision, tol in (("fp64", 1e-12), ("split", 1e-5)):
            got = {k: np.zeros((n, a["nfreqs"])) for k in ("S_ray", "dtau_ray", "u_ray")}
            nt = C.c_uint32(0)
            assert emu.mgr_emu_image_for_point(C.byref(desc), _abi.PRECISION[precision], rr, p, C.byref(nt),
                                               got["S_ray"].ctypes.data_as(p64), got["dtau_ray"].ctypes.data_as(p64),
                                               got["u_ray"].ctypes.data_as(p64), n) == 0
            assert nt.value == n
            for k in got:
                # split precision's single-precision sources underflow far in the line wings,
                # and its per-pair sources and optical depths there carry FP32 profile
                # roundings (1e-4); u keeps the imagers' 1e-5
                floor = 1e-300 if precision == "fp64" else 1e-10 * np.abs(ref[k]).max()
                kt = tol if (precision == "fp64" or k == "u_ray") else 1e-4
                assert H.max_rel(got[k], ref[k], floor=floor) < kt, (rr, p, precision, k)


@pytest.mark.parametrize("bc", ["cmb", "thermal"])
def test_split_boundary_intensity_equals_fp64(emu, bc):
    """Without opacity J is the Doppler-shifted boundary intensity alone.  Split
    precision evaluates it in double-float arithmetic (h nu / k T rounded once to the
    float expm1f takes, as the reference rounds it; nu^3 / expm1f as double-float
    products and quotient) and forms the boundary row's h = dtau (1 + dtau/2) in FP64,
    so it equals the FP64 mode's to ~1e-14 and meets the reference's analytic bar
    (all_zero_single_ray.py: 6.41e-6) as the FP64 mode does.  Both ends carry the same
    temperature: with two different boundary intensities the FP32 optical depths of
    the two boundary pairs weigh them (a ~1e-8 effect, inside the split bar)."""
    raw = H.all_zero_model()
    if bc == "thermal":
        raw.boundary_condition[:] = S.BC_THERMAL
        raw.boundary_temperature[:] = 211.0
    a = H.setup(raw)
    J64, _ = run(emu, a, "fp64")
    J32, _ = run(emu, a, "split")
    assert H.max_rel(J32, J64) < 1e-12
    if bc == "cmb":
        err = np.abs(H.relative_error(H.all_zero_solution(raw), J32[:, 0]))
        assert np.max(err) < 6.41e-6


BAND_MODELS = {
    "cube8": lambda: S.grid_cube(n=8, nquads=5),
    "sphere10": lambda: S.grid_sphere(n=10, nside=1, nquads=5),
    "sph_velocity": lambda: S.velocity_gradient_1d(npoints=30, nrays=8, nquads=5),
}


@pytest.mark.parametrize("name", sorted(BAND_MODELS))
@pytest.mark.parametrize("n_off_diag", [1, 2, 4])
def test_emulated_band_alo_matches_oracle(emu, name, n_off_diag):
    """The banded formal solve (n_off_diag > 0): the emulated lane code's band elements
    next to the origin (two sweeps' last rows continued past the origin) against the
    oracle's update_Lambda lists built from the whole banded inverse
    (solver.tpp:2319-2355, :1760-1850), and its diagonal against the ordinary solve."""
    a = H.setup(BAND_MODELS[name]())
    ref = O.Oracle(a).formal_solve_fo2_alo(n_off_diag)
    P, L, R = a["npoints"], a["nlines"], a["hnrays"]
    off = np.zeros((P, L, R, 2 * n_off_diag))
    nr = np.zeros((P, L, R, 2 * n_off_diag), np.uint32)
    emu.mgr_emu_fo2_alo.argtypes = [C.POINTER(_abi.MgrModelDesc), C.c_uint32, C.POINTER(C.c_double),
                                    C.POINTER(C.c_uint32)]
    emu.mgr_emu_fo2_alo.restype = C.c_int
    desc, keep = _abi.make_desc(a)
    rc = emu.mgr_emu_fo2_alo(C.byref(desc), n_off_diag, off.ctypes.data_as(C.POINTER(C.c_double)),
                             nr.ctypes.data_as(C.POINTER(C.c_uint32)))
    assert rc == 0
    J, lam = run(emu, a, "fp64")
    assert H.max_rel(J, ref["J"]) < 1e-12
    assert np.count_nonzero(off) > 0
    assert H.band_alo_error(off, nr, lam, ref) < 1e-12
