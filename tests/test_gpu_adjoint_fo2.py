"""Differentiable formal solve on the GPU (mgr_formal_solve_fo2_smooth_device,
mgr_formal_solve_fo2_adjoint_device, magritte_gb300.adjoint.FormalSolver).

* The smooth J equals the emulated lane code (1e-10 relative; checked against the
  oracle's smooth formal solve in test_adjoint_fo2_emulation.py) and stays within the
  formal solve's 1e-5 bar of the oracle's reference arithmetic.
* A list of origins gives the same rows as the full solve, bit for bit.
* The adjoint kernel equals the emulated adjoint (checked against the oracle's finite
  differences in test_adjoint_fo2_emulation.py) to 1e-9 of the largest entry.
* End to end through torch.autograd (FormalSolver): d(loss)/d(velocity, temperature,
  turbulence, abundance) of a sum of squared J differences against FP64 central
  differences of the same forward, along random directions of each sampled point's
  parameters.  Bar: 1e-4 relative."""
import ctypes as C

import numpy as np
import pytest

import helpers as H
import oracle as O
from magritte_gb300 import _abi, build
from magritte_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

_f64p = C.POINTER(C.c_double)


def _p(x):
    return x.ctypes.data_as(_f64p)


@pytest.fixture(scope="module")
def emu():
    lib = C.CDLL(build.build_emu())
    lib.mgr_emu_fo2_smooth.argtypes = [C.POINTER(_abi.MgrModelDesc), _f64p]
    lib.mgr_emu_fo2_adjoint.argtypes = [C.POINTER(_abi.MgrModelDesc)] + [_f64p] * 7
    return lib


def models():
    return {"sphere": H.setup(S.grid_sphere(n=12, nside=1, nquads=5)),
            "cube": H.setup(S.grid_cube(n=8, nquads=7)),
            "cube-None": H.setup(S.grid_cube(n=8, nquads=7), approx="None")}


def gpu_J(dev, origins=None):
    import torch
    J = torch.zeros((dev.P, dev.F), dtype=torch.float64, device="cuda")
    lib = _abi.load()
    if origins is None:
        _abi._check(lib.mgr_formal_solve_fo2_smooth_device(dev.h, None, 0, C.c_void_p(J.data_ptr())))
    else:
        o = torch.tensor(origins, dtype=torch.int32, device="cuda")
        _abi._check(lib.mgr_formal_solve_fo2_smooth_device(dev.h, C.c_void_p(o.data_ptr()), len(origins),
                                                           C.c_void_p(J.data_ptr())))
    return J.cpu().numpy()


@pytest.mark.parametrize("name", ["sphere", "cube", "cube-None"])
def test_smooth_J_matches_emulation_and_oracle(gpu_lib, emu, name):
    a = models()[name]
    dev = _abi.DeviceModel(a)
    try:
        got = gpu_J(dev)
        desc, keep = _abi.make_desc(a)
        ref = np.zeros_like(got)
        assert emu.mgr_emu_fo2_smooth(C.byref(desc), _p(ref)) == 0
        # the lane code compiled for the device contracts multiply-adds the host build
        # keeps apart; the None approximation's sums over every line amplify those ulps
        assert H.max_rel(got, ref) < 1e-10
        O.set_erf_mode(0)
        orc = O.Oracle(a).formal_solve_fo2()["J"]
        assert H.max_rel(got, orc) < 1e-5
        rows = np.arange(0, dev.P, 7)
        sub = gpu_J(dev, rows)
        np.testing.assert_array_equal(sub[rows], got[rows])
        assert not sub[np.setdiff1d(np.arange(dev.P), rows)].any()
    finally:
        dev.close()


@pytest.mark.parametrize("name", ["sphere", "cube"])
def test_adjoint_kernel_matches_emulation(gpu_lib, emu, name):
    import torch
    a = models()[name]
    P, L, F = a["npoints"], a["nlines"], a["nfreqs"]
    rng = np.random.default_rng(5)
    gJ = rng.normal(size=(P, F))
    desc, keep = _abi.make_desc(a)
    ref = {k: np.zeros((P, L)) for k in ("em", "op", "iw", "Sp")}
    ref["vel"] = np.zeros((P, 3))
    ref["nu"] = np.zeros((P, F))
    assert emu.mgr_emu_fo2_adjoint(C.byref(desc), _p(gJ), _p(ref["em"]), _p(ref["op"]), _p(ref["iw"]),
                                   _p(ref["Sp"]), _p(ref["vel"]), _p(ref["nu"])) == 0
    dev = _abi.DeviceModel(a)
    try:
        t = lambda x: torch.tensor(x, dtype=torch.float64, device="cuda")
        gJd = t(gJ)
        g = {k: torch.zeros_like(t(v)) for k, v in ref.items()}
        ptr = lambda x: C.c_void_p(x.data_ptr())
        _abi._check(_abi.load().mgr_formal_solve_fo2_adjoint_device(
            dev.h, None, 0, ptr(gJd), ptr(g["em"]), ptr(g["op"]), ptr(g["iw"]), ptr(g["Sp"]), ptr(g["vel"]),
            ptr(g["nu"])))
        for k in ref:
            scale = np.abs(ref[k]).max()
            assert scale > 0, k
            # summation order (warp sums, atomics) and CUDA's vs the host's FP64 libm
            assert np.abs(g[k].cpu().numpy() - ref[k]).max() <= 1e-9 * scale, k
    finally:
        dev.close()


def _core(raw):
    from magritte_gb300 import loader
    m = loader.to_core(raw, precision="fp64")
    m.compute_spectral_discretisation()
    m.compute_inverse_line_widths()
    m.compute_LTE_level_populations()
    return m


def test_autograd_gradients_match_finite_differences(gpu_lib):
    import torch
    from magritte_gb300 import adjoint

    raw = S.grid_sphere(n=12, nside=1, nquads=5)
    solver = adjoint.FormalSolver(_core(raw))
    dev = dict(dtype=torch.float64, device="cuda")
    v0 = torch.tensor(raw.velocity, **dev)
    T0 = torch.tensor(raw.temperature, **dev)
    vt0 = torch.tensor(raw.vturb2, **dev)
    ab0 = torch.tensor(raw.abundance, **dev)
    rng = np.random.default_rng(3)
    with torch.no_grad():
        target = solver(v0 * 1.05, T0 * 1.1, vt0, ab0)
        # the smooth J equals the drop-in solve within the formal solve's bar
        ref = solver.model
        ref.compute_radiation_field_feautrier_order_2()
        J_ref = np.array(ref.radiation.J).reshape(raw.npoints, -1)
        assert H.max_rel(solver(v0, T0, vt0, ab0).cpu().numpy(), J_ref) < 1e-5
    solver.refresh()

    def loss_of(v, T, vt, ab):
        return ((solver(v, T, vt, ab) - target) ** 2).sum()

    params = [t.clone().requires_grad_(True) for t in (v0, T0, vt0, ab0)]
    loss = loss_of(*params)
    loss.backward()
    grads = [p.grad.detach().clone() for p in params]
    assert all(torch.isfinite(g).all() for g in grads)
    gv = grads[0].norm(dim=1).cpu().numpy()
    interior = np.setdiff1d(np.arange(raw.npoints), raw.boundary2point)
    pts = np.unique(np.concatenate([np.argsort(gv)[-4:], rng.choice(interior, 6, replace=False)]))
    checked = 0
    for p in pts:
        dirv = [torch.zeros_like(t) for t in params]
        u = rng.normal(size=6)
        dirv[0][p] = torch.tensor(u[:3], **dev) * 1e-4 * v0.abs().max()
        dirv[1][p] = u[3] * 1e-4 * T0[p]
        dirv[2][p] = u[4] * 1e-4 * vt0[p]
        dirv[3][p, 0] = u[5] * 1e-4 * ab0[p, 0]
        an = sum(float((g * dv).sum()) for g, dv in zip(grads, dirv))

        def central(eps):
            with torch.no_grad():
                lp = loss_of(*[t + eps * dv for t, dv in zip((v0, T0, vt0, ab0), dirv)])
                lm = loss_of(*[t - eps * dv for t, dv in zip((v0, T0, vt0, ab0), dirv)])
            return float(lp - lm) / (2 * eps)

        c1, c2 = central(1.0), central(0.5)
        if abs(c1 - c2) > 1e-3 * abs(c2):
            continue  # the step crossed a held branch (large-shift test, line bracket)
        fd = (4.0 * c2 - c1) / 3.0
        assert abs(an - fd) <= 1e-4 * abs(fd) + 1e-9 * abs(loss.item()), (p, an, fd)
        checked += 1
    assert checked >= 6


def test_drop_in_solve_after_differentiable_solve_sees_host_state(gpu_lib):
    """FormalSolver runs on the core.Model's own device copy and replaces its
    velocities, frequencies and line data; the next drop-in solve of that model must
    still solve the host state (bit for bit the J of a solve before)."""
    import torch
    from magritte_gb300 import adjoint

    raw = S.grid_sphere(n=10, nside=1, nquads=5)
    model = _core(raw)
    solver = adjoint.FormalSolver(model)
    model.compute_radiation_field_feautrier_order_2()
    J0 = np.array(model.radiation.J).copy()
    dev = dict(dtype=torch.float64, device="cuda")
    with torch.no_grad():
        solver(torch.tensor(raw.velocity, **dev) * 1.05, torch.tensor(raw.temperature, **dev) * 1.1,
               torch.tensor(raw.vturb2, **dev), torch.tensor(raw.abundance, **dev))
    model.compute_radiation_field_feautrier_order_2()
    assert np.array_equal(np.array(model.radiation.J), J0)
