"""Differentiable new imager and formal solve: gradients of compute_image_new images
and of the mean intensity J of compute_radiation_field_feautrier_order_2 with respect
to the per-point velocity, temperature, turbulence and abundance of a model.

The reference has no derivatives.  Its imager (Model::compute_image_new,
src/model/model.cpp:977-1013 -> Solver::image_feautrier_order_2_new_imager,
src/solver/solver.tpp:576-627) becomes a differentiable function in two layers:

* ``ImageNewFunction`` (torch.autograd.Function): image I [nx*ny][F] of one
  direction as a function of the per-point velocity [P][3] (v/c) and line data
  emissivity, opacity, inverse line width [P][L].  Forward and backward are the
  library's CUDA kernels (mgr_image_new_smooth_device / mgr_image_new_adjoint_device):
  the smooth FP64 image (the reference's single-precision powf / expf / expm1f / erff
  in double precision) and its hand-written adjoint, which recomputes each ray's
  elimination factors instead of storing them.  The ray traces, interpolation
  points, CloseLines brackets, the large-shift branch and the dtau clamp are held
  at their values for the model's current state (trace-fixed derivatives).
* ``NewImager``: the line data from temperature, turbulence and abundance through
  LTE level populations (LineProducingSpecies::update_using_LTE,
  lineProducingSpecies.tpp:52-75), Lines::set_emissivity_and_opacity (lines.tpp:29-40)
  and Lines::set_inverse_width (lines.tpp:45-59), written as torch operations so
  autograd chains them into the kernel's derivatives.

The formal solve (Model::compute_radiation_field_feautrier_order_2, model.cpp:353-390
-> Solver::solve_feautrier_order_2, solver.tpp:458-540, :2193-2318) is differentiated the
same way:

* ``FormalSolveFunction``: J [P][F] as a function of the velocity, the line data and
  the frequencies nu [P][F] (which move with the line widths: Model::
  compute_spectral_discretisation, model.cpp:70-161).  Forward and backward are
  mgr_formal_solve_fo2_smooth_device / mgr_formal_solve_fo2_adjoint_device: the smooth
  FP64 two-sided Feautrier solve and its adjoint, which recomputes every ray pair's
  elimination factors in the backward pass.  An optional list of origins restricts
  both to those rows of J.
* ``FormalSolver``: line data and frequencies from temperature, turbulence and
  abundance as torch operations.

PyTorch is the autograd plumbing here; every image, J and adjoint is computed by the
library's kernels, and the calls fail if the CUDA library is missing."""
import ctypes as C

import numpy as np
import torch

from . import _abi

# Physical constants of the library and the reference (src/tools/constants.hpp).
KB = 1.38064852e-23
HH = 6.62607004e-34
CC = 2.99792458e8
AMU = 1.66053904e-27
CC_SQUARED = 8.98755179e16
HH_OVER_FOUR_PI = HH / (4.0 * np.pi)
TWO_KB_OVER_AMU_CC_SQUARED = 2.0 * KB / (AMU * CC_SQUARED)


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _check_f64_cuda(t, name):
    if t.dtype != torch.float64 or not t.is_cuda or not t.is_contiguous():
        raise TypeError(f"{name} must be a contiguous float64 CUDA tensor")


class ImageNewFunction(torch.autograd.Function):
    """I = image_new(velocity, emissivity, opacity, inverse_width) for one direction."""

    @staticmethod
    def forward(ctx, handle, raydir, nx, ny, F, velocity, emissivity, opacity, inverse_width):
        lib = _abi.load()
        for t, n in ((velocity, "velocity"), (emissivity, "emissivity"), (opacity, "opacity"),
                     (inverse_width, "inverse_width")):
            _check_f64_cuda(t, n)
        torch.cuda.current_stream().synchronize()  # inputs written on torch's stream
        d = np.ascontiguousarray(raydir, np.float64)
        _abi._check(lib.mgr_model_set_velocity_device(handle, _ptr(velocity)))
        _abi._check(lib.mgr_model_set_line_data_device(handle, _ptr(emissivity), _ptr(opacity), _ptr(inverse_width)))
        I = torch.empty((nx * ny, F), dtype=torch.float64, device=velocity.device)
        _abi._check(lib.mgr_image_new_smooth_device(handle, d.ctypes.data_as(_abi._f64p), nx, ny, _ptr(I), None,
                                                    None))
        ctx.handle, ctx.raydir, ctx.nx, ctx.ny = handle, d, nx, ny
        ctx.save_for_backward(velocity, emissivity, opacity, inverse_width)
        return I

    @staticmethod
    def backward(ctx, gI):
        lib = _abi.load()
        velocity, em, op, iw = ctx.saved_tensors
        gI = gI.contiguous().to(torch.float64)
        torch.cuda.current_stream().synchronize()
        # the model may have been re-targeted by another forward since: restore this one's inputs
        _abi._check(lib.mgr_model_set_velocity_device(ctx.handle, _ptr(velocity)))
        _abi._check(lib.mgr_model_set_line_data_device(ctx.handle, _ptr(em), _ptr(op), _ptr(iw)))
        g_em, g_op, g_iw, g_Sp = (torch.zeros_like(em) for _ in range(4))
        g_vel = torch.zeros_like(velocity)
        _abi._check(lib.mgr_image_new_adjoint_device(ctx.handle, ctx.raydir.ctypes.data_as(_abi._f64p), ctx.nx,
                                                     ctx.ny, _ptr(gI), _ptr(g_em), _ptr(g_op), _ptr(g_iw),
                                                     _ptr(g_Sp), _ptr(g_vel)))
        # the kernel's line source is the library's quotient Sp = em / op
        g_em = g_em + g_Sp / op
        g_op = g_op - g_Sp * em / (op * op)
        return None, None, None, None, None, g_vel, g_em, g_op, g_iw


def _species(model, device):
    """Per-species line data of a core.Model as torch tensors."""
    dev = dict(dtype=torch.float64, device=device)
    out = []
    for ls in model.lines.lineProducingSpecies:
        ld = ls.linedata
        out.append(dict(
            num=int(ld.num), nlev=int(ld.nlev), nrad=int(ld.nrad), inverse_mass=float(ld.inverse_mass),
            energy=torch.tensor(np.array(ld.energy), **dev), weight=torch.tensor(np.array(ld.weight), **dev),
            frequency=torch.tensor(np.array(ld.frequency), **dev), A=torch.tensor(np.array(ld.A), **dev),
            Ba=torch.tensor(np.array(ld.Ba), **dev), Bs=torch.tensor(np.array(ld.Bs), **dev),
            irad=torch.tensor(np.array(ld.irad), dtype=torch.long, device=device),
            jrad=torch.tensor(np.array(ld.jrad), dtype=torch.long, device=device),
            roots=torch.tensor(np.array(ls.quadrature.roots), **dev)))
    return out


def line_data(species, min_em, min_op, temperature, vturb2, abundance):
    """Emissivity, opacity and inverse width [P][L] from temperature [P], vturb2 [P]
    ((v_turb/c)^2) and abundance [P][nspecs] (number densities): LTE populations
    (LineProducingSpecies::update_using_LTE, lineProducingSpecies.tpp:52-75),
    Lines::set_emissivity_and_opacity with the reference's floors (lines.tpp:29-40),
    Lines::set_inverse_width (lines.tpp:45-59), as torch operations."""
    em_cols, op_cols, iw_cols = [], [], []
    T = temperature[:, None]
    for s in species:
        pop = s["weight"][None, :] * torch.exp(-s["energy"][None, :] / (KB * T))
        pop = pop * (abundance[:, s["num"]][:, None] / pop.sum(dim=1, keepdim=True))
        up, lo = pop[:, s["irad"]], pop[:, s["jrad"]]
        nu = s["frequency"][None, :]
        em = nu * HH_OVER_FOUR_PI * s["A"][None, :] * up
        op = nu * HH_OVER_FOUR_PI * (lo * s["Ba"][None, :] - up * s["Bs"][None, :])
        em_cols.append(torch.clamp(em, min=min_em))
        op_cols.append(torch.clamp(op, min=min_op))
        width = nu * torch.sqrt(TWO_KB_OVER_AMU_CC_SQUARED * s["inverse_mass"] * T + vturb2[:, None])
        iw_cols.append(1.0 / width)
    return (torch.cat(em_cols, dim=1).contiguous(), torch.cat(op_cols, dim=1).contiguous(),
            torch.cat(iw_cols, dim=1).contiguous())


def line_frequencies(species, temperature, vturb2):
    """nu [P][F] of the line spectral discretisation (Model::compute_spectral_discretisation,
    model.cpp:70-161): nu(p, f) = line + width(p) root_z for f = line * nquads + z, with the
    line's Doppler width from temperature and turbulence."""
    cols = []
    T = temperature[:, None]
    for s in species:
        pw = torch.sqrt(TWO_KB_OVER_AMU_CC_SQUARED * s["inverse_mass"] * T + vturb2[:, None])  # [P][1]
        for k in range(s["nrad"]):
            line = s["frequency"][k]
            cols.append(line + (line * pw) * s["roots"][None, :])
    return torch.cat(cols, dim=1).contiguous()


class FormalSolveFunction(torch.autograd.Function):
    """J = formal_solve(velocity, emissivity, opacity, inverse_width, nu) [P][F]; with
    ``origins`` (an int32 CUDA tensor) only those rows are computed (others are 0)."""

    @staticmethod
    def forward(ctx, handle, origins, P, F, velocity, emissivity, opacity, inverse_width, nu):
        lib = _abi.load()
        for t, n in ((velocity, "velocity"), (emissivity, "emissivity"), (opacity, "opacity"),
                     (inverse_width, "inverse_width"), (nu, "nu")):
            _check_f64_cuda(t, n)
        torch.cuda.current_stream().synchronize()
        _set_inputs(lib, handle, velocity, emissivity, opacity, inverse_width, nu)
        J = torch.zeros((P, F), dtype=torch.float64, device=velocity.device)
        optr, n_o = (None, 0) if origins is None else (_ptr(origins), int(origins.numel()))
        _abi._check(lib.mgr_formal_solve_fo2_smooth_device(handle, optr, n_o, _ptr(J)))
        ctx.handle, ctx.origins = handle, origins
        ctx.save_for_backward(velocity, emissivity, opacity, inverse_width, nu)
        return J

    @staticmethod
    def backward(ctx, gJ):
        lib = _abi.load()
        velocity, em, op, iw, nu = ctx.saved_tensors
        gJ = gJ.contiguous().to(torch.float64)
        torch.cuda.current_stream().synchronize()
        _set_inputs(lib, ctx.handle, velocity, em, op, iw, nu)
        g_em, g_op, g_iw, g_Sp = (torch.zeros_like(em) for _ in range(4))
        g_vel = torch.zeros_like(velocity)
        g_nu = torch.zeros_like(nu)
        optr, n_o = (None, 0) if ctx.origins is None else (_ptr(ctx.origins), int(ctx.origins.numel()))
        _abi._check(lib.mgr_formal_solve_fo2_adjoint_device(ctx.handle, optr, n_o, _ptr(gJ), _ptr(g_em), _ptr(g_op),
                                                            _ptr(g_iw), _ptr(g_Sp), _ptr(g_vel), _ptr(g_nu)))
        g_em = g_em + g_Sp / op
        g_op = g_op - g_Sp * em / (op * op)
        return None, None, None, None, g_vel, g_em, g_op, g_iw, g_nu


def _set_inputs(lib, handle, velocity, em, op, iw, nu):
    _abi._check(lib.mgr_model_set_velocity_device(handle, _ptr(velocity)))
    _abi._check(lib.mgr_model_set_line_data_device(handle, _ptr(em), _ptr(op), _ptr(iw)))
    _abi._check(lib.mgr_model_set_frequencies_device(handle, _ptr(nu)))


class FormalSolver:
    """Differentiable Model::compute_radiation_field_feautrier_order_2 of a core.Model:
    J [P][F] from velocity [P][3] (v/c), temperature [P], vturb2 [P] and abundance
    [P][nspecs] (number densities), with the line data and the line frequencies
    recomputed in torch.  The model needs its line spectral discretisation, line widths
    and level populations set up; its device copy (core.Model.upload) is used, and its
    velocities, line data and frequencies are replaced by each call.  The trace-fixed
    structure (interpolation points, line brackets, large-shift branches) follows the
    model's host state at construction or ``refresh()``."""

    def __init__(self, model, device=None):
        self.model = model
        prm = model.parameters
        self.P, self.F, self.L = prm.npoints(), prm.nfreqs(), prm.nlines()
        self.device = torch.device(device if device is not None else "cuda")
        self.min_em = float(prm.min_line_emissivity)
        self.min_op = float(prm.min_line_opacity)
        self.species = _species(model, self.device)
        self.handle = None
        self.refresh()

    def refresh(self):
        self.model.release_device()
        self.handle = C.c_void_p(self.model.upload())

    def solve(self, velocity, emissivity, opacity, inverse_width, nu, origins=None):
        """J [P][F] from the kernel's direct inputs (differentiable)."""
        return FormalSolveFunction.apply(self.handle, origins, self.P, self.F, velocity.contiguous(), emissivity,
                                         opacity, inverse_width, nu)

    def __call__(self, velocity, temperature, vturb2, abundance, origins=None):
        em, op, iw = line_data(self.species, self.min_em, self.min_op, temperature, vturb2, abundance)
        nu = line_frequencies(self.species, temperature, vturb2)
        return self.solve(velocity, em, op, iw, nu, origins)


class NewImager:
    """Differentiable Model::compute_image_new(raydir, nx, ny) of a core.Model.

    The model must have its spectral discretisation (usually an imaging one,
    compute_spectral_discretisation(nu_min, nu_max, n)), line widths and level
    populations set up; its device copy (core.Model.upload) is used and its line
    data and velocities are replaced by each call.  ``refresh()`` re-derives the
    trace-fixed structure (interpolation points, line brackets) from the model's
    host state."""

    def __init__(self, model, nx, ny, device=None):
        self.model = model
        self.nx, self.ny = int(nx), int(ny)
        prm = model.parameters
        self.P, self.F, self.L = prm.npoints(), prm.nfreqs(), prm.nlines()
        self.device = torch.device(device if device is not None else "cuda")
        self.min_em = float(prm.min_line_emissivity)
        self.min_op = float(prm.min_line_opacity)
        self.species = _species(model, self.device)
        self.handle = None
        self.refresh()

    def refresh(self):
        """(Re)upload the model: the interpolation points, brackets and branch
        thresholds follow the model's current host state."""
        self.model.release_device()
        self.handle = C.c_void_p(self.model.upload())

    def line_data(self, temperature, vturb2, abundance):
        """Emissivity, opacity and inverse width [P][L] (torch, differentiable) from
        temperature [P], vturb2 [P] ((v_turb/c)^2) and abundance [P][nspecs]
        (number densities)."""
        return line_data(self.species, self.min_em, self.min_op, temperature, vturb2, abundance)

    def render(self, raydir, velocity, emissivity, opacity, inverse_width):
        """Image [nx*ny][F] along raydir from velocity / line data (differentiable)."""
        return ImageNewFunction.apply(self.handle, np.asarray(raydir, np.float64), self.nx, self.ny, self.F,
                                      velocity.contiguous(), emissivity, opacity, inverse_width)

    def __call__(self, raydir, velocity, temperature, vturb2, abundance):
        em, op, iw = self.line_data(temperature, vturb2, abundance)
        return self.render(raydir, velocity, em, op, iw)

    def image_coordinates(self, raydir):
        """Pixel coordinates (ImX, ImY) [nx*ny] of the image plane of raydir."""
        lib = _abi.load()
        npix = self.nx * self.ny
        X, Y = np.empty(npix), np.empty(npix)
        I = torch.empty((npix, self.F), dtype=torch.float64, device=self.device)
        d = np.ascontiguousarray(raydir, np.float64)
        _abi._check(lib.mgr_image_new_smooth_device(self.handle, d.ctypes.data_as(_abi._f64p), self.nx, self.ny,
                                                    _ptr(I), X.ctypes.data_as(_abi._f64p),
                                                    Y.ctypes.data_as(_abi._f64p)))
        return X, Y


def inclination_direction(deg):
    """Unit ray direction at inclination ``deg`` from the z axis in the x-z plane."""
    t = np.deg2rad(deg)
    return np.array([np.sin(t), 0.0, np.cos(t)])
