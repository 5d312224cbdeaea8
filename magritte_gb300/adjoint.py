"""Differentiable new imager: gradients of compute_image_new images with respect to
the per-point velocity, temperature, turbulence and abundance of a model.

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

PyTorch is the autograd plumbing here; every image and adjoint is computed by the
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
        dev = dict(dtype=torch.float64, device=self.device)
        self.species = []
        for ls in model.lines.lineProducingSpecies:
            ld = ls.linedata
            self.species.append(dict(
                num=int(ld.num), nlev=int(ld.nlev), nrad=int(ld.nrad), inverse_mass=float(ld.inverse_mass),
                energy=torch.tensor(np.array(ld.energy), **dev), weight=torch.tensor(np.array(ld.weight), **dev),
                frequency=torch.tensor(np.array(ld.frequency), **dev), A=torch.tensor(np.array(ld.A), **dev),
                Ba=torch.tensor(np.array(ld.Ba), **dev), Bs=torch.tensor(np.array(ld.Bs), **dev),
                irad=torch.tensor(np.array(ld.irad), dtype=torch.long, device=self.device),
                jrad=torch.tensor(np.array(ld.jrad), dtype=torch.long, device=self.device)))
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
        em_cols, op_cols, iw_cols = [], [], []
        T = temperature[:, None]
        for s in self.species:
            pop = s["weight"][None, :] * torch.exp(-s["energy"][None, :] / (KB * T))
            pop = pop * (abundance[:, s["num"]][:, None] / pop.sum(dim=1, keepdim=True))
            up, lo = pop[:, s["irad"]], pop[:, s["jrad"]]
            nu = s["frequency"][None, :]
            em = nu * HH_OVER_FOUR_PI * s["A"][None, :] * up
            op = nu * HH_OVER_FOUR_PI * (lo * s["Ba"][None, :] - up * s["Bs"][None, :])
            em_cols.append(torch.clamp(em, min=self.min_em))
            op_cols.append(torch.clamp(op, min=self.min_op))
            width = nu * torch.sqrt(TWO_KB_OVER_AMU_CC_SQUARED * s["inverse_mass"] * T + vturb2[:, None])
            iw_cols.append(1.0 / width)
        return (torch.cat(em_cols, dim=1).contiguous(), torch.cat(op_cols, dim=1).contiguous(),
                torch.cat(iw_cols, dim=1).contiguous())

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
