"""ctypes binding of libmgr_gpu.so (the C ABI declared in include/magritte_gb300.h).

This is the thin Python view of the drop-in boundary: ``DeviceModel`` owns one
``MgrModel`` and calls the formal-solve entry points with host numpy buffers.
It fails loudly when the library is missing or no CUDA device is present; there
is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libmgr_gpu.so")

MGR_OK = 0
# MgrStatus codes (include/magritte_gb300.h)
MGR_ERR_ARGUMENT, MGR_ERR_CUDA, MGR_ERR_NO_DEVICE = -1, -2, -3
MGR_ERR_TRACE, MGR_ERR_CAPACITY, MGR_ERR_NONFINITE, MGR_ERR_UNSUPPORTED = -4, -5, -6, -7
PRECISION = {"fp64": 0, "split": 1}
APPROX = {"None": 0, "OneLine": 1, "CloseLines": 2}

_u32p = C.POINTER(C.c_uint32)
_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)

DESC_FIELDS = [
    ("npoints", C.c_uint32), ("nrays", C.c_uint32), ("hnrays", C.c_uint32), ("nlines", C.c_uint32),
    ("nquads", C.c_uint32), ("nfreqs", C.c_uint32), ("nlspecs", C.c_uint32), ("nboundary", C.c_uint32),
    ("position", _f64p), ("velocity", _f64p), ("n_neighbors", _u32p), ("cum_n_neighbors", _u32p),
    ("neighbors", _u32p), ("point2boundary", _u32p), ("boundary_condition", _i32p),
    ("boundary_temperature", _f64p), ("ray_direction", _f64p), ("ray_weight", _f64p), ("antipod", _u32p),
    ("line", _f64p), ("sorted_line", _f64p), ("sorted_line_map", _u32p), ("max_inverse_mass", C.c_double),
    ("emissivity", _f64p), ("opacity", _f64p), ("inverse_width", _f64p), ("interp_criterion", _f64p),
    ("temperature", _f64p), ("vturb2", _f64p), ("dshift_max", _f64p), ("nu", _f64p),
    ("corr_line", _u32p), ("corr_lspec", _u32p), ("corr_k", _u32p), ("corr_z", _u32p),
    ("in_line_integral", _u8p), ("nrad", _u32p), ("nrad_cum", _u32p), ("line_A", _f64p),
    ("lspec_inverse_mass", _f64p), ("quad_weights", _f64p), ("quad_roots", _f64p),
    ("min_opacity", C.c_double), ("min_dtau", C.c_double), ("max_interpolation_diff", C.c_double),
    ("max_distance_opacity_contribution", C.c_double), ("approx", C.c_int32), ("spherical_symmetry", C.c_int32),
    ("use_adaptive_directions", C.c_int32),
]
_FLAGS = ("spherical_symmetry", "use_adaptive_directions")

_PTR_TYPES = {_u32p: np.uint32, _i32p: np.int32, _f64p: np.float64, _u8p: np.uint8}


class MgrModelDesc(C.Structure):
    _fields_ = DESC_FIELDS


class MgrCollisionPartnerDesc(C.Structure):
    _fields_ = [("num_col_partner", C.c_uint32), ("ortho_para", C.c_int32), ("ncol", C.c_uint32),
                ("ntmp", C.c_uint32), ("icol", _u32p), ("jcol", _u32p), ("tmp", _f64p), ("Cd", _f64p),
                ("Ce", _f64p)]


class MgrSpeciesDesc(C.Structure):
    _fields_ = [("num", C.c_uint32), ("nlev", C.c_uint32), ("nrad", C.c_uint32), ("ncolpar", C.c_uint32),
                ("energy", _f64p), ("weight", _f64p), ("irad", _u32p), ("jrad", _u32p), ("A", _f64p),
                ("Bs", _f64p), ("Ba", _f64p), ("frequency", _f64p),
                ("colpar", C.POINTER(MgrCollisionPartnerDesc))]


class MgrAliParams(C.Structure):
    _fields_ = [("pop_prec", C.c_double), ("min_rel_pop_for_convergence", C.c_double),
                ("convergence_fraction", C.c_double), ("population_inversion_fraction", C.c_double),
                ("min_line_opacity", C.c_double), ("min_line_emissivity", C.c_double),
                ("Ng_acceleration_mem_limit", C.c_uint32), ("adaptive_Ng_acceleration_min_order", C.c_uint32),
                ("Ng_acceleration_remove_N_its", C.c_uint32), ("use_adaptive_Ng_acceleration", C.c_int32),
                ("adaptive_Ng_acceleration_use_max_criterion", C.c_int32)]


# Defaults of Magritte's Parameters (src/model/parameters/parameters.hpp:76-103).
ALI_DEFAULTS = dict(pop_prec=1.0e-6, min_rel_pop_for_convergence=1.0e-10, convergence_fraction=0.995,
                    population_inversion_fraction=-1.0, min_line_opacity=1.0e-13, min_line_emissivity=1.0e-50,
                    Ng_acceleration_mem_limit=9, adaptive_Ng_acceleration_min_order=2,
                    Ng_acceleration_remove_N_its=0, use_adaptive_Ng_acceleration=1,
                    adaptive_Ng_acceleration_use_max_criterion=1)


# mgr_reduce_fn: (user, J_dev, nJ, lambda_diag_dev, nlam, stream) -> 0 on success.
REDUCE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_void_p)

# Every exported symbol of include/magritte_gb300.h with its ctypes signature.
SIGNATURES = {
    "mgr_last_error": (C.c_char_p, []),
    "mgr_version": (C.c_int, []),
    "mgr_device_count": (C.c_int, [C.POINTER(C.c_int)]),
    "mgr_model_create": (C.c_int, [C.POINTER(MgrModelDesc), C.POINTER(C.c_void_p)]),
    "mgr_model_free": (None, [C.c_void_p]),
    "mgr_model_set_line_data": (C.c_int, [C.c_void_p, _f64p, _f64p, _f64p, _f64p]),
    "mgr_ray_lengths_max": (C.c_int, [C.c_void_p, _u32p]),
    "mgr_trace_ray_pair": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _u32p, _u32p,
                                     _u32p, _u32p, _f64p, _f64p, _f64p]),
    "mgr_formal_solve_fo2": (C.c_int, [C.c_void_p, C.c_int, _f64p, _f64p, _f64p]),
    "mgr_formal_solve_fo2_device": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mgr_formal_solve_fo2_rays": (C.c_int, [C.c_void_p, C.c_int, C.c_uint32, C.c_uint32, _f64p, _f64p]),
    "mgr_model_set_n_off_diag": (C.c_int, [C.c_void_p, C.c_uint32]),
    "mgr_formal_solve_fo2_alo_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                  C.c_void_p]),
    "mgr_formal_solve_fo2_alo": (C.c_int, [C.c_void_p, _f64p, _f64p, _f64p, _f64p, _u32p]),
    "mgr_formal_solve_fo2_rays_device": (C.c_int, [C.c_void_p, C.c_int, C.c_uint32, C.c_uint32, C.c_void_p,
                                                   C.c_void_p]),
    "mgr_set_ray_shard": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, REDUCE_FN, C.c_void_p, C.c_int]),
    "mgr_formal_solve_sc0": (C.c_int, [C.c_void_p, C.c_int, _f64p, _f64p, _f64p, _f64p, _f64p]),
    "mgr_formal_solve_sc0_device": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_void_p]),
    "mgr_image": (C.c_int, [C.c_void_p, C.c_int, C.c_uint32, _f64p, _f64p, _f64p]),
    "mgr_image_new": (C.c_int, [C.c_void_p, C.c_int, _f64p, C.c_uint32, C.c_uint32, _f64p, _f64p, _f64p]),
    "mgr_image_optical_depth": (C.c_int, [C.c_void_p, C.c_int, C.c_uint32, _f64p, _f64p, _f64p]),
    "mgr_image_optical_depth_new": (C.c_int, [C.c_void_p, C.c_int, _f64p, C.c_uint32, C.c_uint32, _f64p, _f64p,
                                              _f64p]),
    "mgr_image_for_point": (C.c_int, [C.c_void_p, C.c_int, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32), _f64p,
                                      _f64p, _f64p, C.c_uint32]),
    "mgr_set_column": (C.c_int, [C.c_void_p, _f64p, _f64p]),
    "mgr_formal_solve_fo2_device_noalloc": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mgr_ray_statistics": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                     C.POINTER(C.c_uint64)]),
    "mgr_trace_self_check": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                        C.POINTER(C.c_uint64)]),
    "mgr_set_tuning": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "mgr_autotune_fo2": (C.c_int, [C.c_void_p, C.c_int, C.c_uint32, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(C.c_float)]),
    "mgr_model_set_species": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(MgrSpeciesDesc), C.c_uint32, _f64p,
                                        C.POINTER(_f64p)]),
    "mgr_compute_jeff": (C.c_int, [C.c_void_p, C.c_uint32, _f64p, _f64p, _f64p]),
    "mgr_compute_jeff_sparse": (C.c_int, [C.c_void_p, C.c_uint32, _f64p, _f64p]),
    "mgr_formal_solve_fo2_sparse": (C.c_int, [C.c_void_p, C.c_int, _f64p, _f64p]),
    "mgr_formal_solve_fo2_anis": (C.c_int, [C.c_void_p, C.c_int, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p]),
    "mgr_formal_solve_fo2_uv": (C.c_int, [C.c_void_p, C.c_int, _f64p, _f64p]),
    "mgr_formal_solve_fo2_sparse_device": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "mgr_compute_level_populations_sparse": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_long,
                                                       C.POINTER(MgrAliParams), C.POINTER(C.c_int), _f64p, _f64p,
                                                       C.c_uint32]),
    "mgr_compute_level_populations": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_long, C.POINTER(MgrAliParams),
                                                C.POINTER(C.c_int), _f64p, _f64p, C.c_uint32]),
    "mgr_get_populations": (C.c_int, [C.c_void_p, C.c_uint32, _f64p]),
    "mgr_get_line_data": (C.c_int, [C.c_void_p, _f64p, _f64p]),
    "mgr_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_uint32, C.POINTER(C.c_void_p)]),
    "mgr_batch_free": (None, [C.c_void_p]),
    "mgr_batch_set_tuning": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "mgr_batch_formal_solve_fo2_device": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p),
                                                    C.POINTER(C.c_void_p)]),
    "mgr_batch_formal_solve_fo2": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(_f64p), C.POINTER(_f64p)]),
    "mgr_batch_timings": (C.c_int, [C.c_void_p, _f64p, _f64p]),
    "mgr_batch_stream": (C.c_void_p, [C.c_void_p]),
    "mgr_model_set_velocity_device": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mgr_model_set_line_data_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mgr_image_new_smooth_device": (C.c_int, [C.c_void_p, _f64p, C.c_uint32, C.c_uint32, C.c_void_p, _f64p,
                                              _f64p]),
    "mgr_image_new_adjoint_device": (C.c_int, [C.c_void_p, _f64p, C.c_uint32, C.c_uint32, C.c_void_p,
                                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mgr_sync": (C.c_int, [C.c_void_p]),
    "mgr_model_stream": (C.c_void_p, [C.c_void_p]),
    "mgr_launch_count": (C.c_uint64, []),
    "mgr_model_set_frequencies_device": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mgr_model_restore_inputs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "mgr_formal_solve_fo2_smooth_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "mgr_formal_solve_fo2_adjoint_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p,
                                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                      C.c_void_p]),
    "mgr_ali_phase_times": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "mgr_measure_pipe_rate": (C.c_int, [C.c_int, C.c_uint32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                        C.POINTER(C.c_float)]),
}

_lib = None


class MgrError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"magritte_gb300 error {code}: {msg}")
        self.code = code


def load():
    """Load libmgr_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -m magritte_gb300.build` first")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _check(rc):
    if rc != MGR_OK:
        raise MgrError(rc, load().mgr_last_error().decode())


def _ptr(a, t):
    return None if a is None else a.ctypes.data_as(t)


def make_desc(arrays):
    """MgrModelDesc over a dict of numpy arrays/scalars (keys = field names).
    Returns (desc, keepalive list)."""
    desc = MgrModelDesc()
    keep = []
    for name, typ in DESC_FIELDS:
        v = arrays[name] if name not in _FLAGS else int(arrays.get(name, 0))
        if typ in _PTR_TYPES:
            a = np.ascontiguousarray(v, dtype=_PTR_TYPES[typ])
            keep.append(a)
            setattr(desc, name, _ptr(a, typ))
        else:
            setattr(desc, name, v)
    return desc, keep


class DeviceModel:
    """A model resident on the GPU (mgr_model_create / mgr_model_free)."""

    def __init__(self, arrays):
        lib = load()
        self.a = arrays
        self.P = int(arrays["npoints"])
        self.F = int(arrays["nfreqs"])
        self.L = int(arrays["nlines"])
        self.R = int(arrays["hnrays"])
        desc, keep = make_desc(arrays)
        h = C.c_void_p()
        _check(lib.mgr_model_create(C.byref(desc), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            load().mgr_model_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_line_data(self, emissivity=None, opacity=None, inverse_width=None, interp_criterion=None):
        conv = lambda x: None if x is None else np.ascontiguousarray(x, np.float64)
        e, o, i, c = conv(emissivity), conv(opacity), conv(inverse_width), conv(interp_criterion)
        _check(load().mgr_model_set_line_data(self.h, _ptr(e, _f64p), _ptr(o, _f64p), _ptr(i, _f64p),
                                              _ptr(c, _f64p)))

    def ray_lengths_max(self):
        n = C.c_uint32()
        _check(load().mgr_ray_lengths_max(self.h, C.byref(n)))
        return n.value

    def trace(self, o, rr, l, capacity=4096):
        nr = np.zeros(capacity, np.uint32)
        ni = np.zeros(capacity, np.uint32)
        fac = np.zeros(capacity)
        sh = np.zeros(capacity)
        dz = np.zeros(capacity)
        n_tot = C.c_uint32()
        centre = C.c_uint32()
        _check(load().mgr_trace_ray_pair(self.h, o, rr, l, capacity, C.byref(n_tot), C.byref(centre),
                                         _ptr(nr, _u32p), _ptr(ni, _u32p), _ptr(fac, _f64p), _ptr(sh, _f64p),
                                         _ptr(dz, _f64p)))
        n = n_tot.value
        return dict(centre=centre.value, nr=nr[:n].copy(), nr_interp=ni[:n].copy(), interp_factor=fac[:n].copy(),
                    shift=sh[:n].copy(), dZ=dz[:n - 1].copy())

    def formal_solve_fo2(self, precision="fp64", want_u=False, want_lambda=True):
        J = np.empty((self.P, self.F))
        u = np.empty((self.R, self.P, self.F)) if want_u else None
        lam = np.empty((self.P, self.L)) if want_lambda else None
        _check(load().mgr_formal_solve_fo2(self.h, PRECISION[precision], _ptr(J, _f64p), _ptr(u, _f64p),
                                           _ptr(lam, _f64p)))
        return dict(J=J, u=u, lambda_diag=lam)

    def formal_solve_fo2_rays(self, rr_begin, rr_end, precision="fp64", want_lambda=True):
        """Partial J and ALO diagonal summed over the ray pairs [rr_begin, rr_end)."""
        J = np.empty((self.P, self.F))
        lam = np.empty((self.P, self.L)) if want_lambda else None
        _check(load().mgr_formal_solve_fo2_rays(self.h, PRECISION[precision], rr_begin, rr_end, _ptr(J, _f64p),
                                                _ptr(lam, _f64p)))
        return dict(J=J, lambda_diag=lam)

    def formal_solve_fo2_rays_device(self, precision, rr_begin, rr_end, J_dev, lam_dev=None):
        """Enqueue the partial solve of [rr_begin, rr_end) on the model stream (device pointers)."""
        _check(load().mgr_formal_solve_fo2_rays_device(self.h, PRECISION[precision], rr_begin, rr_end,
                                                       C.c_void_p(J_dev), C.c_void_p(lam_dev) if lam_dev else None))

    def set_ray_shard(self, rr_begin, rr_end, reduce=None, capturable=False):
        """Restrict the ALI loop's formal solves to [rr_begin, rr_end); ``reduce`` is a
        Python callable (J_dev, nJ, lam_dev, nlam, stream) -> None that sums the shards
        in place (it may raise).  reduce=None with the full range restores the default."""
        if reduce is None:
            cb = REDUCE_FN()
        else:
            def _cb(user, J, nJ, lam, nlam, stream):
                try:
                    reduce(J, nJ, lam, nlam, stream)
                    return 0
                except Exception as e:  # reported as an error of the ALI call
                    self._shard_error = e
                    return 1
            cb = REDUCE_FN(_cb)
        self._shard_cb = cb  # the library keeps the pointer: hold the thunk
        _check(load().mgr_set_ray_shard(self.h, rr_begin, rr_end, cb, None, int(bool(capturable))))

    def image(self, ray_nr, precision="fp64"):
        I = np.empty((self.P, self.F))
        X, Y = np.empty(self.P), np.empty(self.P)
        _check(load().mgr_image(self.h, PRECISION[precision], ray_nr, _ptr(I, _f64p), _ptr(X, _f64p),
                                _ptr(Y, _f64p)))
        return dict(I=I, ImX=X, ImY=Y)

    def image_for_point(self, ray_nr, p, precision="fp64"):
        """S_ray, dtau_ray, u_ray [n_tot][F] of point p's ray ray_nr."""
        lib = load()
        n = C.c_uint32(0)
        _check(lib.mgr_image_for_point(self.h, PRECISION[precision], ray_nr, p, C.byref(n), None, None, None, 0))
        out = {k: np.empty((n.value, self.F)) for k in ("S_ray", "dtau_ray", "u_ray")}
        _check(lib.mgr_image_for_point(self.h, PRECISION[precision], ray_nr, p, C.byref(n),
                                       _ptr(out["S_ray"], _f64p), _ptr(out["dtau_ray"], _f64p),
                                       _ptr(out["u_ray"], _f64p), n.value))
        return out

    def set_column(self, density):
        """column [nrays][P] of density [P]."""
        rho = np.ascontiguousarray(density, np.float64)
        col = np.empty((int(self.a["nrays"]), self.P))
        _check(load().mgr_set_column(self.h, _ptr(rho, _f64p), _ptr(col, _f64p)))
        return col

    def image_optical_depth(self, ray_nr, precision="fp64"):
        I = np.empty((self.P, self.F))
        X, Y = np.empty(self.P), np.empty(self.P)
        _check(load().mgr_image_optical_depth(self.h, PRECISION[precision], ray_nr, _ptr(I, _f64p), _ptr(X, _f64p),
                                              _ptr(Y, _f64p)))
        return dict(I=I, ImX=X, ImY=Y)

    def image_optical_depth_new(self, raydir, nx, ny, precision="fp64"):
        I = np.empty((nx * ny, self.F))
        X, Y = np.empty(nx * ny), np.empty(nx * ny)
        d = np.ascontiguousarray(raydir, np.float64)
        _check(load().mgr_image_optical_depth_new(self.h, PRECISION[precision], _ptr(d, _f64p), nx, ny,
                                                  _ptr(I, _f64p), _ptr(X, _f64p), _ptr(Y, _f64p)))
        return dict(I=I, ImX=X, ImY=Y)

    def image_new(self, raydir, nx, ny, precision="fp64"):
        I = np.empty((nx * ny, self.F))
        X, Y = np.empty(nx * ny), np.empty(nx * ny)
        d = np.ascontiguousarray(raydir, np.float64)
        _check(load().mgr_image_new(self.h, PRECISION[precision], _ptr(d, _f64p), nx, ny, _ptr(I, _f64p),
                                    _ptr(X, _f64p), _ptr(Y, _f64p)))
        return dict(I=I, ImX=X, ImY=Y)

    def formal_solve_sc0(self, precision="fp64", want_I=False, want_uv=False, want_lambda=True):
        J = np.empty((self.P, self.F))
        I = np.empty((2 * self.R, self.P, self.F)) if want_I else None
        u = np.empty((self.R, self.P, self.F)) if want_uv else None
        v = np.empty((self.R, self.P, self.F)) if want_uv else None
        lam = np.empty((self.P, self.L)) if want_lambda else None
        _check(load().mgr_formal_solve_sc0(self.h, PRECISION[precision], _ptr(J, _f64p), _ptr(I, _f64p),
                                           _ptr(u, _f64p), _ptr(v, _f64p), _ptr(lam, _f64p)))
        return dict(J=J, I=I, u=u, v=v, lambda_diag=lam)

    def formal_solve_fo2_device(self, precision, J_dev, u_dev=None, lam_dev=None):
        """Enqueue on the model stream with device pointers (ints); no synchronisation."""
        _check(load().mgr_formal_solve_fo2_device(self.h, PRECISION[precision], C.c_void_p(J_dev),
                                                  C.c_void_p(u_dev) if u_dev else None,
                                                  C.c_void_p(lam_dev) if lam_dev else None))

    def set_n_off_diag(self, n_off_diag):
        """Parameters::n_off_diag: band elements of the non-local ALO on each side."""
        _check(load().mgr_model_set_n_off_diag(self.h, int(n_off_diag)))
        self.n_off_diag = int(n_off_diag)

    def formal_solve_fo2_alo(self):
        """The banded FP64 formal solve (n_off_diag > 0): J [P][F], u [hnrays][P][F], the
        ALO diagonal [P][L] and the band elements alo_off / alo_nr [P][L][hnrays][2 n_off_diag]."""
        import torch

        K = getattr(self, "n_off_diag", 0)
        dev = torch.device("cuda")
        J = torch.empty((self.P, self.F), dtype=torch.float64, device=dev)
        lam = torch.empty((self.P, self.L), dtype=torch.float64, device=dev)
        off = torch.empty((self.P, self.L, self.R, 2 * max(K, 1)), dtype=torch.float64, device=dev)
        nr = torch.empty((self.P, self.L, self.R, 2 * max(K, 1)), dtype=torch.int32, device=dev)
        u = torch.empty((self.R, self.P, self.F), dtype=torch.float64, device=dev)
        torch.cuda.synchronize(dev)
        _check(load().mgr_formal_solve_fo2_alo_device(self.h, C.c_void_p(J.data_ptr()), C.c_void_p(u.data_ptr()),
                                                      C.c_void_p(lam.data_ptr()), C.c_void_p(off.data_ptr()),
                                                      C.c_void_p(nr.data_ptr())))
        self.sync()
        return dict(J=J.cpu().numpy(), u=u.cpu().numpy(), lambda_diag=lam.cpu().numpy(), alo_off=off.cpu().numpy(),
                    alo_nr=nr.cpu().numpy().view(np.uint32))

    def ray_statistics(self):
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(load().mgr_ray_statistics(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return dict(steps=a.value, neighbor_reads=b.value, elements=c.value)

    def sync(self):
        _check(load().mgr_sync(self.h))

    def autotune(self, precision="split", sample_points=0):
        return autotune(self.h, precision, sample_points)

    def stream(self):
        """The model's CUDA stream handle (cudaStream_t as an int)."""
        return load().mgr_model_stream(self.h)

    # ---- level populations ----
    def set_species(self, linedata, abundance, populations):
        """Attach line-producing species (``magritte_gb300.synthetic.Linedata`` list),
        abundances [P][nspecs] and populations (list of [P][nlev])."""
        keep = []

        def arr(x, dt):
            a = np.ascontiguousarray(x, dtype=dt)
            keep.append(a)
            return a

        sp = (MgrSpeciesDesc * len(linedata))()
        for l, ld in enumerate(linedata):
            cps = (MgrCollisionPartnerDesc * max(1, len(ld.colpar)))()
            keep.append(cps)
            for c, cp in enumerate(ld.colpar):
                cps[c].num_col_partner = cp.num_col_partner
                cps[c].ortho_para = {"n": 0, "o": 1, "p": 2}[cp.orth_or_para_H2]
                cps[c].ncol, cps[c].ntmp = cp.ncol, cp.ntmp
                cps[c].icol = _ptr(arr(cp.icol, np.uint32), _u32p)
                cps[c].jcol = _ptr(arr(cp.jcol, np.uint32), _u32p)
                cps[c].tmp = _ptr(arr(cp.tmp, np.float64), _f64p)
                cps[c].Cd = _ptr(arr(cp.Cd, np.float64), _f64p)
                cps[c].Ce = _ptr(arr(cp.Ce, np.float64), _f64p)
            d = sp[l]
            d.num, d.nlev, d.nrad, d.ncolpar = ld.num, ld.nlev, ld.nrad, len(ld.colpar)
            d.energy = _ptr(arr(ld.energy, np.float64), _f64p)
            d.weight = _ptr(arr(ld.weight, np.float64), _f64p)
            d.irad = _ptr(arr(ld.irad, np.uint32), _u32p)
            d.jrad = _ptr(arr(ld.jrad, np.uint32), _u32p)
            d.A = _ptr(arr(ld.A, np.float64), _f64p)
            d.Bs = _ptr(arr(ld.Bs, np.float64), _f64p)
            d.Ba = _ptr(arr(ld.Ba, np.float64), _f64p)
            d.frequency = _ptr(arr(ld.frequency, np.float64), _f64p)
            d.colpar = cps
        ab = arr(abundance, np.float64)
        pops = [arr(p, np.float64) for p in populations]
        pp = (_f64p * len(pops))(*[_ptr(p, _f64p) for p in pops])
        self.nlev = [ld.nlev for ld in linedata]
        self.nrad = [ld.nrad for ld in linedata]
        _check(load().mgr_model_set_species(self.h, len(linedata), sp, ab.shape[1], _ptr(ab, _f64p), pp))

    def compute_jeff(self, l=0):
        out = [np.empty((self.P, self.nrad[l])) for _ in range(3)]
        _check(load().mgr_compute_jeff(self.h, l, *[_ptr(o, _f64p) for o in out]))
        return dict(Jlin=out[0], Jeff=out[1], Jdif=out[2])

    def formal_solve_fo2_sparse(self, precision="fp64"):
        """Memory-lean solve: line-integrated J [P][L] and ALO diagonal [P][L]."""
        Jl = np.empty((self.P, self.L))
        lam = np.empty((self.P, self.L))
        _check(load().mgr_formal_solve_fo2_sparse(self.h, PRECISION[precision], _ptr(Jl, _f64p), _ptr(lam, _f64p)))
        return dict(Jlin=Jl, lambda_diag=lam)

    def formal_solve_fo2_uv(self, precision="fp64"):
        u = np.empty((self.R, self.P, self.F))
        v = np.empty((self.R, self.P, self.F))
        _check(load().mgr_formal_solve_fo2_uv(self.h, PRECISION[precision], _ptr(u, _f64p), _ptr(v, _f64p)))
        return dict(u=u, v=v)

    def formal_solve_fo2_anis(self, precision="fp64"):
        """Anisotropic solve: line-integrated J and the J2 tensor elements [P][L]."""
        keys = ("J", "J2_0", "J2_1_Re", "J2_1_Im", "J2_2_Re", "J2_2_Im")
        out = {k: np.empty((self.P, self.L)) for k in keys}
        _check(load().mgr_formal_solve_fo2_anis(self.h, PRECISION[precision], *[_ptr(out[k], _f64p) for k in keys]))
        return out

    def compute_jeff_sparse(self, l=0):
        out = {k: np.empty((self.P, self.nrad[l])) for k in ("Jlin", "Jeff")}
        _check(load().mgr_compute_jeff_sparse(self.h, l, _ptr(out["Jlin"], _f64p), _ptr(out["Jeff"], _f64p)))
        return out

    def compute_level_populations_sparse(self, precision="fp64", use_ng=True, max_it=100, **params):
        return self.compute_level_populations(precision, use_ng, max_it, _sparse=True, **params)

    def compute_level_populations(self, precision="fp64", use_ng=True, max_it=100, _sparse=False, **params):
        prm = dict(ALI_DEFAULTS)
        prm.update(params)
        p = MgrAliParams(**prm)
        it = C.c_int()
        cap = max_it * len(self.nlev)
        em, ex = np.zeros(cap), np.zeros(cap)
        self._shard_error = None
        try:
            fn = load().mgr_compute_level_populations_sparse if _sparse else load().mgr_compute_level_populations
            _check(fn(self.h, PRECISION[precision], int(use_ng), max_it, C.byref(p), C.byref(it), _ptr(em, _f64p),
                      _ptr(ex, _f64p), cap))
        except MgrError as e:
            if self._shard_error is not None:
                raise e from self._shard_error
            raise
        n = it.value * len(self.nlev)
        return dict(iterations=it.value, error_mean=em[:n], error_max=ex[:n])

    def populations(self, l=0):
        out = np.empty((self.P, self.nlev[l]))
        _check(load().mgr_get_populations(self.h, l, _ptr(out, _f64p)))
        return out

    def line_data(self):
        em, op = np.empty((self.P, self.L)), np.empty((self.P, self.L))
        _check(load().mgr_get_line_data(self.h, _ptr(em, _f64p), _ptr(op, _f64p)))
        return em, op


class Batch:
    """Many DeviceModels solved in one persistent launch (mgr_batch_*).  The models
    must stay open while the batch is used."""

    def __init__(self, devs):
        lib = load()
        self.devs = list(devs)
        hs = (C.c_void_p * len(self.devs))(*[d.h.value for d in self.devs])
        h = C.c_void_p()
        _check(lib.mgr_batch_create(hs, len(self.devs), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            load().mgr_batch_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tuning(self, min_blocks_per_sm=0, warps_per_block=0):
        _check(load().mgr_batch_set_tuning(self.h, min_blocks_per_sm, warps_per_block))

    def formal_solve_fo2(self, precision="fp64", want_lambda=True):
        n = len(self.devs)
        Js = [np.empty((d.P, d.F)) for d in self.devs]
        Ls = [np.empty((d.P, d.L)) if want_lambda else None for d in self.devs]
        Jp = (_f64p * n)(*[_ptr(x, _f64p) for x in Js])
        Lp = (_f64p * n)(*[_ptr(x, _f64p) for x in Ls]) if want_lambda else None
        _check(load().mgr_batch_formal_solve_fo2(self.h, PRECISION[precision], Jp, Lp))
        return [dict(J=J, lambda_diag=L) for J, L in zip(Js, Ls)]

    def formal_solve_fo2_device(self, precision, J_ptrs, lam_ptrs=None):
        """Enqueue on the batch stream with lists of device pointers (ints)."""
        n = len(self.devs)
        Jp = (C.c_void_p * n)(*J_ptrs)
        Lp = (C.c_void_p * n)(*lam_ptrs) if lam_ptrs is not None else None
        _check(load().mgr_batch_formal_solve_fo2_device(self.h, PRECISION[precision], Jp, Lp))

    def timings(self):
        """(start_ms, finish_ms) per model of the last solve, since the launch began."""
        n = len(self.devs)
        s, f = np.empty(n), np.empty(n)
        _check(load().mgr_batch_timings(self.h, _ptr(s, _f64p), _ptr(f, _f64p)))
        return s, f

    def stream(self):
        return load().mgr_batch_stream(self.h)


def autotune(handle, precision="split", sample_points=0):
    """Pick the fastest launch shape of the formal solve for this model (mgr_autotune_fo2)."""
    mb, w, ms = C.c_int(), C.c_int(), C.c_float()
    _check(load().mgr_autotune_fo2(handle, PRECISION[precision], sample_points, C.byref(mb), C.byref(w),
                                   C.byref(ms)))
    return {"min_blocks_per_sm": mb.value, "warps_per_block": w.value, "sample_ms": ms.value}


PIPE_KINDS = {"dfma": 0, "dadd": 1, "dmul": 2, "dsetp": 3, "f2f": 4, "mufu_rcp64": 5}


def pipe_rate(kind, iterations=4096):
    """Measured rate of one instruction kind (mgr_measure_pipe_rate): thread operations
    per second, per SM clock per SM, and the probe's launch time in ms."""
    ops, per_clk, ms = C.c_double(), C.c_double(), C.c_float()
    _check(load().mgr_measure_pipe_rate(PIPE_KINDS[kind], iterations, C.byref(ops), C.byref(per_clk), C.byref(ms)))
    return dict(thread_ops_per_s=ops.value, thread_ops_per_clk_per_sm=per_clk.value, ms=ms.value)


def launch_count():
    return int(load().mgr_launch_count())


def device_count():
    n = C.c_int()
    rc = load().mgr_device_count(C.byref(n))
    return n.value if rc == MGR_OK else 0
