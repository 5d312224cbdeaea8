"""Oracle for the Magritte formal-solve hot path -- TEST INFRASTRUCTURE ONLY.

Two parts:
  * ``reference_setup``: a numpy restatement of the reference's model set-up
    (Model::compute_spectral_discretisation, model.cpp:70-161; LTE populations,
    lineProducingSpecies.tpp:52-75; emissivity/opacity, :23-44;
    Lines::set_inverse_width, lines.tpp:45-59; Model::set_dshift_max,
    model.cpp:1158-1178; InterpHelper criterion, solver_interp_helper.hpp:15-24).
    Populations are kept in double precision where the reference keeps long double.
  * ctypes bindings to ``_build/libmgr_oracle.so`` (mgr_oracle.c).

Only the test-suite, the smoke check and bench.py's CPU-baseline leg use this
module; the product library never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmgr_oracle.so")

CC = 2.99792458e8
HH = 6.62607004e-34
KB = 1.38064852e-23
AMU = 1.66053904e-27
CC_SQUARED = 8.98755179e16
TWO_KB_OVER_AMU_CC_SQUARED = 2.0 * KB / (AMU * CC_SQUARED)
HH_OVER_FOUR_PI = HH / (4.0 * np.pi)

APPROX = {"None": 0, "OneLine": 1, "CloseLines": 2}


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()  # make is incremental: rebuilds a library older than its sources
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


# ---------------------------------------------------------------------------
# Reference model set-up (numpy restatement)
# ---------------------------------------------------------------------------
def reference_setup(raw, approx="CloseLines", max_width_fraction=0.35, min_opacity=1.0e-26,
                    min_line_opacity=1.0e-13, min_line_emissivity=1.0e-50, min_dtau=1.0e-15,
                    max_interpolation_diff=1.4, max_distance_opacity_contribution=10.0,
                    populations=None, image_freqs=None):
    """Arrays of the OrcModel struct for a ``magritte_gb300.synthetic.RawModel``.
    ``populations`` (list per species of [P, nlev]) overrides the LTE populations.
    ``image_freqs = (nu_min, nu_max, n)`` selects the imaging spectral discretisation
    (model.cpp:229-275): n evenly spaced frequencies, the same at every point."""
    P = raw.npoints
    nrays = raw.nrays
    Q = raw.nquads
    lds = raw.linedata
    nlspecs = len(lds)
    nrad = np.array([ld.nrad for ld in lds], dtype=np.uint32)
    nrad_cum = np.zeros(nlspecs, dtype=np.uint32)
    for l in range(1, nlspecs):
        nrad_cum[l] = nrad_cum[l - 1] + nrad[l - 1]
    L = int(nrad.sum())
    F = L * Q
    line = np.concatenate([ld.frequency for ld in lds]).astype(np.float64)
    # Lines::read sorts with heapsort (lines.cpp:43-61); a stable sort gives the same
    # order for distinct line frequencies.
    sorted_line_map = np.argsort(line, kind="stable").astype(np.uint32)
    sorted_line = line[sorted_line_map].copy()
    max_inverse_mass = max(ld.inverse_mass for ld in lds)
    T = raw.temperature.astype(np.float64)
    vt2 = raw.vturb2.astype(np.float64)

    # compute_spectral_discretisation (model.cpp:70-161)
    nu = np.zeros((P, F))
    corr_line = np.zeros(F, np.uint32)
    corr_lspec = np.zeros(F, np.uint32)
    corr_k = np.zeros(F, np.uint32)
    corr_z = np.zeros(F, np.uint32)
    in_line = np.ones(F, np.uint8)
    for l, ld in enumerate(lds):
        pw = np.sqrt(TWO_KB_OVER_AMU_CC_SQUARED * ld.inverse_mass * T + vt2)
        for k in range(ld.nrad):
            lid = int(nrad_cum[l]) + k
            width = line[lid] * pw
            for z in range(Q):
                f = lid * Q + z
                nu[:, f] = line[lid] + width * raw.quad_roots[l][z]
                corr_line[f] = lid
                corr_lspec[f] = l
                corr_k[f] = k
                corr_z[f] = z

    if image_freqs is not None:
        nu_min, nu_max, n = image_freqs
        F = int(n)
        # long double step as the reference (model.cpp:257-262)
        dnu = (np.longdouble(nu_max) - np.longdouble(nu_min)) / (F - 1) if F > 1 else np.longdouble(0)
        row = (np.array([float(np.longdouble(nu_min) + f * dnu) for f in range(F)]) if F > 1
               else np.array([(nu_min + nu_max) / 2.0]))
        nu = np.tile(row, (P, 1))
        corr_line = np.zeros(F, np.uint32)  # not set by the reference for this discretisation
        corr_lspec = np.full(F, F, np.uint32)
        corr_k = np.full(F, F, np.uint32)
        corr_z = np.full(F, F, np.uint32)
        in_line = np.zeros(F, np.uint8)

    # LTE populations (lineProducingSpecies.tpp:52-75) and emissivity/opacity (:23-44)
    emissivity = np.zeros((P, L))
    opacity = np.zeros((P, L))
    inverse_width = np.zeros((P, L))
    criterion = np.zeros((P, L))
    pops = []
    for l, ld in enumerate(lds):
        pop_tot = raw.abundance[:, ld.num].astype(np.float64)
        if populations is None:
            pop = ld.weight[None, :] * np.exp(-ld.energy[None, :] / (KB * T[:, None]))
            pf = np.zeros(P)
            for i in range(ld.nlev):
                pf = pf + pop[:, i]
            pop = pop * (pop_tot / pf)[:, None]
        else:
            pop = np.asarray(populations[l], dtype=np.float64)
        pops.append(pop)
        freq = ld.frequency
        for k in range(ld.nrad):
            lid = int(nrad_cum[l]) + k
            i, j = int(ld.irad[k]), int(ld.jrad[k])
            em = freq[k] * HH_OVER_FOUR_PI * ld.A[k] * pop[:, i]
            op = freq[k] * HH_OVER_FOUR_PI * (pop[:, j] * ld.Ba[k] - pop[:, i] * ld.Bs[k])
            emissivity[:, lid] = np.maximum(em, min_line_emissivity)
            opacity[:, lid] = np.maximum(op, min_line_opacity)
            inverse_width[:, lid] = 1.0 / (freq[k] * np.sqrt(TWO_KB_OVER_AMU_CC_SQUARED * ld.inverse_mass * T + vt2))
            criterion[:, lid] = opacity[:, lid] / pop_tot

    # set_dshift_max (model.cpp:1158-1178)
    dshift_max = np.full(P, np.finfo(np.float64).max)
    for ld in lds:
        cand = max_width_fraction * np.sqrt(TWO_KB_OVER_AMU_CC_SQUARED * ld.inverse_mass * T + vt2)
        dshift_max = np.minimum(dshift_max, cand)

    from magritte_gb300.healpix import antipodes  # geometry helper shared with the host side

    cum = np.zeros(P, np.uint32)
    cum[1:] = np.cumsum(raw.n_neighbors.astype(np.uint64))[:-1].astype(np.uint32)
    p2b = np.full(P, P, np.uint32)
    p2b[raw.boundary2point] = np.arange(len(raw.boundary2point), dtype=np.uint32)

    return dict(
        npoints=P, nrays=nrays, hnrays=nrays // 2, nlines=L, nquads=Q, nfreqs=F, nlspecs=nlspecs,
        nboundary=len(raw.boundary2point),
        position=np.ascontiguousarray(raw.position, np.float64),
        velocity=np.ascontiguousarray(raw.velocity, np.float64),
        n_neighbors=np.ascontiguousarray(raw.n_neighbors, np.uint32), cum_n_neighbors=cum,
        neighbors=np.ascontiguousarray(raw.neighbors, np.uint32), point2boundary=p2b,
        boundary_condition=np.ascontiguousarray(raw.boundary_condition, np.int32),
        boundary_temperature=np.ascontiguousarray(raw.boundary_temperature, np.float64),
        # adaptive ray directions: per point [P][nrays] (rays.cpp:94-146); the antipode
        # table is shared by all points
        ray_direction=np.ascontiguousarray(raw.ray_direction if raw.adaptive_direction is None
                                           else raw.adaptive_direction.reshape(-1, 3), np.float64),
        ray_weight=np.ascontiguousarray(raw.ray_weight if raw.adaptive_weight is None
                                        else raw.adaptive_weight.reshape(-1), np.float64),
        antipod=antipodes(raw.ray_direction),
        use_adaptive_directions=int(raw.adaptive_direction is not None),
        line=line, sorted_line=sorted_line, sorted_line_map=sorted_line_map,
        max_inverse_mass=float(max_inverse_mass),
        emissivity=emissivity, opacity=opacity, inverse_width=inverse_width, interp_criterion=criterion,
        temperature=T, vturb2=vt2, dshift_max=dshift_max, nu=nu,
        corr_line=corr_line, corr_lspec=corr_lspec, corr_k=corr_k, corr_z=corr_z, in_line_integral=in_line,
        nrad=nrad, nrad_cum=nrad_cum,
        line_A=np.concatenate([ld.A for ld in lds]).astype(np.float64),
        lspec_inverse_mass=np.array([ld.inverse_mass for ld in lds], np.float64),
        quad_weights=np.ascontiguousarray(np.stack(raw.quad_weights), np.float64),
        quad_roots=np.ascontiguousarray(np.stack(raw.quad_roots), np.float64),
        min_opacity=min_opacity, min_dtau=min_dtau, max_interpolation_diff=max_interpolation_diff,
        max_distance_opacity_contribution=max_distance_opacity_contribution,
        approx=APPROX[approx], spherical_symmetry=int(bool(getattr(raw, "spherical_symmetry", False))),
        populations=pops,
    )


# ---------------------------------------------------------------------------
# ctypes
# ---------------------------------------------------------------------------
_u32p = C.POINTER(C.c_uint32)
_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)

_FIELDS = [
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
    ("max_distance_opacity_contribution", C.c_double), ("approx", C.c_int), ("spherical_symmetry", C.c_int),
    ("use_adaptive_directions", C.c_int),
]


_FLAGS = ("spherical_symmetry", "use_adaptive_directions")


class OrcModel(C.Structure):
    _fields_ = _FIELDS


class OrcRay(C.Structure):
    _fields_ = [("capacity", C.c_uint32), ("centre", C.c_uint32), ("first", C.c_uint32),
                ("last", C.c_uint32), ("nr", _u32p), ("nr_interp", _u32p), ("interp_factor", _f64p),
                ("shift", _f64p), ("dZ", _f64p)]


def set_erf_mode(mode):
    """0: libm erff as the reference (default); 1: correctly rounded erff (GPU FP64 mode)."""
    lib().orc_set_erf_mode(int(mode))


def set_smooth(on):
    """Smooth arithmetic for gradient checks: pow / exp / expm1 / erf in double
    precision instead of the reference's single-precision calls (off by default)."""
    lib().orc_set_smooth(int(bool(on)))


def _declare(l):
    l.orc_set_erf_mode.restype = None
    l.orc_set_erf_mode.argtypes = [C.c_int]
    l.orc_set_smooth.restype = None
    l.orc_set_smooth.argtypes = [C.c_int]
    l.orc_ray_lengths_max.restype = C.c_uint32
    l.orc_ray_lengths_max.argtypes = [C.POINTER(OrcModel), C.c_int]
    l.orc_trace_ray_pair_for_line.restype = C.c_int
    l.orc_trace_ray_pair_for_line.argtypes = [C.POINTER(OrcModel), C.c_uint32, C.c_uint32, C.c_uint32,
                                              C.POINTER(OrcRay)]
    l.orc_formal_solve_fo2.restype = C.c_int
    l.orc_formal_solve_fo2.argtypes = [C.POINTER(OrcModel), _f64p, _f64p, _f64p, _u8p, C.c_int]
    l.orc_formal_solve_fo2_range.restype = C.c_int
    l.orc_formal_solve_fo2_range.argtypes = [C.POINTER(OrcModel), C.c_uint32, C.c_uint32, C.c_uint32,
                                             C.c_uint32, _f64p, C.c_int]
    l.orc_formal_solve_fo2_origins.restype = C.c_int
    l.orc_formal_solve_fo2_origins.argtypes = [C.POINTER(OrcModel), _u32p, C.c_uint32, _f64p, _f64p, _u8p,
                                               C.c_int]
    l.orc_formal_solve_sc0.restype = C.c_int
    l.orc_formal_solve_sc0.argtypes = [C.POINTER(OrcModel), _f64p, _f64p, _f64p, _f64p, _f64p, _u8p, C.c_int]
    l.orc_image_fo2.restype = C.c_int
    l.orc_image_fo2.argtypes = [C.POINTER(OrcModel), C.c_uint32, _f64p, C.c_int]


def _ptr(a, t):
    return a.ctypes.data_as(t) if a is not None else None


class Oracle:
    """Holds an OrcModel and the numpy arrays it points into."""

    def __init__(self, arrays):
        self.a = arrays
        self.m = OrcModel()
        for name, typ in _FIELDS:
            v = arrays[name] if name not in _FLAGS else int(arrays.get(name, 0))
            if typ in (_u32p, _i32p, _f64p, _u8p):
                setattr(self.m, name, _ptr(v, typ))
            else:
                setattr(self.m, name, v)

    def ray_lengths_max(self, nthreads=0):
        return lib().orc_ray_lengths_max(C.byref(self.m), nthreads)

    def trace(self, o, rr, l, capacity=None):
        if capacity is None:
            capacity = 2 * self.ray_lengths_max() + 1
        nr = np.zeros(capacity, np.uint32)
        ni = np.zeros(capacity, np.uint32)
        fac = np.zeros(capacity)
        sh = np.zeros(capacity)
        dz = np.zeros(capacity)
        ray = OrcRay(capacity, 0, 0, 0, _ptr(nr, _u32p), _ptr(ni, _u32p), _ptr(fac, _f64p), _ptr(sh, _f64p),
                     _ptr(dz, _f64p))
        rc = lib().orc_trace_ray_pair_for_line(C.byref(self.m), o, rr, l, C.byref(ray))
        if rc != 0:
            raise RuntimeError(f"oracle trace failed ({rc})")
        s = slice(ray.first, ray.last + 1)
        return dict(centre=ray.centre - ray.first, nr=nr[s].copy(), nr_interp=ni[s].copy(),
                    interp_factor=fac[s].copy(), shift=sh[s].copy(), dZ=dz[ray.first:ray.last].copy())

    def formal_solve_fo2(self, want_u=False, nthreads=0):
        P, F, L, R = self.a["npoints"], self.a["nfreqs"], self.a["nlines"], self.a["hnrays"]
        J = np.zeros((P, F))
        u = np.zeros((R, P, F)) if want_u else None
        lam = np.zeros((P, L))
        has = np.zeros((P, L), np.uint8)
        rc = lib().orc_formal_solve_fo2(C.byref(self.m), _ptr(J, _f64p), _ptr(u, _f64p), _ptr(lam, _f64p),
                                        _ptr(has, _u8p), nthreads)
        if rc != 0:
            raise RuntimeError(f"oracle formal solve failed ({rc})")
        return dict(J=J, u=u, lambda_diag=lam, lambda_has=has)

    def formal_solve_fo2_uv(self, nthreads=0):
        P, F, R = self.a["npoints"], self.a["nfreqs"], self.a["hnrays"]
        u = np.zeros((R, P, F))
        v = np.zeros((R, P, F))
        l = lib()
        l.orc_formal_solve_fo2_uv.restype = C.c_int
        l.orc_formal_solve_fo2_uv.argtypes = [C.POINTER(OrcModel), _f64p, _f64p, C.c_int]
        rc = l.orc_formal_solve_fo2_uv(C.byref(self.m), _ptr(u, _f64p), _ptr(v, _f64p), nthreads)
        if rc != 0:
            raise RuntimeError(f"oracle uv solve failed ({rc})")
        return dict(u=u, v=v)

    def formal_solve_fo2_anis(self):
        """Solver::solve_feautrier_order_2_anis (solver.tpp:366-456) from this oracle's u:
        per line, du = (w_z w_rr) u, J += 2 du and the J2 tensor elements += wt_x(n) du,
        ray pair outer, quadrature point inner.  Returns [P][L] arrays."""
        a = self.a
        P, L, R = a["npoints"], a["nlines"], a["hnrays"]
        u = self.formal_solve_fo2(want_u=True)["u"]
        sqrt3, inv_sqrt2 = np.sqrt(3.0), 1.0 / np.sqrt(2.0)
        out = {k: np.zeros((P, L)) for k in ("J", "J2_0", "J2_1_Re", "J2_1_Im", "J2_2_Re", "J2_2_Im")}
        fq = [[None] * a["nquads"] for _ in range(L)]
        for f in range(a["nfreqs"]):
            fq[a["corr_line"][f]][a["corr_z"][f]] = f
        nrays = a["nrays"]
        adaptive = int(a.get("use_adaptive_directions", 0))
        for rr in range(R):
            # Rays::get_direction / get_weight (rays.cpp:94-146): per point when adaptive
            if adaptive:
                nx, ny, nz = a["ray_direction"].reshape(P, nrays, 3)[:, rr].T
                wt = a["ray_weight"].reshape(P, nrays)[:, rr]
            else:
                nx, ny, nz = a["ray_direction"][rr]
                wt = a["ray_weight"][rr]
            w = {"J2_0": inv_sqrt2 * (3.0 * nz * nz - 1.0), "J2_1_Re": -sqrt3 * nx * nz,
                 "J2_1_Im": -sqrt3 * ny * nz, "J2_2_Re": 0.5 * sqrt3 * (nx * nx - ny * ny),
                 "J2_2_Im": sqrt3 * nx * ny}
            for l in range(L):
                for z in range(a["nquads"]):
                    f = fq[l][z]
                    du = (a["quad_weights"][a["corr_lspec"][f], z] * wt) * u[rr, :, f]
                    out["J"][:, l] += 2.0 * du
                    for k, wk in w.items():
                        out[k][:, l] += wk * du
        return out

    def formal_solve_fo2_range(self, rr0, rr1, o0, o1, nthreads=0):
        P, F = self.a["npoints"], self.a["nfreqs"]
        J = np.zeros((P, F))
        rc = lib().orc_formal_solve_fo2_range(C.byref(self.m), rr0, rr1, o0, o1, _ptr(J, _f64p), nthreads)
        if rc != 0:
            raise RuntimeError(f"oracle formal solve failed ({rc})")
        return J

    def formal_solve_fo2_origins(self, origins, nthreads=0):
        """J [n][F] and the ALO diagonal [n][L] at the given origins (every ray pair)."""
        P, F, L = self.a["npoints"], self.a["nfreqs"], self.a["nlines"]
        orig = np.ascontiguousarray(origins, np.uint32)
        J = np.zeros((P, F))
        lam = np.zeros((P, L))
        has = np.zeros((P, L), np.uint8)
        rc = lib().orc_formal_solve_fo2_origins(C.byref(self.m), _ptr(orig, _u32p), len(orig), _ptr(J, _f64p),
                                                _ptr(lam, _f64p), _ptr(has, _u8p), nthreads)
        if rc != 0:
            raise RuntimeError(f"oracle formal solve failed ({rc})")
        return dict(J=J[orig], lambda_diag=lam[orig])

    def formal_solve_sc0(self, nthreads=0):
        P, F, L, R = self.a["npoints"], self.a["nfreqs"], self.a["nlines"], self.a["hnrays"]
        J = np.zeros((P, F))
        I = np.zeros((2 * R, P, F))
        u = np.zeros((R, P, F))
        v = np.zeros((R, P, F))
        lam = np.zeros((P, L))
        has = np.zeros((P, L), np.uint8)
        rc = lib().orc_formal_solve_sc0(C.byref(self.m), _ptr(J, _f64p), _ptr(I, _f64p), _ptr(u, _f64p),
                                        _ptr(v, _f64p), _ptr(lam, _f64p), _ptr(has, _u8p), nthreads)
        if rc != 0:
            raise RuntimeError(f"oracle short-char solve failed ({rc})")
        return dict(J=J, I=I, u=u, v=v, lambda_diag=lam, lambda_has=has)

    def image_new(self, raydir, nx, ny, nthreads=0):
        P, F = self.a["npoints"], self.a["nfreqs"]
        I = np.zeros((nx * ny, F))
        X = np.zeros(nx * ny)
        Y = np.zeros(nx * ny)
        d = np.ascontiguousarray(raydir, np.float64)
        l = lib()
        l.orc_image_new.restype = C.c_int
        l.orc_image_new.argtypes = [C.POINTER(OrcModel), _f64p, C.c_uint32, C.c_uint32, _f64p, _f64p, _f64p, C.c_int]
        rc = l.orc_image_new(C.byref(self.m), _ptr(d, _f64p), nx, ny, _ptr(I, _f64p), _ptr(X, _f64p),
                             _ptr(Y, _f64p), nthreads)
        if rc != 0:
            raise RuntimeError(f"oracle new imager failed ({rc})")
        return dict(I=I, ImX=X, ImY=Y)

    def image_optical_depth(self, rr, nthreads=0):
        P, F = self.a["npoints"], self.a["nfreqs"]
        I = np.zeros((P, F))
        l = lib()
        l.orc_image_optical_depth.restype = C.c_int
        l.orc_image_optical_depth.argtypes = [C.POINTER(OrcModel), C.c_uint32, _f64p, C.c_int]
        rc = l.orc_image_optical_depth(C.byref(self.m), rr, _ptr(I, _f64p), nthreads)
        if rc != 0:
            raise RuntimeError(f"oracle optical-depth imager failed ({rc})")
        return I

    def image_optical_depth_new(self, raydir, nx, ny, nthreads=0):
        F = self.a["nfreqs"]
        I = np.zeros((nx * ny, F))
        X = np.zeros(nx * ny)
        Y = np.zeros(nx * ny)
        d = np.ascontiguousarray(raydir, np.float64)
        l = lib()
        l.orc_image_optical_depth_new.restype = C.c_int
        l.orc_image_optical_depth_new.argtypes = [C.POINTER(OrcModel), _f64p, C.c_uint32, C.c_uint32, _f64p, _f64p,
                                                  _f64p, C.c_int]
        rc = l.orc_image_optical_depth_new(C.byref(self.m), _ptr(d, _f64p), nx, ny, _ptr(I, _f64p), _ptr(X, _f64p),
                                           _ptr(Y, _f64p), nthreads)
        if rc != 0:
            raise RuntimeError(f"oracle optical-depth new imager failed ({rc})")
        return dict(I=I, ImX=X, ImY=Y)

    def image_for_point(self, rr, p):
        """Solver::image_feautrier_order_2_for_point (solver.tpp:629-653): S_ray, dtau_ray,
        u_ray [n_tot][F] of point p's ray rr (zeros for a ray of one element)."""
        F = self.a["nfreqs"]
        l = lib()
        l.orc_image_for_point.restype = C.c_int
        l.orc_image_for_point.argtypes = [C.POINTER(OrcModel), C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32),
                                          _f64p, _f64p, _f64p, C.c_uint32]
        n = C.c_uint32(0)
        rc = l.orc_image_for_point(C.byref(self.m), rr, p, C.byref(n), None, None, None, 0)
        if rc not in (0, -3):
            raise RuntimeError(f"oracle image_for_point failed ({rc})")
        out = {k: np.zeros((n.value, F)) for k in ("S_ray", "dtau_ray", "u_ray")}
        rc = l.orc_image_for_point(C.byref(self.m), rr, p, C.byref(n), _ptr(out["S_ray"], _f64p),
                                   _ptr(out["dtau_ray"], _f64p), _ptr(out["u_ray"], _f64p), n.value)
        if rc != 0:
            raise RuntimeError(f"oracle image_for_point failed ({rc})")
        return out

    def formal_solve_fo2_alo(self, n_off_diag, nthreads=0):
        """The formal solve with n_off_diag > 0 (solver.tpp:2319-2355) and its non-local
        ALO (update_Lambda, solver.tpp:1760-1850): J [P][F] and the Lambda lists per
        (point, line): n [P][L], nr / Ls [P][L][cap], in the reference's insertion order."""
        l = lib()
        l.orc_formal_solve_fo2_alo.restype = C.c_int
        l.orc_formal_solve_fo2_alo.argtypes = [C.POINTER(OrcModel), C.c_uint32, _f64p, C.c_uint32,
                                               C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), _f64p, C.c_int]
        P, F, L = self.a["npoints"], self.a["nfreqs"], self.a["nlines"]
        cap = 2 * n_off_diag * self.a["hnrays"] + 1
        J = np.zeros((P, F))
        n = np.zeros((P, L), np.uint32)
        nr = np.zeros((P, L, cap), np.uint32)
        ls = np.zeros((P, L, cap))
        rc = l.orc_formal_solve_fo2_alo(C.byref(self.m), n_off_diag, _ptr(J, _f64p), cap,
                                        n.ctypes.data_as(C.POINTER(C.c_uint32)),
                                        nr.ctypes.data_as(C.POINTER(C.c_uint32)), _ptr(ls, _f64p), nthreads)
        if rc != 0:
            raise RuntimeError(f"oracle formal_solve_fo2_alo failed ({rc})")
        return dict(J=J, alo_n=n, alo_nr=nr, alo_ls=ls)

    def feautrier_bands(self, o, rr, f, n_off_diag):
        """Solver::solve_feautrier_order_2 with n_off_diag > 0 (solver.tpp:2319-2355) for one
        ray pair and frequency: A, C, L_diag [n_tot] and L_upper, L_lower [n_off_diag][n_tot]
        indexed from the first element (None for a ray of at most two elements)."""
        l = lib()
        l.orc_feautrier_bands.restype = C.c_int
        l.orc_feautrier_bands.argtypes = [C.POINTER(OrcModel), C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                          C.POINTER(C.c_uint32), _f64p, _f64p, _f64p, _f64p, _f64p, C.c_uint32]
        n = C.c_uint32(0)
        z = np.zeros(1)
        rc = l.orc_feautrier_bands(C.byref(self.m), o, rr, f, n_off_diag, C.byref(n), _ptr(z, _f64p),
                                   _ptr(z, _f64p), _ptr(z, _f64p), _ptr(z, _f64p), _ptr(z, _f64p), 0)
        if rc not in (0, -3):
            raise RuntimeError(f"oracle feautrier_bands failed ({rc})")
        N = n.value
        if N <= 2:
            return None
        out = dict(A=np.zeros(N), C=np.zeros(N), L_diag=np.zeros(N), L_upper=np.zeros((n_off_diag, N)),
                   L_lower=np.zeros((n_off_diag, N)))
        rc = l.orc_feautrier_bands(C.byref(self.m), o, rr, f, n_off_diag, C.byref(n), _ptr(out["A"], _f64p),
                                   _ptr(out["C"], _f64p), _ptr(out["L_diag"], _f64p), _ptr(out["L_upper"], _f64p),
                                   _ptr(out["L_lower"], _f64p), N)
        if rc != 0:
            raise RuntimeError(f"oracle feautrier_bands failed ({rc})")
        return out

    def set_column(self, density, nthreads=0):
        """Solver::set_column (solver.tpp:2953-2991): column [nrays][P]."""
        P, R = self.a["npoints"], self.a["nrays"]
        rho = np.ascontiguousarray(density, np.float64)
        col = np.zeros((R, P))
        l = lib()
        l.orc_set_column.restype = C.c_int
        l.orc_set_column.argtypes = [C.POINTER(OrcModel), _f64p, _f64p, C.c_int]
        rc = l.orc_set_column(C.byref(self.m), _ptr(rho, _f64p), _ptr(col, _f64p), nthreads)
        if rc != 0:
            raise RuntimeError(f"oracle set_column failed ({rc})")
        return col

    def image_fo2(self, rr, nthreads=0):
        P, F = self.a["npoints"], self.a["nfreqs"]
        I = np.zeros((P, F))
        rc = lib().orc_image_fo2(C.byref(self.m), rr, _ptr(I, _f64p), nthreads)
        if rc != 0:
            raise RuntimeError(f"oracle imager failed ({rc})")
        return I


# ---------------------------------------------------------------------------
# ALI level populations (mgr_oracle_ali.c)
# ---------------------------------------------------------------------------
class OrcColPar(C.Structure):
    _fields_ = [("num_col_partner", C.c_uint32), ("ortho_para", C.c_int32), ("ncol", C.c_uint32),
                ("ntmp", C.c_uint32), ("icol", _u32p), ("jcol", _u32p), ("tmp", _f64p), ("Cd", _f64p),
                ("Ce", _f64p)]


class OrcSpecies(C.Structure):
    _fields_ = [("num", C.c_uint32), ("nlev", C.c_uint32), ("nrad", C.c_uint32), ("ncolpar", C.c_uint32),
                ("line_offset", C.c_uint32), ("energy", _f64p), ("weight", _f64p), ("irad", _u32p),
                ("jrad", _u32p), ("A", _f64p), ("Bs", _f64p), ("Ba", _f64p), ("frequency", _f64p),
                ("colpar", C.POINTER(OrcColPar))]


class OrcAliParams(C.Structure):
    _fields_ = [("pop_prec", C.c_double), ("min_rel_pop_for_convergence", C.c_double),
                ("convergence_fraction", C.c_double), ("population_inversion_fraction", C.c_double),
                ("min_line_opacity", C.c_double), ("min_line_emissivity", C.c_double),
                ("Ng_acceleration_mem_limit", C.c_uint32), ("adaptive_Ng_acceleration_min_order", C.c_uint32),
                ("Ng_acceleration_remove_N_its", C.c_uint32), ("use_adaptive_Ng_acceleration", C.c_int32),
                ("adaptive_Ng_acceleration_use_max_criterion", C.c_int32), ("n_off_diag", C.c_uint32),
                ("global_stateq", C.c_int32)]


# Defaults of src/model/parameters/parameters.hpp:76-103.
ALI_DEFAULTS = dict(pop_prec=1.0e-6, min_rel_pop_for_convergence=1.0e-10, convergence_fraction=0.995,
                    population_inversion_fraction=-1.0, min_line_opacity=1.0e-13, min_line_emissivity=1.0e-50,
                    Ng_acceleration_mem_limit=9, adaptive_Ng_acceleration_min_order=2,
                    Ng_acceleration_remove_N_its=0, use_adaptive_Ng_acceleration=1,
                    adaptive_Ng_acceleration_use_max_criterion=1, n_off_diag=0,
                    # the oracle's own switch: the global rate system also for n_off_diag = 0
                    global_stateq=0)

_ORTHO_PARA = {"n": 0, "o": 1, "p": 2}


def species_structs(raw, nrad_cum):
    """(OrcSpecies array, keepalive list) for the line-producing species of a RawModel."""
    keep = []

    def arr(x, dt):
        a = np.ascontiguousarray(x, dtype=dt)
        keep.append(a)
        return a

    sp = (OrcSpecies * len(raw.linedata))()
    for l, ld in enumerate(raw.linedata):
        cps = (OrcColPar * max(1, len(ld.colpar)))()
        keep.append(cps)
        for c, cp in enumerate(ld.colpar):
            cps[c].num_col_partner = cp.num_col_partner
            cps[c].ortho_para = _ORTHO_PARA[cp.orth_or_para_H2]
            cps[c].ncol = cp.ncol
            cps[c].ntmp = cp.ntmp
            cps[c].icol = _ptr(arr(cp.icol, np.uint32), _u32p)
            cps[c].jcol = _ptr(arr(cp.jcol, np.uint32), _u32p)
            cps[c].tmp = _ptr(arr(cp.tmp, np.float64), _f64p)
            cps[c].Cd = _ptr(arr(cp.Cd, np.float64), _f64p)
            cps[c].Ce = _ptr(arr(cp.Ce, np.float64), _f64p)
        s = sp[l]
        s.num, s.nlev, s.nrad, s.ncolpar = ld.num, ld.nlev, ld.nrad, len(ld.colpar)
        s.line_offset = int(nrad_cum[l])
        s.energy = _ptr(arr(ld.energy, np.float64), _f64p)
        s.weight = _ptr(arr(ld.weight, np.float64), _f64p)
        s.irad = _ptr(arr(ld.irad, np.uint32), _u32p)
        s.jrad = _ptr(arr(ld.jrad, np.uint32), _u32p)
        s.A = _ptr(arr(ld.A, np.float64), _f64p)
        s.Bs = _ptr(arr(ld.Bs, np.float64), _f64p)
        s.Ba = _ptr(arr(ld.Ba, np.float64), _f64p)
        s.frequency = _ptr(arr(ld.frequency, np.float64), _f64p)
        s.colpar = cps
    return sp, keep


def _declare_ali(l):
    l.orc_compute_jeff.restype = C.c_int
    l.orc_compute_jeff.argtypes = [C.POINTER(OrcModel), C.c_uint32, C.POINTER(OrcSpecies), _f64p, _f64p,
                                   C.POINTER(_f64p), C.POINTER(_f64p), C.POINTER(_f64p), C.POINTER(_f64p)]
    l.orc_stateq.restype = C.c_int
    l.orc_stateq.argtypes = [C.POINTER(OrcSpecies), C.c_uint32, _f64p, C.c_uint32, _f64p, _f64p, _f64p, _f64p,
                             C.c_double, _f64p]
    l.orc_ali_run.restype = C.c_int
    l.orc_ali_run.argtypes = [C.POINTER(OrcModel), _f64p, _f64p, _f64p, C.c_uint32, C.POINTER(OrcSpecies),
                              C.c_uint32, _f64p, C.POINTER(OrcAliParams), C.c_int, C.c_long, C.POINTER(_f64p),
                              _f64p, _f64p, C.POINTER(_f64p), C.c_int]


def _ptr_array(arrays):
    out = (_f64p * len(arrays))()
    for i, a in enumerate(arrays):
        out[i] = _ptr(a, _f64p)
    return out


class AliOracle:
    """The oracle's compute_Jeff / statistical equilibrium / ALI loop on a RawModel.

    ``arrays`` is the dict of ``reference_setup(raw)`` (its populations are the
    initial, LTE, ones); emissivity, opacity and the interpolation criterion in it
    are updated in place by ``run``."""

    def __init__(self, raw, arrays):
        self.raw = raw
        self.a = arrays
        self.orc = Oracle(arrays)
        self.sp, self._keep = species_structs(raw, arrays["nrad_cum"])
        self.abundance = np.ascontiguousarray(raw.abundance, np.float64)
        _declare_ali(lib())

    def compute_jeff(self, J, lam, pops):
        P = self.a["npoints"]
        pops = [np.ascontiguousarray(p, np.float64) for p in pops]
        outs = [[np.zeros((P, ld.nrad)) for ld in self.raw.linedata] for _ in range(3)]
        rc = lib().orc_compute_jeff(C.byref(self.orc.m), len(self.raw.linedata), self.sp,
                                    _ptr(np.ascontiguousarray(J), _f64p), _ptr(np.ascontiguousarray(lam), _f64p),
                                    _ptr_array(pops), _ptr_array(outs[0]), _ptr_array(outs[1]), _ptr_array(outs[2]))
        if rc != 0:
            raise RuntimeError("oracle Jeff failed")
        return dict(Jlin=outs[0], Jeff=outs[1], Jdif=outs[2])

    def stateq(self, l, Jeff, Ls, pop, min_line_opacity=1.0e-13):
        P = self.a["npoints"]
        out = np.zeros((P, self.raw.linedata[l].nlev))
        rc = lib().orc_stateq(C.byref(self.sp[l]), P, _ptr(self.abundance, _f64p), self.abundance.shape[1],
                              _ptr(self.a["temperature"], _f64p), _ptr(np.ascontiguousarray(Jeff), _f64p),
                              _ptr(np.ascontiguousarray(Ls), _f64p), _ptr(np.ascontiguousarray(pop), _f64p),
                              min_line_opacity, _ptr(out, _f64p))
        if rc != 0:
            raise RuntimeError("oracle statistical equilibrium failed")
        return out

    def run(self, use_ng=True, max_it=100, nthreads=0, **params):
        prm = dict(ALI_DEFAULTS)
        prm.update(params)
        p = OrcAliParams(**prm)
        pops = [np.ascontiguousarray(x, np.float64).copy() for x in self.a["populations"]]
        nls = len(self.raw.linedata)
        err_mean = np.zeros(max_it * nls)
        err_max = np.zeros(max_it * nls)
        Jeff = [np.zeros((self.a["npoints"], ld.nrad)) for ld in self.raw.linedata]
        it = lib().orc_ali_run(C.byref(self.orc.m), _ptr(self.a["emissivity"], _f64p),
                               _ptr(self.a["opacity"], _f64p), _ptr(self.a["interp_criterion"], _f64p), nls,
                               self.sp, self.abundance.shape[1], _ptr(self.abundance, _f64p), C.byref(p),
                               int(use_ng), max_it, _ptr_array(pops), _ptr(err_mean, _f64p), _ptr(err_max, _f64p),
                               _ptr_array(Jeff), nthreads)
        if it < 0:
            raise RuntimeError(f"oracle ALI failed ({it})")
        return dict(iterations=it, populations=pops, Jeff=Jeff, error_mean=err_mean[:it * nls],
                    error_max=err_max[:it * nls])
