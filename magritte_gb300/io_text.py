"""Magritte's plain-text model format: read a model folder into a ``RawModel`` (and from
there ``loader.to_core``) and write one.

The layout is the reference's IoText (src/io/cpp/io_cpp_text.cpp): one ``.txt`` file per
field under the model folder, numbers one per line for lists, rows of tab-separated
values for arrays, ``true`` / ``false`` for booleans, and the paths the reference's
``read`` methods use:

  .npoints .nrays .nboundary .nspecs .nlspecs .nquads .dimension .spherical_symmetry ...
  geometry/points/{position,velocity,n_neighbors,neighbors}        (points.cpp:13-60)
  geometry/rays/{direction,weight}                                 (rays.cpp:5-66)
  geometry/boundary/{boundary2point,boundary_temperature,boundary_condition}
                                                                   (boundary.cpp:7-48)
  chemistry/species/{abundance,species}                            (species.cpp:7-30)
  thermodynamics/temperature/gas, thermodynamics/turbulence/vturb2
  lines/lineProducingSpecies_<l>/linedata/{.num,.sym,.inverse_mass,.nlev,.nrad,irad,jrad,
      energy,weight,frequency,A,Bs,Ba}, .../collisionPartner_<c>/{.num_col_partner,
      .orth_or_para_H2,tmp,icol,jcol,Ce,Cd}                        (linedata.cpp:12-70,
                                                                    collisionPartner.cpp:11-45)
  lines/lineProducingSpecies_<l>/quadrature/{weights,roots}        (quadrature.cpp:9-24)
  lines/lineProducingSpecies_<l>/{population_tot,population}       (lineProducingSpecies.cpp:43-135)

A length is the number of lines of a file, or, when the file does not exist, the number
of consecutively numbered siblings (``lineProducingSpecies_0``, ``_1``, ...), as
IoText::read_length counts them.  Numbers are written as the reference writes them
(``%.16e`` for reals, plain integers for sizes)."""
import os
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import synthetic as S


def _path(folder, name):
    return os.path.join(folder, name + ".txt")


def _exists(folder, name):
    return os.path.exists(_path(folder, name))


def _length(folder, name):
    """IoText::read_length: lines of name.txt, else the count of name0, name1, ..."""
    if _exists(folder, name):
        with open(_path(folder, name)) as f:
            return sum(1 for _ in f)
    n = 0
    while os.path.exists(os.path.join(folder, name + str(n))):
        n += 1
    return n


def _word(folder, name, default=None):
    if not _exists(folder, name):
        return default
    with open(_path(folder, name)) as f:
        tok = f.read().split()
    return tok[0] if tok else default


def _number(folder, name, kind=float, default=None):
    w = _word(folder, name)
    if w is None:
        return default
    return kind(float(w)) if kind is int else kind(w)


def _bool(folder, name, default=False):
    w = _word(folder, name)
    return default if w is None else w == "true"


def _list(folder, name, dtype=np.float64):
    with open(_path(folder, name)) as f:
        tok = f.read().split()
    if dtype == np.float64:
        return np.array([float(t) for t in tok], dtype=np.float64)
    return np.array([int(float(t)) for t in tok], dtype=dtype)


def _array(folder, name, ncols=None):
    rows = []
    with open(_path(folder, name)) as f:
        for line in f:
            tok = line.split()
            if tok:
                rows.append([float(t) for t in tok])
    a = np.array(rows, dtype=np.float64)
    if ncols is not None and a.size == 0:
        a = a.reshape(0, ncols)
    return a


@dataclass
class TextModel:
    """A model read from a folder: the arrays, the level populations per species when
    the folder holds them, and the parameters written there."""
    raw: S.RawModel
    populations: Optional[List[np.ndarray]] = None
    population_tot: Optional[List[np.ndarray]] = None
    parameters: Dict[str, object] = field(default_factory=dict)


_PARAM_NUMBERS = ("n_off_diag", "max_width_fraction", "convergence_fraction", "min_rel_pop_for_convergence",
                  "pop_prec", "min_opacity", "Ng_acceleration_mem_limit")
_PARAM_BOOLS = ("store_intensities", "one_line_approximation", "use_adaptive_Ng_acceleration", "use_scattering",
                "adaptive_ray_tracing")


def read(folder) -> TextModel:
    """Reads a Magritte model folder written by the reference's IoText (or by write)."""
    folder = os.path.join(folder, "")
    P = _length(folder, "geometry/points/position")
    position = _array(folder, "geometry/points/position", 3).reshape(P, 3)
    velocity = _array(folder, "geometry/points/velocity", 3).reshape(P, 3)
    n_neighbors = _list(folder, "geometry/points/n_neighbors", np.uint32)
    neighbors = _list(folder, "geometry/points/neighbors", np.uint32)
    nrays = _number(folder, ".nrays", int)
    direction = _array(folder, "geometry/rays/direction", 3)
    weight = _list(folder, "geometry/rays/weight")
    adaptive = direction.shape[0] == nrays * P and direction.shape[0] != nrays
    b2p = _list(folder, "geometry/boundary/boundary2point", np.uint32)
    bt = _list(folder, "geometry/boundary/boundary_temperature")
    bc = _list(folder, "geometry/boundary/boundary_condition", np.int32)
    abundance = _array(folder, "chemistry/species/abundance")
    if abundance.ndim == 1:
        abundance = abundance.reshape(P, -1)
    temperature = _list(folder, "thermodynamics/temperature/gas")
    vturb2 = _list(folder, "thermodynamics/turbulence/vturb2")
    nlspecs = _length(folder, "lines/lineProducingSpecies_")
    lds, roots, weights, pops, tots = [], [], [], [], []
    have_pops = True
    for l in range(nlspecs):
        pl = f"lines/lineProducingSpecies_{l}/"
        pld = pl + "linedata/"
        colpars = []
        for c in range(_length(folder, pld + "collisionPartner_")):
            pc = pld + f"collisionPartner_{c}/"
            ncol = _length(folder, pc + "icol")
            colpars.append(S.CollisionPartner(
                num_col_partner=_number(folder, pc + ".num_col_partner", int),
                orth_or_para_H2=_word(folder, pc + ".orth_or_para_H2", "n"),
                icol=_list(folder, pc + "icol", np.uint32), jcol=_list(folder, pc + "jcol", np.uint32),
                tmp=_list(folder, pc + "tmp"), Cd=_array(folder, pc + "Cd", ncol), Ce=_array(folder, pc + "Ce", ncol)))
        lds.append(S.Linedata(
            num=_number(folder, pld + ".num", int), sym=_word(folder, pld + ".sym", ""),
            inverse_mass=_number(folder, pld + ".inverse_mass"),
            energy=_list(folder, pld + "energy"), weight=_list(folder, pld + "weight"),
            irad=_list(folder, pld + "irad", np.int64), jrad=_list(folder, pld + "jrad", np.int64),
            A=_list(folder, pld + "A"), colpar=colpars, frequency_given=_list(folder, pld + "frequency"),
            Bs_given=_list(folder, pld + "Bs"), Ba_given=_list(folder, pld + "Ba")))
        weights.append(_list(folder, pl + "quadrature/weights"))
        roots.append(_list(folder, pl + "quadrature/roots"))
        if _exists(folder, pl + "population") and _exists(folder, pl + "population_tot"):
            pops.append(_array(folder, pl + "population").reshape(P, -1))
            tots.append(_list(folder, pl + "population_tot"))
        else:
            have_pops = False
    raw = S.RawModel(
        name=os.path.basename(os.path.normpath(folder)), dimension=_number(folder, ".dimension", int, 3),
        position=position, velocity=velocity, neighbors=neighbors, n_neighbors=n_neighbors,
        boundary2point=b2p, boundary_condition=bc, boundary_temperature=bt,
        ray_direction=direction[:nrays].copy() if adaptive else direction,
        ray_weight=weight[:nrays].copy() if adaptive else weight,
        abundance=abundance, temperature=temperature, vturb2=vturb2, linedata=lds, quad_roots=roots,
        quad_weights=weights, nquads=_number(folder, ".nquads", int, len(roots[0]) if roots else 0),
        spherical_symmetry=_bool(folder, ".spherical_symmetry"),
        adaptive_direction=direction.reshape(P, nrays, 3) if adaptive else None,
        adaptive_weight=weight.reshape(P, nrays) if adaptive else None)
    params = {k: _number(folder, "." + k) for k in _PARAM_NUMBERS if _exists(folder, "." + k)}
    params.update({k: _bool(folder, "." + k) for k in _PARAM_BOOLS if _exists(folder, "." + k)})
    return TextModel(raw=raw, populations=pops if have_pops and nlspecs else None,
                     population_tot=tots if have_pops and nlspecs else None, parameters=params)


def _write_word(folder, name, word):
    os.makedirs(os.path.dirname(_path(folder, name)), exist_ok=True)
    with open(_path(folder, name), "w") as f:
        f.write(str(word))


def _write_number(folder, name, x):
    _write_word(folder, name, str(int(x)) if isinstance(x, (int, np.integer)) else "%.16e" % x)


def _write_list(folder, name, a):
    a = np.asarray(a)
    os.makedirs(os.path.dirname(_path(folder, name)), exist_ok=True)
    with open(_path(folder, name), "w") as f:
        if np.issubdtype(a.dtype, np.integer):
            f.writelines("%d\n" % v for v in a.ravel())
        else:
            f.writelines("%.16e\n" % v for v in a.ravel())


def _write_array(folder, name, a):
    a = np.asarray(a, dtype=np.float64)
    os.makedirs(os.path.dirname(_path(folder, name)), exist_ok=True)
    with open(_path(folder, name), "w") as f:
        for row in a:
            f.write("".join("%.16e\t" % v for v in row) + "\n")


def write(raw: S.RawModel, folder, populations=None, parameters=None, species_symbols=None):
    """Writes a RawModel (and optionally level populations [P][nlev] per species and
    the ALI parameters) as a Magritte text model folder."""
    folder = os.path.join(folder, "")
    os.makedirs(folder, exist_ok=True)
    P = raw.npoints
    nrays = raw.nrays
    _write_word(folder, ".version", "0.9.3")
    for k, v in (("dimension", raw.dimension), ("npoints", P), ("nrays", nrays), ("hnrays", nrays // 2),
                 ("nboundary", len(raw.boundary2point)), ("nspecs", raw.abundance.shape[1]),
                 ("nlspecs", len(raw.linedata)), ("nlines", int(sum(ld.nrad for ld in raw.linedata))),
                 ("nquads", raw.nquads)):
        _write_number(folder, "." + k, int(v))
    _write_word(folder, ".spherical_symmetry", "true" if raw.spherical_symmetry else "false")
    for k, v in (parameters or {}).items():
        if isinstance(v, bool):
            _write_word(folder, "." + k, "true" if v else "false")
        else:
            _write_number(folder, "." + k, v)
    _write_array(folder, "geometry/points/position", raw.position)
    _write_array(folder, "geometry/points/velocity", raw.velocity)
    _write_list(folder, "geometry/points/n_neighbors", np.asarray(raw.n_neighbors, np.int64))
    _write_list(folder, "geometry/points/neighbors", np.asarray(raw.neighbors, np.int64))
    if raw.adaptive_direction is not None:
        _write_array(folder, "geometry/rays/direction", raw.adaptive_direction.reshape(-1, 3))
        _write_list(folder, "geometry/rays/weight", raw.adaptive_weight.reshape(-1))
    else:
        _write_array(folder, "geometry/rays/direction", raw.ray_direction)
        _write_list(folder, "geometry/rays/weight", raw.ray_weight)
    _write_list(folder, "geometry/boundary/boundary2point", np.asarray(raw.boundary2point, np.int64))
    _write_list(folder, "geometry/boundary/boundary_temperature", raw.boundary_temperature)
    _write_list(folder, "geometry/boundary/boundary_condition", np.asarray(raw.boundary_condition, np.int64))
    _write_array(folder, "chemistry/species/abundance", raw.abundance)
    syms = species_symbols or [f"s{i}" for i in range(raw.abundance.shape[1])]
    _write_word(folder, "chemistry/species/species", "\n".join(syms) + "\n")
    _write_list(folder, "thermodynamics/temperature/gas", raw.temperature)
    _write_list(folder, "thermodynamics/turbulence/vturb2", raw.vturb2)
    for l, ld in enumerate(raw.linedata):
        pl = f"lines/lineProducingSpecies_{l}/"
        pld = pl + "linedata/"
        _write_number(folder, pld + ".num", int(ld.num))
        _write_word(folder, pld + ".sym", ld.sym or f"species{l}")
        _write_number(folder, pld + ".inverse_mass", float(ld.inverse_mass))
        _write_number(folder, pld + ".nlev", int(ld.nlev))
        _write_number(folder, pld + ".nrad", int(ld.nrad))
        _write_list(folder, pld + "irad", np.asarray(ld.irad, np.int64))
        _write_list(folder, pld + "jrad", np.asarray(ld.jrad, np.int64))
        for k in ("energy", "weight", "frequency", "A", "Bs", "Ba"):
            _write_list(folder, pld + k, np.asarray(getattr(ld, k), np.float64))
        for c, cp in enumerate(ld.colpar):
            pc = pld + f"collisionPartner_{c}/"
            _write_number(folder, pc + ".num_col_partner", int(cp.num_col_partner))
            _write_word(folder, pc + ".orth_or_para_H2", cp.orth_or_para_H2)
            _write_list(folder, pc + "tmp", cp.tmp)
            _write_list(folder, pc + "icol", np.asarray(cp.icol, np.int64))
            _write_list(folder, pc + "jcol", np.asarray(cp.jcol, np.int64))
            _write_array(folder, pc + "Ce", cp.Ce)
            _write_array(folder, pc + "Cd", cp.Cd)
        _write_list(folder, pl + "quadrature/weights", raw.quad_weights[l])
        _write_list(folder, pl + "quadrature/roots", raw.quad_roots[l])
        if populations is not None:
            pop = np.asarray(populations[l], np.float64).reshape(P, -1)
            _write_array(folder, pl + "population", pop)
            _write_list(folder, pl + "population_tot", raw.abundance[:, ld.num])


def to_core(folder, precision="fp64", approx="CloseLines"):
    """A magritte_gb300.core.Model from a model folder, with its level populations when
    the folder holds them (else the caller computes LTE populations)."""
    from . import loader
    tm = read(folder)
    model = loader.to_core(tm.raw, precision=precision, approx=approx)
    if tm.populations is not None:
        for l, (pop, tot) in enumerate(zip(tm.populations, tm.population_tot)):
            lsp = model.lines.lineProducingSpecies[l]
            lsp.population.set(np.ascontiguousarray(pop.ravel(), np.float64))
            lsp.population_tot.set(np.ascontiguousarray(tot, np.float64))
    return model
