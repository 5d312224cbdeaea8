"""Magritte's plain-text model format (magritte_gb300.io_text): the reference's IoText
layout (src/io/cpp/io_cpp_text.cpp) written and read back.

* Round trip: every array of a model written and read back is bit-identical (reals are
  written with 17 significant digits, as IoText writes them), for a Cartesian cube, the
  non-LTE Delaunay sphere with its collision partner, and a model with adaptive rays.
* The folder's layout is the one the reference's read methods open (file names checked).
* The formal solve of the read-back model equals the original's (oracle, bit for bit),
  and core.Model built from the folder carries the written level populations."""
import os

import numpy as np
import pytest

import helpers as H
import oracle as O
from magritte_gb300 import io_text
from magritte_gb300 import synthetic as S

MODELS = {"cube": lambda: S.grid_cube(n=6, nquads=5),
          "nlte": lambda: S.nlte_sphere(npoints=300, nside=1, nside_out=2, nside_in=1),
          "adaptive": lambda: S.with_adaptive_rays(S.grid_cube(n=5, nquads=3))}


def _same(a, b):
    np.testing.assert_array_equal(np.asarray(a), np.asarray(b))


@pytest.mark.parametrize("name", sorted(MODELS))
def test_round_trip_is_exact(tmp_path, name):
    raw = MODELS[name]()
    io_text.write(raw, str(tmp_path / "model"))
    back = io_text.read(str(tmp_path / "model")).raw
    for k in ("position", "velocity", "neighbors", "n_neighbors", "boundary2point", "boundary_condition",
              "boundary_temperature", "ray_direction", "ray_weight", "abundance", "temperature", "vturb2"):
        _same(getattr(back, k), getattr(raw, k))
    assert back.nquads == raw.nquads and back.dimension == raw.dimension
    if raw.adaptive_direction is not None:
        _same(back.adaptive_direction, raw.adaptive_direction)
        _same(back.adaptive_weight, raw.adaptive_weight)
    for la, lb in zip(raw.linedata, back.linedata):
        for k in ("energy", "weight", "irad", "jrad", "A", "frequency", "Bs", "Ba"):
            _same(getattr(lb, k), getattr(la, k))
        assert lb.num == la.num and lb.inverse_mass == la.inverse_mass
        assert len(lb.colpar) == len(la.colpar)
        for ca, cb in zip(la.colpar, lb.colpar):
            for k in ("icol", "jcol", "tmp", "Cd", "Ce"):
                _same(getattr(cb, k), getattr(ca, k))
            assert cb.num_col_partner == ca.num_col_partner and cb.orth_or_para_H2 == ca.orth_or_para_H2
    for a, b in zip(raw.quad_roots + raw.quad_weights, back.quad_roots + back.quad_weights):
        _same(b, a)


def test_layout_is_the_references(tmp_path):
    raw = MODELS["nlte"]()
    folder = str(tmp_path / "model")
    io_text.write(raw, folder, populations=[np.ones((raw.npoints, raw.linedata[0].nlev))])
    for rel in (".npoints", ".nrays", ".nboundary", ".nspecs", ".nlspecs", ".nquads", ".spherical_symmetry",
                "geometry/points/position", "geometry/points/velocity", "geometry/points/n_neighbors",
                "geometry/points/neighbors", "geometry/rays/direction", "geometry/rays/weight",
                "geometry/boundary/boundary2point", "geometry/boundary/boundary_temperature",
                "geometry/boundary/boundary_condition", "chemistry/species/abundance", "chemistry/species/species",
                "thermodynamics/temperature/gas", "thermodynamics/turbulence/vturb2",
                "lines/lineProducingSpecies_0/linedata/.nlev", "lines/lineProducingSpecies_0/linedata/frequency",
                "lines/lineProducingSpecies_0/linedata/collisionPartner_0/Ce",
                "lines/lineProducingSpecies_0/linedata/collisionPartner_0/.orth_or_para_H2",
                "lines/lineProducingSpecies_0/quadrature/roots", "lines/lineProducingSpecies_0/population",
                "lines/lineProducingSpecies_0/population_tot"):
        assert os.path.exists(os.path.join(folder, rel + ".txt")), rel
    # arrays are rows of tab-separated values (IoText::write_array)
    with open(os.path.join(folder, "geometry/points/position.txt")) as f:
        assert f.readline().count("\t") == 3


def test_read_back_model_solves_identically(tmp_path):
    raw = MODELS["cube"]()
    io_text.write(raw, str(tmp_path / "model"))
    back = io_text.read(str(tmp_path / "model")).raw
    J0 = O.Oracle(H.setup(raw)).formal_solve_fo2()["J"]
    J1 = O.Oracle(H.setup(back)).formal_solve_fo2()["J"]
    _same(J1, J0)


def test_core_model_from_folder_keeps_populations(tmp_path):
    pytest.importorskip("magritte_gb300.core")
    raw = MODELS["nlte"]()
    rng = np.random.default_rng(0)
    nlev = raw.linedata[0].nlev
    pop = rng.uniform(0.1, 1.0, size=(raw.npoints, nlev))
    pop *= (raw.abundance[:, raw.linedata[0].num] / pop.sum(axis=1))[:, None]
    io_text.write(raw, str(tmp_path / "model"), populations=[pop], parameters={"pop_prec": 1.0e-6})
    tm = io_text.read(str(tmp_path / "model"))
    assert tm.parameters["pop_prec"] == 1.0e-6
    model = io_text.to_core(str(tmp_path / "model"))
    got = np.array(model.lines.lineProducingSpecies[0].population).reshape(raw.npoints, nlev)
    _same(got, pop)
