"""Loads a ``synthetic.RawModel`` into the host ``core.Model`` through the same
setters a Magritte user calls (magritte/setup.py style)."""
import numpy as np


def to_core(raw, precision="fp64", approx="CloseLines"):
    from . import core

    model = core.Model()
    prm = model.parameters
    prm.set_model_name(raw.name)
    prm.set_dimension(raw.dimension)
    prm.set_npoints(raw.npoints)
    prm.set_nrays(raw.nrays)
    prm.set_nspecs(raw.abundance.shape[1])
    prm.set_nlspecs(len(raw.linedata))
    prm.set_nquads(raw.nquads)
    prm.set_spherical_symmetry(bool(raw.spherical_symmetry))
    prm.precision = precision
    prm.one_line_approximation = approx == "OneLine"
    prm.sum_opacity_emissivity_over_all_lines = approx == "None"

    g = model.geometry
    g.points.position.set(np.ascontiguousarray(raw.position, np.float64))
    g.points.velocity.set(np.ascontiguousarray(raw.velocity, np.float64))
    g.points.neighbors.set(np.ascontiguousarray(raw.neighbors, np.uint32))
    g.points.n_neighbors.set(np.ascontiguousarray(raw.n_neighbors, np.uint32))
    if raw.adaptive_direction is not None:
        # per-point rays (Rays::use_adaptive_directions): [npoints * nrays]
        g.rays.use_adaptive_directions = True
        g.rays.direction.set(np.ascontiguousarray(raw.adaptive_direction.reshape(-1, 3), np.float64))
        g.rays.weight.set(np.ascontiguousarray(raw.adaptive_weight.reshape(-1), np.float64))
    else:
        g.rays.direction.set(np.ascontiguousarray(raw.ray_direction, np.float64))
        g.rays.weight.set(np.ascontiguousarray(raw.ray_weight, np.float64))
    g.boundary.boundary2point.set(np.ascontiguousarray(raw.boundary2point, np.uint32))
    prm.set_nboundary(len(raw.boundary2point))
    g.boundary.boundary_condition.set(np.ascontiguousarray(raw.boundary_condition, np.int32))
    g.boundary.boundary_temperature.set(np.ascontiguousarray(raw.boundary_temperature, np.float64))

    model.chemistry.species.abundance = np.ascontiguousarray(raw.abundance, np.float64)
    model.thermodynamics.temperature.gas.set(np.ascontiguousarray(raw.temperature, np.float64))
    model.thermodynamics.turbulence.vturb2.set(np.ascontiguousarray(raw.vturb2, np.float64))

    model.lines.resize_LineProducingSpecies(len(raw.linedata))
    for l, ld in enumerate(raw.linedata):
        lsp = model.lines.lineProducingSpecies[l]
        d = lsp.linedata
        d.num = int(ld.num)
        d.sym = ld.sym
        d.inverse_mass = float(ld.inverse_mass)
        d.nlev = int(ld.nlev)
        d.nrad = int(ld.nrad)
        d.energy = [float(x) for x in ld.energy]
        d.weight = [float(x) for x in ld.weight]
        d.irad = [int(x) for x in ld.irad]
        d.jrad = [int(x) for x in ld.jrad]
        d.A = [float(x) for x in ld.A]
        d.frequency = [float(x) for x in ld.frequency]
        d.Bs = [float(x) for x in ld.Bs]
        d.Ba = [float(x) for x in ld.Ba]
        cps = []
        for c in ld.colpar:
            cp = core.CollisionPartner()
            cp.num_col_partner = int(c.num_col_partner)
            cp.orth_or_para_H2 = c.orth_or_para_H2
            cp.ncol = int(c.ncol)
            cp.ntmp = int(c.ntmp)
            cp.icol = [int(x) for x in c.icol]
            cp.jcol = [int(x) for x in c.jcol]
            cp.tmp = [float(x) for x in c.tmp]
            cp.Cd = [[float(x) for x in row] for row in c.Cd]
            cp.Ce = [[float(x) for x in row] for row in c.Ce]
            cps.append(cp)
        d.colpar = core.vCollisionPartner(cps)
        lsp.linedata = d
        lsp.quadrature.roots.set(np.asarray(raw.quad_roots[l], np.float64))
        lsp.quadrature.weights.set(np.asarray(raw.quad_weights[l], np.float64))
    return model
