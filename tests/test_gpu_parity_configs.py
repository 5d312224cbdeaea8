"""GPU parity on the benchmark set's own configurations, against the oracle, through
the C ABI.

The workloads are the ones the benchmark times and states:
  * config 0: the 20^3 Cartesian cube (6 ray pairs, one line x 11 quadrature points),
    every origin;
  * config 1 (the benchmarked model): the 64^3 grid cut to a sphere (130,536 points,
    24 ray pairs, 4 lines x 31), every 50th origin with every ray pair;
  * config 2 family: the non-LTE Delaunay sphere (density ~ r^-2, 15 km/s wind,
    192 rays, 10-level rotor x 21) at 20,000 interior points, every 40th origin; and
    its ALI level populations at 1,000 interior points (8 iterations, Ng every 4).

Two oracle arithmetics are compared.  Erf mode 1 is the correctly rounded erff that
the GPU's FP64 mode uses; erf mode 0 is the reference's own arithmetic, glibc's erff
(the reference subtracts two single-precision erff values, solver.tpp:2450, so the two
differ by up to a few 1e-6 of J on Doppler-shifted models).  Bars:
  * GPU FP64 and split precision against both modes: 1e-5 relative in J and in the
    ALO diagonal, at every sampled (origin, frequency);
  * ALI populations: 1e-6 (FP64 mode) and 1e-5 (split) of the oracle after the same
    iterations."""
import numpy as np
import pytest

import helpers as H
import oracle as O
from magritte_gb300 import _abi
from magritte_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def _rel(x, ref, floor=1e-300):
    return float(np.max(np.abs(x - ref) / np.maximum(np.abs(ref), floor)))


def _oracle_modes(a, origins):
    orc = O.Oracle(a)
    out = {}
    try:
        for mode in (0, 1):
            O.set_erf_mode(mode)
            out[mode] = orc.formal_solve_fo2_origins(origins)
    finally:
        O.set_erf_mode(0)
    return out


def _gpu(a):
    dev = _abi.DeviceModel(a)
    try:
        return {p: dev.formal_solve_fo2(p) for p in ("fp64", "split")}
    finally:
        dev.close()


def _check(gpu, ref, origins, what):
    lines = []
    for prec in ("fp64", "split"):
        J = gpu[prec]["J"][origins]
        lam = gpu[prec]["lambda_diag"][origins]
        for mode in (0, 1):
            eJ = _rel(J, ref[mode]["J"])
            eL = _rel(lam, ref[mode]["lambda_diag"])
            lines.append(f"{what} {prec} vs erf mode {mode}: J {eJ:.3e}  ALO {eL:.3e}")
            assert eJ < 1e-5 and eL < 1e-5, lines[-1]
    print("\n".join(lines))


def test_config0_cube_every_origin(gpu_lib):
    a = H.setup(S.grid_cube())
    origins = np.arange(a["npoints"])
    _check(_gpu(a), _oracle_modes(a, origins), origins, "config 0")


def test_config1_benchmarked_model_sample(gpu_lib):
    a = H.setup(S.grid_sphere(n=64))
    origins = np.arange(0, a["npoints"], 50)
    _check(_gpu(a), _oracle_modes(a, origins), origins, "config 1 (64^3)")


def test_config2_family_formal_solve_sample(gpu_lib):
    a = H.setup(S.nlte_sphere(npoints=20_000, nside=4))
    origins = np.arange(0, a["npoints"], 40)
    _check(_gpu(a), _oracle_modes(a, origins), origins, "config 2 family (20k)")


def test_config2_family_ali_populations(gpu_lib):
    """8 ALI iterations (Default Ng every 4, no early stop) on 1,000 interior points of
    the non-LTE sphere with an nside-8 outer shell; populations against the oracle's
    loop in the GPU FP64 mode's arithmetic."""
    raw = S.nlte_sphere(npoints=1000, nside=4, nside_out=8)
    params = dict(use_adaptive_Ng_acceleration=0, Ng_acceleration_mem_limit=4, pop_prec=0.0)
    O.set_erf_mode(1)
    try:
        ref = O.AliOracle(raw, H.setup(raw)).run(use_ng=True, max_it=8, **params)
    finally:
        O.set_erf_mode(0)
    tot = raw.abundance[:, raw.linedata[0].num][:, None]
    errs = {}
    for prec, bar in (("fp64", 1e-6), ("split", 1e-5)):
        a = H.setup(raw)
        dev = _abi.DeviceModel(a)
        try:
            dev.set_species(raw.linedata, raw.abundance, a["populations"])
            got = dev.compute_level_populations(prec, use_ng=True, max_it=8, **params)
            assert got["iterations"] == ref["iterations"] == 8
            errs[prec] = _rel(dev.populations(0), ref["populations"][0], 1e-10 * tot)
        finally:
            dev.close()
        assert errs[prec] < bar, (prec, errs[prec])
    print(f"config 2 family ALI populations vs oracle: fp64 {errs['fp64']:.3e}  split {errs['split']:.3e}")
