"""The non-local ALO (n_off_diag > 0) on the GPU against the oracle, through the C ABI.

* The banded FP64 formal solve (mgr_formal_solve_fo2_alo_device): J, the ALO diagonal
  and the band elements next to the origin against the oracle's update_Lambda lists
  (solver.tpp:2319-2355, :1760-1850; Lambda::add_element, lambda.tpp:74-86), within the
  FP64 bar of the formal-solve tests (1e-5: the single-precision libm calls differ by
  a few ulp between glibc and CUDA; relative to each list's largest element for the
  band elements), and J and the diagonal equal to the ordinary FP64 solve's (1e-13).
* The ALI loop with the band elements (mgr_compute_level_populations with
  mgr_model_set_n_off_diag): Jeff with the band terms and the global rate system
  (lineProducingSpecies.tpp:377-581), solved here by block-Jacobi-preconditioned
  BiCGSTAB and by the oracle with a dense direct solve.  Populations within 1e-6
  relative of the oracle after one iteration (where the band elements move the
  populations by ~1e-4 against the diagonal ALO) and after a run with Ng acceleration,
  with the same number of iterations.
* The cases the reference refuses or this library does not offer: the memory-lean
  (sparse) update with n_off_diag != 0 (lineProducingSpecies.tpp:592-593), split
  precision and n_off_diag above 4."""
import numpy as np
import pytest

import helpers as H
import oracle as O
from magritte_gb300 import _abi
from magritte_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _oracle_with_correctly_rounded_erf():
    O.set_erf_mode(1)
    yield
    O.set_erf_mode(0)


MODELS = {
    "cube8": lambda: S.grid_cube(n=8, nquads=5),
    "sphere10": lambda: S.grid_sphere(n=10, nside=1, nquads=5),
    "sph_velocity": lambda: S.velocity_gradient_1d(npoints=30, nrays=8, nquads=5),
}


@pytest.mark.parametrize("name", sorted(MODELS))
@pytest.mark.parametrize("n_off_diag", [1, 2, 4])
def test_banded_solve_matches_oracle(gpu_lib, name, n_off_diag):
    a = H.setup(MODELS[name]())
    ref = O.Oracle(a).formal_solve_fo2_alo(n_off_diag)
    dev = _abi.DeviceModel(a)
    try:
        dev.set_n_off_diag(n_off_diag)
        out = dev.formal_solve_fo2_alo()
        assert H.max_rel(out["J"], ref["J"]) < 1e-5
        assert np.count_nonzero(out["alo_off"]) > 0
        assert H.band_alo_error(out["alo_off"], out["alo_nr"], out["lambda_diag"], ref) < 1e-5
        # the band elements' points are the oracle's exactly (traces are bit-exact)
        for p in range(0, a["npoints"], 7):
            for l in range(a["nlines"]):
                mine = set(out["alo_nr"][p, l][out["alo_off"][p, l] != 0.0].tolist()) | {p}
                theirs = set(ref["alo_nr"][p, l, :ref["alo_n"][p, l]].tolist())
                assert mine <= theirs | {p}, (p, l)
        # the ordinary FP64 solve: the same J, u and diagonal, up to the compiler's
        # contraction of FP64 multiply-adds in the two kernels' lane code, where an ulp of
        # a single-precision profile or erff argument can flip its rounding (measured
        # 8.5e-9 before the frequency products were explicitly rounded): 1e-6, far inside
        # the 1e-5 parity bar
        plain = dev.formal_solve_fo2("fp64", want_u=True)
        assert H.max_rel(plain["J"], out["J"]) < 1e-6
        assert H.max_rel(plain["u"], out["u"]) < 1e-6
        has = plain["lambda_diag"] != 0.0
        assert H.max_rel(out["lambda_diag"][has], plain["lambda_diag"][has]) < 1e-6
    finally:
        dev.close()


def _ali_pair(raw, n_off_diag, **run):
    ref = O.AliOracle(raw, H.setup(raw)).run(n_off_diag=n_off_diag, **run)
    a = H.setup(raw)
    dev = _abi.DeviceModel(a)
    try:
        dev.set_species(raw.linedata, raw.abundance, a["populations"])
        dev.set_n_off_diag(n_off_diag)
        prm = {k: v for k, v in run.items() if k not in ("use_ng", "max_it")}
        got = dev.compute_level_populations("fp64", use_ng=run["use_ng"], max_it=run["max_it"], **prm)
        pops = [dev.populations(l) for l in range(len(raw.linedata))]
    finally:
        dev.close()
    return ref, got, pops


ALI_MODELS = {
    "cube6": lambda: S.grid_cube(n=6, nquads=5),
    "sphere8": lambda: S.grid_sphere(n=8, nside=1, nquads=7),
}


@pytest.mark.parametrize("name", sorted(ALI_MODELS))
@pytest.mark.parametrize("n_off_diag", [1, 2])
def test_ali_one_iteration_matches_oracle(gpu_lib, name, n_off_diag):
    raw = ALI_MODELS[name]()
    ref, got, pops = _ali_pair(raw, n_off_diag, use_ng=False, max_it=1)
    diag = O.AliOracle(raw, H.setup(raw)).run(use_ng=False, max_it=1)
    tot = raw.abundance[:, raw.linedata[0].num][:, None]
    err = np.max(np.abs(pops[0] - ref["populations"][0]) / np.maximum(np.abs(ref["populations"][0]), 1e-10 * tot))
    moved = np.max(np.abs(diag["populations"][0] / ref["populations"][0] - 1.0))
    assert got["iterations"] == ref["iterations"] == 1
    assert moved > 10 * 1e-6  # the band elements matter at this bar
    assert err < 1e-6, (err, moved)


@pytest.mark.parametrize("name", sorted(ALI_MODELS))
def test_ali_with_ng_matches_oracle(gpu_lib, name):
    raw = ALI_MODELS[name]()
    ref, got, pops = _ali_pair(raw, 1, use_ng=True, max_it=12, Ng_acceleration_mem_limit=4)
    tot = raw.abundance[:, raw.linedata[0].num][:, None]
    err = np.max(np.abs(pops[0] - ref["populations"][0]) / np.maximum(np.abs(ref["populations"][0]), 1e-10 * tot))
    assert got["iterations"] == ref["iterations"]
    assert err < 1e-6, err
    np.testing.assert_allclose(got["error_max"], ref["error_max"], rtol=1e-3, atol=1e-12)


def test_banded_ali_refusals(gpu_lib):
    raw = S.grid_cube(n=6, nquads=5)
    a = H.setup(raw)
    dev = _abi.DeviceModel(a)
    try:
        with pytest.raises(_abi.MgrError):
            dev.set_n_off_diag(5)
        dev.set_species(raw.linedata, raw.abundance, a["populations"])
        dev.set_n_off_diag(1)
        with pytest.raises(_abi.MgrError, match="sparse"):
            dev.compute_level_populations_sparse("fp64", use_ng=False, max_it=1)
        with pytest.raises(_abi.MgrError, match="FP64"):
            dev.compute_level_populations("split", use_ng=False, max_it=1)
        # back to the diagonal ALO: the ordinary loop runs again
        dev.set_n_off_diag(0)
        got = dev.compute_level_populations("fp64", use_ng=False, max_it=1)
        assert got["iterations"] == 1
    finally:
        dev.close()


def test_core_model_banded_solve_and_jeff(gpu_lib):
    """The drop-in API with parameters.n_off_diag = 2: compute_level_populations for one
    iteration (against the oracle), then compute_radiation_field_feautrier_order_2 and
    compute_Jeff with the band elements: Jeff = Jlin - h/(4 pi) sum over the (point,
    line) Lambda list of Ls population(nr, upper) (model.cpp:514-545), the lists from
    the oracle's banded solve on the oracle's line data after the same iteration."""
    from magritte_gb300 import loader

    K = 2
    raw = S.grid_cube(n=6, nquads=5)
    ref_arrays = H.setup(raw)
    ref = O.AliOracle(raw, ref_arrays).run(use_ng=False, max_it=1, n_off_diag=K)
    model = loader.to_core(raw, precision="fp64")
    model.parameters.n_off_diag = K
    model.compute_spectral_discretisation()
    model.compute_inverse_line_widths()
    model.compute_LTE_level_populations()
    assert model.compute_level_populations(False, 1) == 1
    pop = np.array(model.lines.lineProducingSpecies[0].population).reshape(raw.npoints, -1)
    tot = raw.abundance[:, raw.linedata[0].num][:, None]
    ref_pop = ref["populations"][0]
    assert np.max(np.abs(pop - ref_pop) / np.maximum(np.abs(ref_pop), 1e-10 * tot)) < 1e-6
    model.compute_radiation_field_feautrier_order_2()
    model.compute_Jeff()
    lists = O.Oracle(ref_arrays).formal_solve_fo2_alo(K)
    a = ref_arrays
    P, Q, ld = raw.npoints, a["nquads"], raw.linedata[0]
    Jlin = np.zeros((P, ld.nrad))
    for f in range(a["nfreqs"]):
        Jlin[:, a["corr_line"][f]] += a["quad_weights"][0, a["corr_z"][f]] * lists["J"][:, f]
    diff = np.zeros((P, ld.nrad))
    for p in range(P):
        for k in range(ld.nrad):
            for i in range(lists["alo_n"][p, k]):
                diff[p, k] += lists["alo_ls"][p, k, i] * ref_pop[lists["alo_nr"][p, k, i], ld.irad[k]]
    hh4pi = S.HH / (4.0 * np.pi)
    Jeff_ref = Jlin - hh4pi * diff
    got = np.array(model.lines.lineProducingSpecies[0].Jeff).reshape(P, -1)
    assert np.max(np.abs(got - Jeff_ref) / np.max(np.abs(Jeff_ref))) < 1e-6
    # the band terms matter at this bar
    lam_only = Jlin - hh4pi * np.array([[lists["alo_ls"][p, k, 0] * ref_pop[p, ld.irad[k]]
                                         for k in range(ld.nrad)] for p in range(P)])
    assert np.max(np.abs(lam_only - Jeff_ref) / np.max(np.abs(Jeff_ref))) > 1e-5
