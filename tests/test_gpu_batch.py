"""Many-model batch (mgr_batch_*): every model's J and ALO diagonal from the one
persistent launch equal its own single-model formal solve (same lane code, same
order of the sums) and the oracle within the single-model bars."""
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


def _rel(x, ref):
    return float(np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1e-300)))


RAWS = [
    lambda: S.grid_cube(n=8, nquads=5),
    lambda: S.grid_sphere(n=14, nside=1, nquads=11),
    lambda: S.grid_cube(n=12, nquads=7, seed=3),
    lambda: S.grid_sphere(n=16, nside=2, nquads=5),
    lambda: S.grid_cube(n=10, nquads=11, seed=5),
]


@pytest.mark.parametrize("approx", ["CloseLines", "None"])
def test_batch_matches_single_model_solves(gpu_lib, approx):
    arrays = [H.setup(r(), approx=approx) for r in RAWS]
    devs = [_abi.DeviceModel(a) for a in arrays]
    batch = _abi.Batch(devs)
    try:
        for prec in ("fp64", "split"):
            got = batch.formal_solve_fo2(prec)
            # Split precision: the same lane code and order of the sums, 1e-13.  FP64 mode:
            # the two kernels' lane code may round an FP64 multiply-add differently (the
            # compiler's contraction of each instantiation), which can move a
            # single-precision erff argument by an ulp; the same-wing erf differences
            # amplify that (measured 8.5e-9 under CloseLines, 1.3e-8 under None): 1e-6,
            # far inside the 1e-5 parity bar.
            bar = 1e-6 if prec == "fp64" else 1e-13
            for d, g in zip(devs, got):
                ref = d.formal_solve_fo2(prec)
                assert _rel(g["J"], ref["J"]) < bar
                assert _rel(g["lambda_diag"], ref["lambda_diag"]) < bar
        start, finish = batch.timings()
        assert np.all(start >= 0) and np.all(finish >= start)
        got = batch.formal_solve_fo2("fp64")
        for a, g in zip(arrays, got):
            ref = O.Oracle(a).formal_solve_fo2()
            has = ref["lambda_has"].astype(bool)
            # the FP64 bar of the single-model solve (libm differences of expf / powf)
            assert H.max_rel(g["J"], ref["J"]) < 1e-5
            assert H.max_rel(g["lambda_diag"][has], ref["lambda_diag"][has]) < 1e-5
    finally:
        batch.close()
        for d in devs:
            d.close()


def test_batch_tuning_shapes_agree(gpu_lib):
    arrays = [H.setup(r()) for r in RAWS[:3]]
    devs = [_abi.DeviceModel(a) for a in arrays]
    batch = _abi.Batch(devs)
    try:
        base = batch.formal_solve_fo2("split")
        for minb, warps in ((3, 4), (4, 8), (2, 2)):
            batch.set_tuning(minb, warps)
            got = batch.formal_solve_fo2("split")
            for g, b in zip(got, base):
                np.testing.assert_array_equal(g["J"], b["J"])
        with pytest.raises(_abi.MgrError):
            batch.set_tuning(5, 0)
    finally:
        batch.close()
        for d in devs:
            d.close()


def test_batch_rejects_mixed_approximations(gpu_lib):
    a = H.setup(RAWS[0](), approx="CloseLines")
    b = H.setup(RAWS[0](), approx="None")
    da, db = _abi.DeviceModel(a), _abi.DeviceModel(b)
    try:
        with pytest.raises(_abi.MgrError):
            _abi.Batch([da, db])
    finally:
        da.close()
        db.close()


def test_batch_refuses_other_geometries(gpu_lib):
    """Batches take general-geometry models with shared rays; a spherically symmetric
    model is refused with an error (it is solved by its own mgr_formal_solve_fo2)."""
    devs = [_abi.DeviceModel(H.setup(S.grid_cube(n=6, nquads=3))),
            _abi.DeviceModel(H.setup(S.density_distribution_1d("a", npoints=20, nrays=8, nquads=3)))]
    try:
        with pytest.raises(_abi.MgrError, match="spherically symmetric"):
            _abi.Batch(devs)
    finally:
        for d in devs:
            d.close()
