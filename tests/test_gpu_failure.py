"""Failure detection on the GPU without a fault: a bounded device-side wait
that runs out reports EXAFAC_ERR_TIMEOUT through the session's status word,
the context stays usable, and the step does no work with the unsorted hits.
The wait is made to run out by a test hook (a sort tile that publishes no
status, and a short poll limit), not by breaking anything on the device.
Also: factors with a NaN are refused on the host before any launch."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from rdist_tensor_gb300 import _lib

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return _lib


def optimizer(precision, sampler="cp_arls_lev"):
    from rdist_tensor_gb300 import synthetic
    from rdist_tensor_gb300.api import (AccumulatorStationary, CP_ARLS_LEV, Grid, LowRankTensor, STS_CP,
                                        SparseTensor, TensorGrid)

    dims, idx, vals = synthetic.planted_uniform(dims=(60, 50, 40), nnz=100000, rank=5, seed=3, nonneg=False)
    tg = TensorGrid(dims, Grid(np.ones(3, dtype=np.int32)))
    st = SparseTensor(tg, idx, vals, "none")
    lr = LowRankTensor(5, tg)
    lr.set_factors(synthetic.gaussian_factors(dims, 5, seed=6))
    s = CP_ARLS_LEV(lr) if sampler == "cp_arls_lev" else STS_CP(lr)
    opt = AccumulatorStationary(st, lr, s, max_samples=4096, precision=precision)
    opt.initialize_ground_truth_for_als()
    return opt, lr


def raw_info(lib, opt):
    out = lib.StepInfo()
    lib.call("exafac_als_step_info", opt._h, ctypes.byref(out), ctypes.c_void_p(0))
    return out


@pytest.mark.parametrize("precision", ["fp64", "tf32"])
def test_lookback_wait_runs_out_and_reports_timeout(lib, precision):
    opt, lr = optimizer(precision)
    opt.execute_ALS_step(0, 4096)
    info = raw_info(lib, opt)
    assert info.device_status == 0
    assert info.hits > 3 * 4096  # the row sort of a step spans several 4096-hit tiles
    lib.call("exafac_als_set_wait_limit", opt._h, 256, 0)  # tile 0 publishes nothing
    opt.execute_ALS_step(1, 4096)
    torch.cuda.synchronize()  # the step finished: every wait ran out and returned
    info = raw_info(lib, opt)
    assert info.device_status == 4  # EXAFAC_ERR_TIMEOUT
    assert info.touched_rows == 0  # no work was done with the unsorted hits
    with pytest.raises(lib.ExafacError, match="wait ran out"):
        opt.step_info()
    opt.deinitialize()
    # the context is still usable: a fresh session steps normally
    torch.cuda.synchronize()
    opt2, _ = optimizer(precision)
    for n in range(3):
        opt2.execute_ALS_step(n, 4096)
    assert raw_info(lib, opt2).device_status == 0
    assert 0.0 < opt2.compute_exact_fit() < 1.0
    opt2.deinitialize()


def test_nan_factor_refused_on_host(lib):
    from rdist_tensor_gb300 import synthetic
    from rdist_tensor_gb300.api import AccumulatorStationary, CP_ARLS_LEV, Grid, LowRankTensor, SparseTensor, TensorGrid

    dims, idx, vals = synthetic.random_sparse((20, 15, 10), 500, seed=1)
    tg = TensorGrid(dims, Grid(np.ones(3, dtype=np.int32)))
    st = SparseTensor(tg, idx, vals, "none")
    lr = LowRankTensor(4, tg)
    f = synthetic.gaussian_factors(dims, 4, seed=2)
    f[1][3, 2] = np.nan
    lr.set_factors(f)
    opt = AccumulatorStationary(st, lr, CP_ARLS_LEV(lr), max_samples=256)
    launches = lib.load().exafac_kernel_launches()
    with pytest.raises(ValueError, match="non-finite"):
        opt.initialize_ground_truth_for_als()
    assert lib.load().exafac_kernel_launches() == launches


def test_rank_deficient_factors_take_the_pseudo_inverse(lib, oracle_mod):
    """Singular design Gram (a factor of rank 2 < R = 4): the eigenvalue cut
    of the pseudo-inverse, as the reference's compute_pinv_square; the step
    matches the oracle."""
    from rdist_tensor_gb300 import synthetic
    from rdist_tensor_gb300.api import AccumulatorStationary, CP_ARLS_LEV, Grid, LowRankTensor, SparseTensor, TensorGrid

    dims, idx, vals = synthetic.random_sparse((30, 25, 20), 3000, seed=4)
    f = synthetic.gaussian_factors(dims, 4, seed=5)
    f[1] = np.ascontiguousarray(f[1][:, :2] @ np.random.default_rng(6).standard_normal((2, 4)))
    f[2] = np.ascontiguousarray(f[2][:, :2] @ np.random.default_rng(7).standard_normal((2, 4)))
    tg = TensorGrid(dims, Grid(np.ones(3, dtype=np.int32)))
    st = SparseTensor(tg, idx, vals, "none")
    lr = LowRankTensor(4, tg)
    lr.set_factors(f)
    opt = AccumulatorStationary(st, lr, CP_ARLS_LEV(lr), max_samples=2000)
    opt.initialize_ground_truth_for_als()
    ora = oracle_mod.OracleALS(dims, idx, vals, f, "cp_arls_lev")
    uni = np.random.default_rng(8).random((3, 2000))
    opt.execute_ALS_step(0, 2000, torch.as_tensor(uni, device="cuda"))
    out = ora.step(0, 2000, uni)
    got = lr.factors[0].data.cpu().numpy()
    assert np.all(np.isfinite(got))
    assert np.max(np.abs(got - out["factor"])) / np.max(np.abs(out["factor"])) < 1e-8
    opt.deinitialize()
