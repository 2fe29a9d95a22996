"""No kernel may read session workspace it has not written: the same sweeps
with the workspace filled with zero bytes and with 0xFF bytes (a NaN in
every float and double) give bitwise equal, finite results, for every form
and both samplers, at R <= 32 and R > 32.  (A padded FP32 MTTKRP row that the
carry fix-up left unwritten once turned such a NaN into NaN factors.)"""
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


def run(dims, idx, vals, factors, sampler, precision, fill, J=4096, sweeps=3):
    from rdist_tensor_gb300.api import (AccumulatorStationary, CP_ARLS_LEV, Grid, LowRankTensor, STS_CP,
                                        SparseTensor, TensorGrid)

    tg = TensorGrid(dims, Grid(np.ones(len(dims), dtype=np.int32)))
    st = SparseTensor(tg, idx, vals, "none")
    lr = LowRankTensor(factors[0].shape[1], tg)
    lr.set_factors(factors)
    s = CP_ARLS_LEV(lr) if sampler == "cp_arls_lev" else STS_CP(lr)
    opt = AccumulatorStationary(st, lr, s, max_samples=J, precision=precision, workspace_fill=fill)
    opt.initialize_ground_truth_for_als()
    for _ in range(sweeps):
        for n in range(len(dims)):
            opt.execute_ALS_step(n, J)
    assert opt.step_info().device_status == 0
    fit = opt.compute_exact_fit()
    out = [f.data.clone() for f in lr.factors] + [lr.sigma.clone()]
    opt.deinitialize()
    return out, fit


@pytest.mark.parametrize("R", [5, 48])
@pytest.mark.parametrize("precision", ["fp64", "tf32", "bf16"])
@pytest.mark.parametrize("sampler", ["cp_arls_lev", "sts_cp"])
def test_results_do_not_depend_on_workspace_contents(lib, sampler, precision, R):
    from rdist_tensor_gb300 import synthetic

    dims, idx, vals = synthetic.planted_uniform(dims=(60, 50, 40), nnz=100000, rank=5, seed=3, nonneg=False)
    factors = synthetic.gaussian_factors(dims, R, seed=6)
    a, fa = run(dims, idx, vals, factors, sampler, precision, 0x00)
    b, fb = run(dims, idx, vals, factors, sampler, precision, 0xFF)
    for x, y in zip(a, b):
        assert bool(torch.isfinite(x).all())
        assert torch.equal(x, y)
    assert fa == fb and np.isfinite(fa)
