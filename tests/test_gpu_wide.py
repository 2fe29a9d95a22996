"""GPU parity of the 32 < R <= 128 path (wide_kernels.cu): the FP64 form
against the oracle over a full sweep (1e-8, as for R <= 32), and the mixed
forms (FP32 design rows, MTTKRP, solve and STS-CP descents) against the FP64
form driven by the same uniforms over several sweeps: the fit within 1e-3 (the
spec bar), the factor error after each sweep reported."""
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


def rel_err(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def optimizer(dims, idx, vals, factors, sampler, J, precision):
    from rdist_tensor_gb300.api import (AccumulatorStationary, CP_ARLS_LEV, Grid, LowRankTensor, STS_CP,
                                        SparseTensor, TensorGrid)

    N = len(dims)
    tg = TensorGrid(np.asarray(dims, dtype=np.int64), Grid(np.ones(N, dtype=np.int32)))
    st = SparseTensor(tg, idx, vals, "none")
    lr = LowRankTensor(factors[0].shape[1], tg)
    lr.set_factors(factors)
    s = CP_ARLS_LEV(lr) if sampler == "cp_arls_lev" else STS_CP(lr)
    opt = AccumulatorStationary(st, lr, s, max_samples=J, precision=precision)
    opt.initialize_ground_truth_for_als()
    return opt, lr


@pytest.mark.parametrize("R", [48, 64, 100, 128])
@pytest.mark.parametrize("sampler", ["cp_arls_lev", "sts_cp"])
def test_fp64_wide_sweep_matches_oracle(lib, oracle_mod, sampler, R):
    from rdist_tensor_gb300 import synthetic

    dims, idx, vals = synthetic.planted_uniform(dims=(300, 250, 200), nnz=60000, rank=5, seed=3)
    J = 8192
    factors = synthetic.gaussian_factors(dims, R, seed=5)
    opt, lr = optimizer(dims, idx, vals, factors, sampler, J, "fp64")
    ora = oracle_mod.OracleALS(dims, idx, vals, factors, sampler)
    rng = np.random.default_rng(12 + R)
    for n in range(3):
        uni = rng.random((3, J) if sampler == "cp_arls_lev" else (3, 2, J))
        opt.execute_ALS_step(n, J, torch.as_tensor(uni, device="cuda"))
        out = ora.step(n, J, uni)
        assert opt.step_info().hits == out["hits"]
        assert rel_err(lr.factors[n].data.cpu().numpy(), out["factor"]) < 1e-8, n
        assert rel_err(lr.sigma.cpu().numpy(), out["sigma"]) < 1e-8, n
    assert abs(opt.compute_exact_fit() - ora.fit()) < 1e-8
    opt.deinitialize()


def planted(R_true, seed):
    from rdist_tensor_gb300 import synthetic

    # a convergent problem with every mode longer than R = 128: 37 % of a
    # 160 x 150 x 140 planted tensor observed
    return synthetic.planted_uniform(dims=(160, 150, 140), nnz=1_250_000, rank=R_true, seed=seed, nonneg=False)


@pytest.mark.parametrize("R", [64, 128])
@pytest.mark.parametrize("precision", ["tf32", "bf16"])
@pytest.mark.parametrize("sampler", ["sts_cp", "cp_arls_lev"])
def test_mixed_wide_equal_fit(lib, sampler, precision, R):
    """Mixed vs FP64 form at R = 64 / 128, the same uniforms, 6 sweeps: the
    fit after the last three within 1e-3 of the FP64 form's.  R is
    far above the planted rank, so the factors are poorly determined: the
    factor error between the forms is large while the fits agree (it is
    printed, not bounded).  CP-ARLS-LEV draws the same samples in both forms,
    so its first sweep (from random factors, the steepest) is also held to
    2e-3; the mixed STS-CP draws are other samples of the same distribution
    (Cholesky factors of the sampling matrices), so its first-sweep gap is
    sampling noise and only the fixed-sweep bar applies."""
    from rdist_tensor_gb300 import synthetic

    dims, idx, vals = planted(8, 7)
    J = 32768
    factors = synthetic.gaussian_factors(dims, R, seed=9)
    per = (3, J) if sampler == "cp_arls_lev" else (3, 2, J)
    rng = np.random.default_rng(31)
    uniforms = [torch.as_tensor(rng.random(per), device="cuda") for _ in range(18)]
    fits, facs = {}, {}
    for prec in ("fp64", precision):
        opt, lr = optimizer(dims, idx, vals, factors, sampler, J, prec)
        fl, fc = [], []
        for s in range(6):
            for n in range(3):
                opt.execute_ALS_step(n, J, uniforms[3 * s + n])
            fl.append(opt.compute_exact_fit())
            fc.append([f.data.cpu().numpy().copy() for f in lr.factors])
            assert opt.step_info().device_status == 0
        fits[prec], facs[prec] = fl, fc
        opt.deinitialize()
    err = [max(rel_err(a, b) for a, b in zip(facs[precision][s], facs["fp64"][s])) for s in range(6)]
    gaps = [abs(a - b) for a, b in zip(fits[precision], fits["fp64"])]
    print(f"{sampler} {precision} R={R}: fp64 fit {fits['fp64'][-1]:.6f}, gaps "
          + " ".join(f"{g:.1e}" for g in gaps) + ", factor error " + " ".join(f"{e:.1e}" for e in err))
    assert fits["fp64"][-1] > 0.1, fits
    assert max(gaps[-3:]) < 1e-3, gaps
    if sampler == "cp_arls_lev":
        assert max(gaps) < 2e-3, gaps
