"""The zero-sampling fit estimate (exafac_als_estimated_fit; the reference's
legacy compute_estimated_fit, exafac/low_rank_tensor.py:110-184) against the
oracle's restatement on the same zero samples (1e-10; the kept count exact),
including the 5-mode tensor whose fibre keys need more than 64 bits; its
Philox form is repeatable and close to the exact fit; factors written to a
file and read back resume the decomposition exactly."""
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


def optimizer(dims, idx, vals, factors, sampler="cp_arls_lev", J=2000):
    from rdist_tensor_gb300.api import (AccumulatorStationary, CP_ARLS_LEV, Grid, LowRankTensor, STS_CP,
                                        SparseTensor, TensorGrid)

    N = len(dims)
    tg = TensorGrid(np.asarray(dims, dtype=np.int64), Grid(np.ones(N, dtype=np.int32)))
    st = SparseTensor(tg, idx, vals, "none")
    lr = LowRankTensor(factors[0].shape[1], tg)
    lr.set_factors(factors)
    s = CP_ARLS_LEV(lr) if sampler == "cp_arls_lev" else STS_CP(lr)
    opt = AccumulatorStationary(st, lr, s, max_samples=J)
    opt.initialize_ground_truth_for_als()
    return opt, lr


def zero_coords(dims, idx, Z, seed):
    """Uniform coordinates, a quarter of them copied from nonzeros (collisions)."""
    rng = np.random.default_rng(seed)
    z = np.stack([rng.integers(0, d, size=Z) for d in dims], axis=1).astype(np.int64)
    pick = rng.choice(len(idx), size=Z // 4, replace=False)
    z[: Z // 4] = idx[pick]
    return z


def test_estimated_fit_matches_oracle(lib, oracle_mod):
    from rdist_tensor_gb300 import synthetic

    dims, idx, vals = synthetic.random_sparse((30, 25, 20), 3000, seed=4)
    factors = synthetic.gaussian_factors(dims, 6, seed=5)
    opt, lr = optimizer(dims, idx, vals, factors)
    for n in range(3):
        opt.execute_ALS_step(n, 2000)
    ora = oracle_mod.OracleALS(dims, idx, vals, [f.data.cpu().numpy() for f in lr.factors], "cp_arls_lev")
    ora.sigma = lr.sigma.cpu().numpy()
    z = zero_coords(dims, idx, 4000, 6)
    est, kept = opt.compute_estimated_fit(zero_coords=z)
    ref, ref_kept = oracle_mod.estimated_fit(ora, z)
    assert kept == ref_kept and kept <= 4000 - 1000
    assert abs(est - ref) < 1e-10, (est, ref)
    # the Philox draws: repeatable for a seed, and close to the exact fit on
    # this 20 %-dense tensor (15 000 cells, 3000 zero samples)
    a, ka = opt.compute_estimated_fit(seed=11)
    b, kb = opt.compute_estimated_fit(seed=11)
    assert a == b and ka == kb and 0 < ka <= 3000
    exact = opt.compute_exact_fit()
    assert abs(a - exact) < 0.05, (a, exact)
    opt.deinitialize()


def test_estimated_fit_membership_with_128bit_keys(lib, golden, oracle_mod):
    g = golden("keys128.npz")
    dims = [int(d) for d in g["dims"]]
    R = int(g["R"])
    factors = []
    for k in range(len(dims)):
        U = np.zeros((dims[k], R))
        U[g[f"rows{k}"].astype(np.int64)] = g[f"fvals{k}"]
        factors.append(U)
    opt, lr = optimizer(dims, g["idx"], g["vals"], factors, "sts_cp", 1500)
    ora = oracle_mod.OracleALS(dims, g["idx"], g["vals"], factors, "sts_cp")
    # zero samples on the support grid, where collisions are frequent
    rng = np.random.default_rng(3)
    rows = [g[f"rows{k}"].astype(np.int64) for k in range(len(dims))]
    z = np.stack([r[rng.integers(0, len(r), size=3000)] for r in rows], axis=1)
    est, kept = opt.compute_estimated_fit(zero_coords=z)
    ref, ref_kept = oracle_mod.estimated_fit(ora, z)
    assert kept == ref_kept and 0 < kept < 3000
    # the zero samples sit on the support, where the model is large: a large
    # negative estimate, compared relatively
    assert abs(est - ref) <= 1e-12 * max(1.0, abs(ref)), (est, ref)
    opt.deinitialize()


def test_factor_file_resumes_the_decomposition(lib, tmp_path):
    from rdist_tensor_gb300 import synthetic

    dims, idx, vals = synthetic.random_sparse((30, 25, 20), 3000, seed=4)
    factors = synthetic.gaussian_factors(dims, 6, seed=5)
    opt, lr = optimizer(dims, idx, vals, factors, "sts_cp")
    for n in range(3):
        opt.execute_ALS_step(n, 2000)
    fit = opt.compute_exact_fit()
    path = lr.write_to_file(str(tmp_path / "factors"), fmt="npz")
    opt.deinitialize()
    opt2, lr2 = optimizer(dims, idx, vals, synthetic.gaussian_factors(dims, 6, seed=9), "sts_cp")
    opt2.deinitialize()
    lr2.read_from_file(path)
    opt2.initialize_ground_truth_for_als()
    assert opt2.compute_exact_fit() == fit
    for a, b in zip(lr.factors, lr2.factors):
        assert torch.equal(a.data, b.data)
    opt2.deinitialize()
