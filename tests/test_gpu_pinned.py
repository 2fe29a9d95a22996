"""GPU parity on the paths the first fixtures left open, against the
reference's own outputs (tests/golden/make_golden.py):

* a 5-mode tensor whose packed off-mode coordinates need more than 64 bits
  (128-bit fibre keys in the lookup and the deduplication), both samplers;
* ExactALS (exact_als.hpp:90-143), the "-p exact" preprocessing;
* 20 sweeps of the 2000^3 / 2e6-nonzero STS-CP workload (R=25, J=65536): the
  fit after every sweep;
* the statistics JSON of execute_ALS_rounds (keys and nesting).

Bars as in test_gpu_parity: indices bit-exact, weights and sampled MTTKRP
1e-12 relative, factors/sigma/fits 1e-8 over one sweep; the fit after each
of 20 sweeps within 1e-3 (and bitwise-close while no sampled index differs)."""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if b.size == 0:
        return 0.0
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def lib():
    from rdist_tensor_gb300 import _lib

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return _lib


def dev(a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype).contiguous()


def optimizer(dims, idx, vals, factors, sampler, J_max, precision="fp64"):
    from exafac.cpp_ext.py_module import (AccumulatorStationary, CP_ARLS_LEV, Grid, LowRankTensor, STS_CP,
                                          SparseTensor, TensorGrid)

    N = len(dims)
    tg = TensorGrid(np.asarray(dims, dtype=np.int64), Grid(np.ones(N, dtype=np.int32)))
    st = SparseTensor(tg, np.asarray(idx, dtype=np.uint32), np.asarray(vals, dtype=np.float64), "none")
    lr = LowRankTensor(factors[0].shape[1], tg)
    lr.set_factors(factors)
    s = CP_ARLS_LEV(lr) if sampler == "cp_arls_lev" else STS_CP(lr)
    opt = AccumulatorStationary(st, lr, s, max_samples=J_max, precision=precision)
    opt.initialize_ground_truth_for_als()
    return opt, lr


def key_bits(dims, skip):
    return sum(max(1, int(np.ceil(np.log2(d)))) for k, d in enumerate(dims) if k != skip)


@pytest.mark.parametrize("sampler", ["cp_arls_lev", "sts_cp"])
def test_128bit_fibre_keys_sweep_matches_reference(lib, golden, sampler):
    g = golden("keys128.npz")
    dims = [int(d) for d in g["dims"]]
    N, R, J = len(dims), int(g["R"]), int(g["J"])
    # modes 1..4 pack their off-mode coordinates into more than 64 bits
    assert [key_bits(dims, n) > 64 for n in range(N)] == [False, True, True, True, True]
    assert key_bits(dims, 0) == 64
    rows = [g[f"rows{k}"].astype(np.int64) for k in range(N)]
    factors = []
    for k in range(N):
        U = np.zeros((dims[k], R))
        U[rows[k]] = g[f"fvals{k}"]
        factors.append(U)
    opt, lr = optimizer(dims, g["idx"], g["vals"], factors, sampler, J)
    p = f"{sampler}_"
    assert abs(opt.compute_exact_fit() - float(g[p + "fit0"])) < 1e-10
    for t in range(N):
        n = t
        uni = dev(g[f"{p}s{t}_uniforms"], torch.float64)
        perms = dev(g[f"{p}s{t}_perms"].astype(np.int32), torch.int32) if sampler == "cp_arls_lev" else None
        samples, weights = opt.draw(n, J, uni, perms)
        assert np.array_equal(samples.cpu().numpy().astype(np.uint32), g[f"{p}s{t}_samples"]), f"step {t}"
        assert rel_err(weights.cpu().numpy(), g[f"{p}s{t}_weights"]) < 1e-12
        M = opt.sampled_mttkrp(n, g[f"{p}s{t}_samples_dedup"], g[f"{p}s{t}_spmm_design"]).cpu().numpy()
        assert opt.step_info().hits == int(g[f"{p}s{t}_spmm_found"])
        assert int(g[f"{p}s{t}_spmm_found"]) > 0
        assert rel_err(M[rows[n]], g[f"{p}s{t}_spmm_out_rows"]) < 1e-12
        assert not np.any(np.delete(M, rows[n], axis=0))
        opt.execute_ALS_step(n, J, uni, perms)
        info = opt.step_info()
        assert info.hits == int(g[f"{p}s{t}_hits"])
        sd, wd, _, _ = opt.last_dedup()
        sd, wd = sd.cpu().numpy().astype(np.uint32), wd.cpu().numpy()
        ref_sd, ref_wd = g[f"{p}s{t}_samples_dedup"], g[f"{p}s{t}_weights_dedup"]
        cols = [k for k in range(N) if k != n]
        o1 = np.lexsort(tuple(sd[:, k] for k in reversed(cols)))
        o2 = np.lexsort(tuple(ref_sd[:, k] for k in reversed(cols)))
        assert np.array_equal(sd[o1][:, cols], ref_sd[o2][:, cols])
        assert rel_err(wd[o1], ref_wd[o2]) < 1e-12
        U = lr.factors[n].data.cpu().numpy()
        assert rel_err(U[rows[n]], g[f"{p}s{t}_factor_rows"]) < 1e-8, f"step {t}"
        assert not np.any(np.delete(U, rows[n], axis=0))
        assert rel_err(lr.sigma.cpu().numpy(), g[f"{p}s{t}_sigma"]) < 1e-8
    assert abs(opt.compute_exact_fit() - float(g[p + "fit1"])) < 1e-8
    opt.deinitialize()


@pytest.mark.parametrize("case", ["e3", "e4"])
def test_exact_als_matches_reference(lib, golden, case):
    from exafac.cpp_ext.py_module import ExactALS, Grid, LowRankTensor, SparseTensor, TensorGrid

    g = golden("exact.npz")
    dims = [int(d) for d in g[f"{case}_dims"]]
    N = len(dims)
    factors = [g[f"{case}_U{k}"] for k in range(N)]
    tg = TensorGrid(np.asarray(dims, dtype=np.int64), Grid(np.ones(N, dtype=np.int32)))
    st = SparseTensor(tg, g[f"{case}_idx"], g[f"{case}_vals"], "none")
    lr = LowRankTensor(factors[0].shape[1], tg)
    lr.set_factors(factors)
    opt = ExactALS(st, lr)
    opt.initialize_ground_truth_for_als()
    assert abs(opt.compute_exact_fit() - float(g[f"{case}_fit0"])) < 1e-10
    for t in range(2 * N):
        opt.execute_ALS_step(t % N, 0)
        assert rel_err(lr.factors[t % N].data.cpu().numpy(), g[f"{case}_s{t}_factor"]) < 1e-8, f"step {t}"
        assert rel_err(lr.sigma.cpu().numpy(), g[f"{case}_s{t}_sigma"]) < 1e-8, f"step {t}"
    assert abs(opt.compute_exact_fit() - float(g[f"{case}_fit1"])) < 1e-8
    opt.deinitialize()


TWENTY = {
    # 2000^3 planted, 2e6 nonzeros, R=25, J=65536 (the plain STS-CP workload)
    "sweeps20.npz": dict(gen=lambda s: s.planted_uniform(seed=0), factor_seed=1),
    # 150^3 planted rank 8, 30 % observed, R=8, J=16384 (fit converges to ~0.16)
    "sweeps20_dense.npz": dict(gen=lambda s: s.planted_uniform(dims=(150, 150, 150), nnz=1_012_500, rank=8, seed=5,
                                                              nonneg=False), factor_seed=6),
}


@pytest.mark.parametrize("name", sorted(TWENTY))
def test_twenty_sweeps_fit_matches_reference(lib, golden, oracle_mod, name):
    """20 STS-CP sweeps with the reference's uniform stream replayed: the fit
    after every sweep within 1e-3 of the reference's (the correctness bar of
    the sampled solver).  While the samples are identical the FP64 path tracks
    the reference to rounding (fits to 1e-8, sigma to 1e-8 relative): checked
    over the first 5 sweeps.  Later, the rounding differences (summation
    order) carried through 3 pseudo-inverses per sweep can move one sampled
    index, after which the two runs are different draws of the same sampler."""
    from rdist_tensor_gb300 import synthetic

    g = golden(name)
    dims, idx, vals = TWENTY[name]["gen"](synthetic)
    R, J, sweeps = int(g["R"]), int(g["J"]), int(g["sweeps"])
    factors = synthetic.gaussian_factors(dims, R, seed=TWENTY[name]["factor_seed"])
    opt, lr = optimizer(dims, idx, vals, factors, "sts_cp", J)
    ref_fits, ref_sig = g["fits"], g["sigmas"]
    assert abs(opt.compute_exact_fit() - ref_fits[0]) < 1e-10
    streams = oracle_mod.sts_uniform_stream(int(g["seeds"][0]), 3, J, 3 * sweeps)
    gaps, sig_err = [], []
    for s in range(sweeps):
        for n in range(3):
            opt.execute_ALS_step(n, J, dev(streams[3 * s + n], torch.float64))
            sig_err.append(rel_err(lr.sigma.cpu().numpy(), ref_sig[3 * s + n]))
        gaps.append(abs(opt.compute_exact_fit() - ref_fits[s + 1]))
    print(f"{name}: fit gaps", " ".join(f"{x:.1e}" for x in gaps), "max sigma error", f"{max(sig_err):.1e}")
    assert max(gaps) < 1e-3, gaps
    assert max(gaps[:5]) < 1e-8, gaps
    assert max(sig_err[:15]) < 1e-8, sig_err
    opt.deinitialize()


@pytest.mark.parametrize("sampler", ["sts_cp", "cp_arls_lev"])
def test_statistics_json_schema(lib, sampler):
    """execute_ALS_rounds + get_statistics_json: same keys, nesting and
    round bookkeeping as the reference's JSON (captured from the reference
    on the same small problem)."""
    from rdist_tensor_gb300 import synthetic

    with open(os.path.join(HERE, "golden", f"stats_{sampler}.json")) as f:
        ref = json.load(f)
    dims, idx, vals = synthetic.random_sparse((30, 25, 20), 2000, seed=61)
    factors = synthetic.gaussian_factors(dims, 4, seed=62)
    opt, lr = optimizer(dims, idx, vals, factors, sampler, 500)
    opt.execute_ALS_rounds(2, 500, 1)
    got = json.loads(opt.get_statistics_json())
    assert set(got) == set(ref)
    for k, v in ref.items():
        if isinstance(v, dict):
            assert set(got[k]) == set(v), k
            assert got[k]["std"] is None and v["std"] is None
            assert got[k]["min"] == got[k]["mean"] == got[k]["max"]
        elif isinstance(v, list):
            assert len(got[k]) == len(v), k
    assert got["rounds"] == ref["rounds"] == [0, 1, 2]
    assert got["num_rounds"] == ref["num_rounds"] == 2
    assert got["fits"][0] == 0.0 and got["als_times"][0] == 0.0
    assert got["als_times"][2] >= got["als_times"][1] > 0.0
    assert got["als_total_time"] == got["als_times"][2]
    assert got["sum_nonzeros_iterated"] > 0
    assert got["avg_nonzeros_iterated"]["mean"] == got["sum_nonzeros_iterated"]
    for r in ("leverage_sampling_time", "design_matrix_prep_time", "spmm_time", "postprocessing_time",
              "sampler_update_time"):
        assert got[r]["mean"] > 0.0, r
    assert got["row_gather_time"]["mean"] == 0.0 and got["dense_reduce_time"]["mean"] == 0.0
    # the region timers sum to no more than the round timer
    regions = sum(got[r]["mean"] for r in ref if isinstance(ref[r], dict) and r != "avg_nonzeros_iterated")
    assert regions <= got["als_total_time"] * 1.05 + 1e-4
    opt.deinitialize()
