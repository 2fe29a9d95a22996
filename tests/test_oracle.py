"""Pins the oracle (oracle/oracle.py + oracle_kernels.c) against the golden
fixtures made by running the reference's own C++ (tests/golden/make_golden.py).

Sampled indices are compared exactly; floating-point outputs within the stated
relative tolerances (the oracle's BLAS/LAPACK calls sum in a different order
than the reference's OpenBLAS kernels)."""
import json

import numpy as np
import pytest


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(np.max(np.abs(b)), 1e-300) if b.size else 1.0
    return float(np.max(np.abs(a - b)) / scale) if b.size else 0.0


@pytest.mark.parametrize("name", ["t_partial", "t_eigen", "t_rows", "t_single"])
def test_partition_tree_matches_reference(golden, oracle_mod, name):
    g = golden("units.npz")
    U, F, x, draws = g[f"{name}_U"], int(g[f"{name}_F"]), g[f"{name}_x"], g[f"{name}_draws"]
    n, R = U.shape
    tree = oracle_mod.PartitionTree(n, F, R)
    tree.build(U)
    Gref = g[f"{name}_G"].reshape(-1, R, R)
    iu = np.triu_indices(R)
    assert rel_err(tree.G[:, iu[0], iu[1]], Gref[:, iu[0], iu[1]]) < 1e-13
    h = np.ones_like(x)
    idx = tree.sample(U, x, h, draws)
    assert np.array_equal(idx, g[f"{name}_idx"])
    assert np.array_equal(h, g[f"{name}_h"])


@pytest.mark.parametrize("case", ["full", "deficient"])
def test_pinv_matches_reference(golden, oracle_mod, case):
    g = golden("units.npz")
    out = oracle_mod.pinv_square(g[f"pinv_{case}_in"])
    ref = g[f"pinv_{case}_out"]
    iu = np.triu_indices(ref.shape[0])
    assert rel_err(out[iu], ref[iu]) < 1e-10


def _cases(golden):
    g = golden("steps.npz")
    return g, json.loads(str(g["meta"]))


STEP_CASES = ["c3_cp_arls_lev", "c3_sts_cp", "c4_cp_arls_lev", "c4_sts_cp", "dup_cp_arls_lev", "dup_sts_cp",
              "one_cp_arls_lev", "one_sts_cp", "logc_cp_arls_lev"]


def _problem(g, meta, key, oracle_mod):
    m = meta[key]
    base = key.split("_")[0]
    dims = m["dims"]
    factors = [g[f"{base}_U{k}"] for k in range(len(dims))]
    return oracle_mod.OracleALS(dims, g[f"{base}_idx"], g[f"{base}_vals"], factors, m["sampler"],
                                m.get("preprocessing", "none")), m


@pytest.mark.parametrize("key", STEP_CASES)
def test_sweep_matches_reference(golden, oracle_mod, key):
    g, meta = _cases(golden)
    ora, m = _problem(g, meta, key, oracle_mod)
    N, J = len(m["dims"]), m["J"]
    assert abs(ora.fit() - float(g[f"{key}_fit0"])) < 1e-10
    for t in range(m["steps"]):
        n = t % N
        uni = g[f"{key}_s{t}_uniforms"]
        perms = g[f"{key}_s{t}_perms"] if m["sampler"] == "cp_arls_lev" else None
        has_detail = f"{key}_s{t}_samples" in g
        if has_detail:
            samples, weights = ora.draw(n, J, uni, perms)
            assert np.array_equal(samples, g[f"{key}_s{t}_samples"]), f"step {t}: sampled indices differ"
            assert rel_err(weights, g[f"{key}_s{t}_weights"]) < 1e-12
            sd, wd = oracle_mod.deduplicate(samples, weights, n)
            ref_sd = g[f"{key}_s{t}_samples_dedup"]
            cols = [k for k in range(N) if k != n]
            assert np.array_equal(sd[:, cols], ref_sd[:, cols])
            assert rel_err(wd, g[f"{key}_s{t}_weights_dedup"]) < 1e-12
            M, found = ora.lookups[n].sampled_mttkrp(ref_sd, g[f"{key}_s{t}_spmm_design"], m["dims"][n])
            assert found == int(g[f"{key}_s{t}_spmm_found"])
            assert rel_err(M, g[f"{key}_s{t}_spmm_out"]) < 1e-13
        out = ora.step(n, J, uni, perms)
        assert out["hits"] == int(g[f"{key}_s{t}_hits"])
        assert rel_err(out["factor"], g[f"{key}_s{t}_factor"]) < 1e-8, f"step {t}"
        assert rel_err(out["sigma"], g[f"{key}_s{t}_sigma"]) < 1e-8
    assert abs(ora.fit() - float(g[f"{key}_fit1"])) < 1e-8


@pytest.mark.slow
def test_workload1_sweep_matches_reference(golden, oracle_mod):
    """2000^3 planted tensor, 2e6 nonzeros, R=25, J=65536, STS-CP: one sweep
    of the oracle against the reference (tensor and uniforms regenerated)."""
    from rdist_tensor_gb300 import synthetic

    g = golden("workload1.npz")
    dims, idx, vals = synthetic.planted_uniform(seed=0)
    R, J = int(g["R"]), int(g["J"])
    factors = synthetic.gaussian_factors(dims, R, seed=1)
    ora = oracle_mod.OracleALS(dims, idx, vals, factors, "sts_cp")
    assert abs(ora.fit() - float(g["fit0"])) < 1e-10
    streams = oracle_mod.sts_uniform_stream(int(g["seeds"][0]), 3, J, 3)
    for t in range(3):
        out = ora.step(t, J, streams[t])
        assert out["hits"] == int(g[f"s{t}_hits"])
        assert rel_err(out["factor"], g[f"s{t}_factor"]) < 1e-9
        assert rel_err(out["sigma"], g[f"s{t}_sigma"]) < 1e-9
    assert abs(ora.fit() - float(g["fit1"])) < 1e-9
