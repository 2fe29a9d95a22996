"""Generates the golden fixtures in tests/golden/ by running the reference's
own C++ (exafac/cpp_ext, compiled here by oracle/build_ref.sh into
oracle/_ref/exafac_ref*.so) on seeded inputs with injected random streams.

    OMP_NUM_THREADS=1 python tests/golden/make_golden.py

Every fixture stores its inputs (or the seeds that regenerate them) and the
reference's outputs.  The reference draws its uniforms from std::mt19937
streams; the harness reseeds them and replays them on copies, so the fixtures
hold the exact uniforms and per-mode permutations each draw consumed.

Fixtures:
  units.npz      PartitionTree build + PTSample on given matrices; pinv.
  steps.npz      small tensors (3 and 4 modes, edge shapes): one full sweep per
                 case with both samplers — draws, dedup, sampled MTTKRP, the
                 updated factors, sigma, hit counts, fits.
  workload1.npz  the 2000^3 / 2e6-nonzero planted tensor, R=25, J=65536,
                 STS-CP, one sweep (tensor and uniforms regenerated from seeds).
"""
import json
import os
import sys

os.environ.setdefault("OMP_NUM_THREADS", "1")
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import exafac_ref as REF  # noqa: E402
from rdist_tensor_gb300 import synthetic  # noqa: E402


def units():
    rng = np.random.default_rng(7)
    out = {}
    for name, (n, R, F, J) in {"t_partial": (37, 5, 5, 400), "t_eigen": (25, 25, 1, 300),
                               "t_rows": (203, 8, 8, 600), "t_single": (1, 4, 4, 50)}.items():
        U = rng.standard_normal((n, R))
        sh = rng.standard_normal((J, R))
        draws = rng.random(J)
        idx, h, G = REF.pt_sample(U, F, sh, draws)
        out.update({f"{name}_U": U, f"{name}_F": np.int64(F), f"{name}_x": sh, f"{name}_draws": draws,
                    f"{name}_idx": idx, f"{name}_h": h, f"{name}_G": G})
    A = rng.standard_normal((40, 6))
    out["pinv_full_in"] = A.T @ A
    out["pinv_full_out"] = REF.pinv_square(A.T @ A)
    B = rng.standard_normal((6, 3))
    out["pinv_deficient_in"] = B @ B.T
    out["pinv_deficient_out"] = REF.pinv_square(B @ B.T)
    np.savez_compressed(os.path.join(HERE, "units.npz"), **out)


def make_problem(dims, idx, vals, R, factors, sampler, seeds, preprocessing="none"):
    dims32 = np.asarray(dims, dtype=np.int32)
    g = REF.Grid(np.ones(len(dims), dtype=np.int32))
    tg = REF.TensorGrid(dims32, g)
    st = REF.SparseTensor(tg, np.ascontiguousarray(idx, dtype=np.uint32), np.asarray(vals, dtype=np.float64),
                          preprocessing)
    st.set_indices(np.ascontiguousarray(idx, dtype=np.uint32))  # undo the random relabelling
    lr = REF.LowRankTensor(R, tg)
    for k, U in enumerate(factors):
        lr.set_factor(k, U)
    lr.set_sigma(np.ones(R))
    s = REF.CP_ARLS_LEV(lr) if sampler == "cp_arls_lev" else REF.STS_CP(lr)
    opt = REF.AccumulatorStationary(st, lr, s)
    opt.initialize_ground_truth_for_als()
    s.reseed(*seeds)
    # Grid/TensorGrid are held by reference on the C++ side: keep them alive.
    return (g, tg), st, lr, s, opt


def run_sweep(dims, idx, vals, R, factors, sampler, J, seeds, steps, preprocessing="none", detail=True):
    keep, st, lr, s, opt = make_problem(dims, idx, vals, R, factors, sampler, seeds, preprocessing)
    N = len(dims)
    rec = {"fit0": opt.compute_exact_fit()}
    for t in range(steps):
        n = t % N
        saved = s.save_streams()
        if sampler == "cp_arls_lev":
            smp, w, uni, perm = s.draw(J, n)
            rec[f"s{t}_perms"] = perm
        else:
            smp, w, uni = s.draw(J, n)
        s.restore_streams(saved)
        rec[f"s{t}_uniforms"] = uni
        if detail:
            rec[f"s{t}_samples"] = smp
            rec[f"s{t}_weights"] = w
            sd, wd = opt.dedup(smp, w, n)
            rec[f"s{t}_samples_dedup"] = sd
            rec[f"s{t}_weights_dedup"] = wd
            # Sampled MTTKRP of the reference's lookup on a seeded design matrix.
            D = np.random.default_rng(100 + t).standard_normal((len(sd), R))
            M, found = opt.spmm(n, sd, D, int(dims[n]) + 1)
            rec[f"s{t}_spmm_design"] = D
            rec[f"s{t}_spmm_out"] = M[: int(dims[n])]
            rec[f"s{t}_spmm_found"] = np.int64(found)
        before = opt.nonzeros_iterated
        opt.execute_ALS_step(n, J)
        rec[f"s{t}_hits"] = np.int64(round(opt.nonzeros_iterated - before))
        rec[f"s{t}_factor"] = lr.get_factor(n)
        rec[f"s{t}_sigma"] = lr.get_sigma()[0]
    rec["fit1"] = opt.compute_exact_fit()
    return rec


def steps():
    out = {}
    cases = {
        "c3": dict(dims=(50, 40, 30), nnz=3000, R=6, J=800, seed=1),
        "c4": dict(dims=(20, 30, 12, 9), nnz=1500, R=5, J=700, seed=2),
        "dup": dict(dims=(6, 5, 4), nnz=60, R=3, J=500, seed=3),
        "one": dict(dims=(1, 30, 20), nnz=300, R=4, J=400, seed=4),
    }
    meta = {}
    for name, c in cases.items():
        dims, idx, vals = synthetic.random_sparse(c["dims"], c["nnz"], seed=c["seed"])
        factors = synthetic.gaussian_factors(dims, c["R"], seed=c["seed"] + 50)
        for sampler in ("cp_arls_lev", "sts_cp"):
            key = f"{name}_{sampler}"
            rec = run_sweep(dims, idx, vals, c["R"], factors, sampler, c["J"], (1000 + c["seed"], 2000 + c["seed"]),
                            steps=len(dims) + 1)
            for k, v in rec.items():
                out[f"{key}_{k}"] = v
            meta[key] = dict(c, sampler=sampler, steps=len(dims) + 1)
        out[f"{name}_idx"] = idx
        out[f"{name}_vals"] = vals
        for k, U in enumerate(factors):
            out[f"{name}_U{k}"] = U
    # log_count preprocessing on integer counts
    dims, idx, vals = synthetic.random_sparse((30, 25, 20), 2000, seed=9)
    vals = np.floor(vals * 20.0)
    factors = synthetic.gaussian_factors(dims, 4, seed=59)
    rec = run_sweep(dims, idx, vals, 4, factors, "cp_arls_lev", 600, (1009, 2009), steps=3,
                    preprocessing="log_count")
    for k, v in rec.items():
        out[f"logc_cp_arls_lev_{k}"] = v
    out["logc_idx"], out["logc_vals"] = idx, vals
    for k, U in enumerate(factors):
        out[f"logc_U{k}"] = U
    meta["logc_cp_arls_lev"] = dict(dims=(30, 25, 20), nnz=2000, R=4, J=600, seed=9, sampler="cp_arls_lev",
                                    steps=3, preprocessing="log_count")
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, "steps.npz"), **out)


def workload1():
    """2000^3, 2e6 nonzeros, planted rank 10, R=25, J=65536, STS-CP, one sweep."""
    dims, idx, vals = synthetic.planted_uniform(seed=0)
    R, J = 25, 65536
    factors = synthetic.gaussian_factors(dims, R, seed=1)
    seeds = (4242, 4343)
    rec = run_sweep(dims, idx, vals, R, factors, "sts_cp", J, seeds, steps=3, detail=False)
    out = {"seeds": np.array(seeds, dtype=np.int64), "R": np.int64(R), "J": np.int64(J),
           "fit0": rec["fit0"], "fit1": rec["fit1"]}
    for t in range(3):
        out[f"s{t}_hits"] = rec[f"s{t}_hits"]
        out[f"s{t}_factor"] = rec[f"s{t}_factor"]
        out[f"s{t}_sigma"] = rec[f"s{t}_sigma"]
    np.savez_compressed(os.path.join(HERE, "workload1.npz"), **out)


if __name__ == "__main__":
    which = sys.argv[1:] or ["units", "steps", "workload1"]
    for w in which:
        globals()[w]()
        print("wrote", w)
