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
  keys128.npz    a 5-mode tensor whose packed off-mode keys need 64 to 73 bits,
                 one sweep per sampler.
  sweeps20.npz, sweeps20_dense.npz
                 20 sweeps of STS-CP (the 2000^3 workload; a 150^3 tensor with
                 30 % observed): fit after every sweep, sigma after every step.
  exact.npz      ExactALS, two sweeps on a 3- and a 4-mode tensor.
  stats_*.json   the statistics JSON of execute_ALS_rounds.
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


def support_tensor(dims, support, nnz, R, seed):
    """A tensor whose nonzeros sit on a small grid of coordinates spread over
    large modes (the highest coordinate of every mode included, so every bit of
    the packed keys is exercised), and factors that are nonzero only on those
    rows: sampled fibres then hold nonzeros, as they do after the exact-ALS
    preprocessing of a sparse tensor."""
    rng = np.random.default_rng(seed)
    rows = []
    for d, s in zip(dims, support):
        r = np.sort(rng.choice(d - 1, size=s - 1, replace=False))
        rows.append(np.concatenate([r, [d - 1]]).astype(np.uint32))
    cells = int(np.prod(support))
    lin = rng.choice(cells, size=nnz, replace=False)
    local = np.stack(np.unravel_index(lin, tuple(support)), axis=1)
    idx = np.stack([rows[k][local[:, k]] for k in range(len(dims))], axis=1).astype(np.uint32)
    vals = rng.random(nnz) + 0.5
    fvals = []
    for k, d in enumerate(dims):
        v = rng.standard_normal((len(rows[k]), R))
        v /= np.sqrt((v * v).sum(axis=0))[None, :]
        fvals.append(v)
    return np.ascontiguousarray(idx), vals, rows, fvals


def dense_factors(dims, rows, fvals):
    out = []
    for d, r, v in zip(dims, rows, fvals):
        U = np.zeros((int(d), v.shape[1]))
        U[r] = v
        out.append(U)
    return out


def keys128():
    """5-mode tensor whose packed off-mode coordinates need more than 64 bits
    for modes 1-4 (65, 65, 65, 73 bits) and exactly 64 for mode 0; one full
    sweep per sampler.  Factor rows are stored on the support only (the other
    rows are zero before and after every step)."""
    dims = (300_000, 250_000, 200_000, 150_000, 900)
    support = (12, 10, 9, 8, 6)
    R, J, nnz = 6, 1500, 4000
    idx, vals, rows, fvals = support_tensor(dims, support, nnz, R, seed=21)
    factors = dense_factors(dims, rows, fvals)
    out = {"dims": np.array(dims, dtype=np.int64), "R": np.int64(R), "J": np.int64(J), "idx": idx, "vals": vals}
    for k in range(len(dims)):
        out[f"rows{k}"] = rows[k]
        out[f"fvals{k}"] = fvals[k]
    for sampler in ("cp_arls_lev", "sts_cp"):
        rec = run_sweep(dims, idx, vals, R, factors, sampler, J, (31, 32), steps=len(dims))
        for t in range(len(dims)):
            U = rec.pop(f"s{t}_factor")
            n = t % len(dims)
            assert not np.any(np.delete(U, rows[n], axis=0)), "factor rows outside the support"
            rec[f"s{t}_factor_rows"] = U[rows[n]]
            rec[f"s{t}_spmm_out_rows"] = rec.pop(f"s{t}_spmm_out")[rows[n]]
        for k, v in rec.items():
            out[f"{sampler}_{k}"] = v
    np.savez_compressed(os.path.join(HERE, "keys128.npz"), **out)


def sweeps20(dense=False):
    """20 full sweeps of STS-CP by the reference with its local stream
    reseeded: the fit after every sweep and sigma after every step.  Default:
    the 2000^3 / 2e6-nonzero planted tensor, R=25, J=65536 (its fit stays near
    zero: 2.5e-4 of the entries are observed).  dense=True: a 150^3 planted
    rank-8 tensor with 30 % of its entries observed, R=8, J=16384, whose fit
    converges to a clearly positive value."""
    if dense:
        dims, idx, vals = synthetic.planted_uniform(dims=(150, 150, 150), nnz=1_012_500, rank=8, seed=5,
                                                    nonneg=False)
        R, J, sweeps = 8, 16384, 20
        factors = synthetic.gaussian_factors(dims, R, seed=6)
        seeds = (5353, 5454)
        name = "sweeps20_dense.npz"
    else:
        dims, idx, vals = synthetic.planted_uniform(seed=0)
        R, J, sweeps = 25, 65536, 20
        factors = synthetic.gaussian_factors(dims, R, seed=1)
        seeds = (5151, 5252)
        name = "sweeps20.npz"
    keep, st, lr, s, opt = make_problem(dims, idx, vals, R, factors, "sts_cp", seeds)
    N = len(dims)
    fits = [opt.compute_exact_fit()]
    sigmas = []
    for _ in range(sweeps):
        for n in range(N):
            opt.execute_ALS_step(n, J)
            sigmas.append(lr.get_sigma()[0])
        fits.append(opt.compute_exact_fit())
        print(f"sweep {len(fits) - 1}: fit {fits[-1]:.8f}", flush=True)
    out = {"seeds": np.array(seeds, dtype=np.int64), "R": np.int64(R), "J": np.int64(J), "sweeps": np.int64(sweeps),
           "fits": np.array(fits), "sigmas": np.array(sigmas),
           "final_factor0_head": lr.get_factor(0)[:64]}
    np.savez_compressed(os.path.join(HERE, name), **out)


def sweeps20_dense():
    sweeps20(dense=True)


def exact():
    """ExactALS (exact_als.hpp:90-143): two sweeps from given factors on a
    3-mode and a 4-mode tensor; factors and sigma after every step, fits."""
    out = {}
    for name, (d, nnz, R, seed) in {"e3": ((40, 35, 30), 2500, 5, 41), "e4": ((15, 12, 10, 9), 900, 4, 42)}.items():
        dims, idx, vals = synthetic.random_sparse(d, nnz, seed=seed)
        factors = synthetic.gaussian_factors(dims, R, seed=seed + 1)
        dims32 = np.asarray(dims, dtype=np.int32)
        g = REF.Grid(np.ones(len(dims), dtype=np.int32))
        tg = REF.TensorGrid(dims32, g)
        st = REF.SparseTensor(tg, np.ascontiguousarray(idx, dtype=np.uint32), np.asarray(vals, dtype=np.float64),
                              "none")
        st.set_indices(np.ascontiguousarray(idx, dtype=np.uint32))
        lr = REF.LowRankTensor(R, tg)
        for k, U in enumerate(factors):
            lr.set_factor(k, U)
        lr.set_sigma(np.ones(R))
        opt = REF.ExactALS(st, lr)
        opt.initialize_ground_truth_for_als()
        out[f"{name}_fit0"] = opt.compute_exact_fit()
        N = len(dims)
        for t in range(2 * N):
            opt.execute_ALS_step(t % N, 0)
            out[f"{name}_s{t}_factor"] = lr.get_factor(t % N)
            out[f"{name}_s{t}_sigma"] = lr.get_sigma()[0]
        out[f"{name}_fit1"] = opt.compute_exact_fit()
        out[f"{name}_idx"], out[f"{name}_vals"] = idx, vals
        out[f"{name}_dims"] = np.asarray(dims, dtype=np.int64)
        for k, U in enumerate(factors):
            out[f"{name}_U{k}"] = U
    np.savez_compressed(os.path.join(HERE, "exact.npz"), **out)


def stats_schema():
    """The statistics JSON of ALS_Optimizer::execute_ALS_rounds
    (als_optimizer.hpp:40-124, compute_dstat common.h:613-675) at one rank:
    two rounds on a small tensor, fit every round.  Timings vary run to run;
    the tests compare keys, nesting and the non-timing values."""
    dims, idx, vals = synthetic.random_sparse((30, 25, 20), 2000, seed=61)
    factors = synthetic.gaussian_factors(dims, 4, seed=62)
    for sampler in ("sts_cp", "cp_arls_lev"):
        keep, st, lr, s, opt = make_problem(dims, idx, vals, 4, factors, sampler, (71, 72))
        opt.execute_ALS_rounds(2, 500, 1)
        text = opt.get_statistics_json()
        with open(os.path.join(HERE, f"stats_{sampler}.json"), "w") as f:
            f.write(text + "\n")


if __name__ == "__main__":
    which = sys.argv[1:] or ["units", "steps", "workload1", "keys128", "sweeps20", "sweeps20_dense", "exact",
                             "stats_schema"]
    for w in which:
        globals()[w]()
        print("wrote", w)
