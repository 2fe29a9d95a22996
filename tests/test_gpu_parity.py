"""GPU parity: the CUDA path (libexafac_gb300.so through its C ABI) against the
reference's own outputs (golden fixtures) and the oracle.

Bars: sampled indices bit-exact; weights and sampled MTTKRP within 1e-12
relative (of the largest magnitude); factors, sigma and fits within 1e-8
(they pass through the R x R pseudo-inverse, whose conditioning multiplies
the ~1e-16 differences in summation order)."""
import ctypes
import json

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


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


def P(t):
    return ctypes.c_void_p(t.data_ptr())


def unpack(Gp, R):
    nodes = Gp.shape[0]
    out = np.zeros((nodes, R, R))
    iu = np.triu_indices(R)
    out[:, iu[0], iu[1]] = Gp
    out[:, iu[1], iu[0]] = Gp
    return out


@pytest.mark.parametrize("name", ["t_partial", "t_eigen", "t_rows", "t_single"])
def test_tree_build_and_sample(lib, golden, name):
    g = golden("units.npz")
    U, F, x, draws = g[f"{name}_U"], int(g[f"{name}_F"]), g[f"{name}_x"], g[f"{name}_draws"]
    n, R = U.shape
    J = x.shape[0]
    nodes = lib.load().exafac_tree_node_count(n, F)
    Ud = dev(U, torch.float64)
    G = torch.zeros((nodes, R * (R + 1) // 2), dtype=torch.float64, device="cuda")
    lib.call("exafac_tree_build", n, F, R, P(Ud), P(G), None)
    Gref = g[f"{name}_G"].reshape(-1, R, R)
    iu = np.triu_indices(R)
    assert rel_err(G.cpu().numpy(), Gref[:, iu[0], iu[1]]) < 1e-13
    xd = dev(x, torch.float64)
    h = torch.ones((J, R), dtype=torch.float64, device="cuda")
    dd = dev(draws, torch.float64)
    rows = torch.zeros(J, dtype=torch.int32, device="cuda")
    lib.call("exafac_tree_sample", n, F, R, P(G), P(Ud), J, P(xd), P(h), P(dd), P(rows), 1, None)
    torch.cuda.synchronize()
    assert np.array_equal(rows.cpu().numpy().astype(np.uint32), g[f"{name}_idx"])
    assert np.array_equal(h.cpu().numpy(), g[f"{name}_h"])


@pytest.mark.parametrize("case", ["full", "deficient"])
def test_pinv_square(lib, golden, case):
    g = golden("units.npz")
    A = g[f"pinv_{case}_in"]
    R = A.shape[0]
    Ad = dev(A, torch.float64)
    out = torch.zeros((R, R), dtype=torch.float64, device="cuda")
    nbytes = lib.load().exafac_dense_workspace_bytes(R)
    ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    lib.call("exafac_pinv_square", R, P(Ad), P(out), ctypes.c_double(1e-11), P(ws), ctypes.c_size_t(nbytes), None)
    ref = g[f"pinv_{case}_out"]
    iu = np.triu_indices(R)
    assert rel_err(out.cpu().numpy()[iu], ref[iu]) < 1e-10


@pytest.mark.parametrize("R,rank", [(92, 92), (93, 93), (128, 128), (128, 70)])
def test_pinv_square_large_rank(lib, R, rank):
    """Ranks on both sides of the largest one whose Cholesky buffers fit in
    shared memory (92); above it the Jacobi path runs alone."""
    rng = np.random.default_rng(R + rank)
    B = rng.standard_normal((R + 5, rank))
    A = B[:R] @ B[:R].T if rank < R else B.T @ B
    Ad = dev(A, torch.float64)
    out = torch.zeros((R, R), dtype=torch.float64, device="cuda")
    nbytes = lib.load().exafac_dense_workspace_bytes(R)
    ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    lib.call("exafac_pinv_square", R, P(Ad), P(out), ctypes.c_double(1e-11), P(ws), ctypes.c_size_t(nbytes), None)
    ref = np.linalg.pinv(A, rcond=1e-10, hermitian=True)
    assert rel_err(out.cpu().numpy(), ref) < 1e-9


def test_syev_matches_lapack(lib):
    rng = np.random.default_rng(3)
    for R in (1, 2, 5, 25, 32, 64):
        A = rng.standard_normal((R + 7, R))
        M = A.T @ A
        lam_ref, V_ref = np.linalg.eigh(M)
        Md = dev(M, torch.float64)
        V = torch.zeros((R, R), dtype=torch.float64, device="cuda")
        lam = torch.zeros(R, dtype=torch.float64, device="cuda")
        nbytes = lib.load().exafac_dense_workspace_bytes(R)
        ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        lib.call("exafac_syev", R, P(Md), P(V), P(lam), P(ws), ctypes.c_size_t(nbytes), None)
        lam_g, V_g = lam.cpu().numpy(), V.cpu().numpy()
        assert rel_err(lam_g, lam_ref) < 1e-13
        # eigenvectors up to sign
        dots = np.abs(np.sum(V_g * V_ref, axis=0))
        assert np.max(np.abs(dots - 1.0)) < 1e-10


STEP_CASES = ["c3_cp_arls_lev", "c3_sts_cp", "c4_cp_arls_lev", "c4_sts_cp", "dup_cp_arls_lev", "dup_sts_cp",
              "one_cp_arls_lev", "one_sts_cp", "logc_cp_arls_lev"]


def make_optimizer(dims, idx, vals, factors, sampler, J_max, preprocessing="none"):
    from exafac.cpp_ext.py_module import (AccumulatorStationary, CP_ARLS_LEV, Grid, LowRankTensor, STS_CP,
                                          SparseTensor, TensorGrid)

    N = len(dims)
    grid = Grid(np.ones(N, dtype=np.int32))
    tg = TensorGrid(np.asarray(dims, dtype=np.int32), grid)
    st = SparseTensor(tg, np.asarray(idx, dtype=np.uint32), np.asarray(vals, dtype=np.float64), preprocessing)
    lr = LowRankTensor(factors[0].shape[1], tg)
    lr.set_factors(factors)
    s = CP_ARLS_LEV(lr) if sampler == "cp_arls_lev" else STS_CP(lr)
    opt = AccumulatorStationary(st, lr, s, max_samples=J_max)
    opt.initialize_ground_truth_for_als()
    return opt, lr


def lex_sorted(a, cols):
    order = np.lexsort(tuple(a[:, k] for k in reversed(cols)))
    return order


@pytest.mark.parametrize("key", STEP_CASES)
def test_sweep_matches_reference(lib, golden, key):
    g = golden("steps.npz")
    meta = json.loads(str(g["meta"]))
    m = meta[key]
    base = key.split("_")[0]
    dims, J = m["dims"], m["J"]
    N = len(dims)
    factors = [g[f"{base}_U{k}"] for k in range(N)]
    opt, lr = make_optimizer(dims, g[f"{base}_idx"], g[f"{base}_vals"], factors, m["sampler"], J,
                             m.get("preprocessing", "none"))
    assert abs(opt.compute_exact_fit() - float(g[f"{key}_fit0"])) < 1e-10
    for t in range(m["steps"]):
        n = t % N
        uni = dev(g[f"{key}_s{t}_uniforms"], torch.float64)
        perms = dev(g[f"{key}_s{t}_perms"].astype(np.int32), torch.int32) if m["sampler"] == "cp_arls_lev" else None
        if f"{key}_s{t}_samples" in g:
            samples, weights = opt.draw(n, J, uni, perms)
            assert np.array_equal(samples.cpu().numpy().astype(np.uint32), g[f"{key}_s{t}_samples"]), f"step {t}"
            assert rel_err(weights.cpu().numpy(), g[f"{key}_s{t}_weights"]) < 1e-12
            sd_ref = g[f"{key}_s{t}_samples_dedup"]
            M = opt.sampled_mttkrp(n, sd_ref, g[f"{key}_s{t}_spmm_design"])
            assert rel_err(M.cpu().numpy(), g[f"{key}_s{t}_spmm_out"]) < 1e-12
            assert opt.step_info().hits == int(g[f"{key}_s{t}_spmm_found"])
        opt.execute_ALS_step(n, J, uni, perms)
        info = opt.step_info()
        assert info.hits == int(g[f"{key}_s{t}_hits"])
        if f"{key}_s{t}_samples_dedup" in g:
            sd, wd, _, _ = opt.last_dedup()
            sd, wd = sd.cpu().numpy().astype(np.uint32), wd.cpu().numpy()
            ref_sd, ref_wd = g[f"{key}_s{t}_samples_dedup"], g[f"{key}_s{t}_weights_dedup"]
            cols = [k for k in range(N) if k != n]
            o1, o2 = lex_sorted(sd, cols), lex_sorted(ref_sd, cols)
            assert np.array_equal(sd[o1][:, cols], ref_sd[o2][:, cols])
            assert rel_err(wd[o1], ref_wd[o2]) < 1e-12
        assert rel_err(lr.factors[n].data.cpu().numpy(), g[f"{key}_s{t}_factor"]) < 1e-8, f"step {t}"
        assert rel_err(lr.sigma.cpu().numpy(), g[f"{key}_s{t}_sigma"]) < 1e-8
    assert abs(opt.compute_exact_fit() - float(g[f"{key}_fit1"])) < 1e-8
    opt.deinitialize()


def test_workload1_sweep_matches_reference(lib, golden, oracle_mod):
    """2000^3 planted tensor, 2e6 nonzeros, R=25, J=65536, STS-CP: one sweep on
    the GPU against the reference (tensor and uniform stream regenerated)."""
    from rdist_tensor_gb300 import synthetic

    g = golden("workload1.npz")
    dims, idx, vals = synthetic.planted_uniform(seed=0)
    R, J = int(g["R"]), int(g["J"])
    factors = synthetic.gaussian_factors(dims, R, seed=1)
    opt, lr = make_optimizer(dims, idx, vals, factors, "sts_cp", J)
    assert abs(opt.compute_exact_fit() - float(g["fit0"])) < 1e-10
    streams = oracle_mod.sts_uniform_stream(int(g["seeds"][0]), 3, J, 3)
    for t in range(3):
        opt.execute_ALS_step(t, J, dev(streams[t], torch.float64))
        assert opt.step_info().hits == int(g[f"s{t}_hits"])
        assert rel_err(lr.factors[t].data.cpu().numpy(), g[f"s{t}_factor"]) < 1e-8
        assert rel_err(lr.sigma.cpu().numpy(), g[f"s{t}_sigma"]) < 1e-8
    assert abs(opt.compute_exact_fit() - float(g["fit1"])) < 1e-8
    opt.deinitialize()


@pytest.mark.parametrize("sampler", ["cp_arls_lev", "sts_cp"])
def test_exact_then_sampled_against_oracle(lib, oracle_mod, sampler):
    """One exact-ALS sweep (the -p exact preprocessing) then a sampled sweep
    with the GPU's own uniforms, replayed through the oracle."""
    from rdist_tensor_gb300 import synthetic

    dims, idx, vals = synthetic.zipf_tensor((3000, 2500, 300, 60), 60000, alpha=1.2, seed=4)
    vals = vals.astype(np.float64)
    R, J = 8, 4096
    factors = synthetic.gaussian_factors(dims, R, seed=5)
    opt, lr = make_optimizer(dims, idx, vals, factors, sampler, J)
    ora = oracle_mod.OracleALS(dims, idx, vals, factors, sampler)
    for n in range(4):
        opt.exact_step(n)
    oracle_mod.exact_als_sweep(ora, 1)
    for n in range(4):
        assert rel_err(lr.factors[n].data.cpu().numpy(), ora.factors[n]) < 1e-9
    assert abs(opt.compute_exact_fit() - ora.fit()) < 1e-9
    rng = np.random.default_rng(11)
    for n in range(4):
        shape = (4, J) if sampler == "cp_arls_lev" else (4, 2, J)
        uni = rng.random(shape)
        opt.execute_ALS_step(n, J, dev(uni, torch.float64))
        out = ora.step(n, J, uni)
        assert opt.step_info().hits == out["hits"]
        assert rel_err(lr.factors[n].data.cpu().numpy(), out["factor"]) < 1e-8
    assert abs(opt.compute_exact_fit() - ora.fit()) < 1e-8
    opt.deinitialize()


def make_optimizer_prec(dims, idx, vals, factors, sampler, J_max, precision):
    from exafac.cpp_ext.py_module import (AccumulatorStationary, CP_ARLS_LEV, Grid, LowRankTensor, STS_CP,
                                          SparseTensor, TensorGrid)

    N = len(dims)
    grid = Grid(np.ones(N, dtype=np.int32))
    tg = TensorGrid(np.asarray(dims, dtype=np.int32), grid)
    st = SparseTensor(tg, np.asarray(idx, dtype=np.uint32), np.asarray(vals, dtype=np.float64), "none")
    lr = LowRankTensor(factors[0].shape[1], tg)
    lr.set_factors(factors)
    s = CP_ARLS_LEV(lr) if sampler == "cp_arls_lev" else STS_CP(lr)
    opt = AccumulatorStationary(st, lr, s, max_samples=J_max, precision=precision)
    opt.initialize_ground_truth_for_als()
    return opt, lr


def sts_quadratic_forms(factors, samples, n):
    """h^T Phi h for each sample's rows: h the product of the sampled modes'
    rows, Phi the pseudo-inverse of the Hadamard product of their Grams (the
    FP64 oracle's, eigenvalues <= 1e-8 dropped as in sts_cp.hpp:110-153)."""
    N, R = len(factors), factors[0].shape[1]
    G = np.ones((R, R))
    h = np.ones((samples.shape[0], R))
    for k in range(N):
        if k == n:
            continue
        G = G * (factors[k].T @ factors[k])
        h = h * factors[k][samples[:, k].astype(np.int64)]
    lam, V = np.linalg.eigh(G)
    keep = lam > 1e-8
    Phi = (V[:, keep] / lam[keep]) @ V[:, keep].T
    return np.einsum("jr,rs,js->j", h, Phi, h)


@pytest.mark.parametrize("precision", ["fp64", "tf32", "bf16"])
@pytest.mark.parametrize("R", [3, 10, 40])
def test_mixed_sts_distribution(lib, oracle_mod, precision, R):
    """The STS-CP draws follow the exact leverage distribution of the
    Khatri-Rao product: P(rows) = h^T Phi h / rank(Phi) (the reference's
    sampler, sts_cp.hpp:203-300, draws exactly from it).  A 40 x 12 x 9
    tensor, all 108 (mode 1, mode 2) cells for mode 0 and 360 cells for mode
    1, J = 2^18 seeded draws; Pearson's chi-square against the exact cell
    probabilities, p > 1e-4.  R = 10 exceeds the 9 rows of mode 2, so its
    Gram is singular and the pivoted Cholesky of the mixed forms stops short
    of full rank; R = 40 takes the mixed forms' tensor-core level and leaf
    kernels, every row tree a single partial leaf."""
    from scipy.stats import chi2

    from rdist_tensor_gb300 import synthetic

    dims = (40, 12, 9)
    rng = np.random.default_rng(7)
    nnz = 2000
    idx = np.stack([rng.integers(0, d, nnz) for d in dims], axis=1).astype(np.uint32)
    idx = np.unique(idx, axis=0)
    vals = rng.standard_normal(idx.shape[0])
    factors = synthetic.gaussian_factors(dims, R, seed=11)
    J = 1 << 18
    opt, lr = make_optimizer_prec(dims, idx, vals, factors, "sts_cp", J, precision)
    for n in (0, 1):
        modes = [k for k in range(3) if k != n]
        uni = dev(rng.random((3, 2, J)), torch.float64)
        s, w = opt.draw(n, J, uni)
        s = s.cpu().numpy().astype(np.int64)
        cells = np.array([(a, b) for a in range(dims[modes[0]]) for b in range(dims[modes[1]])])
        full = np.zeros((cells.shape[0], 3), dtype=np.uint32)
        full[:, modes[0]], full[:, modes[1]] = cells[:, 0], cells[:, 1]
        q = sts_quadratic_forms(factors, full, n)
        p = q / q.sum()
        obs = np.bincount(s[:, modes[0]] * dims[modes[1]] + s[:, modes[1]], minlength=cells.shape[0])
        exp = p * J
        live = exp > 0
        assert obs[~live].sum() == 0
        stat = float(np.sum((obs[live] - exp[live]) ** 2 / exp[live]))
        pval = float(chi2.sf(stat, live.sum() - 1))
        print(f"{precision} R={R} mode {n}: chi2 {stat:.1f} dof {live.sum() - 1} p {pval:.3g}")
        assert pval > 1e-4
        w = w.cpu().numpy()
        qs = sts_quadratic_forms(factors, s.astype(np.uint32), n)
        assert rel_err(w, R / (qs * J)) < (1e-12 if precision == "fp64" else 1e-5)
    opt.deinitialize()


@pytest.mark.parametrize("precision", ["fp64", "tf32"])
@pytest.mark.parametrize("R", [16, 40])
def test_mixed_sts_distribution_many_leaves(lib, oracle_mod, precision, R):
    """The STS-CP draws through row trees of many leaves: a 40 x 4000 x 9
    tensor, draws for mode 0, whose mode-1 tree has 4000 / R leaves (250 at
    R = 16 on the CUDA-core leaf kernel, 100 at R = 40 on the tensor-core
    one), so that leaf boundaries fall anywhere inside the leaf stage's slot
    tiles.  J = 2^18 seeded draws; Pearson's chi-square of the mode-1 and
    mode-2 marginals against the exact leverage distribution, p > 1e-4."""
    from scipy.stats import chi2

    from rdist_tensor_gb300 import synthetic

    dims = (40, 4000, 9)
    rng = np.random.default_rng(17)
    nnz = 20000
    idx = np.stack([rng.integers(0, d, nnz) for d in dims], axis=1).astype(np.uint32)
    idx = np.unique(idx, axis=0)
    vals = rng.standard_normal(idx.shape[0])
    factors = synthetic.gaussian_factors(dims, R, seed=13)
    J = 1 << 18
    opt, lr = make_optimizer_prec(dims, idx, vals, factors, "sts_cp", J, precision)
    uni = dev(rng.random((3, 2, J)), torch.float64)
    s, w = opt.draw(0, J, uni)
    s = s.cpu().numpy().astype(np.int64)
    cells = np.array([(a, b) for a in range(dims[1]) for b in range(dims[2])])
    full = np.zeros((cells.shape[0], 3), dtype=np.uint32)
    full[:, 1], full[:, 2] = cells[:, 0], cells[:, 1]
    p = sts_quadratic_forms(factors, full, 0)
    p = (p / p.sum()).reshape(dims[1], dims[2])
    for k, marg in ((1, p.sum(axis=1)), (2, p.sum(axis=0))):
        obs = np.bincount(s[:, k], minlength=dims[k])
        exp = marg * J
        live = exp > 0
        assert obs[~live].sum() == 0
        stat = float(np.sum((obs[live] - exp[live]) ** 2 / exp[live]))
        pval = float(chi2.sf(stat, live.sum() - 1))
        print(f"{precision} R={R} mode-{k} marginal: chi2 {stat:.1f} dof {live.sum() - 1} p {pval:.3g}")
        assert pval > 1e-4
    qs = sts_quadratic_forms(factors, s.astype(np.uint32), 0)
    assert rel_err(w.cpu().numpy(), R / (qs * J)) < (1e-12 if precision == "fp64" else 1e-5)
    opt.deinitialize()


@pytest.mark.parametrize("R", [16, 48, 100])
@pytest.mark.parametrize("precision", ["tf32", "bf16"])
@pytest.mark.parametrize("sampler", ["cp_arls_lev", "sts_cp"])
def test_mixed_first_step_accuracy(lib, oracle_mod, precision, sampler, R):
    """First step of the mixed forms against the oracle.

    Draws: CP-ARLS-LEV samples from the FP64 leverage scores and CDF, so its
    indices equal the oracle's.  The mixed STS-CP draws take Cholesky factors
    of the sampling matrices in place of the reference's scaled eigenvectors
    and descend FP32 copies of the trees: the rows follow the same
    distribution (test_mixed_sts_distribution) but are other samples.  Each
    weight must still be R / (J h^T Phi h) for the rows drawn (h the product
    of the rows, Phi the oracle's FP64 pseudo-inverse): within 1e-5, the FP32
    quadratic form.

    Solve: the oracle is run on the GPU's own draws, so the factor error is
    that of the mixed arithmetic alone: FP32 design rows and MTTKRP, and Phi,
    the pseudo-inverse of a Gram formed on the tensor cores from TF32 (10-bit)
    or BF16 (7-bit mantissa) inputs: factor within 1e-3 (TF32) / 2e-2
    (BF16)."""
    from rdist_tensor_gb300 import synthetic

    dims, idx, vals = synthetic.planted_uniform(dims=(300, 250, 200), nnz=60000, rank=5, seed=3)
    J = 8192
    factors = synthetic.gaussian_factors(dims, R, seed=5)
    opt, lr = make_optimizer_prec(dims, idx, vals, factors, sampler, J, precision)
    ora = oracle_mod.OracleALS(dims, idx, vals, factors, sampler)
    rng = np.random.default_rng(12)
    shape = (3, J) if sampler == "cp_arls_lev" else (3, 2, J)
    uni = rng.random(shape)
    ud = dev(uni, torch.float64)
    s_gpu, w_gpu = opt.draw(0, J, ud)
    s_gpu = s_gpu.cpu().numpy().astype(np.uint32)
    w_gpu = w_gpu.cpu().numpy()
    if sampler == "cp_arls_lev":
        s_ora, w_ora = ora.draw(0, J, uni)
        assert np.array_equal(s_gpu, np.asarray(s_ora))
        assert rel_err(w_gpu, w_ora) < 1e-12
    else:
        q = sts_quadratic_forms(factors, s_gpu, 0)
        assert rel_err(w_gpu, R / (q * J)) < 1e-5
    opt.execute_ALS_step(0, J, ud)
    out = ora.step(0, J, uni, draws=(s_gpu, w_gpu))
    assert opt.step_info().hits == out["hits"]
    tol = 1e-3 if precision == "tf32" else 2e-2
    err_u = rel_err(lr.factors[0].data.cpu().numpy(), out["factor"])
    err_s = rel_err(lr.sigma.cpu().numpy(), out["sigma"])
    print(f"{precision} {sampler} R={R}: factor {err_u:.2e} sigma {err_s:.2e}")
    assert err_u < tol and err_s < tol
    opt.deinitialize()


@pytest.mark.parametrize("precision", ["tf32", "bf16"])
@pytest.mark.parametrize("sampler", ["cp_arls_lev", "sts_cp"])
def test_mixed_equal_fit(lib, precision, sampler):
    """Fit after 20 sweeps on a planted rank-5 tensor (signed factors) with 5/6
    of its entries observed (the fit converges, so sampling noise is small):
    mixed form within 1e-3 of the FP64 form driven by the same uniforms."""
    from rdist_tensor_gb300 import synthetic

    dims, idx, vals = synthetic.planted_uniform(dims=(60, 50, 40), nnz=100000, rank=5, seed=3, nonneg=False)
    R, J = 5, 4096
    factors = synthetic.gaussian_factors(dims, R, seed=6)
    fits = {}
    for prec in ("fp64", precision):
        opt, lr = make_optimizer_prec(dims, idx, vals, factors, sampler, J, prec)
        for _ in range(20):
            for n in range(3):
                opt.execute_ALS_step(n, J)
        fits[prec] = opt.compute_exact_fit()
        opt.deinitialize()
    assert fits["fp64"] > 0.5, fits
    assert abs(fits[precision] - fits["fp64"]) < 1e-3, fits


@pytest.mark.parametrize("precision", ["fp64", "tf32"])
@pytest.mark.parametrize("sampler", ["cp_arls_lev", "sts_cp"])
def test_sessions_repeat_bitwise(lib, precision, sampler):
    """Two sessions on the same input, stepped alike, stay bitwise equal:
    every reduction on the path has a fixed order."""
    from rdist_tensor_gb300 import synthetic

    dims, idx, vals = synthetic.planted_uniform(dims=(300, 250, 200), nnz=60000, rank=5, seed=3)
    factors = synthetic.gaussian_factors(dims, 16, seed=5)
    a, la = make_optimizer_prec(dims, idx, vals, factors, sampler, 4096, precision)
    b, lb = make_optimizer_prec(dims, idx, vals, factors, sampler, 4096, precision)
    for _ in range(3):
        for n in range(3):
            a.execute_ALS_step(n, 4096)
            b.execute_ALS_step(n, 4096)
    for k in range(3):
        assert torch.equal(la.factors[k].data, lb.factors[k].data), k
    assert torch.equal(la.sigma, lb.sigma)
    a.deinitialize()
    b.deinitialize()


@pytest.mark.parametrize("precision", ["fp64", "tf32"])
@pytest.mark.parametrize("sampler", ["cp_arls_lev", "sts_cp"])
def test_graph_sweeps_match_steps(lib, precision, sampler):
    """execute_sweeps (a captured sweep replayed as a CUDA graph) gives the
    same factors, bit for bit, as the same sweeps run step by step: with the
    session's Philox stream, and with explicit uniforms refilled in place."""
    from rdist_tensor_gb300 import synthetic

    dims, idx, vals = synthetic.planted_uniform(dims=(300, 250, 200), nnz=60000, rank=5, seed=3)
    factors = synthetic.gaussian_factors(dims, 16, seed=5)
    J = 4096
    a, la = make_optimizer_prec(dims, idx, vals, factors, sampler, J, precision)
    b, lb = make_optimizer_prec(dims, idx, vals, factors, sampler, J, precision)
    a.execute_sweeps(4, J)
    for _ in range(4):
        for n in range(3):
            b.execute_ALS_step(n, J)
    for k in range(3):
        assert torch.equal(la.factors[k].data, lb.factors[k].data), k
    per_step = 3 * (2 if sampler == "sts_cp" else 1) * J
    buf = torch.empty(3 * per_step, dtype=torch.float64, device="cuda")
    rng = np.random.default_rng(8)
    for _ in range(3):
        u = dev(rng.random(3 * per_step), torch.float64)
        buf.copy_(u)
        a.execute_sweeps(1, J, buf)
        for n in range(3):
            b.execute_ALS_step(n, J, u[n * per_step:(n + 1) * per_step])
    for k in range(3):
        assert torch.equal(la.factors[k].data, lb.factors[k].data), k
    assert torch.equal(la.sigma, lb.sigma)
    assert a.compute_exact_fit() == b.compute_exact_fit()
    a.deinitialize()
    b.deinitialize()
