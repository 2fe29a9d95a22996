"""Generalized CP: the sampled-model autograd Function and its hand-written
adjoint, against finite differences and a dense FP64 reference gradient;
the stratified entry sampler; a short Poisson fit."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from rdist_tensor_gb300 import gcp

    return gcp


def _all_entries(dims):
    grids = np.meshgrid(*[np.arange(d) for d in dims], indexing="ij")
    return np.stack([g.reshape(-1) for g in grids], axis=1).astype(np.int32)


def _dense_model(factors):
    N = len(factors)
    letters = "abcdefgh"[:N]
    expr = ",".join(f"{c}r" for c in letters) + "->" + letters
    return torch.einsum(expr, *factors)


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_model_matches_dense(dtype):
    gcp = _cuda()
    dt = getattr(torch, dtype)
    dims = (7, 6, 5)
    g = torch.Generator(device="cuda").manual_seed(1)
    U = [torch.randn((d, 4), generator=g, device="cuda", dtype=dt) for d in dims]
    idx = torch.as_tensor(_all_entries(dims), device="cuda")
    m = gcp.sampled_model(idx, U)
    ref = _dense_model([u.double() for u in U]).reshape(-1)
    tol = 1e-5 if dtype == "float32" else 1e-13
    assert torch.max(torch.abs(m.double() - ref)).item() <= tol * torch.max(torch.abs(ref)).item()


def test_adjoint_matches_finite_differences():
    """FP64 kernels: autograd gradient of a weighted Poisson objective on 60
    sampled entries (with repeats) against central differences."""
    gcp = _cuda()
    dims, R = (6, 5, 4), 3
    rng = np.random.default_rng(3)
    idx = torch.as_tensor(np.stack([rng.integers(0, d, 60) for d in dims], axis=1).astype(np.int32), device="cuda")
    x = torch.as_tensor(rng.poisson(2.0, 60).astype(np.float64), device="cuda")
    w = torch.as_tensor(rng.uniform(0.5, 2.0, 60), device="cuda")
    U = [torch.as_tensor(rng.uniform(0.2, 1.0, (d, R)), device="cuda").requires_grad_() for d in dims]

    def objective(fs):
        m = gcp.sampled_model(idx, fs)
        return (w * gcp.loss_values("poisson", x, m)).sum()

    objective(U).backward()
    h = 1e-6
    for k, Uk in enumerate(U):
        fd = torch.zeros_like(Uk)
        for i in range(dims[k]):
            for r in range(R):
                with torch.no_grad():
                    base = [u.detach().clone() for u in U]
                    plus = [u.clone() for u in base]
                    minus = [u.clone() for u in base]
                    plus[k][i, r] += h
                    minus[k][i, r] -= h
                    fd[i, r] = (objective(plus) - objective(minus)) / (2 * h)
        err = torch.max(torch.abs(Uk.grad - fd)).item() / torch.max(torch.abs(fd)).item()
        assert err < 1e-7, (k, err)


@pytest.mark.parametrize("dtype,tol", [("float32", 2e-4), ("float64", 1e-11)])
def test_adjoint_matches_dense_fp64_gradient(dtype, tol):
    """All 200^3 entries of a Poisson count tensor as the sample (weight 1):
    the kernels' gradient of the Poisson objective against the dense FP64
    gradient einsum(Y, U_j, U_k), Y = df/dm over the dense tensor."""
    gcp = _cuda()
    from rdist_tensor_gb300 import synthetic

    dims, R = (200, 200, 200), 32
    d, nz_idx, nz_vals, _ = synthetic.poisson_counts(dims, 400_000, rank=16, seed=5)
    X = torch.zeros(dims, dtype=torch.float64, device="cuda")
    X[tuple(torch.as_tensor(nz_idx.astype(np.int64), device="cuda").T)] = torch.as_tensor(
        nz_vals.astype(np.float64), device="cuda")
    dt = getattr(torch, dtype)
    g = torch.Generator(device="cuda").manual_seed(7)
    U64 = [torch.rand((n, R), generator=g, device="cuda", dtype=torch.float64) * 0.3 + 0.05 for n in dims]
    U = [u.to(dt).requires_grad_() for u in U64]
    idx = torch.as_tensor(_all_entries(dims), device="cuda")
    x = X.reshape(-1).to(dt)
    m = gcp.sampled_model(idx, U)
    gcp.loss_values("poisson", x, m).sum().backward()
    Ud = [u.detach().double() for u in U]
    M = _dense_model(Ud)
    Y = 1.0 - X / (M + gcp.EPS)
    ref = [torch.einsum("ijk,jr,kr->ir", Y, Ud[1], Ud[2]), torch.einsum("ijk,ir,kr->jr", Y, Ud[0], Ud[2]),
           torch.einsum("ijk,ir,jr->kr", Y, Ud[0], Ud[1])]
    for k in range(3):
        err = torch.max(torch.abs(U[k].grad.double() - ref[k])).item() / torch.max(torch.abs(ref[k])).item()
        print(f"{dtype} mode {k}: max rel err {err:.2e}")
        assert err < tol, (k, err)


def test_sampler_strata():
    gcp = _cuda()
    from rdist_tensor_gb300 import synthetic

    dims = (300, 200, 100)
    _, nz_idx, nz_vals = synthetic.random_sparse(dims, 5000, seed=2)
    idx = torch.as_tensor(nz_idx.astype(np.int32), device="cuda")
    vals = torch.as_tensor(nz_vals, device="cuda")
    J_nz, J_z = 4000, 6000
    s_idx, s_x, s_w = gcp.sample_entries(idx, vals, dims, J_nz, J_z, seed=11, counter=0)
    s_idx, s_x, s_w = s_idx.cpu().numpy(), s_x.cpu().numpy(), s_w.cpu().numpy()
    lookup = {tuple(c): v for c, v in zip(nz_idx.tolist(), nz_vals.tolist())}
    for c, v in zip(s_idx[:J_nz].tolist(), s_x[:J_nz].tolist()):
        assert lookup[tuple(c)] == v
    assert np.all(s_x[J_nz:] == 0.0)
    for k, dk in enumerate(dims):
        assert s_idx[:, k].min() >= 0 and s_idx[:, k].max() < dk
    assert np.allclose(s_w[:J_nz], 5000 / J_nz)
    assert np.allclose(s_w[J_nz:], (np.prod(dims) - 5000) / J_z)
    # a different counter gives a different sample
    s2, _, _ = gcp.sample_entries(idx, vals, dims, J_nz, J_z, seed=11, counter=1)
    assert not np.array_equal(s2.cpu().numpy(), s_idx)


def test_out_of_range_entry_is_skipped_and_flagged():
    gcp = _cuda()
    dims, R = (5, 4, 3), 2
    U = [torch.rand((d, R), device="cuda", dtype=torch.float64).requires_grad_() for d in dims]
    idx = torch.tensor([[0, 0, 0], [5, 1, 1], [4, 3, 2]], dtype=torch.int32, device="cuda")
    m = gcp.SampledCPModel.apply(idx, *U)
    assert m[1].item() == 0.0
    m.sum().backward()
    # the skipped entry adds nothing: compare with the two valid entries alone
    V = [u.detach().clone().requires_grad_() for u in U]
    gcp.sampled_model(idx[[0, 2]].contiguous(), V).sum().backward()
    for a, b in zip(U, V):
        assert torch.equal(a.grad, b.grad)


def test_poisson_fit_decreases_objective():
    gcp = _cuda()
    from rdist_tensor_gb300 import synthetic

    dims = (60, 50, 40)
    _, nz_idx, nz_vals, _ = synthetic.poisson_counts(dims, 20_000, rank=4, seed=9)
    model = gcp.GCP(nz_idx, nz_vals, dims, rank=4, loss="poisson", seed=0)
    idx_all = torch.as_tensor(_all_entries(dims), device="cuda")
    X = torch.zeros(dims, dtype=torch.float32, device="cuda")
    X[tuple(torch.as_tensor(nz_idx.astype(np.int64), device="cuda").T)] = torch.as_tensor(nz_vals, device="cuda")
    x_all = X.reshape(-1)
    ones = torch.ones_like(x_all)

    def full():
        with torch.no_grad():
            return model.objective(idx_all, x_all, ones).item()

    f0 = full()
    model.fit(200, J_nz=4096, J_z=4096, lr=2e-2)
    f1 = full()
    assert np.isfinite(f1) and f1 < 0.9 * f0, (f0, f1)


def test_full_objective_matches_dense():
    """The exact Poisson objective over every entry (model mass from column
    sums, nonzero terms from the kernels) against the dense FP64 sum."""
    gcp = _cuda()
    from rdist_tensor_gb300 import synthetic

    dims = (30, 20, 10)
    _, nz_idx, nz_vals, _ = synthetic.poisson_counts(dims, 900, rank=3, seed=4)
    model = gcp.GCP(nz_idx, nz_vals, dims, rank=5, loss="poisson", dtype=torch.float64, seed=2)
    X = torch.zeros(dims, dtype=torch.float64, device="cuda")
    X[tuple(torch.as_tensor(nz_idx.astype(np.int64), device="cuda").T)] = torch.as_tensor(
        nz_vals.astype(np.float64), device="cuda")
    M = _dense_model([u.detach() for u in model.factors])
    ref = float((M - X * torch.log(M + gcp.EPS)).sum())
    got = model.full_objective(chunk=256)  # several chunks
    assert abs(got - ref) <= 1e-10 * abs(ref), (got, ref)
    assert abs(model.model_mass() - float(M.sum())) <= 1e-12 * float(M.sum())


def test_poisson_counts_device():
    """The device generator of the count tensors: distinct in-range
    coordinates, positive integer counts, and a mean count near the planted
    model's mean rate at those coordinates."""
    _cuda()
    from rdist_tensor_gb300 import synthetic

    dims = (20_000, 20_000, 500)
    d, idx, vals, A = synthetic.poisson_counts_device(dims, 200_000, rank=16, seed=3)
    assert idx.shape == (200_000, 3) and idx.dtype == torch.int32
    for k in range(3):
        assert int(idx[:, k].min()) >= 0 and int(idx[:, k].max()) < dims[k]
    key = (idx[:, 0].long() * dims[1] + idx[:, 1].long()) * dims[2] + idx[:, 2].long()
    assert torch.unique(key).numel() == idx.shape[0]
    assert bool((vals >= 1).all()) and bool((vals == torch.round(vals)).all())
    rows = idx.long()
    lam = (A[0][rows[:, 0]] * A[1][rows[:, 1]] * A[2][rows[:, 2]]).sum(dim=1).double()
    # E[max(Poisson(lam), 1)] = lam + exp(-lam)
    expect = float((lam + torch.exp(-lam)).mean())
    assert abs(float(vals.double().mean()) - expect) < 0.02 * expect
    # Gamma(0.5, 1) factors: mean 0.5, variance 0.5
    a = torch.cat([x.reshape(-1) for x in A]).double()
    assert abs(float(a.mean()) - 0.5) < 0.01 and abs(float(a.var()) - 0.5) < 0.03


def test_gcp_reduced_count_tensor_decreases_objective():
    """The GCP workload's step (R = 32, J = 2^17 entries, Adam lr = 1e-2) on a
    reduced count tensor, 1e5 x 1e5 x 1e3 with 5e6 nonzeros: the exact
    objective over all entries falls (by two orders of magnitude in a torch
    CPU restatement of the same steps), and every sampled objective is
    finite."""
    gcp = _cuda()
    from rdist_tensor_gb300 import synthetic

    dims, idx, vals, _ = synthetic.poisson_counts_device((100_000, 100_000, 1_000), 5_000_000, rank=16, seed=1)
    model = gcp.GCP(idx, vals, dims, rank=32, loss="poisson", seed=1)
    f0 = model.full_objective()
    hist = model.fit(60, J_nz=1 << 16, J_z=1 << 16, lr=1e-2)
    f1 = model.full_objective()
    assert bool(torch.isfinite(hist).all())
    assert np.isfinite(f1) and f1 < 0.1 * f0, (f0, f1)
    assert min(float(u.detach().min()) for u in model.factors) >= 0.0


@pytest.mark.parametrize("dtype,tol", [("float32", 1e-6), ("float64", 1e-14)])
def test_fused_adam_matches_torch_adam(dtype, tol):
    """The fused Adam + projection kernel against torch.optim.Adam followed by
    clamp_min over six steps: sizes that are and are not multiples of four,
    one parameter without a gradient, and one with a misaligned (offset)
    storage that takes the scalar path."""
    gcp = _cuda()
    dt = getattr(torch, dtype)
    g = torch.Generator(device="cuda").manual_seed(4)
    base = torch.rand(1003 * 7 + 1, generator=g, device="cuda", dtype=dt)
    shapes = [(1000, 32), (37, 5), (1003, 7)]
    ours = [torch.rand(s, generator=g, device="cuda", dtype=dt) for s in shapes[:2]]
    ours.append(base[1:].view(shapes[2]))  # storage offset by one element
    ref = [p.detach().clone() for p in ours]
    # the aligned pair takes the float4 body (FP32); the offset tensor, in a
    # launch of its own, the scalar path
    opts = [gcp.FusedAdam(ours[:2], lr=3e-2, betas=(0.85, 0.995), eps=1e-7, lower=0.0),
            gcp.FusedAdam(ours[2:], lr=3e-2, betas=(0.85, 0.995), eps=1e-7, lower=0.0)]
    moments = [(o, k) for o in opts for k in range(len(o.params))]
    topt = torch.optim.Adam(ref, lr=3e-2, betas=(0.85, 0.995), eps=1e-7)
    for step in range(6):
        grads = [torch.randn(s, generator=g, device="cuda", dtype=dt) for s in shapes]
        for k, (p, q) in enumerate(zip(ours, ref)):
            if k == 1 and step % 2 == 1:  # no gradient on odd steps
                p.grad, q.grad = None, torch.zeros_like(q)
            else:
                p.grad, q.grad = grads[k], grads[k].clone()
        for o in opts:
            o.step()
        topt.step()
        with torch.no_grad():
            for q in ref:
                q.clamp_(min=0.0)
    for k, (p, q) in enumerate(zip(ours, ref)):
        err = torch.max(torch.abs(p - q)).item()
        assert err <= tol, (k, err)
        st = topt.state[q]
        o, j = moments[k]
        assert torch.allclose(o.exp_avg[j], st["exp_avg"], rtol=tol * 10, atol=tol)
        assert torch.allclose(o.exp_avg_sq[j], st["exp_avg_sq"], rtol=tol * 10, atol=tol)
    assert min(float(p.min()) for p in ours) >= 0.0
