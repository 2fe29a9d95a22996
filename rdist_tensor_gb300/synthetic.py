"""Seeded synthetic sparse tensors with the shapes and value distributions of
the sampled-ALS workloads (the reference ships no tensors; its FROSTT inputs
are loaded from HDF5 files that are not part of the repository).

All generators are deterministic functions of their seed.

* ``planted_uniform``: coordinates uniform without replacement over the full
  index space; values from a planted nonnegative CP model (|N(0,1)| factor
  entries) plus Gaussian noise.  Workload "3-mode 2000^3, 2e6 nonzeros, planted
  rank 10, noise variance 0.01".
* ``zipf_tensor``: per-mode Zipf(alpha) coordinates truncated to the mode
  range, deduplicated; values log-normal(0, 1) or N(0, 1) in float32.
  Workloads "4-mode 5e6 x 5e6 x 2e4 x 1e3, 1e8 nonzeros, alpha 1.2" and
  "5-mode 1e6 x 1e6 x 1e5 x 1e3 x 100, 2e8 nonzeros, alpha 1.1".
* ``poisson_counts``: counts ~ Poisson(planted nonnegative CP with Gamma(0.5, 1)
  factors) on a Zipf support (generalized-CP workload).
"""
from __future__ import annotations

import numpy as np


def planted_uniform(dims=(2000, 2000, 2000), nnz=2_000_000, rank=10, noise_var=0.01, seed=0, nonneg=True):
    rng = np.random.default_rng(seed)
    dims = tuple(int(d) for d in dims)
    total = int(np.prod(np.array(dims, dtype=np.float64)))
    # Uniform without replacement: oversample, deduplicate, keep the first nnz
    # in draw order.
    lin = np.empty(0, dtype=np.int64)
    while len(lin) < nnz:
        extra = rng.integers(0, total, size=int((nnz - len(lin)) * 1.05) + 16, dtype=np.int64)
        cand = np.concatenate([lin, extra])
        _, first = np.unique(cand, return_index=True)
        lin = cand[np.sort(first)]
    lin = lin[:nnz]
    idx = np.stack(np.unravel_index(lin, dims), axis=1).astype(np.uint32)
    A = [rng.standard_normal((d, rank)) for d in dims]
    if nonneg:
        A = [np.abs(a) for a in A]
    model = np.ones((nnz, rank))
    for k, Ak in enumerate(A):
        model *= Ak[idx[:, k]]
    vals = model.sum(axis=1) + rng.normal(0.0, np.sqrt(noise_var), size=nnz)
    return np.array(dims, dtype=np.int64), np.ascontiguousarray(idx), np.ascontiguousarray(vals)


def random_sparse(dims, nnz, seed=0):
    """Uniform coordinates without replacement and U(0,1) values (small cases)."""
    rng = np.random.default_rng(seed)
    dims = tuple(int(d) for d in dims)
    total = int(np.prod(dims))
    lin = rng.choice(total, size=min(nnz, total), replace=False)
    idx = np.stack(np.unravel_index(lin, dims), axis=1).astype(np.uint32)
    vals = rng.random(len(lin))
    return np.array(dims, dtype=np.int64), np.ascontiguousarray(idx), np.ascontiguousarray(vals)


def zipf_coords(rng, dim: int, alpha: float, n: int) -> np.ndarray:
    """Zipf(alpha) over {0..dim-1} (rank k+1 has mass proportional to (k+1)^-alpha),
    by inverse-CDF search on the exact truncated distribution."""
    k = np.arange(1, dim + 1, dtype=np.float64)
    cdf = np.cumsum(k ** (-alpha))
    cdf /= cdf[-1]
    u = rng.random(n)
    return np.minimum(np.searchsorted(cdf, u, side="right"), dim - 1).astype(np.uint32)


def zipf_tensor(dims, nnz, alpha=1.2, values="lognormal", seed=0, max_rounds=8):
    """Per-mode Zipf coordinates, deduplicated; oversamples until ``nnz`` unique
    coordinates are found or ``max_rounds`` rounds ran (the achieved count is
    then smaller, and is what the returned arrays hold)."""
    rng = np.random.default_rng(seed)
    dims = [int(d) for d in dims]
    N = len(dims)
    bits = [max(1, int(np.ceil(np.log2(d)))) for d in dims]
    have = np.zeros((0, N), dtype=np.uint32)
    want = nnz
    for _ in range(max_rounds):
        m = int(want * 1.3) + 1024
        cand = np.stack([zipf_coords(rng, d, alpha, m) for d in dims], axis=1)
        allc = np.concatenate([have, cand])
        keys = _pack(allc, bits)
        _, first = np.unique(keys, axis=0, return_index=True)
        have = allc[np.sort(first)]
        if len(have) >= nnz:
            break
        want = nnz - len(have)
    have = have[:nnz]
    if values == "lognormal":
        vals = rng.lognormal(0.0, 1.0, size=len(have)).astype(np.float32)
    else:
        vals = rng.standard_normal(len(have)).astype(np.float32)
    return np.array(dims, dtype=np.int64), np.ascontiguousarray(have), vals


def zipf_tensor_device(dims, nnz, alpha=1.2, values="lognormal", seed=0, max_rounds=12, device="cuda"):
    """Same construction as ``zipf_tensor`` with torch on a CUDA device (the
    1e8-nonzero workloads take minutes in numpy): per-mode exact truncated
    Zipf(alpha) by inverse-CDF search, deduplicated on a packed 128-bit key,
    first occurrences kept, oversampled in rounds until ``nnz`` unique
    coordinates exist (or ``max_rounds`` ran; the returned count is then what
    was reached).  Deterministic for a seed on a given torch build.  Returns
    (dims int64 numpy, idx int32 [nnz, N] device tensor, values float32 device
    tensor)."""
    import torch

    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed))
    dims = [int(d) for d in dims]
    N = len(dims)
    bits = [max(1, int(np.ceil(np.log2(d)))) for d in dims]
    if sum(bits) > 126:
        raise ValueError("coordinates need more than 126 key bits")
    cdfs = []
    for d in dims:
        # Summed on the host, in order: a device scan need not add in the same
        # order on every run, and a last-bit change of one CDF entry moves the
        # rare draw that lands on it, which changes the tensor.
        k = np.arange(1, d + 1, dtype=np.float64)
        c = np.cumsum(k ** (-alpha))
        cdfs.append(torch.from_numpy(c / c[-1]).to(device))

    def pack(idx):
        hi = torch.zeros(idx.shape[0], dtype=torch.int64, device=device)
        lo = torch.zeros(idx.shape[0], dtype=torch.int64, device=device)
        total = 0
        for k in range(N - 1, -1, -1):
            c = idx[:, k].to(torch.int64)
            if total < 63 and total + bits[k] <= 63:
                lo |= c << total
            elif total >= 63:
                hi |= c << (total - 63)
            else:
                lo |= (c & ((1 << (63 - total)) - 1)) << total
                hi |= c >> (63 - total)
            total += bits[k]
        return hi, lo

    have = torch.zeros((0, N), dtype=torch.int32, device=device)
    want = int(nnz)
    for _ in range(max_rounds):
        m = int(want * 1.3) + 1024
        cand = torch.stack([torch.clamp(torch.searchsorted(cdfs[k], torch.rand(m, dtype=torch.float64, device=device,
                                                                                 generator=gen), right=True),
                                        max=dims[k] - 1).to(torch.int32) for k in range(N)], dim=1)
        allc = torch.cat([have, cand])
        hi, lo = pack(allc)
        pos = torch.arange(allc.shape[0], device=device)
        # stable two-key sort: by lo, then by hi
        o = torch.sort(lo, stable=True).indices
        o = o[torch.sort(hi[o], stable=True).indices]
        hs, ls, ps = hi[o], lo[o], pos[o]
        first = torch.ones_like(hs, dtype=torch.bool)
        first[1:] = (hs[1:] != hs[:-1]) | (ls[1:] != ls[:-1])
        keep = torch.sort(ps[first]).values  # first occurrences in draw order
        have = allc[keep]
        del allc, hi, lo, pos, o, hs, ls, ps, first, keep, cand
        if have.shape[0] >= nnz:
            break
        want = int(nnz) - have.shape[0]
    have = have[:nnz].contiguous()
    if values == "lognormal":
        vals = torch.exp(torch.randn(have.shape[0], dtype=torch.float32, device=device, generator=gen))
    else:
        vals = torch.randn(have.shape[0], dtype=torch.float32, device=device, generator=gen)
    return np.array(dims, dtype=np.int64), have, vals


def _pack(idx, bits):
    """Packs coordinates into two uint64 words per row (most significant mode first)."""
    hi = np.zeros(len(idx), dtype=np.uint64)
    lo = np.zeros(len(idx), dtype=np.uint64)
    for k, b in enumerate(bits):
        b = np.uint64(b)
        hi = (hi << b) | (lo >> (np.uint64(64) - b))
        lo = (lo << b) | idx[:, k].astype(np.uint64)
    return np.stack([hi, lo], axis=1)


def poisson_counts(dims, nnz, rank=16, seed=0):
    """Count tensor: Zipf(1.1) support, entries ~ Poisson(planted rank-`rank`
    CP with Gamma(0.5, 1) factors) (zeros redrawn as 1 so every stored entry is
    a nonzero)."""
    rng = np.random.default_rng(seed)
    d, idx, _ = zipf_tensor(dims, nnz, alpha=1.1, seed=seed + 1)
    A = [rng.gamma(0.5, 1.0, size=(int(n), rank)) for n in d]
    rate = np.ones((len(idx), rank))
    for k, Ak in enumerate(A):
        rate *= Ak[idx[:, k]]
    lam = rate.sum(axis=1)
    vals = rng.poisson(lam).astype(np.float32)
    vals[vals == 0] = 1.0
    return d, idx, vals, A


def poisson_counts_device(dims, nnz, rank=16, seed=0, device="cuda"):
    """``poisson_counts`` built with torch on a CUDA device, for the
    5e7-nonzero count tensors: the Zipf(1.1) support of
    ``zipf_tensor_device``, Gamma(0.5, 1) planted factors drawn as Z^2 / 2
    with Z ~ N(0, 1) (the chi-square with one degree of freedom, halved),
    entries ~ Poisson(sum_r prod_k A_k[i_k, r]) with zeros redrawn as 1.
    Returns (dims int64 numpy, idx int32 [nnz, N] device tensor, float32
    values device tensor, planted factors as float32 device tensors)."""
    import torch

    d, idx, _ = zipf_tensor_device(dims, nnz, alpha=1.1, values="normal", seed=seed + 1, device=device)
    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed))
    A = []
    for n in d:
        z = torch.randn((int(n), rank), dtype=torch.float32, device=device, generator=gen)
        A.append(0.5 * z * z)
    lam = torch.empty(idx.shape[0], dtype=torch.float32, device=device)
    step = 1 << 24
    for a in range(0, idx.shape[0], step):
        rows = idx[a:a + step].to(torch.int64)
        rate = A[0][rows[:, 0]]
        for k in range(1, len(A)):
            rate = rate * A[k][rows[:, k]]
        lam[a:a + step] = rate.sum(dim=1)
    vals = torch.poisson(lam, generator=gen)
    vals[vals == 0] = 1.0
    return d, idx, vals, A


def gaussian_factors(dims, R, seed=0):
    """initialize_factors_gaussian_random (low_rank_tensor.hpp:35-41,
    distmat.hpp:153-168, 85-138): N(0,1) entries, columns normalised."""
    rng = np.random.default_rng(seed)
    out = []
    for d in dims:
        U = rng.standard_normal((int(d), R))
        U /= np.sqrt((U * U).sum(axis=0))[None, :]
        out.append(np.ascontiguousarray(U))
    return out


def deterministic_factors(dims, R):
    """initialize_factors_deterministic (distmat.hpp:140-151) at one rank:
    U[i, j] = cos(i * R + j), columns normalised."""
    out = []
    for d in dims:
        i = np.arange(int(d), dtype=np.float64)[:, None]
        j = np.arange(R, dtype=np.float64)[None, :]
        U = np.cos(i * R + j)
        U /= np.sqrt((U * U).sum(axis=0))[None, :]
        out.append(np.ascontiguousarray(U))
    return out
