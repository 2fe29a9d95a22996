"""ORACLE — CPU restatement of the reference's sampled-ALS hot path.

TEST INFRASTRUCTURE ONLY.  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this module: as the checker, or as
the timed CPU port of the reference.  The product never imports it.

Pinned against the reference itself: ``tests/golden/make_golden.py`` runs the
reference's own C++ (compiled here by ``oracle/build_ref.sh``) with injected
random streams and stores inputs and outputs as fixtures; ``tests/test_oracle.py``
checks this restatement against them.

Layout: loops live in ``oracle_kernels.c`` (``oracle/_build/liboracle.so``);
this file holds the R x R algebra (numpy/LAPACK) and the step orchestration of
``AccumulatorStationary::execute_ALS_step`` at one rank.  Uniforms and per-mode
permutations are explicit inputs (the reference draws them from std::mt19937
streams; the harness exports them).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None


def build() -> str:
    """Compiles oracle_kernels.c (gcc, OpenMP) if needed; returns the .so path."""
    src = os.path.join(_HERE, "oracle_kernels.c")
    if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", _HERE])
    return _LIB_PATH


class _Tree(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in (
        "n", "F", "R", "leaf_count", "node_count", "lfill_level", "lfill_count",
        "nodes_upto_lfill", "nodes_before_lfill", "complete_level_offset")]


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        P = ctypes.c_void_p
        I64 = ctypes.c_int64
        _lib.or_tree_shape.argtypes = [I64, I64, I64, ctypes.POINTER(_Tree)]
        _lib.or_tree_build.argtypes = [ctypes.POINTER(_Tree), P, P]
        _lib.or_tree_hadamard.argtypes = [ctypes.POINTER(_Tree), P, P]
        _lib.or_tree_sample.argtypes = [ctypes.POINTER(_Tree), P, P, I64, P, P, P, P]
        _lib.or_pack_keys.argtypes = [ctypes.c_int, ctypes.c_int, P, I64, P, P, P]
        _lib.or_pack_keys.restype = ctypes.c_int
        _lib.or_radix_sort128.argtypes = [I64, ctypes.c_int, P, P, P]
        _lib.or_apply_perm_u32.argtypes = [I64, ctypes.c_int, P, P, P]
        _lib.or_apply_perm_f64.argtypes = [I64, P, P, P]
        _lib.or_apply_perm_u64.argtypes = [I64, P, P, P]
        _lib.or_sampled_mttkrp.argtypes = [I64, P, P, P, P, I64, P, P, ctypes.c_int, P, I64, P]
        _lib.or_sampled_mttkrp.restype = I64
        _lib.or_fit_residual.argtypes = [ctypes.c_int, ctypes.c_int, I64, P, P, P, P]
        _lib.or_fit_residual.restype = ctypes.c_double
        _lib.or_exact_mttkrp.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, I64, P, P, P, I64, P]
        _lib.or_dagat.argtypes = [I64, ctypes.c_int, P, P, P]
        _lib.or_num_threads.restype = ctypes.c_int
    return _lib


def _p(a: np.ndarray):
    assert a.flags.c_contiguous
    return ctypes.c_void_p(a.ctypes.data)


# --------------------------------------------------------------------------
# Dense helpers (common.h)
# --------------------------------------------------------------------------
def gram(A: np.ndarray) -> np.ndarray:
    """compute_gram (common.h:363-403): full symmetric A^T A."""
    G = A.T @ A
    return np.triu(G) + np.triu(G, 1).T


def pinv_square(M: np.ndarray, tol: float = 1e-11) -> np.ndarray:
    """compute_pinv_square (common.h:405-443): eigendecomposition of the upper
    triangle, columns with eigenvalue <= tol dropped, out = (V L^-1/2)(V L^-1/2)^T."""
    lam, V = np.linalg.eigh(M, UPLO="U")
    W = np.zeros_like(V)
    keep = lam > tol
    W[:, keep] = V[:, keep] / np.sqrt(lam[keep])
    out = W @ W.T
    return np.triu(out) + np.triu(out, 1).T


def dagat(A: np.ndarray, G: np.ndarray) -> np.ndarray:
    """compute_DAGAT (common.h:727-746): res_i = a_i^T G a_i."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    G = np.ascontiguousarray(G, dtype=np.float64)
    res = np.empty(A.shape[0])
    lib().or_dagat(A.shape[0], A.shape[1], _p(A), _p(G), _p(res))
    return res


def seq_sum(x: np.ndarray) -> float:
    """std::accumulate order (sequential left-to-right)."""
    return float(np.cumsum(x)[-1]) if len(x) else 0.0


def discrete_cdf(w: np.ndarray) -> np.ndarray:
    """libstdc++ discrete_distribution::param_type::_M_initialize
    (bits/random.tcc:2657-2678): normalise by the sequential sum, sequential
    partial sums, last entry forced to 1.0.  Fewer than two weights: empty."""
    if len(w) < 2:
        return np.zeros(0)
    s = seq_sum(w)
    cp = np.cumsum(w / s)
    cp[-1] = 1.0
    return cp


# --------------------------------------------------------------------------
# PartitionTree (partition_tree.hpp)
# --------------------------------------------------------------------------
class PartitionTree:
    """Segment tree of R x R Grams over F-row leaves (partition_tree.hpp:48-380)."""

    def __init__(self, n: int, F: int, R: int):
        self.shape = _Tree()
        lib().or_tree_shape(n, F, R, ctypes.byref(self.shape))
        self.n, self.F, self.R = n, F, R
        self.G = np.zeros((self.shape.node_count, R, R))

    def build(self, U: np.ndarray):
        U = np.ascontiguousarray(U[: self.n], dtype=np.float64)
        lib().or_tree_build(ctypes.byref(self.shape), _p(U), _p(self.G))

    def hadamard(self, M: np.ndarray):
        M = np.ascontiguousarray(M, dtype=np.float64)
        lib().or_tree_hadamard(ctypes.byref(self.shape), _p(self.G), _p(M))

    def sample(self, U: np.ndarray, x: np.ndarray, hmul: np.ndarray, draws: np.ndarray) -> np.ndarray:
        """PTSample: descent by x, draws explicit; hmul *= U[row] in place."""
        U = np.ascontiguousarray(U[: self.n], dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        draws = np.ascontiguousarray(draws, dtype=np.float64)
        assert hmul.flags.c_contiguous and hmul.dtype == np.float64
        out = np.empty(x.shape[0], dtype=np.uint32)
        lib().or_tree_sample(ctypes.byref(self.shape), _p(self.G), _p(U), x.shape[0], _p(x), _p(hmul),
                             _p(draws), _p(out))
        return out


# --------------------------------------------------------------------------
# Sorted lookup (sort_lookup.hpp)
# --------------------------------------------------------------------------
def pack_keys(idx: np.ndarray, dims, skip: int):
    idx = np.ascontiguousarray(idx, dtype=np.uint32)
    d = np.ascontiguousarray(np.asarray(dims, dtype=np.int64))
    hi = np.empty(idx.shape[0], dtype=np.uint64)
    lo = np.empty(idx.shape[0], dtype=np.uint64)
    bits = lib().or_pack_keys(idx.shape[1], skip, _p(d), idx.shape[0], _p(idx), _p(hi), _p(lo))
    if bits < 0:
        raise ValueError("coordinates need more than 128 key bits")
    return hi, lo, bits


class SortIdxLookup:
    """Mode-n lookup (sort_lookup.hpp:37-102, reorder=true): nonzeros sorted by
    their coordinates with mode n left out (stable for equal keys)."""

    def __init__(self, idx: np.ndarray, val: np.ndarray, dims, mode: int):
        self.mode = mode
        hi, lo, bits = pack_keys(idx, dims, mode)
        perm = np.empty(idx.shape[0], dtype=np.int64)
        lib().or_radix_sort128(idx.shape[0], bits, _p(hi), _p(lo), _p(perm))
        self.perm = perm
        self.khi = hi[perm]
        self.klo = lo[perm]
        self.rows = np.ascontiguousarray(idx[perm, mode], dtype=np.uint32)
        self.vals = np.ascontiguousarray(val[perm], dtype=np.float64)
        self.dims = list(dims)

    def sampled_mttkrp(self, samples_dedup: np.ndarray, design: np.ndarray, out_rows: int):
        """csr_based_spmm (sort_lookup.hpp:238-375).  Returns (M, hits)."""
        shi, slo, _ = pack_keys(samples_dedup, self.dims, self.mode)
        design = np.ascontiguousarray(design, dtype=np.float64)
        R = design.shape[1]
        out = np.zeros((out_rows, R))
        H = lib().or_sampled_mttkrp(len(self.khi), _p(self.khi), _p(self.klo), _p(self.rows), _p(self.vals),
                                    samples_dedup.shape[0], _p(shi), _p(slo), R, _p(design), out_rows, _p(out))
        return out, int(H)


# --------------------------------------------------------------------------
# Samplers
# --------------------------------------------------------------------------
def arls_leverage(U: np.ndarray) -> np.ndarray:
    """CP_ARLS_LEV::update_sampler (cp_arls_lev.hpp:25-34)."""
    P = pinv_square(gram(U))
    return dagat(U, P)


def arls_draw(scores, J: int, n: int, uniforms: np.ndarray, perms=None):
    """CP_ARLS_LEV::KRPDrawSamples + draw_leverage_score_samples
    (cp_arls_lev.hpp:36-163) at one rank, uniforms [N, J] and permutations
    [N, J] explicit (perms None: identity)."""
    N = len(scores)
    samples = np.zeros((J, N), dtype=np.uint32)
    w = np.full(J, 0.0 - math.log(float(J)))
    for i in range(N):
        if i == n:
            continue
        s = scores[i]
        total = seq_sum(s)
        cp = discrete_cdf(s)
        if len(cp) == 0:
            idx = np.zeros(J, dtype=np.int64)
        else:
            idx = np.searchsorted(cp, uniforms[i], side="left")
        lw = 0.0 + (np.log(total) - np.log(s[idx]))
        if perms is not None:
            p = np.asarray(perms[i], dtype=np.int64)
            idx, lw = idx[p], lw[p]
        samples[:, i] = idx
        w = w + lw
    return samples, np.exp(w)


class STSState:
    """STS_CP (sts_cp.hpp) at one rank: one row tree (F = R) per factor and the
    per-mode Grams; eigen trees are rebuilt per draw in compute_M."""

    def __init__(self, factors):
        self.R = factors[0].shape[1]
        self.trees = []
        self.grams = []
        for U in factors:
            t = PartitionTree(U.shape[0], self.R, self.R)
            self.trees.append(t)
            self.grams.append(None)
        for k, U in enumerate(factors):
            self.update(k, U)

    def update(self, k: int, U: np.ndarray):
        """update_sampler -> ExactLeverageTree::build_tree (exact_leverage_tree.hpp:156-258)."""
        self.trees[k].build(U)
        self.grams[k] = gram(U)

    def compute_M(self, n: int):
        """STS_CP::computeM (sts_cp.hpp:80-188).  Returns Phi and, for each
        sampled mode k, the scaled-eigenvector matrix its eigen tree uses."""
        N, R = len(self.grams), self.R
        P = {}
        last = np.ones((R, R))
        for k in range(N - 1, -1, -1):
            if k != n:
                P[k] = self.grams[k] * last
                last = P[k]
        first = min(k for k in range(N) if k != n)
        lam, V = np.linalg.eigh(P[first], UPLO="U")
        W = np.zeros((R, R))
        for v in range(R):
            if lam[v] > 1e-8:
                W[:, R - 1 - v] = V[:, v] / math.sqrt(lam[v])
        Phi = W @ W.T
        Phi = np.triu(Phi) + np.triu(Phi, 1).T
        E = {N: np.ascontiguousarray(W.T)}
        for k in range(N - 1, 0, -1):
            if k != n:
                Mk = P[k] * Phi
                lk, Vk = np.linalg.eigh(Mk, UPLO="U")
                with np.errstate(invalid="ignore"):
                    E[k] = np.ascontiguousarray((Vk * np.sqrt(lk)[None, :]).T)
        nxt = {}
        for k in range(N):
            if k == n:
                continue
            j = k + 1
            while j < N and j == n:
                j += 1
            nxt[k] = min(j, N)
        return Phi, E, nxt

    def draw(self, factors, J: int, n: int, uniforms: np.ndarray):
        """STS_CP::KRPDrawSamples (sts_cp.hpp:203-300) at one rank; uniforms
        [N, 2, J]: per sampled mode the eigen-tree then the row-tree draws."""
        N, R = len(factors), self.R
        Phi, E, nxt = self.compute_M(n)
        samples = np.zeros((J, N), dtype=np.uint32)
        h = np.ones((J, R))
        for k in range(N):
            if k == n:
                continue
            sh = h.copy()
            et = PartitionTree(R, 1, R)
            et.build(E[nxt[k]])
            et.hadamard(self.grams[k])
            samples[:, n] = et.sample(E[nxt[k]], h, sh, uniforms[k, 0])
            samples[:, k] = self.trees[k].sample(factors[k], sh, h, uniforms[k, 1])
        w = dagat(h, Phi)
        weights = float(R) / (w * float(J))
        return samples, weights, Phi


# --------------------------------------------------------------------------
# The ALS step (accumulator_stationary.hpp:139-295 at one rank)
# --------------------------------------------------------------------------
def deduplicate(samples: np.ndarray, weights: np.ndarray, n: int):
    """deduplicate_design_matrix (als_optimizer.hpp:130-206): lexicographic
    order over the modes != n, weight times multiplicity."""
    N = samples.shape[1]
    cols = [k for k in range(N) if k != n]
    order = np.lexsort(tuple(samples[:, k] for k in reversed(cols)), axis=0) if cols else np.arange(len(samples))
    s = samples[order]
    key = s[:, cols]
    if len(s) == 0:
        return s, weights[:0]
    new = np.ones(len(s), dtype=bool)
    new[1:] = np.any(key[1:] != key[:-1], axis=1)
    starts = np.flatnonzero(new)
    counts = np.diff(np.append(starts, len(s)))
    return np.ascontiguousarray(s[starts]), weights[order][starts] * counts


def design_matrix(factors, samples_dedup: np.ndarray, weights_dedup: np.ndarray, n: int):
    """Design rows, Gram and pinv (accumulator_stationary.hpp:212-249)."""
    R = factors[0].shape[1]
    D = np.ones((samples_dedup.shape[0], R))
    for k in range(len(factors)):
        if k != n:
            D *= factors[k][samples_dedup[:, k].astype(np.int64)]
    sw = np.sqrt(weights_dedup)[:, None]
    D *= sw
    G = gram(D)
    Phi = pinv_square(G)
    D *= sw
    return D, G, Phi


def renormalize(U: np.ndarray):
    """DistMat1D::renormalize_columns (distmat.hpp:85-138)."""
    norms = np.sqrt((U * U).sum(axis=0))
    return U / norms[None, :], norms


class OracleALS:
    """Single-rank restatement of SparseTensor + LowRankTensor + sampler +
    AccumulatorStationary (sparse_tensor.hpp:36-96; low_rank_tensor.hpp;
    accumulator_stationary.hpp:38-295).  The random relabelling of modes
    (sparse_tensor.hpp:76-95) is left out: it is a load-balancing permutation
    that the caller can apply to the coordinates beforehand."""

    def __init__(self, dims, idx, val, factors, sampler: str, preprocessing: str = "none"):
        self.dims = [int(d) for d in dims]
        self.N = len(self.dims)
        self.idx = np.ascontiguousarray(idx, dtype=np.uint32)
        v = np.asarray(val, dtype=np.float64)
        if preprocessing == "log_count":
            v = np.log(v + 1)
        elif preprocessing == "ones":
            v = np.ones_like(v)
        self.val = np.ascontiguousarray(v)
        self.tensor_norm = math.sqrt(float(np.dot(self.val, self.val)))
        self.factors = [np.ascontiguousarray(U, dtype=np.float64).copy() for U in factors]
        self.R = self.factors[0].shape[1]
        self.sigma = np.ones(self.R)
        self.sampler = sampler
        self.lookups = [SortIdxLookup(self.idx, self.val, self.dims, n) for n in range(self.N)]
        if sampler == "cp_arls_lev":
            self.scores = [arls_leverage(U) for U in self.factors]
        elif sampler == "sts_cp":
            self.sts = STSState(self.factors)
        else:
            raise ValueError(sampler)

    def draw(self, n: int, J: int, uniforms, perms=None):
        if self.sampler == "cp_arls_lev":
            return arls_draw(self.scores, J, n, uniforms, perms)
        samples, weights, _ = self.sts.draw(self.factors, J, n, uniforms)
        return samples, weights

    def update_sampler(self, n: int):
        if self.sampler == "cp_arls_lev":
            self.scores[n] = arls_leverage(self.factors[n])
        else:
            self.sts.update(n, self.factors[n])

    def step(self, n: int, J: int, uniforms, perms=None, draws=None) -> dict:
        """One AccumulatorStationary step.  draws: optional (samples, weights)
        to use in place of the oracle's own draw (to check the solve of a
        form whose draws may differ in a few near-tie samples)."""
        samples, weights = self.draw(n, J, uniforms, perms) if draws is None else draws
        sd, wd = deduplicate(samples, weights, n)
        D, G, Phi = design_matrix(self.factors, sd, wd, n)
        M, hits = self.lookups[n].sampled_mttkrp(sd, D, self.dims[n])
        U = M @ Phi
        U, norms = renormalize(U)
        self.factors[n] = U
        self.sigma = norms
        self.update_sampler(n)
        return dict(samples=samples, weights=weights, samples_dedup=sd, weights_dedup=wd, design=D,
                    design_gram=G, design_pinv=Phi, mttkrp=M, hits=hits, factor=U, sigma=norms)

    def fit(self) -> float:
        """SparseTensor::compute_exact_fit (sparse_tensor.hpp:288-356)."""
        R = self.R
        chain = np.ones((R, R))
        for U in self.factors:
            chain = chain * gram(U)
        normsq = float(np.sum(chain * np.outer(self.sigma, self.sigma)))
        Us = [np.ascontiguousarray(U) for U in self.factors]
        arr = (ctypes.c_void_p * self.N)(*[U.ctypes.data for U in Us])
        sig = np.ascontiguousarray(self.sigma)
        bmb = lib().or_fit_residual(self.N, R, self.idx.shape[0], _p(self.idx), _p(self.val), arr, _p(sig))
        return 1.0 - math.sqrt(normsq + bmb) / self.tensor_norm


def mt19937_canonicals(seed: int, count: int) -> np.ndarray:
    """The doubles std::generate_canonical<double, 53>(std::mt19937(seed))
    returns, `count` of them in order (libstdc++ bits/random.tcc:3349-3381:
    two 32-bit outputs, low word first, divided by 2^64, clamped below 1).
    numpy's MT19937 with legacy integer seeding is the same generator."""
    bg = np.random.MT19937()
    bg._legacy_seeding(int(seed))
    raw = bg.random_raw(2 * count)
    u0 = raw[0::2].astype(np.float64)
    u1 = raw[1::2].astype(np.float64)
    r = (u0 + u1 * 4294967296.0) / 18446744073709551616.0
    r[r >= 1.0] = np.nextafter(1.0, 0.0)
    return r


def sts_uniform_stream(seed: int, N: int, J: int, steps: int) -> list:
    """Per-step uniforms [N, 2, J] that STS_CP::KRPDrawSamples consumes from one
    local stream over `steps` consecutive ALS steps (mode t % N at step t):
    per sampled mode, J eigen-tree draws then J row-tree draws
    (sts_cp.hpp:228-255, fill_buffer_random_draws 190-201)."""
    flat = mt19937_canonicals(seed, steps * 2 * (N - 1) * J)
    out, pos = [], 0
    for t in range(steps):
        n = t % N
        u = np.full((N, 2, J), -1.0)
        for k in range(N):
            if k == n:
                continue
            for s in range(2):
                u[k, s] = flat[pos:pos + J]
                pos += J
        out.append(u)
    return out


def exact_als_sweep(ora: "OracleALS", sweeps: int = 1):
    """ExactALS (exact_als.hpp:90-143) at one rank, `sweeps` rounds, applied to
    the oracle's factors in place (decompose.py:82-96 runs one as the
    "-p exact" preprocessing).  Keeps its own Gram matrices, as the reference
    does, and ends by refreshing the sampler."""
    N, R = ora.N, ora.R
    grams = [gram(U) for U in ora.factors]
    for _ in range(sweeps):
        for n in range(N):
            chain = np.ones((R, R))
            for k in range(N):
                if k != n:
                    chain = chain * grams[k]
            Phi = pinv_square(chain)
            Us = [np.ascontiguousarray(U) for U in ora.factors]
            arr = (ctypes.c_void_p * N)(*[U.ctypes.data for U in Us])
            M = np.zeros((ora.dims[n], R))
            lib().or_exact_mttkrp(N, n, R, ora.idx.shape[0], _p(ora.idx), _p(ora.val), arr, ora.dims[n], _p(M))
            U, norms = renormalize(M @ Phi)
            ora.factors[n] = U
            ora.sigma = norms
            grams[n] = gram(U)
    for n in range(N):
        ora.update_sampler(n)


def estimated_fit(ora: "OracleALS", zero_coords: np.ndarray):
    """DistLowRank.compute_estimated_fit (exafac/low_rank_tensor.py:110-184)
    with the zero samples given and an exact membership test: the squared
    error over every nonzero plus the mean squared model value over the zero
    samples that are not nonzeros, scaled by (prod dims - nnz).  Returns
    (estimated fit, zero samples kept)."""
    def model(coords):
        p = np.tile(ora.sigma, (len(coords), 1))
        for k, U in enumerate(ora.factors):
            p = p * U[coords[:, k].astype(np.int64)]
        return p.sum(axis=1)

    nonzero_loss = float(np.sum((ora.val - model(ora.idx)) ** 2))
    present = {tuple(int(x) for x in row) for row in ora.idx}
    keep = np.array([tuple(int(x) for x in row) not in present for row in zero_coords], dtype=bool)
    z = model(np.asarray(zero_coords)[keep])
    kept = int(keep.sum())
    dense = float(np.prod(np.array(ora.dims, dtype=np.float64)))
    zero_loss = float(np.sum(z * z)) * (dense - ora.idx.shape[0]) / kept if kept else 0.0
    return 1.0 - math.sqrt(nonzero_loss + zero_loss) / ora.tensor_norm, kept
