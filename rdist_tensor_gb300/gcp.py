"""Generalized CP (GCP) on sampled entries, on the GPU.

The model at sampled coordinates, m_j = sum_r prod_k U_k[i_jk, r], is a
``torch.autograd.Function`` whose forward and backward are the library's
hand-written kernels (``exafac_cp_sampled_model`` and
``exafac_cp_sampled_adjoint``): the backward is the sampled MTTKRP of the
loss derivatives into every factor, with the Khatri-Rao rows recomputed from
the factors instead of stored.  A loss on the sampled entries (Poisson,
Bernoulli or Gaussian) written in torch then gives gradient-based GCP
(Hong, Kolda and Duersch, "Generalized canonical polyadic tensor
decomposition", SIAM Review 2020) driven by the stratified sampler
``exafac_gcp_sample_entries``.

This part has no counterpart in the reference; its nearest relatives there
are execute_exact_mttkrp (exafac/cpp_ext/sort_lookup.hpp:440-495) and the
zero-sampling fit estimate (exafac/low_rank_tensor.py:110-184).  There is no
CPU path: without the built library or a GPU every call raises.
"""
from __future__ import annotations

import ctypes
from typing import Sequence

import torch

from . import _lib

_DTYPES = {torch.float32: 0, torch.float64: 1}
EPS = 1e-10


def _stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dims_arg(dims: Sequence[int]):
    return (ctypes.c_int64 * len(dims))(*[int(d) for d in dims])


def _ptrs(ts):
    return (ctypes.c_void_p * len(ts))(*[t.data_ptr() if t is not None else None for t in ts])


def _check(idx: torch.Tensor, factors: Sequence[torch.Tensor]):
    if not idx.is_cuda or idx.dtype != torch.int32 or idx.dim() != 2 or not idx.is_contiguous():
        raise ValueError("idx must be a contiguous int32 [J, N] CUDA tensor")
    dt = factors[0].dtype
    if dt not in _DTYPES:
        raise ValueError("factors must be float32 or float64")
    R = factors[0].shape[1]
    for U in factors:
        if not U.is_cuda or U.dtype != dt or U.dim() != 2 or U.shape[1] != R or not U.is_contiguous():
            raise ValueError("factors must be contiguous [dims_k, R] CUDA tensors of one dtype")
    if idx.shape[1] != len(factors):
        raise ValueError("idx has one column per mode")
    return dt, R


class SampledCPModel(torch.autograd.Function):
    """m = SampledCPModel.apply(idx, *factors): model values at the sampled
    coordinates; backward accumulates the sampled MTTKRP of grad_m into the
    factor gradients."""

    @staticmethod
    def forward(ctx, idx: torch.Tensor, *factors: torch.Tensor) -> torch.Tensor:
        dt, R = _check(idx, factors)
        N, J = len(factors), idx.shape[0]
        dims = [U.shape[0] for U in factors]
        m = torch.empty(J, dtype=dt, device=idx.device)
        status = torch.zeros(1, dtype=torch.int32, device=idx.device)
        _lib.call("exafac_cp_sampled_model", N, R, _dims_arg(dims), J, ctypes.c_void_p(idx.data_ptr()),
                  _ptrs(factors), ctypes.c_void_p(m.data_ptr()), _DTYPES[dt], ctypes.c_void_p(status.data_ptr()),
                  _stream())
        ctx.save_for_backward(idx, *factors)
        ctx.status = status
        return m

    @staticmethod
    def backward(ctx, grad_m: torch.Tensor):
        idx, *factors = ctx.saved_tensors
        dt, R = _check(idx, factors)
        N, J = len(factors), idx.shape[0]
        dims = [U.shape[0] for U in factors]
        grads = [torch.zeros_like(U) if ctx.needs_input_grad[1 + k] else None for k, U in enumerate(factors)]
        gm = grad_m.contiguous().to(dt)
        _lib.call("exafac_cp_sampled_adjoint", N, R, _dims_arg(dims), J, ctypes.c_void_p(idx.data_ptr()),
                  ctypes.c_void_p(gm.data_ptr()), _ptrs(factors), _ptrs(grads), _DTYPES[dt],
                  ctypes.c_void_p(ctx.status.data_ptr()), _stream())
        return (None, *grads)


def sampled_model(idx: torch.Tensor, factors: Sequence[torch.Tensor]) -> torch.Tensor:
    return SampledCPModel.apply(idx, *factors)


def loss_values(kind: str, x: torch.Tensor, m: torch.Tensor) -> torch.Tensor:
    """Elementwise GCP losses f(x, m) (Hong, Kolda, Duersch, Table 2.1)."""
    if kind == "poisson":  # identity link, m >= 0
        return m - x * torch.log(m + EPS)
    if kind == "bernoulli":  # odds link, m >= 0
        return torch.log(m + 1.0) - x * torch.log(m + EPS)
    if kind == "gaussian":
        return (x - m) ** 2
    raise ValueError(f"unknown loss {kind!r}")


def sample_entries(idx: torch.Tensor, vals: torch.Tensor, dims: Sequence[int], J_nz: int, J_z: int, seed: int,
                   counter: int):
    """Stratified sample of nonzeros and uniform coordinates (see the C
    header): returns (coordinates [J, N] int32, values [J], weights [J])."""
    N = len(dims)
    dt = vals.dtype
    J = J_nz + J_z
    out_idx = torch.empty((J, N), dtype=torch.int32, device=idx.device)
    x = torch.empty(J, dtype=dt, device=idx.device)
    w = torch.empty(J, dtype=dt, device=idx.device)
    _lib.call("exafac_gcp_sample_entries", N, _dims_arg(dims), idx.shape[0], ctypes.c_void_p(idx.data_ptr()),
              ctypes.c_void_p(vals.data_ptr()), J_nz, J_z, ctypes.c_uint64(seed), ctypes.c_uint64(counter),
              ctypes.c_void_p(out_idx.data_ptr()), ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(w.data_ptr()),
              _DTYPES[dt], _stream())
    return out_idx, x, w


class FusedAdam:
    """Adam over CUDA tensors in one launch per step of the library's fused
    kernel (``exafac_adam_step``): torch.optim.Adam's update without weight
    decay or amsgrad, in the parameters' own precision, followed when
    ``lower`` is given by the projection onto x >= lower.  It reads each
    parameter, gradient and moment once and writes the parameter and moments
    once: 7 words per parameter, where torch's Adam plus a separate
    projection pass moves 9.  A parameter without a gradient takes a zero
    gradient (its moments still decay)."""

    def __init__(self, params, lr: float = 1e-3, betas=(0.9, 0.999), eps: float = 1e-8, lower=None):
        self.params = list(params)
        if not self.params or len(self.params) > 8:
            raise ValueError("FusedAdam takes 1 to 8 tensors")
        dt = self.params[0].dtype
        if dt not in _DTYPES:
            raise ValueError("parameters must be float32 or float64")
        for q in self.params:
            if not q.is_cuda or q.dtype != dt or not q.is_contiguous():
                raise ValueError("parameters must be contiguous CUDA tensors of one dtype")
        self.lr, self.betas, self.eps, self.lower = float(lr), (float(betas[0]), float(betas[1])), float(eps), lower
        self.dtype = dt
        self.exp_avg = [torch.zeros_like(q, memory_format=torch.contiguous_format) for q in self.params]
        self.exp_avg_sq = [torch.zeros_like(q, memory_format=torch.contiguous_format) for q in self.params]
        self.steps = 0
        self._numel = (ctypes.c_int64 * len(self.params))(*[q.numel() for q in self.params])

    def zero_grad(self, set_to_none: bool = True):
        for q in self.params:
            if set_to_none:
                q.grad = None
            elif q.grad is not None:
                q.grad.zero_()

    @torch.no_grad()
    def step(self):
        grads = []
        for q in self.params:
            g = q.grad
            if g is not None and (g.dtype != self.dtype or not g.is_contiguous()):
                g = g.to(self.dtype).contiguous()
            grads.append(g)
        self.steps += 1
        _lib.call("exafac_adam_step", len(self.params), _ptrs(self.params), _ptrs(grads), _ptrs(self.exp_avg),
                  _ptrs(self.exp_avg_sq), self._numel, _DTYPES[self.dtype], self.lr, self.betas[0], self.betas[1],
                  self.eps, self.steps, 0 if self.lower is None else 1,
                  0.0 if self.lower is None else float(self.lower), _stream())


class GCP:
    """Gradient-based GCP of a sparse tensor with stratified entry sampling,
    fused Adam steps, and (for the Poisson and Bernoulli losses) nonnegative
    factors by projection after every step.  Factors start Uniform(0, 0.5)."""

    def __init__(self, idx, vals, dims: Sequence[int], rank: int, loss: str = "poisson",
                 dtype: torch.dtype = torch.float32, seed: int = 0, device: str = "cuda"):
        self.dims = [int(d) for d in dims]
        self.N, self.R, self.loss = len(self.dims), int(rank), loss
        self.idx = torch.as_tensor(idx, device=device).to(torch.int32).contiguous()
        self.vals = torch.as_tensor(vals, device=device).to(dtype).contiguous()
        self.seed, self.counter = int(seed), 0
        g = torch.Generator(device=device)
        g.manual_seed(int(seed))
        self.factors = [torch.rand((d, self.R), generator=g, dtype=dtype, device=device).mul_(0.5).requires_grad_()
                        for d in self.dims]
        self._opt, self._lr = None, None

    def model_mass(self) -> float:
        """Sum of the model over every entry of the tensor:
        sum_r prod_k (sum_i U_k[i, r]), in FP64."""
        with torch.no_grad():
            tot = torch.ones(self.R, dtype=torch.float64, device=self.factors[0].device)
            for U in self.factors:
                tot *= U.detach().double().sum(dim=0)
            return float(tot.sum())

    def full_objective(self, chunk: int = 1 << 24) -> float:
        """The Poisson objective over every entry of the tensor, zeros
        included: sum_all m - sum_nz x log(m + EPS).  The first sum is the
        model mass (column sums), so only the nonzeros are evaluated."""
        if self.loss != "poisson":
            raise ValueError("full_objective is defined for the Poisson loss")
        nz = 0.0
        with torch.no_grad():
            for a in range(0, self.idx.shape[0], chunk):
                m = sampled_model(self.idx[a:a + chunk], self.factors)
                nz += float((self.vals[a:a + chunk].double() * torch.log(m.double() + EPS)).sum())
        return self.model_mass() - nz

    def objective(self, idx, x, w) -> torch.Tensor:
        m = sampled_model(idx, self.factors)
        return (w * loss_values(self.loss, x, m)).sum()

    def step_sample(self, J_nz: int, J_z: int):
        out = sample_entries(self.idx, self.vals, self.dims, J_nz, J_z, self.seed, self.counter)
        self.counter += 1
        return out

    def optimizer(self, lr: float = 1e-2) -> FusedAdam:
        """The model's Adam optimizer, fused with the projection onto
        nonnegative factors for the Poisson and Bernoulli losses; its moments
        persist across steps and fit calls while the rate stays the same."""
        if self._opt is None or self._lr != lr:
            lower = 0.0 if self.loss in ("poisson", "bernoulli") else None
            self._opt = FusedAdam(self.factors, lr=lr, lower=lower)
            self._lr = lr
        return self._opt

    def step(self, J_nz: int, J_z: int, lr: float = 1e-2) -> torch.Tensor:
        """One gradient step: a fresh stratified sample, the weighted loss on
        it, its gradient through the sampled adjoint, and the fused Adam
        update with (for the Poisson and Bernoulli losses) the projection onto
        nonnegative factors.  Returns the sampled objective as a device
        scalar; nothing is read back to the host."""
        opt = self.optimizer(lr)
        idx, x, w = self.step_sample(J_nz, J_z)
        opt.zero_grad(set_to_none=True)
        f = self.objective(idx, x, w)
        f.backward()
        opt.step()
        return f.detach()

    def fit(self, steps: int, J_nz: int, J_z: int, lr: float = 1e-2):
        history = [self.step(J_nz, J_z, lr) for _ in range(steps)]
        return torch.stack(history) if history else torch.empty(0)
