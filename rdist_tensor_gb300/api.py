"""The reference's Python-facing classes (exafac/cpp_ext/py_module.cpp:37-77) on
one GB300: same names, constructor arguments and methods, with torch CUDA
tensors as the device buffers and the sampled-ALS step in
libexafac_gb300.so (C ABI: include/exafac_gb300.h).

One process drives one GPU, so the process grid is 1 x ... x 1: ``Grid`` and
``TensorGrid`` keep their signatures and reject any other shape, as the
reference does when the grid does not match the MPI world (grid.hpp:62-65).
"""
from __future__ import annotations

import ctypes
import json
import time

import numpy as np
import torch

from . import _lib

_REGIONS = ["leverage_sampling_time", "row_gather_time", "design_matrix_prep_time", "spmm_time",
            "dense_reduce_time", "postprocessing_time", "sampler_update_time"]


def _device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("exafac GB300 engine needs a CUDA device (no CPU fallback)")
    return torch.device("cuda", torch.cuda.current_device())


def _stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t: torch.Tensor) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


class Grid:
    """Cartesian processor grid (grid.hpp:16-122); one rank here."""

    def __init__(self, proc_dims):
        self.proc_dims = np.asarray(proc_dims, dtype=np.int32).copy()
        if int(np.prod(self.proc_dims)) != 1:
            raise RuntimeError("The number of MPI ranks does not match the number of processes specified by the grid.")
        self.dim = len(self.proc_dims)
        self.rank = 0
        self.world_size = 1

    def get_dimension(self) -> int:
        return self.dim


class TensorGrid:
    """Per-mode row blocks of the grid (grid.hpp:124-174)."""

    def __init__(self, tensor_dims, grid: Grid):
        self.tensor_dims = np.asarray(tensor_dims, dtype=np.int64).copy()
        self.grid = grid
        self.dim = grid.dim
        self.rank = 0
        if len(self.tensor_dims) != grid.dim:
            raise ValueError("Grid dimension must match tensor dimension")
        # round_to_nearest_integer(n, 1) / 1 = n + 1 (common.h:196-198); the
        # extra row is never part of the factor here.
        self.padded_row_counts = [int(d) + 1 for d in self.tensor_dims]


class DistMat1D:
    """One factor matrix (distmat.hpp:15-193): rows x cols float64 on the GPU."""

    def __init__(self, cols: int, tensor_grid: TensorGrid, slice_dim: int):
        self.cols = int(cols)
        self.tensor_grid = tensor_grid
        self.slice_dim = int(slice_dim)
        self.rows = int(tensor_grid.tensor_dims[slice_dim])
        self.true_row_count = self.rows
        self.data = torch.zeros((self.rows, self.cols), dtype=torch.float64, device=_device())

    def initialize_deterministic(self):
        """distmat.hpp:140-151: U[i, j] = cos(i * cols + j)."""
        i = torch.arange(self.rows, dtype=torch.float64, device=self.data.device)[:, None]
        j = torch.arange(self.cols, dtype=torch.float64, device=self.data.device)[None, :]
        self.data.copy_(torch.cos(i * self.cols + j))

    def initialize_gaussian_random(self, generator=None):
        """distmat.hpp:153-168: N(0, 1) entries."""
        self.data.normal_(0.0, 1.0, generator=generator)

    def renormalize_columns(self, col_norms_out=None):
        """distmat.hpp:85-138."""
        norms = torch.sqrt((self.data * self.data).sum(dim=0))
        self.data.div_(norms[None, :])
        if col_norms_out is not None:
            col_norms_out.copy_(norms)

    def compute_gram_matrix(self) -> torch.Tensor:
        return self.data.T @ self.data


class LowRankTensor:
    """sigma (R) and one DistMat1D per mode (low_rank_tensor.hpp:10-54)."""

    def __init__(self, rank: int, tensor_grid: TensorGrid):
        self.rank = int(rank)
        self.tensor_grid = tensor_grid
        self.sigma = torch.ones(self.rank, dtype=torch.float64, device=_device())
        self.factors = [DistMat1D(self.rank, tensor_grid, i) for i in range(tensor_grid.dim)]

    def initialize_factors_deterministic(self):
        for f in self.factors:
            f.initialize_deterministic()
            f.renormalize_columns(None)
        self.sigma.fill_(1.0)

    def initialize_factors_gaussian_random(self, seed: int | None = None):
        gen = None
        if seed is not None:
            gen = torch.Generator(device=self.sigma.device)
            gen.manual_seed(int(seed))
        for f in self.factors:
            f.initialize_gaussian_random(gen)
            f.renormalize_columns(None)
        self.sigma.fill_(1.0)

    def set_factors(self, mats, sigma=None):
        """Copies host or device matrices into the factors (test and resume helper)."""
        for f, m in zip(self.factors, mats):
            f.data.copy_(torch.as_tensor(np.asarray(m) if not torch.is_tensor(m) else m, dtype=torch.float64))
        if sigma is not None:
            self.sigma.copy_(torch.as_tensor(sigma, dtype=torch.float64))
        else:
            self.sigma.fill_(1.0)

    def write_to_file(self, filename: str, fmt: str | None = None) -> str:
        """LowRankTensor.write_to_file (exafac/low_rank_tensor.py:186-192):
        FACTOR_MODE_i datasets (HDF5 when h5py is importable, else .npz),
        plus SIGMA.  Returns the path written."""
        from . import checkpoint

        return checkpoint.write_factors(filename, [f.data.cpu().numpy() for f in self.factors],
                                        self.sigma.cpu().numpy(), fmt)

    def read_from_file(self, filename: str):
        """Loads factors (and sigma, when the file holds it) written by
        write_to_file, to resume a decomposition."""
        from . import checkpoint

        mats, sigma = checkpoint.read_factors(filename)
        if len(mats) != len(self.factors):
            raise ValueError(f"{filename} holds {len(mats)} factors, the tensor has {len(self.factors)} modes")
        for f, m in zip(self.factors, mats):
            if tuple(m.shape) != tuple(f.data.shape):
                raise ValueError(f"factor shape {m.shape} does not match {tuple(f.data.shape)}")
        self.set_factors(mats, sigma)

    def test_gram_matrix_computation(self):
        """low_rank_tensor.hpp:44-54: prints the Grams of the deterministic factors."""
        for i, f in enumerate(self.factors):
            f.initialize_deterministic()
            print(f"Gram matrix for factor {i}")
            print(f.compute_gram_matrix().cpu().numpy())


class SparseTensor:
    """COO tensor (sparse_tensor.hpp:17-96): coordinates and float64 values on
    the GPU.  ``SparseTensor(tensor_grid, idx, vals, preprocessing)`` takes
    numpy or torch arrays (uint32/int32/int64 coordinates, float32/float64
    values); ``SparseTensor(tensor_grid, I, N, Q)`` builds the reference's
    synthetic block tensor (sparse_tensor.hpp:102-215).

    The reference relabels every mode with a random permutation to balance
    MPI ranks (sparse_tensor.hpp:76-95); with one GPU there is nothing to
    balance and coordinates are kept as given."""

    def __init__(self, tensor_grid: TensorGrid, a, b, c, seed: int = 0):
        self.tensor_grid = tensor_grid
        self.dim = tensor_grid.dim
        if isinstance(c, str):
            idx, vals, self.preprocessing = a, b, c
        else:
            idx, vals = _block_tensor(int(a), int(b), int(c), seed)
            self.preprocessing = "none"
        # Host-side validation first (shape, coordinate range, value count,
        # preprocessing name), before anything reaches the device.
        idx_t = torch.as_tensor(np.ascontiguousarray(idx).astype(np.int64, copy=False) if not torch.is_tensor(idx)
                                else idx)
        if idx_t.dim() != 2 or idx_t.shape[1] != self.dim:
            raise ValueError("indices must be nnz x N")
        self.nnz = int(idx_t.shape[0])
        dims = torch.as_tensor(tensor_grid.tensor_dims, dtype=torch.int64)
        if bool((dims < 1).any()) or bool((dims > 0xffffffff).any()):
            raise ValueError("mode sizes must be in [1, 2^32)")
        if self.nnz and (idx_t.min() < 0 or bool((idx_t.max(dim=0).values >= dims.to(idx_t.device)).any())):
            raise ValueError("coordinate out of range for the tensor grid")
        v = torch.as_tensor(vals) if not torch.is_tensor(vals) else vals
        if v.numel() != self.nnz:
            raise ValueError("values must have one entry per nonzero")
        if self.preprocessing not in _lib.PREPROCESSING:
            raise ValueError(f"unknown preprocessing {self.preprocessing}")
        dev = _device()
        # The engine reads coordinates as uint32 words; they are held in an
        # int32 tensor, where a coordinate in [2^31, 2^32) keeps its bit
        # pattern (two's-complement wrap of the validated int64 value).
        idx64 = idx_t.to(device=dev, dtype=torch.int64)
        self.indices = torch.where(idx64 >= 2 ** 31, idx64 - 2 ** 32, idx64).to(torch.int32).contiguous()
        self.values = v.to(device=dev, dtype=torch.float64).contiguous().reshape(-1)


def _block_tensor(I: int, N: int, Q: int, seed: int):
    """sparse_tensor.hpp:102-215 at one rank: every factor has one basis vector
    per row (uniform over Q); the tensor is the sum of Q rank-one blocks with
    unit entries."""
    if N != 3:
        raise ValueError("Error, dimension must be 3.")
    rng = np.random.default_rng(seed)
    lists = [[[] for _ in range(Q)] for _ in range(N)]
    for i in range(N):
        cols = rng.integers(0, Q, size=I)
        for k, j in enumerate(cols):
            lists[i][j].append(k)
    blocks = []
    for j in range(Q):
        a, b, c = (np.array(lists[i][j], dtype=np.int64) for i in range(3))
        if len(a) and len(b) and len(c):
            g = np.stack(np.meshgrid(a, b, c, indexing="ij"), axis=-1).reshape(-1, 3)
            blocks.append(g)
    idx = np.concatenate(blocks) if blocks else np.zeros((0, 3), dtype=np.int64)
    return idx.astype(np.uint32), np.ones(len(idx))


class Sampler:
    """sampler.hpp:16-41.  The sampler's state lives in the optimizer's session."""

    kind = ""

    def __init__(self, low_rank_tensor: LowRankTensor):
        self.low_rank_tensor = low_rank_tensor


class CP_ARLS_LEV(Sampler):
    """Per-factor leverage-score sampling (cp_arls_lev.hpp)."""

    kind = "cp_arls_lev"


class STS_CP(Sampler):
    """Exact Khatri-Rao leverage sampling through segment trees (sts_cp.hpp)."""

    kind = "sts_cp"


class ALS_Optimizer:
    """Round loop, fit and statistics (als_optimizer.hpp:10-218)."""

    def __init__(self, ground_truth: SparseTensor, low_rank_tensor: LowRankTensor, sampler: Sampler | None,
                 max_samples: int = 1 << 19, precision: str = "fp64", seed: int = 0x5eed,
                 workspace_fill: int | None = None):
        """workspace_fill: a byte value written over the session's device
        workspace before it is used (a test aid: results must not depend on
        what the workspace held; 0xFF makes every float and double a NaN)."""
        self.ground_truth = ground_truth
        self.low_rank_tensor = low_rank_tensor
        self.sampler = sampler
        self.max_samples = int(max_samples)
        self.precision = precision
        self.seed = int(seed)
        self.workspace_fill = workspace_fill
        self.stats = {}
        self._h = None
        self._ws = None
        self.tensor_norm = None
        self.timing = False

    # -- session -----------------------------------------------------------
    def _config(self, J_max: int) -> _lib.AlsConfig:
        gt, lr = self.ground_truth, self.low_rank_tensor
        cfg = _lib.AlsConfig()
        cfg.N = gt.dim
        cfg.R = lr.rank
        for k in range(gt.dim):
            cfg.dims[k] = int(gt.tensor_grid.tensor_dims[k])
        cfg.nnz = gt.nnz
        cfg.J_max = int(J_max)
        kind = self.sampler.kind if self.sampler is not None else "cp_arls_lev"
        cfg.sampler = _lib.SAMPLER[kind]
        cfg.precision = _lib.PRECISION[self.precision]
        cfg.preprocessing = _lib.PREPROCESSING[gt.preprocessing]
        return cfg

    def _factors(self) -> _lib.Factors:
        f = _lib.Factors()
        for k, m in enumerate(self.low_rank_tensor.factors):
            f.U[k] = m.data.data_ptr()
        f.sigma = self.low_rank_tensor.sigma.data_ptr()
        return f

    def _create(self, J_max: int):
        self.deinitialize()
        for k, f in enumerate(self.low_rank_tensor.factors):
            if not bool(torch.isfinite(f.data).all()):
                raise ValueError(f"factor matrix {k} has a non-finite entry")
        if not bool(torch.isfinite(self.low_rank_tensor.sigma).all()):
            raise ValueError("sigma has a non-finite entry")
        cfg = self._config(J_max)
        pers, setup = ctypes.c_size_t(), ctypes.c_size_t()
        _lib.call("exafac_als_workspace_size", ctypes.byref(cfg), ctypes.byref(pers), ctypes.byref(setup))
        dev = _device()
        self._ws = torch.empty(pers.value, dtype=torch.uint8, device=dev)
        setup_ws = torch.empty(setup.value, dtype=torch.uint8, device=dev)
        if self.workspace_fill is not None:
            self._ws.fill_(int(self.workspace_fill))
            setup_ws.fill_(int(self.workspace_fill))
        h = ctypes.c_void_p()
        _lib.call("exafac_als_create", ctypes.byref(cfg), _ptr(self._ws), ctypes.c_size_t(pers.value),
                  ctypes.byref(h))
        self._h = h
        self._cfg = cfg
        _lib.call("exafac_als_set_seed", self._h, ctypes.c_uint64(self.seed))
        norm = ctypes.c_double()
        self._fac = self._factors()
        _lib.call("exafac_als_init", self._h, _ptr(self.ground_truth.indices), _ptr(self.ground_truth.values),
                  ctypes.byref(self._fac), _ptr(setup_ws), ctypes.c_size_t(setup.value), ctypes.byref(norm),
                  _stream())
        del setup_ws
        self.tensor_norm = norm.value
        if self.timing:
            _lib.call("exafac_als_enable_timing", self._h, 1)

    def initialize_ground_truth_for_als(self):
        self._create(self.max_samples)

    def deinitialize(self):
        if self._h is not None:
            torch.cuda.synchronize()
            _lib.load().exafac_als_destroy(self._h)
            self._h = None
            self._ws = None

    def __del__(self):
        try:
            self.deinitialize()
        except Exception:
            pass

    def _require(self):
        if self._h is None:
            raise RuntimeError("initialize_ground_truth_for_als() must be called first")

    # -- reference methods ---------------------------------------------------
    def compute_exact_fit(self) -> float:
        self._require()
        out = ctypes.c_double()
        _lib.call("exafac_als_fit", self._h, ctypes.byref(out), _stream())
        return out.value

    def compute_estimated_fit(self, alpha: float = 0.5, seed: int = 0, zero_coords=None):
        """The reference's legacy zero-sampling fit estimate
        (exafac/low_rank_tensor.py:110-184): the error over every nonzero plus
        (1 / alpha - 1) nnz uniform zero samples (coordinates that are
        nonzeros are found exactly and dropped).  zero_coords: optional
        Z x N coordinates to use instead of the Philox draws.  Returns
        (estimated fit, zero samples kept)."""
        self._require()
        fit, kept = ctypes.c_double(), ctypes.c_int64()
        if zero_coords is not None:
            z = torch.as_tensor(np.asarray(zero_coords, dtype=np.int64) if not torch.is_tensor(zero_coords)
                                else zero_coords)
            if z.dim() != 2 or z.shape[1] != self.ground_truth.dim:
                raise ValueError("zero_coords must be Z x N")
            dims = torch.as_tensor(self.ground_truth.tensor_grid.tensor_dims, dtype=torch.int64)
            if z.numel() and (z.min() < 0 or bool((z.max(dim=0).values >= dims.to(z.device)).any())):
                raise ValueError("zero coordinate out of range")
            z64 = z.to(device=_device(), dtype=torch.int64)
            zd = torch.where(z64 >= 2 ** 31, z64 - 2 ** 32, z64).to(torch.int32).contiguous()
            Z = int(zd.shape[0])
            ptr = _ptr(zd)
        else:
            Z = max(1, int(round((1.0 / float(alpha) - 1.0) * self.ground_truth.nnz)))
            ptr = None
        _lib.call("exafac_als_estimated_fit", self._h, Z, ptr, ctypes.c_uint64(int(seed)), ctypes.byref(fit),
                  ctypes.byref(kept), _stream())
        return fit.value, kept.value

    def execute_ALS_step(self, mode: int, J: int, uniforms: torch.Tensor | None = None,
                         perms: torch.Tensor | None = None):
        self._require()
        if J > self.max_samples:
            self.max_samples = int(J)
            self._create(self.max_samples)
        _lib.call("exafac_als_step", self._h, int(mode), int(J), _ptr(uniforms) if uniforms is not None else None,
                  _ptr(perms) if perms is not None else None, _stream())

    def execute_sweeps(self, num_sweeps: int, J: int, uniforms: torch.Tensor | None = None):
        """num_sweeps sweeps (modes 0..N-1) without per-region timers, replayed
        from one captured CUDA graph once every factor has had a sampled
        update.  uniforms: None for the session's Philox stream, or a device
        tensor of N per-step blocks (as execute_ALS_step takes), read on every
        sweep (refill it in place between calls)."""
        self._require()
        if J > self.max_samples:
            self.max_samples = int(J)
            self._create(self.max_samples)
        if self.timing:
            _lib.call("exafac_als_enable_timing", self._h, 0)
            self.timing = False
        _lib.call("exafac_als_sweeps", self._h, int(J), int(num_sweeps),
                  _ptr(uniforms) if uniforms is not None else None, _stream())

    def execute_ALS_rounds(self, num_rounds: int, J: int, epoch_interval: int):
        """als_optimizer.hpp:40-124; timers are CUDA events on the GPU."""
        self._require()
        if J > self.max_samples:
            self.max_samples = int(J)
            self._create(self.max_samples)
        self.timing = True
        _lib.call("exafac_als_enable_timing", self._h, 1)
        info0 = self.step_info()
        rounds, fits, als_times, fit_times = [0], [0.0], [0.0], [0.0]
        als_total = 0.0
        fit_total = 0.0
        dim = self.ground_truth.dim
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        for rnd in range(1, int(num_rounds) + 1):
            print(f"Starting ALS round {rnd}")
            ev0.record()
            for i in range(dim):
                self.execute_ALS_step(i, J)
            ev1.record()
            ev1.synchronize()
            als_total += ev0.elapsed_time(ev1) * 1e-3
            if epoch_interval and rnd % int(epoch_interval) == 0:
                t = time.perf_counter()
                fit = self.compute_exact_fit()
                fit_total += time.perf_counter() - t
                print(f"Exact fit after {rnd} rounds: {fit}")
                rounds.append(rnd)
                fits.append(fit)
                als_times.append(als_total)
                fit_times.append(fit_total)
        regions = (ctypes.c_double * 7)()
        _lib.call("exafac_als_region_times", self._h, regions)
        info1 = self.step_info()
        nz = float(info1.hits_total - info0.hits_total)

        def dstat(q):
            # compute_dstat (common.h:613-675) at one rank: std is 0/0.
            return {"mean": q, "std": None, "min": q, "max": q}

        st = {"num_rounds": int(num_rounds), "als_total_time": als_total, "fit_computation_time": fit_total}
        for name, v in zip(_REGIONS, regions):
            st[name] = dstat(float(v))
        st["avg_nonzeros_iterated"] = dstat(nz)
        st["sum_nonzeros_iterated"] = nz
        st["rounds"] = rounds
        st["fits"] = fits
        st["als_times"] = als_times
        st["fit_computation_times"] = fit_times
        self.stats = st

    def get_statistics_json(self) -> str:
        return json.dumps(self.stats, indent=4)

    # -- extras --------------------------------------------------------------
    def step_info(self) -> _lib.StepInfo:
        self._require()
        out = _lib.StepInfo()
        _lib.call("exafac_als_step_info", self._h, ctypes.byref(out), _stream())
        if out.device_status != 0:
            what = {4: "a bounded device-side wait ran out; re-initialise the optimizer"}
            raise _lib.ExafacError("device", out.device_status,
                                   what.get(out.device_status, "a kernel reported an out-of-range index"))
        return out

    def draw(self, mode: int, J: int, uniforms: torch.Tensor | None = None, perms: torch.Tensor | None = None):
        """Sampler::KRPDrawSamples for `mode`: returns (samples J x N, weights J)."""
        self._require()
        dev = _device()
        N = self.ground_truth.dim
        samples = torch.empty((J, N), dtype=torch.int32, device=dev)
        weights = torch.empty(J, dtype=torch.float64, device=dev)
        _lib.call("exafac_als_draw", self._h, int(mode), int(J), _ptr(uniforms) if uniforms is not None else None,
                  _ptr(perms) if perms is not None else None, _ptr(samples), _ptr(weights), _stream())
        return samples, weights

    def last_dedup(self):
        """(samples_dedup, weights_dedup, design Gram, its pinv) of the last step."""
        self._require()
        info = self.step_info()
        p = [ctypes.c_void_p() for _ in range(4)]
        _lib.call("exafac_als_last_dedup", self._h, *[ctypes.byref(x) for x in p])
        N, R, Ju = self.ground_truth.dim, self.low_rank_tensor.rank, info.unique_samples
        return (_device_array(p[0].value, (Ju, N), torch.int32), _device_array(p[1].value, (Ju,), torch.float64),
                _device_array(p[2].value, (R, R), torch.float64), _device_array(p[3].value, (R, R), torch.float64))

    def sampled_mttkrp(self, mode: int, samples_dedup, design) -> torch.Tensor:
        """csr_based_spmm on the mode's sorted copy (see exafac_als_sampled_mttkrp)."""
        self._require()
        dev = _device()
        sd = torch.as_tensor(np.asarray(samples_dedup).astype(np.int32) if not torch.is_tensor(samples_dedup)
                             else samples_dedup).to(device=dev, dtype=torch.int32).contiguous()
        D = torch.as_tensor(design).to(device=dev, dtype=torch.float64).contiguous()
        out = torch.empty((int(self.ground_truth.tensor_grid.tensor_dims[mode]), self.low_rank_tensor.rank),
                          dtype=torch.float64, device=dev)
        _lib.call("exafac_als_sampled_mttkrp", self._h, int(mode), int(sd.shape[0]), _ptr(sd), _ptr(D), _ptr(out),
                  _stream())
        return out

    def exact_step(self, mode: int):
        self._require()
        _lib.call("exafac_als_exact_step", self._h, int(mode), _stream())


class _DeviceView:
    """__cuda_array_interface__ over a device address owned by the session."""

    def __init__(self, ptr: int, shape, typestr: str):
        self.__cuda_array_interface__ = {"shape": tuple(int(x) for x in shape), "typestr": typestr,
                                         "data": (int(ptr), False), "version": 2, "strides": None}


def _device_array(ptr: int, shape, dtype) -> torch.Tensor:
    """Copies `shape` elements at a device address into a new tensor."""
    n = int(np.prod(shape))
    if n == 0:
        return torch.empty(shape, dtype=dtype, device=_device())
    typestr = {torch.int32: "<i4", torch.float64: "<f8"}[dtype]
    torch.cuda.current_stream().synchronize()
    return torch.as_tensor(_DeviceView(ptr, shape, typestr), device=_device()).clone()


class AccumulatorStationary(ALS_Optimizer):
    """accumulator_stationary.hpp: at one GPU, one sorted copy per mode."""

    def __init__(self, ground_truth, low_rank_tensor, sampler, **kw):
        super().__init__(ground_truth, low_rank_tensor, sampler, **kw)


class TensorStationary(ALS_Optimizer):
    """tensor_stationary.hpp: at one rank its step computes the same as
    AccumulatorStationary (no samples are filtered out, no reduction)."""

    def __init__(self, ground_truth, low_rank_tensor, sampler, **kw):
        super().__init__(ground_truth, low_rank_tensor, sampler, **kw)


class ExactALS(ALS_Optimizer):
    """exact_als.hpp: exact MTTKRP over all nonzeros; J is ignored."""

    def __init__(self, ground_truth, low_rank_tensor, **kw):
        super().__init__(ground_truth, low_rank_tensor, None, **kw)
        self.max_samples = 1

    def execute_ALS_step(self, mode: int, J: int = 0, uniforms=None, perms=None):
        self._require()
        _lib.call("exafac_als_exact_step", self._h, int(mode), _stream())

    def execute_ALS_rounds(self, num_rounds: int, J: int, epoch_interval: int):
        self._require()
        rounds, fits, als_times, fit_times = [0], [0.0], [0.0], [0.0]
        als_total = fit_total = 0.0
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        for rnd in range(1, int(num_rounds) + 1):
            print(f"Starting ALS round {rnd}")
            ev0.record()
            for i in range(self.ground_truth.dim):
                self.execute_ALS_step(i)
            ev1.record()
            ev1.synchronize()
            als_total += ev0.elapsed_time(ev1) * 1e-3
            if epoch_interval and rnd % int(epoch_interval) == 0:
                t = time.perf_counter()
                fit = self.compute_exact_fit()
                fit_total += time.perf_counter() - t
                print(f"Exact fit after {rnd} rounds: {fit}")
                rounds.append(rnd)
                fits.append(fit)
                als_times.append(als_total)
                fit_times.append(fit_total)
        z = {"mean": 0.0, "std": None, "min": 0.0, "max": 0.0}
        self.stats = {"num_rounds": int(num_rounds), "als_total_time": als_total, "fit_computation_time": fit_total,
                      **{r: dict(z) for r in _REGIONS}, "avg_nonzeros_iterated": dict(z),
                      "sum_nonzeros_iterated": 0.0, "rounds": rounds, "fits": fits, "als_times": als_times,
                      "fit_computation_times": fit_times}
