"""Tensor loaders of the reference (exafac/sparse_tensor_e.py) on one GPU.

``DistSparseTensorE`` reads the HDF5 layout the reference's converters write
(datasets ``MODE_i``, ``VALUES``, ``MIN_MODE_SET``, ``MAX_MODE_SET``;
tensor_io/process_frostt_tensor.cpp); it needs h5py.  ``RandomSparseTensor``
builds the reference's synthetic block tensor.  ``SyntheticSparseTensor`` adds
the seeded workloads used by the benchmarks."""
from __future__ import annotations

import numpy as np

from rdist_tensor_gb300.api import Grid, SparseTensor, TensorGrid


def round_to_nearest(n, m):
    return (n + m - 1) // m * m


def prime_factorization(n):
    factors, i = [], 2
    while i * i <= n:
        if n % i:
            i += 1
        else:
            n //= i
            factors.append(i)
    if n > 1:
        factors.append(n)
    return sorted(factors)


def get_best_mpi_dim(nprocs, global_dims):
    """Processor grid dimensions (sparse_tensor_e.py:31-61); one process here,
    so every dimension is 1."""
    dims = np.ones(len(global_dims), dtype=np.int32)
    if nprocs != 1:
        raise RuntimeError("this engine runs one process per GPU; the processor grid is 1 x ... x 1")
    return dims


class DistSparseTensorE:
    def __init__(self, filename, grid=None, preprocessing="None"):
        try:
            import h5py
        except ImportError as e:  # pragma: no cover - depends on the environment
            raise ImportError("DistSparseTensorE needs h5py to read the HDF5 tensor files") from e
        with h5py.File(filename, "r") as f:
            self.max_idxs = f["MAX_MODE_SET"][:]
            self.min_idxs = f["MIN_MODE_SET"][:]
            self.dim = len(self.max_idxs)
            self.tensor_dims = np.array(self.max_idxs - self.min_idxs + 1, dtype=np.int64)
            self.nnz = len(f["MODE_0"])
            idx = np.zeros((self.nnz, self.dim), dtype=np.uint32)
            for i in range(self.dim):
                idx[:, i] = f[f"MODE_{i}"][:] - self.min_idxs[i]
            vals = f["VALUES"][:]
        self.grid = grid if grid is not None else Grid(get_best_mpi_dim(1, self.tensor_dims))
        self.tensor_grid = TensorGrid(self.tensor_dims, self.grid)
        if self.grid.get_dimension() != self.dim:
            raise ValueError("Grid dimension must match tensor dimension")
        self.tensor_idxs = idx
        self.values = vals
        self.sparse_tensor = SparseTensor(self.tensor_grid, idx, vals, preprocessing)


class RandomSparseTensor:
    def __init__(self, grid, I, N, Q, seed=0):
        self.max_idxs = np.array([I - 1] * N, dtype=np.int64)
        self.min_idxs = np.zeros(N, dtype=np.int64)
        self.dim = N
        self.tensor_dims = np.array(self.max_idxs - self.min_idxs + 1, dtype=np.int64)
        self.grid = grid if grid is not None else Grid(get_best_mpi_dim(1, self.tensor_dims))
        self.tensor_grid = TensorGrid(self.tensor_dims, self.grid)
        if self.grid.get_dimension() != self.dim:
            raise ValueError("Grid dimension must match tensor dimension")
        self.sparse_tensor = SparseTensor(self.tensor_grid, I, N, Q, seed=seed)
        self.nnz = self.sparse_tensor.nnz


class SyntheticSparseTensor:
    """Seeded synthetic workloads (rdist_tensor_gb300.synthetic):
    ``planted`` 2000^3 / 2e6 nonzeros, ``zipf4`` 5e6 x 5e6 x 2e4 x 1e3 / 1e8,
    ``zipf4_small`` a tenth of it, ``zipf5`` 1e6 x 1e6 x 1e5 x 1e3 x 100 / 2e8."""

    def __init__(self, name, grid=None, seed=0):
        from rdist_tensor_gb300 import synthetic

        if name == "planted":
            dims, idx, vals = synthetic.planted_uniform(seed=seed)
        elif name in ("zipf4", "zipf4_small", "zipf5"):
            spec = {"zipf4": ((5_000_000, 5_000_000, 20_000, 1_000), 100_000_000, 1.2, "lognormal"),
                    "zipf4_small": ((500_000, 500_000, 20_000, 1_000), 10_000_000, 1.2, "lognormal"),
                    "zipf5": ((1_000_000, 1_000_000, 100_000, 1_000, 100), 200_000_000, 1.1, "normal")}[name]
            dims, idx, vals = synthetic.zipf_tensor_device(spec[0], spec[1], alpha=spec[2], values=spec[3], seed=seed)
        else:
            raise ValueError(f"unknown synthetic tensor {name}")
        self.tensor_dims = np.asarray(dims, dtype=np.int64)
        self.dim = len(dims)
        self.grid = grid if grid is not None else Grid(np.ones(self.dim, dtype=np.int32))
        self.tensor_grid = TensorGrid(self.tensor_dims, self.grid)
        self.sparse_tensor = SparseTensor(self.tensor_grid, idx, vals, "none")
        self.nnz = self.sparse_tensor.nnz
