"""The HDF5 tensor input of the reference's exafac/sparse_tensor_e.py
(DistSparseTensorE, lines 63-113) on the layout its converters write
(tensor_io/process_frostt_tensor.cpp:67-103: datasets MODE_0 .. MODE_{N-1}
with 1-based or offset coordinates, VALUES, MIN_MODE_SET, MAX_MODE_SET).
h5py is not installed here or on the GPU machine, so the file is a stand-in
module with h5py's File interface (context manager, dataset[:] reads), and
SparseTensor is replaced by a recorder: what is checked is the reader's
arithmetic (offsets, dims, dtypes), not HDF5 itself."""
import sys
import types

import numpy as np
import pytest


class _File:
    def __init__(self, datasets):
        self._d = datasets

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def __getitem__(self, key):
        return self._d[key]


def test_reads_converter_layout(monkeypatch):
    pytest.importorskip("torch")
    import exafac.sparse_tensor_e as ste

    rng = np.random.default_rng(0)
    mins = np.array([1, 1, 5], dtype=np.uint64)
    maxs = np.array([40, 30, 24], dtype=np.uint64)
    nnz = 500
    modes = [rng.integers(mins[i], maxs[i] + 1, nnz).astype(np.uint64) for i in range(3)]
    vals = rng.random(nnz)
    files = {"t.hdf5": {**{f"MODE_{i}": modes[i] for i in range(3)}, "VALUES": vals, "MIN_MODE_SET": mins,
                        "MAX_MODE_SET": maxs}}
    fake = types.ModuleType("h5py")
    fake.File = lambda name, mode="r": _File(files[name])
    monkeypatch.setitem(sys.modules, "h5py", fake)
    seen = {}

    class Recorder:
        def __init__(self, grid, idx, v, prep):
            seen.update(dims=np.asarray(grid.tensor_dims), idx=idx, vals=v, prep=prep)

    monkeypatch.setattr(ste, "SparseTensor", Recorder)
    t = ste.DistSparseTensorE("t.hdf5", None, preprocessing="log_count")
    assert t.dim == 3 and t.nnz == nnz
    assert np.array_equal(seen["dims"], [40, 30, 20])
    assert seen["idx"].dtype == np.uint32
    for i in range(3):
        assert np.array_equal(seen["idx"][:, i], (modes[i] - mins[i]).astype(np.uint32))
    assert np.array_equal(seen["vals"], vals) and seen["prep"] == "log_count"


def test_without_h5py_raises(monkeypatch):
    pytest.importorskip("torch")
    import exafac.sparse_tensor_e as ste

    monkeypatch.setitem(sys.modules, "h5py", None)
    with pytest.raises(ImportError, match="h5py"):
        ste.DistSparseTensorE("missing.hdf5")
