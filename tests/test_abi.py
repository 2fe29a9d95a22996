"""CPU-side checks of the drop-in boundary: the library builds, loads and
exports every entry point include/exafac_gb300.h declares; host-side argument
checks fail with the documented status codes; the 1-rank Grid shim keeps the
reference's error behaviour.  No GPU work is launched."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "exafac_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(exafac_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from rdist_tensor_gb300 import _lib

    return _lib.load()


def test_header_symbols_exported(lib):
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), f"{s} not exported"


def test_ctypes_table_covers_header():
    from rdist_tensor_gb300 import _lib

    assert sorted(_lib.SIGNATURES) == header_symbols()


def test_abi_version(lib):
    assert lib.exafac_abi_version() == 1


def test_workspace_size_and_argument_errors(lib):
    from rdist_tensor_gb300 import _lib

    cfg = _lib.AlsConfig()
    cfg.N, cfg.R, cfg.nnz, cfg.J_max = 3, 25, 2_000_000, 65536
    for k in range(3):
        cfg.dims[k] = 2000
    cfg.sampler, cfg.precision, cfg.preprocessing = 1, 0, 0
    pers, setup = ctypes.c_size_t(), ctypes.c_size_t()
    assert lib.exafac_als_workspace_size(ctypes.byref(cfg), ctypes.byref(pers), ctypes.byref(setup)) == 0
    assert pers.value > 2_000_000 * 3 * 12 and setup.value > 0
    cfg.R = 0
    assert lib.exafac_als_workspace_size(ctypes.byref(cfg), ctypes.byref(pers), ctypes.byref(setup)) == 1
    assert b"R must be" in lib.exafac_last_error()
    cfg.R, cfg.N = 25, 9
    assert lib.exafac_als_workspace_size(ctypes.byref(cfg), ctypes.byref(pers), ctypes.byref(setup)) == 1
    # more than 128 key bits: nine... eight modes of 2^20 each minus one = 140 bits
    cfg.N = 8
    for k in range(8):
        cfg.dims[k] = 1 << 20
    assert lib.exafac_als_workspace_size(ctypes.byref(cfg), ctypes.byref(pers), ctypes.byref(setup)) == 1
    assert b"128 bits" in lib.exafac_last_error()


def test_tree_node_count(lib):
    for n, F in [(1, 4), (2000, 25), (37, 5), (25, 1), (1_000_000, 128)]:
        leaves = (n + F - 1) // F
        assert lib.exafac_tree_node_count(n, F) == 2 * leaves - 1


def test_null_pointer_rejected(lib):
    assert lib.exafac_tree_build(10, 2, 3, None, None, None) == 1


def test_grid_shim_rejects_multi_rank():
    pytest.importorskip("torch")
    from rdist_tensor_gb300.api import Grid

    g = Grid(np.array([1, 1, 1], dtype=np.int32))
    assert g.get_dimension() == 3
    with pytest.raises(RuntimeError, match="number of MPI ranks"):
        Grid(np.array([2, 1, 1], dtype=np.int32))
