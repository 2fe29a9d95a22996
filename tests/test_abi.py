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


def test_adam_and_quad_forms_argument_errors(lib):
    """Host-side checks of the fused Adam step and the quadratic-forms entry
    (they return before any device work)."""
    P = ctypes.c_void_p
    one = (ctypes.c_int64 * 1)(4)
    ptrs = (ctypes.c_void_p * 1)(None)
    adam = lib.exafac_adam_step
    assert adam(9, ptrs, None, ptrs, ptrs, one, 0, 1e-2, 0.9, 0.999, 1e-8, 1, 1, 0.0, None) == 1
    assert b"count" in lib.exafac_last_error()
    assert adam(1, ptrs, None, ptrs, ptrs, one, 0, 1e-2, 0.9, 0.999, 1e-8, 0, 1, 0.0, None) == 1
    assert b"step" in lib.exafac_last_error()
    assert adam(1, ptrs, None, ptrs, ptrs, one, 0, 1e-2, 1.0, 0.999, 1e-8, 1, 1, 0.0, None) == 1
    assert b"betas" in lib.exafac_last_error()
    assert adam(1, ptrs, None, ptrs, ptrs, one, 2, 1e-2, 0.9, 0.999, 1e-8, 1, 1, 0.0, None) == 1
    assert adam(1, ptrs, None, ptrs, ptrs, one, 0, 1e-2, 0.9, 0.999, 1e-8, 1, 1, 0.0, None) == 1  # null tensors
    assert adam(0, None, None, None, None, None, 0, 1e-2, 0.9, 0.999, 1e-8, 1, 1, 0.0, None) == 0  # nothing to do
    quad = lib.exafac_quad_forms_f32
    buf = (ctypes.c_float * 4)()
    p = ctypes.cast(buf, P)
    assert quad(64, 128, None, None, None, None, 1, None) == 1
    assert quad(64, 128, p, p, p, p, 3, None) == 1
    assert b"use_tc" in lib.exafac_last_error()
    assert quad(16, 128, p, p, p, p, 2, None) == 1
    assert b"R >= 32" in lib.exafac_last_error()


def test_fused_adam_refuses_host_tensors():
    torch = pytest.importorskip("torch")
    from rdist_tensor_gb300 import gcp

    with pytest.raises(ValueError, match="CUDA"):
        gcp.FusedAdam([torch.zeros(4)])
    with pytest.raises(ValueError, match="1 to 8"):
        gcp.FusedAdam([])
