"""Failure detection on the host (no GPU): corrupt COO input, an oversize
sample count, shapes the engine does not support, and the wait-limit hook's
argument checks.  Each fails with an exception or a status code before any
device work is queued (the reference exits or throws in the same cases, or
does not check them: accumulator_stationary.hpp:107-110, grid.hpp:62-65)."""
import ctypes

import numpy as np
import pytest


@pytest.fixture(scope="module")
def lib():
    from rdist_tensor_gb300 import _lib

    return _lib.load()


def config(N=3, R=8, nnz=1000, J=4096, dims=(100, 90, 80)):
    from rdist_tensor_gb300 import _lib

    cfg = _lib.AlsConfig()
    cfg.N, cfg.R, cfg.nnz, cfg.J_max = N, R, nnz, J
    for k, d in enumerate(dims):
        cfg.dims[k] = d
    cfg.sampler, cfg.precision, cfg.preprocessing = 1, 0, 0
    return cfg


def sizes(lib, cfg):
    pers, setup = ctypes.c_size_t(), ctypes.c_size_t()
    return lib.exafac_als_workspace_size(ctypes.byref(cfg), ctypes.byref(pers), ctypes.byref(setup))


def test_oversize_sample_count_fails_on_host(lib):
    assert sizes(lib, config(J=(1 << 31) - 1)) == 0
    assert sizes(lib, config(J=1 << 31)) == 1
    assert b"J_max" in lib.exafac_last_error()


def test_keys_beyond_128_bits_rejected(lib):
    dims = (0xffffffff,) * 6
    assert sizes(lib, config(N=6, dims=dims)) == 1  # 5 x 32 = 160 bits off any mode
    assert b"128 bits" in lib.exafac_last_error()
    assert sizes(lib, config(N=5, dims=(0xffffffff,) * 5)) == 0  # exactly 128


@pytest.mark.parametrize("field,value", [("R", 129), ("R", 0), ("nnz", 0), ("N", 1), ("precision", 3),
                                         ("sampler", 2), ("preprocessing", 3)])
def test_unsupported_configs_rejected(lib, field, value):
    cfg = config()
    setattr(cfg, field, value)
    assert sizes(lib, cfg) == 1


def test_mode_size_bounds(lib):
    assert sizes(lib, config(dims=(100, 0, 80))) == 1
    assert sizes(lib, config(dims=(100, 1 << 32, 80))) == 1


def test_wait_limit_hook_arguments(lib):
    """The session object exists on the host alone: exafac_als_create carves
    the workspace without touching it, so a fake aligned address serves."""
    cfg = config()
    pers, setup = ctypes.c_size_t(), ctypes.c_size_t()
    assert lib.exafac_als_workspace_size(ctypes.byref(cfg), ctypes.byref(pers), ctypes.byref(setup)) == 0
    h = ctypes.c_void_p()
    assert lib.exafac_als_create(ctypes.byref(cfg), ctypes.c_void_p(1 << 20), ctypes.c_size_t(pers.value),
                                 ctypes.byref(h)) == 0
    try:
        assert lib.exafac_als_set_wait_limit(h, 256, 0) == 0
        assert lib.exafac_als_set_wait_limit(h, 0, -1) == 0
        assert lib.exafac_als_set_wait_limit(h, 0, -2) == 1
        assert lib.exafac_als_set_wait_limit(None, 0, -1) == 1
    finally:
        lib.exafac_als_destroy(h)
    # misaligned or too small workspaces
    assert lib.exafac_als_create(ctypes.byref(cfg), ctypes.c_void_p((1 << 20) + 8), ctypes.c_size_t(pers.value),
                                 ctypes.byref(h)) == 1
    assert lib.exafac_als_create(ctypes.byref(cfg), ctypes.c_void_p(1 << 20), ctypes.c_size_t(pers.value // 2),
                                 ctypes.byref(h)) == 6


def grid3(dims):
    from rdist_tensor_gb300.api import Grid, TensorGrid

    return TensorGrid(np.asarray(dims, dtype=np.int64), Grid(np.ones(3, dtype=np.int32)))


@pytest.mark.parametrize("case", ["too_large", "negative", "shape", "values", "preprocessing", "mode_size"])
def test_corrupt_coo_rejected_before_the_device(case):
    """SparseTensor validates on the host; these raise on a machine without a
    GPU, before the engine is asked for a device."""
    from rdist_tensor_gb300.api import SparseTensor

    dims = (10, 9, 8)
    idx = np.array([[0, 0, 0], [9, 8, 7], [3, 4, 5]], dtype=np.int64)
    vals = np.ones(3)
    pre = "none"
    if case == "too_large":
        idx[1, 2] = 8
    elif case == "negative":
        idx[2, 0] = -1
    elif case == "shape":
        idx = idx[:, :2]
    elif case == "values":
        vals = np.ones(4)
    elif case == "preprocessing":
        pre = "sqrt"
    elif case == "mode_size":
        dims = (10, 0, 8)
    with pytest.raises(ValueError):
        SparseTensor(grid3(dims), idx, vals, pre)


def test_grid_other_than_one_rank_raises():
    from rdist_tensor_gb300.api import Grid

    with pytest.raises(RuntimeError, match="MPI ranks"):
        Grid(np.array([2, 1, 1], dtype=np.int32))
