"""The allocation-free pseudo-inverse entry point (exafac_pinv_square_static).

It exists for callers that cannot allocate device memory, or size a workspace
up front: its scratch is a static device array shared by every call on the
device.  This test calls it through the C ABI twice in a row and checks each
result against exafac_pinv_square (which takes a caller-allocated
workspace), on a well-conditioned matrix (Cholesky path) and a rank-deficient
one (Jacobi path, which is the part that uses the scratch).  The file sorts
last so that a run stopping at the first failure has run every other test."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_static_scratch_pinv_matches_workspace_pinv():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from rdist_tensor_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(21)
    for R, rank in ((25, 25), (25, 9), (64, 40), (128, 128)):
        B = rng.standard_normal((R + 3, rank))
        if rank < R:
            A = B[:R] @ B[:R].T  # rank-deficient R x R
        else:
            A = B.T @ B
        Ad = torch.as_tensor(A, device="cuda")
        ref = torch.zeros((R, R), dtype=torch.float64, device="cuda")
        nbytes = lib.exafac_dense_workspace_bytes(R)
        ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        _lib.call("exafac_pinv_square", R, ctypes.c_void_p(Ad.data_ptr()), ctypes.c_void_p(ref.data_ptr()),
                  ctypes.c_double(1e-11), ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(nbytes), None)
        for _ in range(2):
            out = torch.full((R, R), float("nan"), dtype=torch.float64, device="cuda")
            _lib.call("exafac_pinv_square_static", R, ctypes.c_void_p(Ad.data_ptr()),
                      ctypes.c_void_p(out.data_ptr()), ctypes.c_double(1e-11), None)
            torch.cuda.synchronize()
            assert rel_err(out.cpu().numpy(), ref.cpu().numpy()) < 1e-12


def test_static_scratch_rejects_large_rank():
    from rdist_tensor_gb300 import _lib

    lib = _lib.load()
    rc = lib.exafac_pinv_square_static(129, None, None, ctypes.c_double(1e-11), None)
    assert rc == 1
    assert b"128" in lib.exafac_last_error()
