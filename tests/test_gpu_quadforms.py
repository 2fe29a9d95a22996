"""The quadratic forms of the mixed forms' breadth-first STS-CP descents
(x^T A x of each sample against its node, the per-level masses of
PartitionTree::PTSample, partition_tree.hpp:204-380) on the tensor cores
(tcgen05, TF32 hi + lo split) and on the CUDA cores, against FP64."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from rdist_tensor_gb300 import _lib

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return _lib


def packed_stride_f32(R):
    return (R * (R + 1) // 2 + 3) & ~3


def make_nodes(R, count, rng):
    """count positive semidefinite R x R node Grams (sums of outer products
    of rank <= R rows, like the tree nodes), packed upper triangles in FP32."""
    Pf = packed_stride_f32(R)
    iu = np.triu_indices(R)
    full = np.zeros((count, R, R))
    packed = np.zeros((count, Pf), dtype=np.float32)
    for c in range(count):
        U = rng.standard_normal((int(rng.integers(1, 3 * R)), R))
        A = (U.T @ U).astype(np.float32).astype(np.float64)
        full[c] = A
        packed[c, : iu[0].size] = A[iu].astype(np.float32)
    return full, packed


@pytest.mark.parametrize("R", [32, 48, 64, 100, 128])
@pytest.mark.parametrize("layout", ["runs", "scattered"])
def test_quad_forms(lib, R, layout):
    """J = 1000 (not a multiple of the 128-slot tile), 37 nodes; "runs":
    slots sorted by node (the descents' layout), "scattered": every slot
    its own run.  |q - q_exact| <= 1e-5 x^T |A| x on every path (FP32, TF32
    hi + lo, and TF32 hi + lo with the node resident), the FP32 and TF32
    paths agree to the same bound, and the two tensor-core kernels agree bit
    for bit."""
    rng = np.random.default_rng(R)
    J, nodes = 1000, 37
    full, packed = make_nodes(R, nodes, rng)
    X = rng.standard_normal((J, R)).astype(np.float32)
    node = rng.integers(0, nodes, J)
    if layout == "runs":
        node = np.sort(node)
    X64 = X.astype(np.float64)
    exact = np.einsum("jr,jrs,js->j", X64, full[node], X64)
    scale = np.einsum("jr,jrs,js->j", np.abs(X64), np.abs(full[node]), np.abs(X64))
    Xd = torch.as_tensor(X).cuda()
    nd = torch.as_tensor(node.astype(np.int64)).cuda()
    Gd = {tc: torch.as_tensor(packed).cuda() for tc in (0, 1, 2)}
    out = {}
    for tc in (0, 1, 2):
        q = torch.full((J,), float("nan"), dtype=torch.float32, device="cuda")
        lib.call("exafac_quad_forms_f32", R, J, ctypes.c_void_p(Xd.data_ptr()), ctypes.c_void_p(nd.data_ptr()),
                 ctypes.c_void_p(Gd[tc].data_ptr()), ctypes.c_void_p(q.data_ptr()), tc, None)
        torch.cuda.synchronize()
        out[tc] = q.cpu().numpy().astype(np.float64)
        err = np.max(np.abs(out[tc] - exact) / scale)
        print(f"R={R} {layout} tc={tc}: max error / (x^T |A| x) = {err:.2e}")
        assert np.all(np.isfinite(out[tc]))
        assert err < 1e-5
    assert np.max(np.abs(out[1] - out[0]) / scale) < 2e-5
    assert np.array_equal(out[2], out[1])


@pytest.mark.parametrize("R", [64, 100, 128])
@pytest.mark.parametrize("layout", ["runs", "scattered"])
def test_quad_forms_resident_many_tiles(lib, R, layout):
    """The resident-node kernel over more tiles than blocks (J = 60,001: 469
    tiles, four per block, a partial last tile): its contiguous tile ranges,
    single slot buffer refilled during the epilogue, and node changes within
    and between tiles; bit for bit equal to bfs_level_tc_kernel and within
    1e-5 x^T |A| x of FP64."""
    rng = np.random.default_rng(7 * R)
    J, nodes = 60_001, 6
    full, packed = make_nodes(R, nodes, rng)
    X = rng.standard_normal((J, R)).astype(np.float32)
    node = rng.integers(0, nodes, J)
    if layout == "runs":
        node = np.sort(node)
    X64 = X.astype(np.float64)
    exact = np.einsum("jr,jrs,js->j", X64, full[node], X64)
    scale = np.einsum("jr,jrs,js->j", np.abs(X64), np.abs(full[node]), np.abs(X64))
    Xd = torch.as_tensor(X).cuda()
    nd = torch.as_tensor(node.astype(np.int64)).cuda()
    Gd = torch.as_tensor(packed).cuda()
    out = {}
    for tc in (1, 2):
        q = torch.full((J,), float("nan"), dtype=torch.float32, device="cuda")
        lib.call("exafac_quad_forms_f32", R, J, ctypes.c_void_p(Xd.data_ptr()), ctypes.c_void_p(nd.data_ptr()),
                 ctypes.c_void_p(Gd.data_ptr()), ctypes.c_void_p(q.data_ptr()), tc, None)
        torch.cuda.synchronize()
        out[tc] = q.cpu().numpy().astype(np.float64)
    err = np.max(np.abs(out[2] - exact) / scale)
    print(f"R={R} {layout}: resident-node kernel max error / (x^T |A| x) = {err:.2e}")
    assert np.all(np.isfinite(out[2])) and err < 1e-5
    assert np.array_equal(out[2], out[1])


def test_quad_forms_repeat(lib):
    """The tensor-core path repeats bit for bit."""
    R, J = 128, 4096
    rng = np.random.default_rng(1)
    _, packed = make_nodes(R, 5, rng)
    X = torch.as_tensor(rng.standard_normal((J, R)).astype(np.float32)).cuda()
    nd = torch.as_tensor(np.sort(rng.integers(0, 5, J)).astype(np.int64)).cuda()
    Gd = torch.as_tensor(packed).cuda()
    res = []
    for _ in range(2):
        q = torch.empty(J, dtype=torch.float32, device="cuda")
        lib.call("exafac_quad_forms_f32", R, J, ctypes.c_void_p(X.data_ptr()), ctypes.c_void_p(nd.data_ptr()),
                 ctypes.c_void_p(Gd.data_ptr()), ctypes.c_void_p(q.data_ptr()), 1, None)
        res.append(q.cpu().numpy())
    assert np.array_equal(res[0], res[1])


@pytest.mark.parametrize("R", [16, 48, 128])
def test_tree_build_f32(lib, R):
    """The mixed forms' tree build from the FP32 factor copy against the FP64
    build of the same values (PartitionTree::build_tree,
    partition_tree.hpp:117-167): every packed node entry within 2e-6 (tensor
    cores, R >= 32: TF32 hi + lo parts) or 1e-12 (compensated FP32 sums,
    R < 32) of the same entry of the tree of |U|.  1000 rows, F = R rows per
    leaf (partial last leaf)."""
    rng = np.random.default_rng(R + 1)
    n, F = 1000, R
    U32 = rng.standard_normal((n, R)).astype(np.float32)
    U64 = U32.astype(np.float64)
    nodes = lib.load().exafac_tree_node_count(n, F)
    P = R * (R + 1) // 2
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a)).cuda()
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())
    out = {}
    for name, U in (("f32", dev(U32)), ("f64", dev(U64)), ("abs", dev(np.abs(U64)))):
        G = torch.zeros((nodes, P), dtype=torch.float64, device="cuda")
        fn = "exafac_tree_build_f32" if name == "f32" else "exafac_tree_build"
        lib.call(fn, n, F, R, ptr(U), ptr(G), None)
        torch.cuda.synchronize()
        out[name] = G.cpu().numpy()
    err = np.max(np.abs(out["f32"] - out["f64"]) / np.maximum(out["abs"], 1e-300))
    print(f"R={R}: max error / |U|^T|U| = {err:.2e}")
    assert err < (2e-6 if R >= 32 else 1e-12)
