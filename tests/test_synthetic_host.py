"""The seeded synthetic generators on a CPU torch device (the same code the
GPU workloads run on CUDA): the Zipf support's distinct in-range
coordinates, and the count tensor's values against its planted model."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_zipf_tensor_device_on_cpu():
    from rdist_tensor_gb300 import synthetic

    dims = (3000, 2000, 50)
    d, idx, vals = synthetic.zipf_tensor_device(dims, 20_000, alpha=1.2, seed=4, device="cpu")
    assert list(d) == list(dims) and idx.shape == (20_000, 3) and idx.dtype == torch.int32
    for k in range(3):
        assert int(idx[:, k].min()) >= 0 and int(idx[:, k].max()) < dims[k]
    key = (idx[:, 0].long() * dims[1] + idx[:, 1].long()) * dims[2] + idx[:, 2].long()
    assert torch.unique(key).numel() == idx.shape[0]
    assert bool((vals > 0).all())  # log-normal
    # Zipf: row 0 is the most frequent coordinate of every mode
    for k in range(3):
        counts = torch.bincount(idx[:, k].long(), minlength=dims[k])
        assert int(counts.argmax()) == 0
    # seeded: the same call repeats
    _, idx2, vals2 = synthetic.zipf_tensor_device(dims, 20_000, alpha=1.2, seed=4, device="cpu")
    assert torch.equal(idx, idx2) and torch.equal(vals, vals2)


def test_poisson_counts_device_on_cpu():
    from rdist_tensor_gb300 import synthetic

    dims = (4000, 4000, 100)
    d, idx, vals, A = synthetic.poisson_counts_device(dims, 50_000, rank=16, seed=2, device="cpu")
    assert idx.shape == (50_000, 3)
    assert bool((vals >= 1).all()) and bool((vals == torch.round(vals)).all())
    rows = idx.long()
    lam = (A[0][rows[:, 0]] * A[1][rows[:, 1]] * A[2][rows[:, 2]]).sum(dim=1).double()
    expect = float((lam + torch.exp(-lam)).mean())  # E[max(Poisson(lam), 1)]
    assert abs(float(vals.double().mean()) - expect) < 0.03 * expect
    a = torch.cat([x.reshape(-1) for x in A]).double()  # Gamma(0.5, 1): mean 0.5, variance 0.5
    assert abs(float(a.mean()) - 0.5) < 0.01 and abs(float(a.var()) - 0.5) < 0.04
    assert np.isfinite(float(vals.sum()))
