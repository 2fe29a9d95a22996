"""Factor output in the reference's FACTOR_MODE_i layout
(exafac/low_rank_tensor.py:186-192, read back as analysis/analysis.py:38-47
does): round trips through the numpy archive and, when h5py is installed,
HDF5.  No GPU."""
import numpy as np
import pytest

from rdist_tensor_gb300 import checkpoint


def factors():
    rng = np.random.default_rng(0)
    return [rng.standard_normal((d, 5)) for d in (7, 6, 4)], rng.random(5)


def test_npz_round_trip(tmp_path):
    mats, sigma = factors()
    path = checkpoint.write_factors(str(tmp_path / "run"), mats, sigma, fmt="npz")
    assert path.endswith(".npz")
    d = checkpoint.load_factors_from_file(path)
    assert sorted(d) == ["FACTOR_MODE_0", "FACTOR_MODE_1", "FACTOR_MODE_2", "SIGMA"]
    got, s = checkpoint.read_factors(path)
    for a, b in zip(got, mats):
        assert np.array_equal(a, b) and a.dtype == np.float64
    assert np.array_equal(s, sigma)
    # the name without the suffix finds the archive too
    got2, _ = checkpoint.read_factors(str(tmp_path / "run"))
    assert np.array_equal(got2[1], mats[1])


def test_npz_without_sigma(tmp_path):
    mats, _ = factors()
    path = checkpoint.write_factors(str(tmp_path / "f.npz"), mats)
    got, s = checkpoint.read_factors(path)
    assert s is None and len(got) == 3


def test_hdf5_round_trip(tmp_path):
    h5py = pytest.importorskip("h5py")
    mats, sigma = factors()
    path = checkpoint.write_factors(str(tmp_path / "f.hdf5"), mats, sigma, fmt="hdf5")
    with h5py.File(path, "r") as f:
        assert sorted(f.keys()) == ["FACTOR_MODE_0", "FACTOR_MODE_1", "FACTOR_MODE_2", "SIGMA"]
    got, s = checkpoint.read_factors(path)
    assert all(np.array_equal(a, b) for a, b in zip(got, mats)) and np.array_equal(s, sigma)


def test_hdf5_unavailable_is_reported(tmp_path, monkeypatch):
    monkeypatch.setattr(checkpoint, "_h5py", lambda: None)
    mats, _ = factors()
    with pytest.raises(RuntimeError, match="h5py"):
        checkpoint.write_factors(str(tmp_path / "f.hdf5"), mats, fmt="hdf5")
    # the default falls back to the archive
    assert checkpoint.write_factors(str(tmp_path / "g"), mats).endswith(".npz")
