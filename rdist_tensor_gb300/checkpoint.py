"""Factor output and resume in the reference's layout.

LowRankTensor.write_to_file (exafac/low_rank_tensor.py:186-192) writes one
dataset per mode, FACTOR_MODE_i (rows x R, float64), to an HDF5 file; the
analysis scripts read every key containing FACTOR_MODE back
(analysis/analysis.py:38-47).  Here the same datasets go to HDF5 when h5py is
importable, otherwise to a numpy .npz archive with the same keys.  SIGMA (the
column norms, R) is written beside them so that a run can resume; readers that
look only for FACTOR_MODE keys skip it."""
from __future__ import annotations

import os

import numpy as np


def _h5py():
    try:
        import h5py  # noqa: F401

        return h5py
    except ImportError:
        return None


def write_factors(filename: str, factors, sigma=None, fmt: str | None = None) -> str:
    """Writes FACTOR_MODE_i (and SIGMA) to `filename`.  fmt: "hdf5", "npz" or
    None (HDF5 when h5py is importable and the name does not end in .npz).
    Returns the path written (".npz" appended for the numpy format when
    missing)."""
    mats = [np.ascontiguousarray(np.asarray(U, dtype=np.float64)) for U in factors]
    if fmt is None:
        fmt = "npz" if (filename.endswith(".npz") or _h5py() is None) else "hdf5"
    if fmt == "hdf5":
        h5py = _h5py()
        if h5py is None:
            raise RuntimeError("writing HDF5 needs h5py, which is not installed; use fmt='npz'")
        with h5py.File(filename, "w") as f:
            for i, U in enumerate(mats):
                f.create_dataset(f"FACTOR_MODE_{i}", data=U)
            if sigma is not None:
                f.create_dataset("SIGMA", data=np.asarray(sigma, dtype=np.float64))
        return filename
    if fmt != "npz":
        raise ValueError(f"unknown factor file format {fmt}")
    path = filename if filename.endswith(".npz") else filename + ".npz"
    arrays = {f"FACTOR_MODE_{i}": U for i, U in enumerate(mats)}
    if sigma is not None:
        arrays["SIGMA"] = np.asarray(sigma, dtype=np.float64)
    np.savez(path, **arrays)
    return path


def load_factors_from_file(filename: str) -> dict:
    """Every FACTOR_MODE key of the file (analysis/analysis.py:38-47), plus
    SIGMA when present."""
    out = {}
    if filename.endswith(".npz") or not os.path.exists(filename) and os.path.exists(filename + ".npz"):
        path = filename if filename.endswith(".npz") else filename + ".npz"
        with np.load(path) as f:
            for key in f.files:
                if "FACTOR_MODE" in key or key == "SIGMA":
                    out[key] = f[key]
        return out
    h5py = _h5py()
    if h5py is None:
        raise RuntimeError("reading HDF5 needs h5py, which is not installed")
    with h5py.File(filename, "r") as f:
        for key in f.keys():
            if "FACTOR_MODE" in key or key == "SIGMA":
                out[key] = f[key][:]
    return out


def read_factors(filename: str):
    """(list of factor matrices in mode order, sigma or None)."""
    d = load_factors_from_file(filename)
    n = len([k for k in d if k.startswith("FACTOR_MODE_")])
    mats = [d[f"FACTOR_MODE_{i}"] for i in range(n)]
    return mats, d.get("SIGMA")
