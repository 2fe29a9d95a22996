"""GB300 (sm_103a) sampled-ALS engine for sparse CP decomposition: the hot path
of the CP-ARLS-LEV and STS-CP solvers of vbharadwaj-bk/rdist_tensor, behind
the reference's own class interface (exafac/cpp_ext/py_module.cpp).

The CUDA library (csrc/, C ABI in include/exafac_gb300.h) is built in-tree by
``rdist_tensor_gb300._build.build()``; ``rdist_tensor_gb300.api`` holds the
classes.  There is no CPU fallback."""

__all__ = ["api", "synthetic"]
