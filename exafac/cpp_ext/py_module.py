"""Same module path and class names as the reference's pybind module
(exafac/cpp_ext/py_module.cpp:37-77); the classes run on the GPU engine."""
from rdist_tensor_gb300.api import (  # noqa: F401
    ALS_Optimizer,
    AccumulatorStationary,
    CP_ARLS_LEV,
    DistMat1D,
    ExactALS,
    Grid,
    LowRankTensor,
    STS_CP,
    Sampler,
    SparseTensor,
    TensorGrid,
    TensorStationary,
)
