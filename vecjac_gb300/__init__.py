"""vecjac_gb300: GB300-native one-sided Jacobi SVD and batched 2x2 Hermitian EVD.

The compute path is libvecjac_gb300.so (hand-written sm_103a CUDA kernels behind a C ABI
whose entry points are VecJac's: dbjac2_/zbjac2_/sbjac2_/cbjac2_, dvjsvd_/zvjsvd_/
svjsvd_/cvjsvd_, pjs). This package only loads it and mirrors the reference's calling
conventions for Python callers (numpy host arrays, or CUDA tensors for the device forms).
There is no CPU fallback: when the library or a GPU is missing, calls raise.
"""
from .api import (  # noqa: F401
    VJ_ERR_ARG, VJ_ERR_CUDA, VJ_ERR_NO_GPU, VJ_ERR_NOMEM, bjac2, bjac2_dev, last_mixed_phases, last_trace, lib, lib_path,
    merge, merge_dev, pjs, pjs_dev, split, split_dev,
    vjsvd, vjsvd_dev, vjsvd_mixed_dev,
)
