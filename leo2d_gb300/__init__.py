"""GB300 implementation of LEO2D's Chebyshev kernel-polynomial-method path.

The product is libleo2d_gb300.so (C ABI in include/leo2d_gpu.h, CUDA kernels
for sm_103a in csrc/, C++ host code in host/) and the `leo2d` driver built
beside it. This package only builds and binds them.
"""
from ._abi import (CSR_KEEP_ZEROS, CSR_WITH_DX, FP32, FP64, MODEL_REF, MODEL_SIMPLE, VEC_GAUSSIAN,
                   VEC_HOST, VEC_PHASE, Geom, KpmCfg, make_geom)
from .api import Batch, Context, Csr, Leo2dError, Mlp, k_grid, k_path, kpm_cfg, run_input, vacancy_rows

__all__ = ["Batch", "Context", "Csr", "Mlp", "Leo2dError", "kpm_cfg", "run_input", "vacancy_rows", "k_grid", "k_path", "Geom", "KpmCfg", "make_geom", "MODEL_REF",
           "MODEL_SIMPLE", "VEC_PHASE", "VEC_HOST", "VEC_GAUSSIAN", "FP32", "FP64", "CSR_KEEP_ZEROS",
           "CSR_WITH_DX"]
