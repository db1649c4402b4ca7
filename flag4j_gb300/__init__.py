"""flag4j_gb300 -- GB300 (sm_103a) engine for Flag4j's product path.

Dense real / Complex128 GEMM (plain FP64 DMMA, FP64-accurate FP8-slice split
GEMM on tcgen05, and Flag4j's own bit-identical order), CSR SpMV / SpMM
(bit-identical to the reference loops), CSR structure kernels and reverse-mode
adjoints, all behind the C ABI of libflag4j_cuda.so (include/flag4j_cuda.h).
This package mirrors the reference types that reach those products.
"""
from ._lib import Flag4jDeviceException, load as load_library  # noqa: F401
from .adjoint import MatMulNode, SpMMNode  # noqa: F401
from .arrays import CMatrix, CooMatrix, CsrCMatrix, CsrMatrix, CVector, Matrix, Shape, Vector  # noqa: F401
from .device import (Context, IllegalArgumentException, LinearAlgebraException, default_context,  # noqa: F401
                     gemm_mode, pinned_empty, set_gemm_mode)

__version__ = "0.1.0"
