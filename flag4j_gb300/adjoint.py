"""Reverse-mode nodes for the product path (no Flag4j counterpart: Flag4j has no
autodiff; the CPU checks restate dA = W.multTranspose(B) and dB = A.T().mult(W)).

  MatMulNode  C = A B (real or Complex128):
              dA = dC B^T (B^H), dB = A^T dC (A^H dC) on the same GEMM kernels with
              transposed operand descriptors; the forward operands stay on the device.
  SpMMNode    C = S X with S in CSR:
              dX = S^T dC through the cached transpose permutation (atomic-free),
              dS = (dC X^T) restricted to pattern(S) through SDDMM.
"""
import ctypes

import numpy as np

from . import _lib
from .arrays import CMatrix, CsrMatrix, Matrix, Shape, ensure_mat_mult_shapes
from .device import check, default_context, gemm_mode


class MatMulNode:
    def __init__(self, A, B, mode=None):
        ensure_mat_mult_shapes(A.shape, B.shape)
        self.A, self.B = A, B
        self.mode = mode
        self.ctx = A._ctx or B._ctx or default_context()
        self.cplx = isinstance(A, CMatrix)
        self.C = A.mult(B, mode=mode)

    def backward(self, dC, need_dA=True, need_dB=True, report=None):
        ctx = self.ctx
        m, k = self.A.shape
        n = self.B.shape[1]
        es = 16 if self.cplx else 8
        dA = ctx.alloc(max(m * k * es, 8)) if need_dA else None
        dB = ctx.alloc(max(k * n * es, 8)) if need_dB else None
        fn = ctx.lib.f4j_zgemm_adjoint if self.cplx else ctx.lib.f4j_dgemm_adjoint
        md = gemm_mode() if self.mode is None else _lib.MODES.get(self.mode, self.mode)
        rep = _lib.f4j_report()
        check(fn(ctx.handle, m, n, k, self.A.device(ctx).handle, self.B.device(ctx).handle, dC.device(ctx).handle,
                 dA.handle if dA else None, dB.handle if dB else None, md, ctypes.byref(rep)))
        if report is not None:
            report.update(rep.as_dict())
        cls = CMatrix if self.cplx else Matrix
        return (cls._from_device(Shape(m, k), dA, ctx) if dA else None,
                cls._from_device(Shape(k, n), dB, ctx) if dB else None)


class SpMMNode:
    def __init__(self, S, X):
        self.S, self.X = S, X
        self.C = S.mult(X)
        self.ctx = self.C._ctx

    def backward(self, dC):
        ctx = self.ctx
        S, X = self.S, self.X
        ncols = X.numCols
        dX = S.multTransposeLeft(dC)
        vals = ctx.alloc(max(8 * S.nnz, 8))
        check(ctx.lib.f4j_sddmm(ctx.handle, S.handle(ctx), dC.device(ctx).handle, X.device(ctx).handle, ncols,
                                vals.handle, None))
        dS = CsrMatrix(S.shape, vals.to_numpy(np.float64, S.nnz), S.rowPointers, S.colIndices, validate=False)
        return dS, dX
