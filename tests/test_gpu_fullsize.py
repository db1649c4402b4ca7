"""The configurations at their full sizes, through size-independent properties.

- C3 real 8192^3 (phi in {0, 8, 32}) and complex 4096^3: the split product's
  largest error against the double-double truth on sampled entries
  (f4j_gemm_check, Dot2) is no larger than the plain DMMA product's on the same
  inputs, and both stay FP64-accurate.
- C4 dense adjoint at 4096 x 2048 x 4096: dA = W B^T and dB = A^T W on the split
  path within 2 k u |W||B^T| and 2 k u |A^T||W| of the oracle's restatement of
  W.multTranspose(B) and A.T().mult(W); the Complex128 Hermitian variant at
  2048^3 within the bound per part.
- C2 structure at 2^20 rows: the stable COO sort and COO -> CSR of 16.8 M
  shuffled triplets equal the oracle's bit for bit.
- C5 sparse adjoint at 2^20 rows x 64 columns: S^T dC is bit-identical to
  S.T().mult(dC) and SDDMM stays within 2 * 64 * u * sum|a||b|.
"""
import ctypes

import numpy as np
import pytest

from conftest import U

pytestmark = pytest.mark.gpu


def sampled_errors(ctx, cplx, m, n, k, dA, dB, dC, samples=4096, seed=1234):
    from flag4j_gb300.device import check
    ea, er = ctypes.c_double(), ctypes.c_double()
    check(ctx.lib.f4j_gemm_check(ctx.handle, int(cplx), m, n, k, dA.handle, 0, dB.handle, 0, dC.handle, samples,
                                 seed, ctypes.byref(ea), ctypes.byref(er)))
    return ea.value, er.value


@pytest.mark.parametrize("phi", [0, 8, 32])
def test_split_8192_no_worse_than_dmma(f4j, phi):
    from flag4j_gb300 import _lib, synth
    from flag4j_gb300.device import check
    ctx = f4j.default_context()
    n = 8192
    dA = ctx.from_numpy(synth.scaled(n, n, phi, 10 + phi, "row"))
    dB = ctx.from_numpy(synth.scaled(n, n, phi, 20 + phi, "col"))
    dC = ctx.alloc(8 * n * n)
    errs = {}
    for mode in ("split", "plain"):
        rep = _lib.f4j_report()
        check(ctx.lib.f4j_dgemm(ctx.handle, n, n, n, dA.handle, 0, dB.handle, 0, dC.handle, _lib.MODES[mode],
                                ctypes.byref(rep)))
        errs[mode] = sampled_errors(ctx, False, n, n, n, dA, dB, dC)
        if mode == "split":
            assert rep.mode_used == _lib.MODE_SPLIT and 2 <= rep.slices <= 12
    assert errs["split"][1] <= errs["plain"][1]
    assert errs["split"][1] < 1e-15


def test_complex_split_4096_no_worse_than_dmma(f4j):
    from flag4j_gb300 import _lib, synth
    from flag4j_gb300.device import check
    ctx = f4j.default_context()
    n = 4096
    dA = ctx.from_numpy(synth.scaled(n, n, 8, 3, "row", cplx=True))
    dB = ctx.from_numpy(synth.scaled(n, n, 8, 4, "col", cplx=True))
    dC = ctx.alloc(16 * n * n)
    errs = {}
    for mode in ("split", "plain"):
        check(ctx.lib.f4j_zgemm(ctx.handle, n, n, n, dA.handle, 0, dB.handle, 0, dC.handle, _lib.MODES[mode], None))
        errs[mode] = sampled_errors(ctx, True, n, n, n, dA, dB, dC)
    assert errs["split"][1] <= errs["plain"][1]
    assert errs["split"][1] < 1e-15


def test_dense_adjoint_full_size(f4j, oracle):
    """C4: A 4096 x 2048, B 2048 x 4096, W 4096 x 4096, N(0,1); the split adjoint."""
    from flag4j_gb300 import synth
    m, k, n = 4096, 2048, 4096
    A, B, W = synth.normal(m, k, 5), synth.normal(k, n, 6), synth.normal(m, n, 7)
    node = f4j.MatMulNode(f4j.Matrix(A), f4j.Matrix(B), mode="split")
    dA, dB = node.backward(f4j.Matrix(W))
    refA = oracle.dgemm_abt(W, B, threads=oracle.threads_default())
    refB = oracle.dgemm(np.ascontiguousarray(A.T), W, threads=oracle.threads_default())
    assert np.all(np.abs(dA.toNumpy() - refA) <= 2 * n * U * (np.abs(W) @ np.abs(B.T)))
    assert np.all(np.abs(dB.toNumpy() - refB) <= 2 * m * U * (np.abs(A.T) @ np.abs(W)))


def test_coo_structure_full_config(f4j, oracle):
    """C2: the 2^20-row Poisson(16) matrix as 16.8 M shuffled COO triplets."""
    from flag4j_gb300 import synth
    n = 1 << 20
    rp, ci, v = synth.csr_poisson(n, n, seed=2024)
    r, c, vv = synth.coo_shuffled(rp, ci, v, seed=7)
    er, ec, ev, _ = oracle.coo_sort(r, c, vv)
    coo = f4j.CooMatrix((n, n), vv.copy(), r.copy(), c.copy()).sortIndices()
    assert np.array_equal(coo.rowIndices, er) and np.array_equal(coo.colIndices, ec)
    assert np.array_equal(coo.data, ev)
    S = coo.toCsr()
    assert np.array_equal(S.rowPointers, oracle.coo_to_csr(n, er))
    assert np.array_equal(S.rowPointers, rp) and np.array_equal(S.colIndices, ci) and np.array_equal(S.data, v)


def test_sparse_adjoint_full_config(f4j, oracle):
    """C5: S of 2^20 rows (Poisson(16)), X and dC 2^20 x 64."""
    from flag4j_gb300 import synth
    from flag4j_gb300.device import check
    n, w = 1 << 20, 64
    rp, ci, v = synth.csr_poisson(n, n, seed=2024)
    X, dC = synth.normal(n, w, 8), synth.normal(n, w, 9)
    S = f4j.CsrMatrix((n, n), v, rp, ci)
    dX = S.multTransposeLeft(f4j.Matrix(dC)).toNumpy()
    trp, tci, tv, _ = oracle.csr_transpose(n, n, rp, ci, v)
    assert np.array_equal(dX, oracle.spmm(trp, tci, tv, dC, threads=oracle.threads_default()))
    ctx = f4j.default_context()
    out = ctx.alloc(8 * len(v))
    dCd, Xd = ctx.from_numpy(dC), ctx.from_numpy(X)
    check(ctx.lib.f4j_sddmm(ctx.handle, S.handle(ctx), dCd.handle, Xd.handle, w, out.handle, None))
    got = out.to_numpy(np.float64, len(v))
    ref = oracle.sddmm(rp, ci, dC, X)
    absab = oracle.sddmm(rp, ci, np.abs(dC), np.abs(X))  # sum |a||b| per nonzero
    assert np.all(np.abs(got - ref) <= 2 * w * U * absab)


def test_complex_hermitian_adjoint_full_size(f4j, oracle):
    """C4's complex variant at 2048^3: dA = W B^H and dB = A^H W (W.mult(B.H()),
    A.H().mult(W)) on the split path within the bound per part of the oracle's
    Complex128 restatement."""
    from flag4j_gb300 import synth
    n = 2048
    A = synth.normal(n, n, 11) + 1j * synth.normal(n, n, 12)
    B = synth.normal(n, n, 13) + 1j * synth.normal(n, n, 14)
    W = synth.normal(n, n, 15) + 1j * synth.normal(n, n, 16)
    node = f4j.MatMulNode(f4j.CMatrix(A), f4j.CMatrix(B), mode="split")
    dA, dB = node.backward(f4j.CMatrix(W))
    t = oracle.threads_default()
    for got, L, R in ((dA.toNumpy(), W, np.ascontiguousarray(B.conj().T)),
                      (dB.toNumpy(), np.ascontiguousarray(A.conj().T), W)):
        ref = oracle.zgemm(L, R, threads=t)
        ab_re = np.abs(L.real) @ np.abs(R.real) + np.abs(L.imag) @ np.abs(R.imag)
        ab_im = np.abs(L.real) @ np.abs(R.imag) + np.abs(L.imag) @ np.abs(R.real)
        assert np.all(np.abs(got.real - ref.real) <= 2 * n * U * ab_re)
        assert np.all(np.abs(got.imag - ref.imag) <= 2 * n * U * ab_im)
