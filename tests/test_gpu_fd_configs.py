"""Central finite differences (h = 1e-6) of the adjoints at the configured sizes.

- Dense, real: A 4096 x 2048, B 2048 x 4096, W 4096 x 4096, all N(0, 1),
  L = sum(W o (A B)); dA = W B^T and dB = A^T W from the plain (DMMA) and the
  split adjoint, checked on 64 seeded entries of A and 64 of B.
- Dense, Complex128 (Hermitian adjoint) at 2048^3: L = Re sum(conj(W) o (A B));
  dA = W B^H, dB = A^H W, checked through the real and imaginary perturbation
  of 64 seeded entries of A and 64 of B.
- Sparse: S with 2^20 rows, Poisson(16) row lengths, X and W 2^20 x 64,
  L = sum(W o (S X)); dX = S^T W (cached transpose permutation) and
  dS = (W X^T) on pattern(S) (SDDMM), checked on 64 seeded nonzeros of S and
  64 entries of X.

The reference products the formulas restate are Matrix.multTranspose
(src/main/java/org/flag4j/arrays/dense/Matrix.java:655-663) and
CsrMatrix.T() (src/main/java/org/flag4j/arrays/sparse/CsrMatrix.java:1431-1433).

Cheap differences: perturbing A[i, j] changes only row i of C, B[j, l] only
column l (computed as the row B[:, l]^T A^T), a nonzero of S only its row, and
X[i, j] only the rows of S with a nonzero in column i.  So L(+h) - L(-h) is
the W-weighted sum of the difference of those entries alone, formed before
the (exact, math.fsum) summation.

Noise floor: the FD quotient carries the forward product's rounding error
divided by 2h.  The forward used for the quotient is the FP64-accurate split
product (its rows differ from the exact ones by about one final rounding of
C), whose FD noise is about 1e-9 of the gradient's scale here; a plain DMMA
forward at k = 2048 carries about 5e-14 per entry of C, i.e. ~3.5e-8 of the
gradient's scale, too close to the 1e-7 bar to be a stable check.  The bar is
|fd - g| <= 1e-7 * max(|g|, rms(g)), rms over the sampled gradient entries:
relative to the entry itself, and to the gradient's scale for the rare entries
near zero whose own size says nothing about the quotient's cancellation.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H = 1e-6
TOL = 1e-7


def _bar(g_samples):
    g = np.asarray(g_samples)
    rms = math.sqrt(float(np.mean(np.abs(g) ** 2)))
    return lambda gv: TOL * max(abs(gv), rms)


def _row_product(ctx, lib, cplx, row, dB, k, n, opB):
    """row (1 x k) times op(B) (k x n) on the split path; returns the 1 x n result."""
    from flag4j_gb300 import _lib
    from flag4j_gb300.device import check
    es = 16 if cplx else 8
    dr = ctx.from_numpy(np.ascontiguousarray(row))
    out = ctx.alloc(es * n)
    fn = lib.f4j_zgemm if cplx else lib.f4j_dgemm
    check(fn(ctx.handle, 1, n, k, dr.handle, 0, dB.handle, opB, out.handle, _lib.MODE_SPLIT, None))
    return out.to_numpy(np.complex128 if cplx else np.float64, n)


def _check_dense(f4j, A, B, W, cplx, mode):
    from flag4j_gb300 import synth
    ctx = f4j.default_context()
    lib = ctx.lib
    m, k = A.shape
    n = B.shape[1]
    cls = f4j.CMatrix if cplx else f4j.Matrix
    node = f4j.MatMulNode(cls(A), cls(B), mode=mode)
    dA, dB = node.backward(cls(W))
    dA, dB = dA.toNumpy(), dB.toNumpy()
    dBdev, dAdev = node.B.device(ctx), node.A.device(ctx)
    rng = synth.rng(4242 + (1 if cplx else 0))
    ia, ja = rng.integers(0, m, 64), rng.integers(0, k, 64)
    ib, lb = rng.integers(0, k, 64), rng.integers(0, n, 64)
    Wc = np.conj(W) if cplx else W

    def dL(Cp, Cm, w):
        d = w * (Cp - Cm)
        return math.fsum(np.real(d).ravel()) / (2 * H)

    units = (1.0, 1j) if cplx else (1.0,)
    worst = 0.0
    gA = [dA[i, j] for i, j in zip(ia, ja)]
    gB = [dB[j, l] for j, l in zip(ib, lb)]
    barA, barB = _bar(gA), _bar(gB)
    for (i, j), g in zip(zip(ia, ja), gA):
        fd = 0.0
        for u in units:  # d/dRe + i d/dIm
            rp, rm = A[i].copy(), A[i].copy()
            rp[j] += u * H
            rm[j] -= u * H
            Cp = _row_product(ctx, lib, cplx, rp, dBdev, k, n, 0)
            Cm = _row_product(ctx, lib, cplx, rm, dBdev, k, n, 0)
            fd += u * dL(Cp, Cm, Wc[i])
        err = abs(fd - g)
        worst = max(worst, err / barA(g) * TOL)
        assert err <= barA(g), "%s dA[%d, %d]: fd %r vs %r" % (mode, i, j, fd, g)
    for (j, l), g in zip(zip(ib, lb), gB):
        fd = 0.0
        for u in units:
            # column l of C as a row: B[:, l]^T A^T (A read transposed in place)
            cp, cm = B[:, l].copy(), B[:, l].copy()
            cp[j] += u * H
            cm[j] -= u * H
            Cp = _row_product(ctx, lib, cplx, cp, dAdev, k, m, 1)
            Cm = _row_product(ctx, lib, cplx, cm, dAdev, k, m, 1)
            fd += u * dL(Cp, Cm, Wc[:, l])
        err = abs(fd - g)
        worst = max(worst, err / barB(g) * TOL)
        assert err <= barB(g), "%s dB[%d, %d]: fd %r vs %r" % (mode, j, l, fd, g)
    return worst


@pytest.mark.parametrize("mode", ["plain", "split"])
def test_dense_adjoint_fd_4096x2048x4096(f4j, mode):
    from flag4j_gb300 import synth
    m, k, n = 4096, 2048, 4096
    A, B, W = synth.normal(m, k, 31), synth.normal(k, n, 32), synth.normal(m, n, 33)
    worst = _check_dense(f4j, A, B, W, False, mode)
    print("real %s: worst |fd - g| / max(|g|, rms) = %.3g" % (mode, worst))


@pytest.mark.parametrize("mode", ["plain", "split"])
def test_complex_hermitian_adjoint_fd_2048cube(f4j, mode):
    from flag4j_gb300 import synth
    n = 2048
    A = synth.normal(n, n, 41) + 1j * synth.normal(n, n, 42)
    B = synth.normal(n, n, 43) + 1j * synth.normal(n, n, 44)
    W = synth.normal(n, n, 45) + 1j * synth.normal(n, n, 46)
    worst = _check_dense(f4j, A, B, W, True, mode)
    print("complex %s: worst |fd - g| / max(|g|, rms) = %.3g" % (mode, worst))


def test_sparse_adjoint_fd_2pow20_rows_64_cols(f4j):
    from flag4j_gb300 import synth
    n, w = 1 << 20, 64
    rp, ci, v = synth.csr_poisson(n, n, seed=2025)
    X, W = synth.normal(n, w, 51), synth.normal(n, w, 52)
    S = f4j.CsrMatrix((n, n), v, rp, ci)
    Xm = f4j.Matrix(X)
    node = f4j.SpMMNode(S, Xm)
    dS, dX = node.backward(f4j.Matrix(W))
    dS, dX = dS.data, dX.toNumpy()
    ctx = f4j.default_context()
    Xdev = Xm.device(ctx)
    rng = synth.rng(777)
    rows_of = np.repeat(np.arange(n, dtype=np.int64), np.diff(rp))

    def sub_product(rows, vals_override=None):
        """CSR of the given full rows of S (values optionally replaced) times the device X."""
        lens = (rp[rows + 1] - rp[rows]).astype(np.int64)
        srp = np.zeros(len(rows) + 1, np.int64)
        np.cumsum(lens, out=srp[1:])
        idx = np.concatenate([np.arange(rp[r], rp[r + 1]) for r in rows])
        vals = v[idx] if vals_override is None else vals_override
        sub = f4j.CsrMatrix((len(rows), n), vals, srp.astype(np.int32), ci[idx])
        return sub.mult(Xm).toNumpy(), idx

    qs = rng.integers(0, len(v), 64)
    gS = [dS[q] for q in qs]
    barS = _bar(gS)
    for q, g in zip(qs, gS):
        r = np.array([rows_of[q]])
        base = v[rp[r[0]]:rp[r[0] + 1]].copy()
        vp, vm = base.copy(), base.copy()
        vp[q - rp[r[0]]] += H
        vm[q - rp[r[0]]] -= H
        Cp, _ = sub_product(r, vp)
        Cm, _ = sub_product(r, vm)
        fd = math.fsum((W[r[0]] * (Cp[0] - Cm[0])).ravel()) / (2 * H)
        assert abs(fd - g) <= barS(g), "dS[%d]: fd %r vs %r" % (q, fd, g)

    order = np.argsort(ci, kind="stable")
    col_start = np.searchsorted(ci[order], np.arange(n + 1))
    cand = np.nonzero(np.diff(col_start) > 0)[0]  # columns of S with a nonzero
    ii = cand[rng.integers(0, len(cand), 64)]
    jj = rng.integers(0, w, 64)
    gX = [dX[i, j] for i, j in zip(ii, jj)]
    barX = _bar(gX)
    for (i, j), g in zip(zip(ii, jj), gX):
        rows = np.unique(rows_of[order[col_start[i]:col_start[i + 1]]])
        x0 = X[i, j]
        off = 8 * (int(i) * w + int(j))
        try:
            Xdev.upload(np.array([x0 + H]), offset=off)
            Cp, _ = sub_product(rows)
            Xdev.upload(np.array([x0 - H]), offset=off)
            Cm, _ = sub_product(rows)
        finally:
            Xdev.upload(np.array([x0]), offset=off)
        fd = math.fsum((W[rows, j] * (Cp[:, j] - Cm[:, j])).ravel()) / (2 * H)
        assert abs(fd - g) <= barX(g), "dX[%d, %d]: fd %r vs %r" % (i, j, fd, g)
