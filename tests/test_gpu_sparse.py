"""CSR products and sparse structure on the GPU: bit-identical to the oracle's
restatement of Flag4j's loops (RealCsrDenseMatMult, RealCsrMatMult,
CooMatrix.toCsr, CooDataSorter, RealCsrOps.transpose); the FMA mode and SDDMM
within 2 k u sum|a||b|."""
import ctypes
import math

import numpy as np
import pytest

from conftest import U

pytestmark = pytest.mark.gpu


def csr_from_dense(f4j, a):
    return f4j.Matrix(a).toCsr()


def test_golden_csr_dense_products(f4j, golden):
    # RealCsrDenseMatMultTests.java:27-88: A.toCsr().mult(B) equals aDense.mult(B)
    cases = [c for c in golden["csr_dense"] if c["call"] == "assertEquals"]
    for c in cases:
        a, b = np.array(c["vars"]["aEntries"]), np.array(c["vars"]["bEntries"])
        A = csr_from_dense(f4j, a)
        exp = f4j.Matrix(a).mult(f4j.Matrix(b), mode="exact")
        assert A.mult(f4j.Matrix(b)) == exp
        for j in range(b.shape[1]):
            assert np.array_equal(A.mult(f4j.Vector(b[:, j])).data, f4j.Matrix(a).mult(
                f4j.Matrix(b[:, j:j + 1]), mode="exact").data)
    bad = [c for c in golden["csr_dense"] if c["call"] == "assertThrows"]
    a, b = np.array(bad[0]["vars"]["aEntries"]), np.array(bad[0]["vars"]["bEntries"])
    with pytest.raises(f4j.LinearAlgebraException):
        csr_from_dense(f4j, a).mult(f4j.Matrix(b))
    with pytest.raises(f4j.IllegalArgumentException, match="Expecting values to be equal"):
        csr_from_dense(f4j, a).mult(f4j.Vector(np.ones(3)))


def test_golden_csr_transpose(f4j, golden):
    # CsrMatrixTransposeTests.java:24-51: A.T() equals denseA.T().toCsr()
    for c in [c for c in golden["csr_transpose"] if c["method"] == "transposeTest" and c["call"] == "assertEquals"]:
        a = np.array(c["vars"]["aDenseEntries"])
        T = csr_from_dense(f4j, a).T()
        E = csr_from_dense(f4j, a.T.copy())
        assert np.array_equal(T.rowPointers, E.rowPointers)
        assert np.array_equal(T.colIndices, E.colIndices)
        assert np.array_equal(T.data, E.data)


@pytest.mark.parametrize("rows,cols,lam,hi", [(1, 1, 1.0, 1), (300, 500, 16.0, 256), (5000, 4000, 16.0, 256),
                                              (2000, 3000, 200.0, 256), (40000, 40000, 3.0, 8)])
@pytest.mark.parametrize("ncols", [1, 3, 32, 64, 100])
def test_spmm_spmv_bit_identical(f4j, oracle, rows, cols, lam, hi, ncols):
    from flag4j_gb300 import synth
    rp, ci, v = synth.csr_poisson(rows, cols, lam=lam, hi=hi, seed=rows + ncols)
    S = f4j.CsrMatrix((rows, cols), v, rp, ci)
    X = synth.normal(cols, ncols, 3)
    assert np.array_equal(S.mult(f4j.Matrix(X)).toNumpy(), oracle.spmm(rp, ci, v, X))
    if ncols == 1:
        assert np.array_equal(S.mult(f4j.Vector(X[:, 0])).data, oracle.spmv(rp, ci, v, X[:, 0]))


def test_empty_rows_and_empty_matrix(f4j, oracle):
    a = np.zeros((70, 9))
    a[3, 2] = 1.5
    a[69, 8] = -2.0
    a[40, :] = np.arange(1, 10)
    S = csr_from_dense(f4j, a)
    X = np.arange(9 * 5, dtype=np.float64).reshape(9, 5)
    assert np.array_equal(S.mult(f4j.Matrix(X)).toNumpy(), oracle.spmm(S.rowPointers, S.colIndices, S.data, X))
    Z = f4j.CsrMatrix((6, 4), np.zeros(0), np.zeros(7, np.int32), np.zeros(0, np.int32))
    assert not Z.mult(f4j.Matrix(np.ones((4, 3)))).toNumpy().any()
    assert not Z.mult(f4j.Vector(np.ones(4))).data.any()


def test_rows_longer_than_a_staging_chunk(f4j, oracle):
    """Rows of 5000 and 1600 nonzeros (longer than the SpMV kernel's shared-memory
    chunk) between empty and short rows; SpMV and SpMM stay bit-identical."""
    rng = np.random.default_rng(17)
    rows, cols = 200, 6000
    lens = rng.integers(0, 40, rows)
    lens[[0, 63, 64, 127, 199]] = [5000, 1600, 0, 3100, 2000]
    lens[100:110] = 0
    rp = np.zeros(rows + 1, np.int32)
    np.cumsum(lens, out=rp[1:])
    ci = np.concatenate([np.sort(rng.choice(cols, n, replace=False)) for n in lens]).astype(np.int32)
    v = rng.standard_normal(len(ci))
    S = f4j.CsrMatrix((rows, cols), v, rp, ci)
    X = rng.standard_normal((cols, 3))
    for j in range(3):
        assert np.array_equal(S.mult(f4j.Vector(X[:, j])).data, oracle.spmv(rp, ci, v, X[:, j]))
        y = S.mult(f4j.Vector(X[:, j]), mode="fma").data
        assert np.all(np.abs(y - oracle.spmv(rp, ci, v, X[:, j])) <= fma_bound(oracle, rp, ci, v, X[:, j:j + 1])[:, 0])
    assert np.array_equal(S.mult(f4j.Matrix(X)).toNumpy(), oracle.spmm(rp, ci, v, X))


def test_full_config_csr_products(f4j, oracle):
    """2^20 x 2^20, Poisson(16) row lengths: SpMV and SpMM (32 columns) bit-identical."""
    from flag4j_gb300 import synth
    n = 1 << 20
    rp, ci, v = synth.csr_poisson(n, n, seed=2024)
    S = f4j.CsrMatrix((n, n), v, rp, ci)
    x = synth.normal(n, 1, 5).ravel()
    assert np.array_equal(S.mult(f4j.Vector(x)).data, oracle.spmv(rp, ci, v, x, threads=8))
    X = synth.normal(n, 32, 6)
    assert np.array_equal(S.mult(f4j.Matrix(X)).toNumpy(), oracle.spmm(rp, ci, v, X, threads=8))


def fma_bound(oracle, rp, ci, v, X, threads=1):
    """2 k u (|S||X|) per row, k = the row's length (the fused and the reference
    rounding each stay within k u |S||X| of the exact product)."""
    k = np.diff(rp).astype(np.float64)[:, None]
    return 2 * k * U * oracle.spmm(rp, ci, np.abs(v), np.abs(X), threads=threads)


@pytest.mark.parametrize("rows,cols,lam,hi", [(1, 1, 1.0, 1), (5000, 4000, 16.0, 256), (2000, 3000, 200.0, 256)])
@pytest.mark.parametrize("ncols", [1, 3, 32, 64, 100])
def test_spmm_spmv_fma_mode_within_bound(f4j, oracle, rows, cols, lam, hi, ncols):
    from flag4j_gb300 import synth
    rp, ci, v = synth.csr_poisson(rows, cols, lam=lam, hi=hi, seed=7 * rows + ncols)
    S = f4j.CsrMatrix((rows, cols), v, rp, ci)
    X = synth.normal(cols, ncols, 11)
    ref = oracle.spmm(rp, ci, v, X)
    bound = fma_bound(oracle, rp, ci, v, X)
    got = S.mult(f4j.Matrix(X), mode="fma").toNumpy()
    assert np.all(np.abs(got - ref) <= bound)
    # the default stays the reference's rounding
    assert np.array_equal(S.mult(f4j.Matrix(X)).toNumpy(), ref)
    if ncols == 1:
        y = S.mult(f4j.Vector(X[:, 0]), mode="fma").data
        assert np.all(np.abs(y - ref[:, 0]) <= bound[:, 0])


def test_fma_mode_full_config_and_complex_rhs(f4j, oracle):
    """2^20 x 2^20, Poisson(16): SpMV and SpMM (32 columns) in the FMA mode within
    the bound; CsrMatrix.mult(CMatrix) in the FMA mode within it per part."""
    from flag4j_gb300 import synth
    n = 1 << 20
    rp, ci, v = synth.csr_poisson(n, n, seed=2024)
    S = f4j.CsrMatrix((n, n), v, rp, ci)
    x = synth.normal(n, 1, 5)
    y = S.mult(f4j.Vector(x.ravel()), mode="fma").data
    assert np.all(np.abs(y - oracle.spmv(rp, ci, v, x.ravel(), threads=8)) <= fma_bound(oracle, rp, ci, v, x, 8)[:, 0])
    X = synth.normal(n, 32, 6)
    got = S.mult(f4j.Matrix(X), mode="fma").toNumpy()
    assert np.all(np.abs(got - oracle.spmm(rp, ci, v, X, threads=8)) <= fma_bound(oracle, rp, ci, v, X, 8))
    rng = np.random.default_rng(3)
    m = 4096
    rp, ci, v = synth.csr_poisson(m, m, seed=31)
    Xz = rng.standard_normal((m, 5)) + 1j * rng.standard_normal((m, 5))
    got = f4j.CsrMatrix((m, m), v, rp, ci).mult(f4j.CMatrix(Xz), mode="fma").toNumpy()
    ref = oracle.spmm_rz(rp, ci, v, Xz)
    assert np.all(np.abs(got.real - ref.real) <= fma_bound(oracle, rp, ci, v, Xz.real))
    assert np.all(np.abs(got.imag - ref.imag) <= fma_bound(oracle, rp, ci, v, Xz.imag))


def test_sparse_mode_rejected(f4j):
    S = f4j.CsrMatrix((2, 2), np.ones(2), np.array([0, 1, 2]), np.array([0, 1]))
    with pytest.raises(f4j.IllegalArgumentException):
        S.mult(f4j.Vector(np.ones(2)), mode="fast")
    ctx = f4j.default_context()
    X = ctx.from_numpy(np.ones((2, 3)))
    Y = ctx.alloc(2 * 3 * 8)
    assert ctx.lib.f4j_spmm_ex(ctx.handle, S.handle(ctx), X.handle, 3, Y.handle, 7, None) != 0
    assert ctx.lib.f4j_spmv_ex(ctx.handle, S.handle(ctx), X.handle, Y.handle, -1, None) != 0


# ------------------------------------------------------------------ structure
def test_coo_to_csr_bit_exact(f4j, oracle):
    from flag4j_gb300 import synth
    rp, ci, v = synth.csr_poisson(20000, 7000, seed=4)
    r = np.repeat(np.arange(20000, dtype=np.int32), np.diff(rp))
    S = f4j.CooMatrix((20000, 7000), v, r, ci).toCsr()
    assert np.array_equal(S.rowPointers, oracle.coo_to_csr(20000, r))
    assert np.array_equal(S.colIndices, ci) and np.array_equal(S.data, v)


def test_coo_sort_stable_bit_exact(f4j, oracle):
    from flag4j_gb300 import synth
    rp, ci, v = synth.csr_poisson(3000, 2000, seed=5)
    r, c, vv = synth.coo_shuffled(rp, ci, v, seed=6)
    # duplicates (same (row, col) twice) must keep their input order
    r = np.concatenate([r, r[:500]])
    c = np.concatenate([c, c[:500]])
    vv = np.concatenate([vv, -vv[:500]])
    er, ec, ev, _ = oracle.coo_sort(r, c, vv)
    coo = f4j.CooMatrix((3000, 2000), vv.copy(), r.copy(), c.copy()).sortIndices()
    assert np.array_equal(coo.rowIndices, er) and np.array_equal(coo.colIndices, ec)
    assert np.array_equal(coo.data, ev)


def _coo_sort_abi(f4j, r, c, v):
    """f4j_coo_sort through the C ABI (no shape validation: negative indices reach it)."""
    ctx = f4j.default_context()
    r, c = np.ascontiguousarray(r, np.int32), np.ascontiguousarray(c, np.int32)
    R, C = ctx.from_numpy(r), ctx.from_numpy(c)
    V = ctx.from_numpy(np.ascontiguousarray(v, np.float64)) if v is not None else None
    assert ctx.lib.f4j_coo_sort(ctx.handle, len(r), R.handle, C.handle, V.handle if V else None) == 0
    ro, co = np.empty_like(r), np.empty_like(c)
    R.download(ro)
    C.download(co)
    vo = None
    if V is not None:
        vo = np.empty(len(r))
        V.download(vo)
    return ro, co, vo


def _shuffled_coo(rng, lens, cols, dup=0):
    r = np.repeat(np.arange(len(lens)), lens)
    c = np.concatenate([rng.choice(cols, n, replace=False) for n in lens]) if len(r) else np.zeros(0, int)
    if dup:
        k = rng.choice(len(r), dup, replace=False)
        r, c = np.concatenate([r, r[k]]), np.concatenate([c, c[k]])
    p = rng.permutation(len(r))
    return r[p], c[p], rng.standard_normal(len(r))


@pytest.mark.parametrize("case", ["segments", "beyond_segment_cap", "no_values"])
def test_coo_sort_row_lengths_and_paths(f4j, oracle, case):
    """Rows of 0..64 entries (ranked in a warp, two keys per lane), 65..4096
    (sorted in shared memory) and beyond 4096 (the radix path), duplicates
    included, with lengths on both sides of 32 and 64."""
    rng = np.random.default_rng(len(case))
    lens = rng.integers(0, 40, 3000)
    if case == "beyond_segment_cap":
        lens[[10, 2000]] = [5000, 4097]
    else:
        lens[[5, 6, 7, 8, 9, 700, 1500, 2999]] = [33, 64, 65, 63, 32, 1000, 4096, 100]
    r, c, v = _shuffled_coo(rng, lens, 6000, dup=700)
    er, ec, ev, _ = oracle.coo_sort(r, c, v)
    ro, co, vo = _coo_sort_abi(f4j, r, c, None if case == "no_values" else v)
    assert np.array_equal(ro, er) and np.array_equal(co, ec)
    if vo is not None:
        assert np.array_equal(vo, ev)


def test_coo_sort_negative_and_sparse_index_ranges(f4j, oracle):
    rng = np.random.default_rng(8)
    # negative indices sort first, as Flag4j's int comparison orders them
    r = rng.integers(-50, 50, 4000)
    c = rng.integers(-1000, 1000, 4000)
    v = rng.standard_normal(4000)
    er, ec, ev, _ = oracle.coo_sort(r, c, v)
    ro, co, vo = _coo_sort_abi(f4j, r, c, v)
    assert np.array_equal(ro, er) and np.array_equal(co, ec) and np.array_equal(vo, ev)
    # a row range far larger than nnz
    r = rng.integers(0, 1 << 30, 3000)
    r[:40] = r[40]  # one row repeated
    c = rng.integers(0, 1 << 30, 3000)
    er, ec, ev, _ = oracle.coo_sort(r, c, v[:3000])
    ro, co, vo = _coo_sort_abi(f4j, r, c, v[:3000])
    assert np.array_equal(ro, er) and np.array_equal(co, ec) and np.array_equal(vo, ev)


def test_transpose_and_permutation_bit_exact(f4j, oracle):
    from flag4j_gb300 import synth
    rows, cols = 9000, 5000
    rp, ci, v = synth.csr_poisson(rows, cols, seed=8)
    S = f4j.CsrMatrix((rows, cols), v, rp, ci)
    trp, tci, tv, perm = oracle.csr_transpose(rows, cols, rp, ci, v)
    T = S.T()
    assert np.array_equal(T.rowPointers, trp) and np.array_equal(T.colIndices, tci)
    assert np.array_equal(T.data, tv)
    assert np.array_equal(S.transposePermutation(), perm)


@pytest.mark.parametrize("ncols", [1, 32, 64, 7])
def test_spmm_transpose_bit_exact(f4j, oracle, ncols):
    """dX = S^T dC without forming S^T equals S.T().mult(dC) of the reference."""
    from flag4j_gb300 import synth
    rows, cols = 12000, 9000
    rp, ci, v = synth.csr_poisson(rows, cols, seed=9)
    S = f4j.CsrMatrix((rows, cols), v, rp, ci)
    dC = synth.normal(rows, ncols, 10)
    trp, tci, tv, _ = oracle.csr_transpose(rows, cols, rp, ci, v)
    assert np.array_equal(S.multTransposeLeft(f4j.Matrix(dC)).toNumpy(), oracle.spmm(trp, tci, tv, dC))


@pytest.mark.parametrize("ncols", [64, 5, 130])
def test_sddmm_within_bound(f4j, oracle, ncols):
    from flag4j_gb300 import synth
    from flag4j_gb300.device import check
    rows, cols = 4000, 3000
    rp, ci, v = synth.csr_poisson(rows, cols, seed=11)
    S = f4j.CsrMatrix((rows, cols), v, rp, ci)
    A, B = synth.normal(rows, ncols, 1), synth.normal(cols, ncols, 2)
    ctx = f4j.default_context()
    out = ctx.alloc(8 * len(v))
    dA, dB = ctx.from_numpy(A), ctx.from_numpy(B)
    check(ctx.lib.f4j_sddmm(ctx.handle, S.handle(ctx), dA.handle, dB.handle, ncols, out.handle, None))
    got = out.to_numpy(np.float64, len(v))
    ref = oracle.sddmm(rp, ci, A, B)
    rows_of = np.repeat(np.arange(rows), np.diff(rp))
    absab = np.sum(np.abs(A[rows_of]) * np.abs(B[ci]), axis=1)
    assert np.all(np.abs(got - ref) <= 2 * ncols * U * absab)


def test_sparse_adjoint_finite_differences(f4j):
    """C = S X, L = sum(W o C): dX = S^T W, dS = (W X^T) on pattern(S); central FD."""
    from flag4j_gb300 import synth
    rows, cols, nc = 3000, 2000, 64
    rp, ci, v = synth.csr_poisson(rows, cols, seed=12)
    X, W = synth.normal(cols, nc, 1), synth.normal(rows, nc, 2)
    node = f4j.SpMMNode(f4j.CsrMatrix((rows, cols), v, rp, ci), f4j.Matrix(X))
    dS, dX = node.backward(f4j.Matrix(W))
    dS, dX = dS.data, dX.toNumpy()
    rng = np.random.default_rng(3)
    h = 1e-6

    def prod(vals, Xm):
        return f4j.CsrMatrix((rows, cols), vals, rp, ci).mult(f4j.Matrix(Xm)).toNumpy()

    def central(Cp, Cm):
        # (L(+h) - L(-h)) / 2h with the difference taken before the sum, which
        # keeps the summation's rounding out of the quotient
        return math.fsum((W * (Cp - Cm)).ravel()) / (2 * h)

    for _ in range(32):
        q = rng.integers(0, len(v))
        vp, vm = v.copy(), v.copy()
        vp[q] += h
        vm[q] -= h
        fd = central(prod(vp, X), prod(vm, X))
        assert abs(fd - dS[q]) <= 1e-7 * max(1.0, abs(dS[q]))
        i, j = rng.integers(0, cols), rng.integers(0, nc)
        Xp, Xm_ = X.copy(), X.copy()
        Xp[i, j] += h
        Xm_[i, j] -= h
        fd = central(prod(v, Xp), prod(v, Xm_))
        assert abs(fd - dX[i, j]) <= 1e-7 * max(1.0, abs(dX[i, j]))


# ------------------------------------------------------------------ validation (host-side faults only)
def _wrap(f4j, rows, cols, rp, ci, v, validate=1):
    from flag4j_gb300.device import check
    ctx = f4j.default_context()
    bufs = [ctx.from_numpy(np.asarray(rp, np.int32)), ctx.from_numpy(np.asarray(ci, np.int32)),
            ctx.from_numpy(np.asarray(v, np.float64))]
    h = ctypes.c_void_p()
    check(ctx.lib.f4j_csr_wrap(ctx.handle, rows, cols, len(v), bufs[0].handle, bufs[1].handle, bufs[2].handle,
                               validate, ctypes.byref(h)))
    ctx.lib.f4j_csr_free(ctx.handle, h)


def test_device_csr_validation_messages(f4j):
    _wrap(f4j, 3, 3, [0, 1, 2, 3], [0, 1, 2], [1.0, 2.0, 3.0])
    with pytest.raises(f4j.IllegalArgumentException, match="monotonically increasing"):
        _wrap(f4j, 3, 3, [0, 2, 1, 3], [0, 1, 2], [1.0, 2.0, 3.0])
    with pytest.raises(f4j.IllegalArgumentException, match="Invalid column index"):
        _wrap(f4j, 3, 3, [0, 1, 2, 3], [0, 5, 2], [1.0, 2.0, 3.0])
    with pytest.raises(f4j.IllegalArgumentException, match="must be positive"):
        _wrap(f4j, 3, 3, [-1, 1, 2, 3], [0, 1, 2], [1.0, 2.0, 3.0])
    with pytest.raises(f4j.IllegalArgumentException, match="elements but nnz"):
        _wrap(f4j, 3, 3, [0, 1, 2, 2], [0, 1, 2], [1.0, 2.0, 3.0])
    with pytest.raises(f4j.IllegalArgumentException, match="Invalid index"):
        f4j.CooMatrix((3, 3), [1.0, 2.0], [0, 3], [0, 1]).toCsr()


# ------------------------------------------------------------------ CSR x CSR
def _bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.int64)


def test_golden_csr_csr_products(f4j, golden):
    # RealCsrCsrMatMultTests.java:34-189: A.mult(B) equals aDense.mult(bDense),
    # A.mult2Csr(B) equals that product's toCsr(); shape mismatches throw
    for c in golden["csr_csr"]:
        a, b = np.array(c["vars"]["aEntries"]), np.array(c["vars"]["bEntries"])
        A, B = f4j.Matrix(a).toCsr(), f4j.Matrix(b).toCsr()
        if c["call"] == "assertThrows":
            with pytest.raises(f4j.LinearAlgebraException):
                A.mult(B) if c["method"] == "multTests" else A.mult2Csr(B)
            continue
        if c["call"] != "assertEquals":
            continue
        exp = f4j.Matrix(a).mult(f4j.Matrix(b), mode="exact")
        if c["method"] == "multTests":
            assert A.mult(B) == exp
        else:
            got, e = A.mult2Csr(B), exp.toCsr()
            assert np.array_equal(got.rowPointers, e.rowPointers) and np.array_equal(got.colIndices, e.colIndices)
            assert np.array_equal(got.data, e.data)


@pytest.mark.parametrize("m,k,n,la,lb", [(1, 1, 1, 1.0, 1.0), (2000, 1500, 1800, 8.0, 6.0), (700, 300, 5000, 40.0, 30.0)])
def test_csr_csr_bit_identical(f4j, oracle, m, k, n, la, lb):
    from flag4j_gb300 import synth
    arp, aci, av = synth.csr_poisson(m, k, lam=la, hi=min(k, 256), seed=m + 1)
    brp, bci, bv = synth.csr_poisson(k, n, lam=lb, hi=min(n, 256), seed=k + 2)
    A, B = f4j.CsrMatrix((m, k), av, arp, aci), f4j.CsrMatrix((k, n), bv, brp, bci)
    assert np.array_equal(_bits(A.mult(B).toNumpy()), _bits(oracle.spgemm_dense(arp, aci, av, brp, bci, bv, n)))
    rp, ci, v = oracle.spgemm_csr(arp, aci, av, brp, bci, bv, n)
    S = A.mult2Csr(B)
    assert S.shape == (m, n) and S.nnz == len(v)
    assert np.array_equal(S.rowPointers, rp) and np.array_equal(S.colIndices, ci)
    assert np.array_equal(_bits(S.data), _bits(v))


def test_csr_csr_cancellations_signed_zeros_and_empty(f4j, oracle):
    # explicit zeros in B, products that cancel, -0.0 first products, empty rows
    rng = np.random.default_rng(12)
    m, k, n = 400, 300, 200
    a = np.where(rng.random((m, k)) < 0.03, rng.choice([-1.0, 1.0, 2.0], (m, k)), 0.0)
    a[50:60] = 0.0
    b = np.where(rng.random((k, n)) < 0.05, rng.choice([-2.0, 2.0, 0.5], (k, n)), 0.0)
    arp, aci, av = _csr_of(a)
    brp, bci, bv = _csr_of(b)
    bv[::7] = 0.0  # stored zeros: products of -0.0 and +0.0
    A, B = f4j.CsrMatrix((m, k), av, arp, aci), f4j.CsrMatrix((k, n), bv, brp, bci)
    assert np.array_equal(_bits(A.mult(B).toNumpy()), _bits(oracle.spgemm_dense(arp, aci, av, brp, bci, bv, n)))
    rp, ci, v = oracle.spgemm_csr(arp, aci, av, brp, bci, bv, n)
    S = A.mult2Csr(B)
    assert np.count_nonzero(v == 0.0) > 0 and np.count_nonzero(np.signbit(v) & (v == 0.0)) > 0
    assert np.array_equal(S.rowPointers, rp) and np.array_equal(S.colIndices, ci)
    assert np.array_equal(_bits(S.data), _bits(v))
    Z = f4j.CsrMatrix((m, k), np.zeros(0), np.zeros(m + 1, np.int32), np.zeros(0, np.int32))
    assert not Z.mult(B).toNumpy().any()
    E = Z.mult2Csr(B)
    assert E.nnz == 0 and not E.rowPointers.any()


def test_csr_csr_mult_transpose(f4j, oracle):
    from flag4j_gb300 import synth
    arp, aci, av = synth.csr_poisson(900, 700, lam=10.0, seed=3)
    brp, bci, bv = synth.csr_poisson(500, 700, lam=12.0, seed=4)
    A, B = f4j.CsrMatrix((900, 700), av, arp, aci), f4j.CsrMatrix((500, 700), bv, brp, bci)
    trp, tci, tv, _ = oracle.csr_transpose(500, 700, brp, bci, bv)
    exp = oracle.spgemm_dense(arp, aci, av, trp, tci, tv, 500)
    assert np.array_equal(_bits(A.multTranspose(B).toNumpy()), _bits(exp))
    with pytest.raises(f4j.LinearAlgebraException):
        A.multTranspose(f4j.CsrMatrix((5, 6), np.ones(1), np.array([0, 1, 1, 1, 1, 1]), np.array([2])))


def _csr_of(a):
    r, c = np.nonzero(a != 0.0)
    rp = np.zeros(a.shape[0] + 1, np.int32)
    np.cumsum(np.bincount(r, minlength=a.shape[0]), out=rp[1:])
    return rp, c.astype(np.int32), a[r, c].copy()


def _cplx(a):
    a = np.asarray(a, dtype=np.float64)
    return a[..., 0] + 1j * a[..., 1]


def test_golden_real_complex_csr_products(f4j, golden):
    # RealComplexCsrCsrMatMultTests.java:37-162: CsrMatrix.mult(CsrCMatrix) equals aDense.mult(bDense),
    # mult2Csr its toCsr(); shape mismatches throw
    for c in golden["csr_csr_rz"]:
        a, b = np.array(c["vars"]["aEntries"]), _cplx(c["vars"]["bEntries"])
        A = f4j.Matrix(a).toCsr()
        B = f4j.CMatrix(b).toCsr()
        if c["call"] == "assertThrows":
            with pytest.raises(f4j.LinearAlgebraException):
                A.mult(B) if c["method"] == "multTests" else A.mult2Csr(B)
            continue
        if c["call"] != "assertEquals":
            continue
        exp = f4j.Matrix(a).mult(f4j.CMatrix(b), mode="exact").toNumpy()
        if c["method"] == "multTests":
            assert np.array_equal(A.mult(B).toNumpy(), exp)
        else:
            got = A.mult2Csr(B)
            assert isinstance(got, f4j.CsrCMatrix)
            r, cc = np.nonzero(exp != 0)
            assert np.array_equal(got.colIndices, cc) and np.array_equal(got.data, exp[r, cc])


def _csr_any(rng, rows, cols, dens, cplx):
    a = np.where(rng.random((rows, cols)) < dens, rng.standard_normal((rows, cols)), 0.0)
    if cplx:
        a = a + 1j * np.where(a != 0, rng.standard_normal((rows, cols)), 0.0)
    r, c = np.nonzero(a != 0)
    rp = np.zeros(rows + 1, np.int32)
    np.cumsum(np.bincount(r, minlength=rows), out=rp[1:])
    return rp, c.astype(np.int32), a[r, c].copy()


@pytest.mark.parametrize("ak,bk", [(0, 1), (1, 0), (1, 1)])
def test_complex_csr_csr_bit_identical(f4j, oracle, ak, bk):
    rng = np.random.default_rng(10 * ak + bk)
    m, k, n = 700, 500, 900
    arp, aci, av = _csr_any(rng, m, k, 0.02, ak)
    brp, bci, bv = _csr_any(rng, k, n, 0.02, bk)
    bv[::9] = 0.0  # stored zeros: signed-zero products
    A = (f4j.CsrCMatrix if ak else f4j.CsrMatrix)((m, k), av, arp, aci)
    B = (f4j.CsrCMatrix if bk else f4j.CsrMatrix)((k, n), bv, brp, bci)
    got = A.mult(B).toNumpy()
    assert np.array_equal(_bits(got.view(np.float64)),
                          _bits(oracle.spgemm_dense_any(arp, aci, av, brp, bci, bv, n).view(np.float64)))
    rp, ci, v = oracle.spgemm_csr_any(arp, aci, av, brp, bci, bv, n)
    S = A.mult2Csr(B)
    assert isinstance(S, f4j.CsrCMatrix) and S.nnz == len(v)
    assert np.array_equal(S.rowPointers, rp) and np.array_equal(S.colIndices, ci)
    assert np.array_equal(_bits(S.data.view(np.float64)), _bits(v.view(np.float64)))
    with pytest.raises(f4j.LinearAlgebraException):
        A.mult(A)


def _adversarial_values(rng, n, specials):
    """Doubles that stress a multiply-then-add chain's rounding: short significands (exact
    ties), N(0,1), magnitudes near overflow and underflow (products and sums leave the normal
    range), subnormals, signed zeros and, with specials, infinities and NaNs."""
    kind = rng.integers(0, 7, n)
    out = rng.standard_normal(n)
    k = kind == 0
    out[k] = rng.integers(-4096, 4097, k.sum()) * np.exp2(rng.integers(-30, 31, k.sum()))
    k = kind == 1
    out[k] = rng.uniform(-2, 2, k.sum()) * np.exp2(rng.integers(480, 1023, k.sum()))
    k = kind == 2
    out[k] = rng.uniform(-2, 2, k.sum()) * np.exp2(rng.integers(-1040, -480, k.sum()))
    k = kind == 3
    out[k] = rng.choice([0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 1.0, -1.0], k.sum())
    k = kind == 4
    out[k] = (1.0 + rng.integers(0, 8, k.sum()) * 2.0 ** -52) * rng.choice([-1.0, 1.0], k.sum())
    if specials:
        k = rng.random(n) < 0.01
        out[k] = rng.choice([np.inf, -np.inf, np.nan], k.sum())
    return out


def _same_bits(a, b):
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint64), b[~nb].view(np.uint64))


@pytest.mark.parametrize("specials", [False, True])
@pytest.mark.parametrize("ncols", [3, 32, 64])
def test_spmm_exact_rounding_adversarial_operands(f4j, oracle, specials, ncols):
    """Exact mode on operands whose products and sums round at ties, cancel, overflow, underflow
    and meet signed zeros and special values: every output, signed zeros included, matches the
    oracle's multiply-then-add chain bit for bit (NaN where the oracle has NaN), for S X and
    S^T X, with the 2-column (128-bit load) and 1-column kernels."""
    from flag4j_gb300 import synth
    rows = cols = 3000
    rng = np.random.default_rng(ncols + 100 * specials)
    rp, ci, _ = synth.csr_poisson(rows, cols, lam=12.0, hi=64, seed=ncols)
    v = _adversarial_values(rng, len(ci), specials)
    X = _adversarial_values(rng, cols * ncols, specials).reshape(cols, ncols)
    X[1::7] = -X[0:-1:7]  # rows that cancel against their neighbours
    S = f4j.CsrMatrix((rows, cols), v, rp, ci)
    assert _same_bits(S.mult(f4j.Matrix(X)).toNumpy(), oracle.spmm(rp, ci, v, X))
    trp, tci, tv, _ = oracle.csr_transpose(rows, cols, rp, ci, v)
    assert _same_bits(S.multTransposeLeft(f4j.Matrix(X)).toNumpy(), oracle.spmm(trp, tci, tv, X))


@pytest.mark.parametrize("specials", [False, True])
def test_spmv_exact_rounding_adversarial_operands(f4j, oracle, specials):
    """The matrix-vector kernel (k_spmv) on the same adversarial values: every
    entry of S x, signed zeros, subnormals and NaN positions included, is the
    oracle's storage-order multiply-then-add result bit for bit."""
    from flag4j_gb300 import synth
    rows = cols = 20000
    rng = np.random.default_rng(7 + specials)
    rp, ci, _ = synth.csr_poisson(rows, cols, lam=12.0, hi=300, seed=33)
    v = _adversarial_values(rng, len(ci), specials)
    x = _adversarial_values(rng, cols, specials)
    S = f4j.CsrMatrix((rows, cols), v, rp, ci)
    assert _same_bits(S.mult(f4j.Vector(x)).data, oracle.spmv(rp, ci, v, x))


@pytest.mark.parametrize("specials", [False, True])
@pytest.mark.parametrize("cp", [False, True])
def test_dense_exact_rounding_adversarial_operands(f4j, oracle, specials, cp):
    """EXACT dense products on the same adversarial values (ties, cancellation,
    overflow, subnormals, signed zeros, and with specials Inf / NaN): bit for
    bit the reference's k-ascending order, real and complex."""
    rng = np.random.default_rng(11 + specials + 2 * cp)
    m, n, k = 150, 70, 260
    A = _adversarial_values(rng, m * k, specials).reshape(m, k)
    B = _adversarial_values(rng, k * n, specials).reshape(k, n)
    if cp:  # real and imaginary parts set directly (1j * inf would also make the real part NaN)
        Az, Bz = np.empty((m, k), np.complex128), np.empty((k, n), np.complex128)
        Az.real, Az.imag = A, _adversarial_values(rng, m * k, specials).reshape(m, k)
        Bz.real, Bz.imag = B, _adversarial_values(rng, k * n, specials).reshape(k, n)
        A, B = Az, Bz
        got = f4j.CMatrix(A).mult(f4j.CMatrix(B), mode="exact").toNumpy()
        ref = oracle.zgemm(A, B)
        assert _same_bits(got.real.copy(), ref.real.copy()) and _same_bits(got.imag.copy(), ref.imag.copy())
    else:
        got = f4j.Matrix(A).mult(f4j.Matrix(B), mode="exact").toNumpy()
        assert _same_bits(got, oracle.dgemm(A, B))


def test_coo_to_csr_range_checks_report_first_bad_entry(f4j):
    """CooMatrix.toCsr checks the indices inside the row count and the column copy: the first
    out-of-range entry by position is reported as SparseValidation.validateCoo words it, for rows
    and columns, in the 16-byte column copy and its tail, and a later bad entry does not win; a
    valid conversion afterwards still works."""
    rng = np.random.default_rng(3)
    n, rows, cols = 100003, 5000, 7000
    r = np.sort(rng.integers(0, rows, n)).astype(np.int32)
    c = rng.integers(0, cols, n).astype(np.int32)
    v = rng.standard_normal(n)
    cases = [[(n - 1, "col", cols)], [(50001, "row", -1)], [(4, "col", -3), (50001, "row", rows)],
             [(n - 2, "row", rows)], [(37, "row", rows + 9), (38, "col", -1)]]
    for bad in cases:
        rr, cc = r.copy(), c.copy()
        for pos, which, val in bad:
            (rr if which == "row" else cc)[pos] = val
        first = bad[0][0]
        with pytest.raises(f4j.IllegalArgumentException,
                           match=r"Invalid index \[%d, %d\]" % (rr[first], cc[first])):
            f4j.CooMatrix((rows, cols), v, rr, cc).toCsr()
    S = f4j.CooMatrix((rows, cols), v, r, c).toCsr()
    assert S.rowPointers[-1] == n
    assert np.array_equal(np.diff(S.rowPointers), np.bincount(r, minlength=rows))
    assert np.array_equal(S.colIndices, c) and np.array_equal(S.data, v)


@pytest.mark.parametrize("rows,lam,p_empty", [(255, 16, 0.0), (256, 16, 0.1), (257, 16, 0.5), (513, 0.5, 0.5),
                                              (3000, 5, 0.9), (2000, 16, 0.02)])
def test_spmv_balanced_lanes_edge_shapes(f4j, oracle, rows, lam, p_empty):
    """The SpMV kernel splits each 256-row block between its 32 lanes by nonzero
    count: blocks of empty rows across block and lane boundaries, trailing empty
    rows and one 3000-nonzero row among short ones stay bit-identical (and within
    the bound in FMA mode)."""
    rng = np.random.default_rng(rows)
    lens = rng.poisson(lam, rows)
    lens[rng.random(rows) < p_empty] = 0
    lens[rows // 3: rows // 3 + rows // 5] = 0
    lens[-3:] = 0
    lens[rng.integers(0, rows - 3)] = 3000
    cols = 4000
    rp = np.zeros(rows + 1, np.int32)
    np.cumsum(lens, out=rp[1:])
    ci = np.concatenate([np.sort(rng.choice(cols, n, replace=False)) for n in lens]).astype(np.int32)
    v = rng.standard_normal(len(ci))
    S = f4j.CsrMatrix((rows, cols), v, rp, ci)
    x = rng.standard_normal(cols)
    ref = oracle.spmv(rp, ci, v, x)
    assert np.array_equal(S.mult(f4j.Vector(x)).data, ref)
    y = S.mult(f4j.Vector(x), mode="fma").data
    assert np.all(np.abs(y - ref) <= fma_bound(oracle, rp, ci, v, x[:, None])[:, 0])
