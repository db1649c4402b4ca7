"""Pins the CPU oracle to Flag4j's own known-answer tests (bit-exact).

Fixtures: tests/golden/reference_golden.json, extracted from the reference's
JUnit sources by tests/golden/make_golden.py.
"""
import numpy as np
import pytest


def cplx(a):
    a = np.asarray(a, dtype=np.float64)
    return a[..., 0] + 1j * a[..., 1]


def test_real_kernels_bit_exact(oracle, golden):
    # src/test/java/org/flag4j/linalg/ops/dense/real/MatrixMultiplyTests.java:13-135
    n = 0
    for c in golden["real_kernels"]:
        v = c["vars"]
        A, B, exp = np.array(v["entriesA"]), np.array(v["entriesB"]), np.array(v["exp"])
        assert np.array_equal(oracle.dgemm(A, B).ravel(), exp), c["line"]
        if c["method"] == "columnVectorTestCase":
            assert np.array_equal(oracle.dgemv_blocked(A, B[:, 0]), exp), c["line"]
        n += 1
    assert n == 20


def test_complex_kernels_bit_exact(oracle, golden):
    # src/test/java/org/flag4j/linalg/ops/dense/complex/CMatrixMultiplyTests.java:13-169
    for c in golden["complex_kernels"]:
        v = c["vars"]
        A, B, exp = cplx(v["entriesA"]), cplx(v["entriesB"]), cplx(v["exp"])
        assert np.array_equal(oracle.zgemm(A, B).ravel(), exp), c["line"]


def test_api_level_products(oracle, golden):
    # MatrixMultTests.java:25-62, CMatrixMultTests.java:62-101, MatrixVectorTests.java:26-58
    mm = [c for c in golden["matrix_mult"] if c["method"] == "matMultTestCase" and c["call"] == "assertEquals"]
    v = mm[0]["vars"]
    assert np.array_equal(oracle.dgemm(np.array(v["aEntries"]), np.array(v["bEntries"])),
                          np.array(v["expEntries"]))
    cm = [c for c in golden["cmatrix_mult"] if c["method"] == "matMultComplexTestCase" and c["call"] == "assertEquals"]
    v = cm[0]["vars"]
    assert np.array_equal(oracle.zgemm(cplx(v["aEntries"]), cplx(v["bEntries"])), cplx(v["expEntries"]))
    mv = [c for c in golden["matrix_vector"] if c["method"] == "matVecMultTestCase" and c["call"] == "assertEquals"]
    v = mv[0]["vars"]
    A, x = np.array(v["aEntries"]), np.array(v["bEntries"])
    assert np.array_equal(oracle.dgemv_blocked(A, x), np.array(v["expEntries"]))


def test_mult_transpose_matches_mult(oracle, golden):
    # MatrixMultTests.java:249-265: A.multTranspose(B) == A.mult(B.T())
    c = [c for c in golden["matrix_mult"] if c["method"] == "multTransposeTestCase"][0]
    A, Bt = np.array(c["vars"]["aEntries"]), np.array(c["vars"]["bEntries"])
    # the test's B = bEntries^T, so multTranspose multiplies by bEntries
    assert np.array_equal(oracle.dgemm_abt(A, Bt.T.copy()), oracle.dgemm(A, Bt))


def _csr_of_dense(a):
    r, c = np.nonzero(a != 0.0)
    rp = oracle_coo_to_csr_rows(a.shape[0], r)
    return rp, c.astype(np.int32), a[r, c]


def oracle_coo_to_csr_rows(rows, r):
    from oracle import oracle as O
    return O.coo_to_csr(rows, r.astype(np.int32))


def test_csr_dense_products_equal_dense(oracle, golden):
    # RealCsrDenseMatMultTests.java:27-88: A.toCsr().mult(B) equals aDense.mult(B) exactly
    cases = [c for c in golden["csr_dense"] if c["call"] == "assertEquals"]
    assert len(cases) == 2
    for c in cases:
        a, b = np.array(c["vars"]["aEntries"]), np.array(c["vars"]["bEntries"])
        rp, ci, v = _csr_of_dense(a)
        assert np.array_equal(oracle.spmm(rp, ci, v, b), oracle.dgemm(a, b))
        for j in range(b.shape[1]):
            assert np.array_equal(oracle.spmv(rp, ci, v, b[:, j].copy()), oracle.dgemm(a, b[:, j:j + 1]).ravel())


def test_csr_transpose_matches_dense_transpose(oracle, golden):
    # CsrMatrixTransposeTests.java:24-51: A.T() equals denseA.T().toCsr()
    cases = [c for c in golden["csr_transpose"] if c["method"] == "transposeTest" and c["call"] == "assertEquals"]
    assert len(cases) == 2
    for c in cases:
        a = np.array(c["vars"]["aDenseEntries"])
        rp, ci, v = _csr_of_dense(a)
        trp, tci, tv, perm = oracle.csr_transpose(a.shape[0], a.shape[1], rp, ci, v)
        erp, eci, ev = _csr_of_dense(a.T.copy())
        assert np.array_equal(trp, erp) and np.array_equal(tci, eci) and np.array_equal(tv, ev)
        assert np.array_equal(v[perm], tv)


def test_csr_csr_products_equal_dense(oracle, golden):
    # RealCsrCsrMatMultTests.java:34-92: A.mult(B) equals aDense.mult(bDense);
    # :94-189: A.mult2Csr(B) equals aDense.mult(bDense).toCsr()
    mult = [c for c in golden["csr_csr"] if c["call"] == "assertEquals"]
    assert [c["method"] for c in mult] == ["multTests", "multTests", "multAsCsrTests", "multAsCsrTests"]
    for c in mult:
        a, b = np.array(c["vars"]["aEntries"]), np.array(c["vars"]["bEntries"])
        (arp, aci, av), (brp, bci, bv) = _csr_of_dense(a), _csr_of_dense(b)
        exp = oracle.dgemm(a, b)
        if c["method"] == "multTests":
            assert np.array_equal(oracle.spgemm_dense(arp, aci, av, brp, bci, bv, b.shape[1]), exp)
        else:
            rp, ci, v = oracle.spgemm_csr(arp, aci, av, brp, bci, bv, b.shape[1])
            erp, eci, ev = _csr_of_dense(exp)
            assert np.array_equal(rp, erp) and np.array_equal(ci, eci) and np.array_equal(v, ev)
    # the shape-mismatch cases keep a.shape[1] != b.shape[0]
    for c in [c for c in golden["csr_csr"] if c["call"] == "assertThrows"]:
        assert np.array(c["vars"]["aEntries"]).shape[1] != np.array(c["vars"]["bEntries"]).shape[0]


def _cplx(a):
    a = np.asarray(a, dtype=np.float64)
    return a[..., 0] + 1j * a[..., 1]


def test_real_complex_csr_products_equal_dense(oracle, golden):
    # RealComplexCsrCsrMatMultTests.java:37-162: CsrMatrix.mult(CsrCMatrix) equals
    # aDense.mult(bDense); mult2Csr equals that product's toCsr()
    cases = [c for c in golden["csr_csr_rz"] if c["call"] == "assertEquals"]
    assert [c["method"] for c in cases] == ["multTests", "multTests", "mult2CsrTests", "mult2CsrTests"]
    for c in cases:
        a, b = np.array(c["vars"]["aEntries"]), _cplx(c["vars"]["bEntries"])
        (arp, aci, av), (brp, bci, bv) = _csr_of_dense(a), _csr_of_dense(b)
        exp = oracle.rzgemm(a, b)
        if c["method"] == "multTests":
            assert np.array_equal(oracle.spgemm_dense_any(arp, aci, av, brp, bci, bv, b.shape[1]), exp)
        else:
            rp, ci, v = oracle.spgemm_csr_any(arp, aci, av, brp, bci, bv, b.shape[1])
            erp, eci, ev = _csr_of_dense(exp)
            assert np.array_equal(rp, erp) and np.array_equal(ci, eci) and np.array_equal(v, ev)


def test_complex_csr_restatements_agree_with_dense(oracle):
    # the three complex variants against dense products of the same matrices
    rng = np.random.default_rng(4)
    a = np.where(rng.random((30, 20)) < 0.2, rng.standard_normal((30, 20)), 0.0)
    b = np.where(rng.random((20, 25)) < 0.2, rng.standard_normal((20, 25)), 0.0)
    az = a * (1 + 0.5j)
    bz = b * (0.25 - 1j)
    for A, B in ((a, bz), (az, b), (az, bz)):
        (arp, aci, av), (brp, bci, bv) = _csr_of_dense(A), _csr_of_dense(B)
        C = oracle.spgemm_dense_any(arp, aci, av, brp, bci, bv, B.shape[1])
        assert np.allclose(C, A @ B, rtol=1e-13, atol=1e-13)
        rp, ci, v = oracle.spgemm_csr_any(arp, aci, av, brp, bci, bv, B.shape[1])
        D = np.zeros(C.shape, complex)
        for i in range(C.shape[0]):
            D[i, ci[rp[i]:rp[i + 1]]] = v[rp[i]:rp[i + 1]]
        assert np.array_equal(D, C)


def test_csr_csr_sparse_result_keeps_cancellations(oracle):
    # standardAsSparse stores every touched column: 1*x + 1*(-x) is an explicit 0.0,
    # and a lone product -1 * 0.0 stays -0.0 (HashMap.merge keeps the first value as is)
    arp, aci, av = np.array([0, 2, 3]), np.array([0, 1, 0]), np.array([1.0, 1.0, -1.0])
    brp, bci, bv = np.array([0, 2, 3]), np.array([0, 2, 0]), np.array([2.5, 0.0, -2.5])
    rp, ci, v = oracle.spgemm_csr(arp, aci, av, brp, bci, bv, 3)
    assert list(rp) == [0, 2, 4] and list(ci) == [0, 2, 0, 2]
    assert v[0] == 0.0 and np.signbit(v[3]) and v[3] == 0.0 and not np.signbit(v[1])
    # the dense result starts from +0.0: 0.0 + -0.0 is +0.0
    C = oracle.spgemm_dense(arp, aci, av, brp, bci, bv, 3)
    assert not np.signbit(C[1, 2])


def test_coo_sort_is_stable_lexicographic(oracle):
    rng = np.random.default_rng(3)
    r = rng.integers(0, 5, 400).astype(np.int32)
    c = rng.integers(0, 4, 400).astype(np.int32)
    vals = np.arange(400, dtype=np.float64)
    rs, cs, vs, perm = oracle.coo_sort(r, c, vals)
    exp = sorted(range(400), key=lambda i: (r[i], c[i], i))
    assert np.array_equal(perm, exp) and np.array_equal(vs, vals[exp])


def test_truth_oracle_is_compensated(oracle):
    # Dot2 recovers a sum that plain FP64 loses entirely.
    A = np.array([[1e16, 1.0, -1e16]])
    B = np.array([[1.0], [1.0], [1.0]])
    hi, lo, ab = oracle.truth_sampled(A, B, [0], [0])
    assert hi[0] + lo[0] == 1.0 and oracle.dgemm(A, B)[0, 0] == 0.0


def test_real_times_complex_golden(oracle, golden):
    # MatrixMultTests.java:66-86 (Matrix.mult(CMatrix)) and MatrixVectorTests.java:66-81
    # (Matrix.mult(CVector)): RealFieldDenseMatMult's k-ascending order, bit-exact
    c = [c for c in golden["matrix_mult"] if c["line"] == 85 and c["call"] == "assertEquals"][0]
    v = c["vars"]
    A, B, exp = np.array(v["aEntries"]), cplx(v["bEntries"]), cplx(v["expCEntries"])
    assert np.array_equal(oracle.rzgemm(A, B), exp)
    # complex x real is the transposed restatement: (B^T A^T)^T with B^T complex
    assert np.array_equal(oracle.zrgemm(B.T.copy(), A.T.copy()).T, oracle.rzgemm(A, B))
    c = [c for c in golden["matrix_vector"] if c["line"] == 81 and c["call"] == "assertEquals"][0]
    v = c["vars"]
    A, x, exp = np.array(v["aEntries"]), cplx(v["bEntries"]), cplx(v["expCEntries"])
    assert np.array_equal(oracle.rzgemm(A, x[:, None]).ravel(), exp)


def test_mixed_sparse_restatements_agree_with_dense(oracle):
    # RealFieldDenseCsrMatMult.java:62-91 and DenseCsrSemiringMatMult.java:59-98 on a
    # matrix with one nonzero per row equal the dense products exactly (one term per sum)
    rng = np.random.default_rng(3)
    rows, cols, nc = 7, 9, 5
    ci = rng.integers(0, cols, size=rows).astype(np.int32)
    rp = np.arange(rows + 1, dtype=np.int32)
    vr = rng.standard_normal(rows)
    vz = vr + 1j * rng.standard_normal(rows)
    X = rng.standard_normal((cols, nc)) + 1j * rng.standard_normal((cols, nc))
    Dr = np.zeros((rows, cols)); Dr[np.arange(rows), ci] = vr
    Dz = np.zeros((rows, cols), np.complex128); Dz[np.arange(rows), ci] = vz
    assert np.array_equal(oracle.spmm_rz(rp, ci, vr, X), oracle.rzgemm(Dr, X))
    # one term per sum: x * v with Complex128.mult's rounding, equal to zgemm's (a * x) products
    assert np.array_equal(oracle.zspmm(rp, ci, vz, X), oracle.zgemm(Dz, X))
