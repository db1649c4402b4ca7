"""Mixed real / complex products on the GPU (through the C ABI via the Flag4j mirror).

- Matrix.mult(CMatrix | CVector): the real GEMM of A with B's interleaved storage
  read as a real k x 2n matrix (MatrixMultiplyDispatcher.java:71-200).
- CMatrix.mult(Matrix | Vector): the complex GEMM with the real operand promoted
  (MatrixMultiplyDispatcher.java:201-260).
- CsrMatrix.mult(CMatrix | CVector): the real SpMM over 2 * ncols interleaved
  columns (RealFieldDenseCsrMatMult.java:62-91).
- CsrCMatrix.mult(CMatrix | CVector): f4j_zspmm (DenseCsrSemiringMatMult.java:59-98).

Bars: EXACT GEMM mode and the sparse products are bit-identical to the
oracle's restatements of those loops (which are pinned to the reference's
golden vectors); PLAIN and SPLIT satisfy |C - C_ref| <= 2 k u |A||B| per part.
"""
import numpy as np
import pytest

from conftest import U

pytestmark = pytest.mark.gpu


def cplx(a):
    a = np.asarray(a, dtype=np.float64)
    return a[..., 0] + 1j * a[..., 1]


def crand(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def test_real_times_complex_golden_exact(f4j, golden):
    # MatrixMultTests.java:66-86 and MatrixVectorTests.java:66-81
    c = [c for c in golden["matrix_mult"] if c["line"] == 85 and c["call"] == "assertEquals"][0]["vars"]
    C = f4j.Matrix(np.array(c["aEntries"])).mult(f4j.CMatrix(cplx(c["bEntries"])), mode="exact")
    assert np.array_equal(C.toNumpy(), cplx(c["expCEntries"]))
    c = [c for c in golden["matrix_vector"] if c["line"] == 81 and c["call"] == "assertEquals"][0]["vars"]
    y = f4j.Matrix(np.array(c["aEntries"])).mult(f4j.CVector(cplx(c["bEntries"])), mode="exact")
    assert np.array_equal(y.data, cplx(c["expCEntries"]))


@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (37, 29, 53), (130, 70, 257)])
def test_mixed_dense_exact_bit_identical(f4j, oracle, m, n, k):
    rng = np.random.default_rng(m * 1000 + n)
    A, Bz = rng.standard_normal((m, k)), crand(rng, k, n)
    got = f4j.Matrix(A).mult(f4j.CMatrix(Bz), mode="exact").toNumpy()
    assert np.array_equal(got, oracle.rzgemm(A, Bz))
    Az, B = crand(rng, m, k), rng.standard_normal((k, n))
    got = f4j.CMatrix(Az).mult(f4j.Matrix(B), mode="exact").toNumpy()
    assert np.array_equal(got, oracle.zrgemm(Az, B))
    x = rng.standard_normal(k)
    got = f4j.CMatrix(Az).mult(f4j.Vector(x), mode="exact").data
    assert np.array_equal(got, oracle.zrgemm(Az, x[:, None]).ravel())


@pytest.mark.parametrize("mode", ["plain", "split"])
def test_mixed_dense_fast_modes_within_bound(f4j, oracle, mode):
    rng = np.random.default_rng(5)
    m, n, k = 96, 80, 300
    A, Bz = rng.standard_normal((m, k)), crand(rng, k, n)
    got = f4j.Matrix(A).mult(f4j.CMatrix(Bz), mode=mode).toNumpy()
    ref = oracle.rzgemm(A, Bz)
    absA = np.abs(A)
    assert np.all(np.abs(got.real - ref.real) <= 2 * k * U * (absA @ np.abs(Bz.real)) + 1e-300)
    assert np.all(np.abs(got.imag - ref.imag) <= 2 * k * U * (absA @ np.abs(Bz.imag)) + 1e-300)
    Az, B = crand(rng, m, k), rng.standard_normal((k, n))
    got = f4j.CMatrix(Az).mult(f4j.Matrix(B), mode=mode).toNumpy()
    ref = oracle.zrgemm(Az, B)
    absB = np.abs(B)
    assert np.all(np.abs(got.real - ref.real) <= 2 * k * U * (np.abs(Az.real) @ absB) + 1e-300)
    assert np.all(np.abs(got.imag - ref.imag) <= 2 * k * U * (np.abs(Az.imag) @ absB) + 1e-300)


@pytest.mark.parametrize("ncols", [1, 5, 32, 33])
def test_csr_times_complex_bit_identical(f4j, oracle, ncols):
    from flag4j_gb300 import synth
    rows, cols = 3000, 2500
    rp, ci, v = synth.csr_poisson(rows, cols, seed=21)
    rng = np.random.default_rng(ncols)
    X = crand(rng, cols, ncols)
    S = f4j.CsrMatrix((rows, cols), v, rp, ci)
    assert np.array_equal(S.mult(f4j.CMatrix(X)).toNumpy(), oracle.spmm_rz(rp, ci, v, X))
    x = X[:, 0].copy()
    assert np.array_equal(S.mult(f4j.CVector(x)).data, oracle.spmm_rz(rp, ci, v, x[:, None]).ravel())


@pytest.mark.parametrize("ncols", [1, 5, 32, 33])
def test_complex_csr_times_complex_bit_identical(f4j, oracle, ncols):
    from flag4j_gb300 import synth
    rows, cols = 3000, 2500
    rp, ci, v = synth.csr_poisson(rows, cols, seed=22)
    rng = np.random.default_rng(100 + ncols)
    vz = v + 1j * rng.standard_normal(len(v))
    X = crand(rng, cols, ncols)
    S = f4j.CsrCMatrix((rows, cols), vz, rp, ci)
    assert np.array_equal(S.mult(f4j.CMatrix(X)).toNumpy(), oracle.zspmm(rp, ci, vz, X))
    x = X[:, 0].copy()
    assert np.array_equal(S.mult(f4j.CVector(x)).data, oracle.zspmm(rp, ci, vz, x[:, None]).ravel())


def test_complex_csr_large_and_empty_rows(f4j, oracle):
    from flag4j_gb300 import synth
    rows, cols = 1 << 17, 1 << 17
    rp, ci, v = synth.csr_poisson(rows, cols, seed=23)
    # empty a stretch of rows (reference semantics: zero output rows)
    cut = rp[100:201].copy()
    lens = np.diff(rp)
    lens[100:200] = 0
    keep = np.ones(len(v), bool)
    keep[cut[0]:cut[-1]] = False
    rp2 = np.zeros(rows + 1, np.int32)
    np.cumsum(lens, out=rp2[1:])
    ci2, v2 = ci[keep], v[keep]
    rng = np.random.default_rng(9)
    vz = v2 + 1j * rng.standard_normal(len(v2))
    X = crand(rng, cols, 8)
    got = f4j.CsrCMatrix((rows, cols), vz, rp2, ci2).mult(f4j.CMatrix(X)).toNumpy()
    ref = oracle.zspmm(rp2, ci2, vz, X, threads=8)
    assert np.array_equal(got, ref)
    assert not np.any(got[100:200])


def test_mixed_shape_errors(f4j):
    from flag4j_gb300 import IllegalArgumentException, LinearAlgebraException
    with pytest.raises(LinearAlgebraException):
        f4j.Matrix(np.ones((3, 4))).mult(f4j.CMatrix(np.ones((5, 2), np.complex128)))
    with pytest.raises(LinearAlgebraException):
        f4j.CMatrix(np.ones((3, 4), np.complex128)).mult(f4j.Matrix(np.ones((5, 2))))
    S = f4j.CsrCMatrix((3, 4), np.ones(2, np.complex128), np.array([0, 1, 2, 2]), np.array([0, 3]))
    with pytest.raises(IllegalArgumentException):
        S.mult(f4j.CVector(np.ones(5, np.complex128)))
    with pytest.raises(LinearAlgebraException):
        S.mult(f4j.CMatrix(np.ones((5, 2), np.complex128)))


@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (45, 33, 70), (130, 64, 129)])
def test_complex_mult_transpose_and_matvec_exact(f4j, oracle, m, n, k):
    # CMatrix.multTranspose -> DenseSemiringMatMultTranspose.java:54-150 (k ascending, running sums)
    # and CMatrix.mult(CVector): both bit-identical to the k-ascending complex restatement
    rng = np.random.default_rng(m + n + k)
    A, B = crand(rng, m, k), crand(rng, n, k)
    got = f4j.CMatrix(A).multTranspose(f4j.CMatrix(B), mode="exact").toNumpy()
    assert np.array_equal(got, oracle.zgemm(A, B.T.copy()))
    x = crand(rng, k)
    got = f4j.CMatrix(A).mult(f4j.CVector(x), mode="exact").data
    assert np.array_equal(got, oracle.zgemm(A, x[:, None]).ravel())
