"""Dense GEMM parity on the GPU through the C ABI (via the Flag4j-mirror API).

Bars: EXACT mode is bit-identical to Flag4j's loops; PLAIN (FP64 DMMA) and
SPLIT (FP8 slices on tcgen05) satisfy |C - C_ref| <= 2 k u |A||B|
(u = 2^-53, k = inner dimension), componentwise.
"""
import ctypes
import math

import numpy as np
import pytest

from conftest import U, assert_within_bound

pytestmark = pytest.mark.gpu


def cplx(a):
    a = np.asarray(a, dtype=np.float64)
    return a[..., 0] + 1j * a[..., 1]


def opx(X, op):
    return X if op == 0 else (X.T if op == 1 else X.conj().T)


def run_gemm(f4j, A, B, opA=0, opB=0, mode="plain"):
    """C = op(A) op(B) through f4j_dgemm / f4j_zgemm with stored A, B."""
    from flag4j_gb300 import _lib
    from flag4j_gb300.device import check
    ctx = f4j.default_context()
    cp = np.iscomplexobj(A) or np.iscomplexobj(B)
    dt = np.complex128 if cp else np.float64
    A = np.ascontiguousarray(A, dt)
    B = np.ascontiguousarray(B, dt)
    m = A.shape[0] if opA == 0 else A.shape[1]
    k = A.shape[1] if opA == 0 else A.shape[0]
    n = B.shape[1] if opB == 0 else B.shape[0]
    dA, dB = ctx.from_numpy(A if A.size else np.zeros(1, dt)), ctx.from_numpy(B if B.size else np.zeros(1, dt))
    dC = ctx.alloc(max(m * n * (16 if cp else 8), 8))
    rep = _lib.f4j_report()
    fn = ctx.lib.f4j_zgemm if cp else ctx.lib.f4j_dgemm
    check(fn(ctx.handle, m, n, k, dA.handle, opA, dB.handle, opB, dC.handle, _lib.MODES[mode], ctypes.byref(rep)))
    C = dC.to_numpy(dt, m * n).reshape(m, n)
    ctx.sync()
    return C, rep


def ref_bound(oracle, A, B, cp):
    if not cp:
        return oracle.dgemm(A, B), oracle.absgemm(A, B)
    ref = oracle.zgemm(A, B)
    ab = np.abs(A.real) @ np.abs(B.real) + np.abs(A.imag) @ np.abs(B.imag)
    ab2 = np.abs(A.real) @ np.abs(B.imag) + np.abs(A.imag) @ np.abs(B.real)
    return ref, ab + 1j * ab2


def check_bound(C, ref, ab, k, what):
    if np.iscomplexobj(C):
        assert_within_bound(C.real, ref.real, ab.real, k, what + " (re)")
        assert_within_bound(C.imag, ref.imag, ab.imag, k, what + " (im)")
    else:
        assert_within_bound(C, ref, ab, k, what)


# ------------------------------------------------------------------ golden
def test_exact_mode_reproduces_golden_vectors(f4j, golden):
    # MatrixMultiplyTests.java / CMatrixMultiplyTests.java known answers, bit for bit
    for c in golden["real_kernels"]:
        v = c["vars"]
        C = f4j.Matrix(v["entriesA"]).mult(f4j.Matrix(v["entriesB"]), mode="exact")
        assert np.array_equal(C.data, np.array(v["exp"])), c["line"]
    for c in golden["complex_kernels"]:
        v = c["vars"]
        C = f4j.CMatrix(cplx(v["entriesA"])).mult(f4j.CMatrix(cplx(v["entriesB"])), mode="exact")
        assert np.array_equal(C.data, cplx(v["exp"]).ravel()), c["line"]


def split_normwise_tol(A, B, F):
    """Documented bound of the split product with F fixed-point bits per element:
    |C - C_true| <= 2^-F (2^e_i |b_j|_1 + 2^f_j |a_i|_1 + 8 k 2^(e_i + f_j)),
    2^e_i > max|a_i.|, 2^f_j > max|b_.j| (real operands; complex via the
    [Re | Im] concatenation)."""
    if np.iscomplexobj(A):
        Ac = np.hstack([A.real, A.imag])
        Bc = np.vstack([np.hstack([B.real, B.imag]), np.hstack([-B.imag, B.real])])
        t = split_normwise_tol(Ac, Bc, F)
        n = B.shape[1]
        return t[:, :n] + 1j * t[:, n:]
    k = A.shape[1]
    ra = np.abs(A).max(axis=1)
    cb = np.abs(B).max(axis=0)
    ea = np.where(ra > 0, np.floor(np.log2(np.where(ra > 0, ra, 1))) + 1, 0)
    fb = np.where(cb > 0, np.floor(np.log2(np.where(cb > 0, cb, 1))) + 1, 0)
    Ea, Fb = np.ldexp(1.0, ea.astype(int))[:, None], np.ldexp(1.0, fb.astype(int))[None, :]
    return np.ldexp(Ea * np.abs(B).sum(axis=0)[None, :] + Fb * np.abs(A).sum(axis=1)[:, None]
                    + 8.0 * k * Ea * Fb, -F)


@pytest.mark.parametrize("mode", ["plain", "split", "auto"])
def test_fast_modes_on_golden_vectors(f4j, golden, oracle, mode):
    for cp, key in ((False, "real_kernels"), (True, "complex_kernels")):
        for c in golden[key]:
            conv = cplx if cp else np.array
            A, B = conv(c["vars"]["entriesA"]), conv(c["vars"]["entriesB"])
            rep = {}
            M = f4j.CMatrix if cp else f4j.Matrix
            C = M(A).mult(M(B), mode=mode, report=rep).toNumpy()
            ref, ab = ref_bound(oracle, A, B, cp)
            if mode == "split":
                # k = 3 with 20-bit spreads: the split keeps its normwise bound
                tol = split_normwise_tol(A, B, rep["frac_bits"])
                assert np.all(np.abs((C - ref).real) <= tol.real + 2 * A.shape[1] * U * ab.real), c["line"]
                if cp:
                    assert np.all(np.abs((C - ref).imag) <= tol.imag + 2 * A.shape[1] * U * ab.imag), c["line"]
            else:
                check_bound(C, ref, ab, A.shape[1], "%s line %d" % (mode, c["line"]))
            if mode == "auto":
                assert rep["mode_used"] == 3 and np.array_equal(C, ref)  # tiny: Flag4j's own order


def test_api_golden_and_shape_errors(f4j, golden):
    c = [c for c in golden["matrix_mult"] if c["method"] == "matMultTestCase"]
    v = c[0]["vars"]
    A, B = f4j.Matrix(v["aEntries"]), f4j.Matrix(v["bEntries"])
    assert A.mult(B, mode="exact") == f4j.Matrix(v["expEntries"])
    v2 = c[1]["vars"]  # MatrixMultTests.java:61: mismatched shapes
    with pytest.raises(f4j.LinearAlgebraException, match=r"Cannot multiply matrices/vector with shapes \(4, 3\) and \(4, 2\)"):
        f4j.Matrix(v2["aEntries"]).mult(f4j.Matrix(v2["bEntries"]))
    mv = [c for c in golden["matrix_vector"] if c["method"] == "matVecMultTestCase"]
    A = f4j.Matrix(mv[0]["vars"]["aEntries"])
    y = A.mult(f4j.Vector(mv[0]["vars"]["bEntries"]), mode="exact")
    assert y == f4j.Vector(mv[0]["vars"]["expEntries"])
    with pytest.raises(f4j.LinearAlgebraException):
        A.mult(f4j.Vector(mv[1]["vars"]["bEntries"]))
    mt = [c for c in golden["matrix_mult"] if c["method"] == "multTransposeTestCase"]
    A, Bs = f4j.Matrix(mt[0]["vars"]["aEntries"]), np.array(mt[0]["vars"]["bEntries"])
    B = f4j.Matrix(Bs.T.copy())
    assert A.multTranspose(B, mode="exact") == A.mult(f4j.Matrix(Bs), mode="exact")
    with pytest.raises(f4j.IllegalArgumentException):
        A.multTranspose(f4j.Matrix(np.array(mt[1]["vars"]["bEntries"]).T.copy()))


# ------------------------------------------------------------------ random sizes
SIZES = [(1, 1, 1), (3, 5, 7), (17, 33, 65), (64, 64, 64), (130, 70, 257), (257, 129, 95), (200, 300, 1000)]


@pytest.mark.parametrize("m,n,k", SIZES)
@pytest.mark.parametrize("cp", [False, True])
def test_exact_mode_bit_identical(f4j, oracle, m, n, k, cp):
    from flag4j_gb300 import synth
    A = synth.uniform(m, k, m + 1)
    B = synth.uniform(k, n, n + 2)
    if cp:
        A = A + 1j * synth.uniform(m, k, 5)
        B = B + 1j * synth.uniform(k, n, 6)
    C, rep = run_gemm(f4j, A, B, mode="exact")
    ref = oracle.zgemm(A, B) if cp else oracle.dgemm(A, B)
    assert np.array_equal(C, ref)


@pytest.mark.parametrize("mode", ["plain", "split"])
@pytest.mark.parametrize("m,n,k", SIZES)
@pytest.mark.parametrize("cp", [False, True])
def test_fast_modes_within_bound(f4j, oracle, mode, m, n, k, cp):
    from flag4j_gb300 import synth
    A = synth.normal(m, k, 11)
    B = synth.normal(k, n, 12)
    if cp:
        A = A + 1j * synth.normal(m, k, 13)
        B = B + 1j * synth.normal(k, n, 14)
    C, rep = run_gemm(f4j, A, B, mode=mode)
    check_bound(C, *ref_bound(oracle, A, B, cp), k, mode)
    if mode == "split" and n == 1:
        # one column: the FP64 FMA matrix-vector product (plain arithmetic)
        assert rep.mode_used == 0 and rep.slices == 0
    elif mode == "split":
        assert rep.mode_used == 1 and 2 <= rep.slices <= 14


@pytest.mark.parametrize("mode", ["plain", "split", "auto"])
@pytest.mark.parametrize("opA", [0, 1, 2])
@pytest.mark.parametrize("cp", [False, True])
@pytest.mark.parametrize("m,k", [(1, 1), (37, 1001), (3000, 257), (5, 40000), (8192, 8192)])
def test_matrix_vector_products(f4j, oracle, mode, opA, cp, m, k):
    """Matrix.mult(Vector) and its transposed / conjugated forms in the fast
    modes: one FP64 FMA dot product per row (warp per row for op(A) = N, a
    K-split column pass for T / C), within 2 k u |A||x|."""
    if opA == 2 and not cp:
        pytest.skip("conjugation is the identity for real data")
    from flag4j_gb300 import synth
    rng = np.random.default_rng(m + k)
    Ast = synth.normal(m, k, 41) if opA == 0 else synth.normal(k, m, 41)
    x = rng.standard_normal((k, 1))
    if cp:
        Ast = Ast + 1j * (synth.normal(m, k, 42) if opA == 0 else synth.normal(k, m, 42))
        x = x + 1j * rng.standard_normal((k, 1))
    C, rep = run_gemm(f4j, Ast, x, opA=opA, mode=mode)
    Aop = opx(Ast, opA)
    ref, ab = ref_bound(oracle, np.ascontiguousarray(Aop), x, cp)
    check_bound(C, ref, ab, k, "gemv")
    if not (mode == "auto" and 2 * m * k * (4 if cp else 1) <= (1 << 24)):
        assert rep.mode_used == 0


def test_matrix_vector_conjugated_vector_and_nonfinite(f4j, oracle):
    rng = np.random.default_rng(3)
    m, k = 300, 500
    A = rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))
    xt = rng.standard_normal((1, k)) + 1j * rng.standard_normal((1, k))  # stored 1 x k, op C -> conj column
    C, _ = run_gemm(f4j, A, xt, opB=2, mode="plain")
    ref, ab = ref_bound(oracle, A, np.ascontiguousarray(xt.conj().T), True)
    check_bound(C, ref, ab, k, "gemv conj x")
    Ar = rng.standard_normal((m, k))
    Ar[7, 3] = np.nan
    Ar[9, 0] = np.inf
    C, _ = run_gemm(f4j, Ar, rng.standard_normal((k, 1)), mode="split")
    assert np.isnan(C[7, 0]) and not np.isfinite(C[9, 0])
    assert np.isfinite(np.delete(C, [7, 9], axis=0)).all()


@pytest.mark.parametrize("mode", ["exact", "plain", "split"])
@pytest.mark.parametrize("opA,opB", [(0, 1), (1, 0), (1, 1), (2, 0), (0, 2), (2, 2)])
def test_transposed_operands(f4j, oracle, mode, opA, opB):
    from flag4j_gb300 import synth
    m, n, k = 70, 45, 133
    for cp in (False, True):
        if not cp and (opA == 2 or opB == 2):
            continue
        As = synth.uniform(m, k, 1) if opA == 0 else synth.uniform(k, m, 1)
        Bs = synth.uniform(k, n, 2) if opB == 0 else synth.uniform(n, k, 2)
        if cp:
            As = As + 1j * synth.uniform(*As.shape, 3)
            Bs = Bs + 1j * synth.uniform(*Bs.shape, 4)
        C, _ = run_gemm(f4j, As, Bs, opA, opB, mode)
        A, B = np.ascontiguousarray(opx(As, opA)), np.ascontiguousarray(opx(Bs, opB))
        ref, ab = ref_bound(oracle, A, B, cp)
        if mode == "exact":
            assert np.array_equal(C, ref)
        else:
            check_bound(C, ref, ab, k, "%s op(%d,%d)" % (mode, opA, opB))


@pytest.mark.parametrize("mode", ["plain", "split", "exact"])
def test_odd_leading_dimensions_and_empty(f4j, oracle, mode):
    # odd real leading dimensions take the DMMA kernel's plain-load path
    from flag4j_gb300 import synth
    for (m, n, k) in [(33, 17, 9), (5, 3, 1), (1, 7, 3)]:
        A, B = synth.uniform(m, k, 7), synth.uniform(k, n, 8)
        C, _ = run_gemm(f4j, A, B, mode=mode)
        check_bound(C, *ref_bound(oracle, A, B, False), k, mode)
    C, _ = run_gemm(f4j, np.zeros((4, 0)), np.zeros((0, 3)), mode=mode)
    assert C.shape == (4, 3) and not C.any()


# ------------------------------------------------------------------ split specifics
def test_split_fp8_accumulation_is_exact(f4j):
    """Known-answer test of the tcgen05 FP32 accumulator: one-digit slices
    (x = d/16, |d| <= 15) make C = sum d_a d_b / 256 exactly representable; an
    adversarial K order (large partial sums first, then +-1 products) must give
    the exact integer result."""
    rng = np.random.default_rng(5)
    m, n, k = 128, 256, 8192
    da = np.empty((m, k), np.int64)
    db = np.empty((k, n), np.int64)
    da[:, : k // 2] = 15
    db[: k // 2, :] = 15
    da[:, k // 2:] = rng.choice([-1, 1], size=(m, k // 2))
    db[k // 2:, :] = rng.choice([-1, 1], size=(k // 2, n))
    da[:, 0] = rng.integers(-15, 16, size=m)
    exact = (da @ db).astype(np.float64) / 256.0
    C, rep = run_gemm(f4j, da / 16.0, db / 16.0, mode="split")
    assert np.array_equal(C, exact)
    # two-digit values: d1/16 + d2/512 -> also exactly representable results
    a2 = rng.integers(-15, 16, (m, 512)) * 32 + rng.integers(-15, 16, (m, 512))
    b2 = rng.integers(-15, 16, (512, n)) * 32 + rng.integers(-15, 16, (512, n))
    a2[:, 0] = 15 * 32
    b2[0, :] = 15 * 32
    C2, _ = run_gemm(f4j, a2 / 512.0, b2 / 512.0, mode="split")
    assert np.array_equal(C2, (a2 @ b2).astype(np.float64) / 512.0 ** 2)


@pytest.mark.parametrize("phi", [0, 8, 32])
def test_split_scaled_inputs(f4j, oracle, phi):
    from flag4j_gb300 import synth
    m = n = k = 384
    A = synth.scaled(m, k, phi, 21, "row")
    B = synth.scaled(k, n, phi, 22, "col")
    C, rep = run_gemm(f4j, A, B, mode="split")
    check_bound(C, *ref_bound(oracle, A, B, False), k, "split phi=%d" % phi)


def test_split_with_wide_spread_picks_more_slices(f4j, oracle):
    from flag4j_gb300 import synth
    A = synth.uniform(64, 256, 1) * np.ldexp(1.0, np.random.default_rng(0).integers(-30, 1, (64, 256)))
    B = synth.uniform(256, 64, 2)
    C, rep = run_gemm(f4j, A, B, mode="split")
    _, rep0 = run_gemm(f4j, synth.uniform(64, 256, 1), B, mode="split")
    assert rep.slices > rep0.slices
    check_bound(C, *ref_bound(oracle, A, B, False), 256, "wide spread")


@pytest.mark.parametrize("cp", [False, True])
@pytest.mark.parametrize("mode", ["split", "plain", "auto"])
def test_extreme_magnitudes(f4j, oracle, mode, cp):
    """Rows of A scaled by 2^e for e from the subnormal range (-1060) to 2^980,
    columns of B by 2^-20 .. 2^20: the split path's per-row and per-column
    exponents and its two-step rescale of the result stay within
    2 k u |A||B| of the reference's order, plus k ulps of the smallest
    subnormal where the reference itself rounds subnormal products."""
    from flag4j_gb300 import synth
    m = n = k = 256
    g = np.random.default_rng(77)
    ea = g.choice([-1060, -1040, -1000, -600, -30, 0, 30, 600, 980], size=m)
    eb = g.integers(-20, 21, size=n)
    A = synth.uniform(m, k, 78)
    B = synth.uniform(k, n, 79)
    if cp:
        A = A + 1j * synth.uniform(m, k, 80)
        B = B + 1j * synth.uniform(k, n, 81)
    A = A * np.ldexp(1.0, ea)[:, None]
    B = B * np.ldexp(1.0, eb)[None, :]
    assert np.isfinite(A).all() and (np.abs(A[ea == -1060]) < 2.0 ** -1022).all()   # subnormal rows
    C, rep = run_gemm(f4j, A, B, mode=mode)
    ref, ab = ref_bound(oracle, A, B, cp)
    slack = 2 * k * 2.0 ** -1074
    parts = [(C.real, ref.real, ab.real), (C.imag, ref.imag, ab.imag)] if cp else [(C, ref, ab)]
    for c, r, a in parts:
        err = np.abs(c - r)
        bound = 2.0 * (2 * k if cp else k) * U * a + slack
        assert np.isfinite(c).all()
        assert not np.any(err > bound), "%d entries outside the bound, worst excess %g" % (
            int((err > bound).sum()), float((err - bound)[err > bound].max()))


@pytest.mark.parametrize("tall", [True, False])
def test_split_beyond_two_million_rows_or_columns(f4j, oracle, tall):
    """More than 2^21 rows of A (tall) or columns of B (wide): the slicing
    kernels cover them with grid.y at its limit of 65535 blocks of 32 targets,
    looping over the rest.  Sampled rows (including the last ones) are within
    2 k u |A||B| of the reference's order."""
    from flag4j_gb300 import synth
    big, small, k = 2_200_000, 64, 100
    m, n = (big, small) if tall else (small, big)
    A = synth.uniform(m, k, 91)
    B = synth.uniform(k, n, 92)
    C, rep = run_gemm(f4j, A, B, mode="split")
    assert rep.mode_used == 1 and rep.slices > 0
    if tall:
        rows = np.r_[0:64, m - 2048:m]   # the last ones are past 65535 x 32 targets
        ref, ab = ref_bound(oracle, A[rows], B, False)
        assert_within_bound(C[rows], ref, ab, k, "tall")
    else:
        cols = np.r_[0:64, n - 2048:n]
        ref, ab = ref_bound(oracle, A, np.ascontiguousarray(B[:, cols]), False)
        assert_within_bound(C[:, cols], ref, ab, k, "wide")


def test_auto_mode_routes_nonfinite_to_dmma(f4j):
    A = np.ones((256, 256))
    A[3, 4] = np.nan
    A[5, 5] = np.inf
    B = np.ones((256, 256))
    C, rep = run_gemm(f4j, A, B, mode="auto")
    assert rep.mode_used == 0
    assert np.isnan(C[3]).all() and np.isinf(C[5]).all() and not np.isnan(C[0]).any()
    # tiny products run Flag4j's own order under AUTO
    _, rep2 = run_gemm(f4j, np.ones((16, 16)), np.ones((16, 16)), mode="auto")
    assert rep2.mode_used == 3


def test_gemm_check_agrees_with_oracle(f4j, oracle):
    from flag4j_gb300 import synth
    from flag4j_gb300.device import check
    ctx = f4j.default_context()
    A, B = synth.normal(300, 500, 1), synth.normal(500, 200, 2)
    C = A @ B + 1e-9  # a deliberately perturbed product
    dA, dB, dC = ctx.from_numpy(A), ctx.from_numpy(B), ctx.from_numpy(C)
    ea, er = ctypes.c_double(), ctypes.c_double()
    check(ctx.lib.f4j_gemm_check(ctx.handle, 0, 300, 200, 500, dA.handle, 0, dB.handle, 0, dC.handle, 256, 99,
                                 ctypes.byref(ea), ctypes.byref(er)))
    ii, jj = np.meshgrid(np.arange(300), np.arange(200), indexing="ij")
    hi, lo, ab = oracle.truth_sampled(A, B, ii.ravel(), jj.ravel())
    full = np.abs((C.ravel() - hi) - lo)
    assert 0 < ea.value <= full.max() * (1 + 1e-12)
    assert ea.value >= 0.5e-9


# ------------------------------------------------------------------ adjoint
@pytest.mark.parametrize("mode", ["exact", "plain", "split"])
def test_dense_adjoint_matches_reference_formulas(f4j, oracle, mode):
    from flag4j_gb300 import synth
    m, k, n = 96, 64, 80
    A, B, W = synth.normal(m, k, 1), synth.normal(k, n, 2), synth.normal(m, n, 3)
    node = f4j.MatMulNode(f4j.Matrix(A), f4j.Matrix(B), mode=mode)
    dA, dB = node.backward(f4j.Matrix(W))
    refA = oracle.dgemm_abt(W, B)             # W.multTranspose(B)
    refB = oracle.dgemm(A.T.copy(), W)        # A.T().mult(W)
    if mode == "exact":
        assert np.array_equal(dA.toNumpy(), refA) and np.array_equal(dB.toNumpy(), refB)
    else:
        check_bound(dA.toNumpy(), refA, np.abs(W) @ np.abs(B.T), n, "dA")
        check_bound(dB.toNumpy(), refB, np.abs(A.T) @ np.abs(W), m, "dB")


def test_complex_hermitian_adjoint(f4j, oracle):
    from flag4j_gb300 import synth
    m, k, n = 48, 40, 56
    A = synth.normal(m, k, 1) + 1j * synth.normal(m, k, 2)
    B = synth.normal(k, n, 3) + 1j * synth.normal(k, n, 4)
    W = synth.normal(m, n, 5) + 1j * synth.normal(m, n, 6)
    node = f4j.MatMulNode(f4j.CMatrix(A), f4j.CMatrix(B), mode="exact")
    dA, dB = node.backward(f4j.CMatrix(W))
    assert np.array_equal(dA.toNumpy(), oracle.zgemm(W, B.conj().T.copy()))   # W.mult(B.H())
    assert np.array_equal(dB.toNumpy(), oracle.zgemm(A.conj().T.copy(), W))   # A.H().mult(W)


@pytest.mark.parametrize("mode", ["plain", "split"])
def test_dense_adjoint_finite_differences(f4j, mode):
    """L = sum(W o (A B)); central differences (h = 1e-6) on 64 seeded entries."""
    from flag4j_gb300 import synth
    m, k, n = 64, 48, 40
    A, B, W = synth.normal(m, k, 1), synth.normal(k, n, 2), synth.normal(m, n, 3)
    node = f4j.MatMulNode(f4j.Matrix(A), f4j.Matrix(B), mode=mode)
    dA, dB = node.backward(f4j.Matrix(W))
    dA, dB = dA.toNumpy(), dB.toNumpy()
    rng = np.random.default_rng(9)
    h = 1e-6

    def prod(Am, Bm):
        return f4j.Matrix(Am).mult(f4j.Matrix(Bm), mode=mode).toNumpy()

    def central(Cp, Cm):
        # (L(+h) - L(-h)) / 2h, difference taken before the (exact) sum
        return math.fsum((W * (Cp - Cm)).ravel()) / (2 * h)

    for _ in range(32):
        i, j = rng.integers(0, m), rng.integers(0, k)
        Ap, Am_ = A.copy(), A.copy()
        Ap[i, j] += h
        Am_[i, j] -= h
        fd = central(prod(Ap, B), prod(Am_, B))
        assert abs(fd - dA[i, j]) <= 1e-7 * max(1.0, abs(dA[i, j]))
        i, j = rng.integers(0, k), rng.integers(0, n)
        Bp, Bm_ = B.copy(), B.copy()
        Bp[i, j] += h
        Bm_[i, j] -= h
        fd = central(prod(A, Bp), prod(A, Bm_))
        assert abs(fd - dB[i, j]) <= 1e-7 * max(1.0, abs(dB[i, j]))


@pytest.mark.parametrize("mode", ["plain", "split"])
def test_wrapped_host_output_matches_device_output(f4j, mode):
    """C written in place into pinned host memory (f4j_buf_wrap) is bitwise the
    C written to device memory; freeing the wrap handle leaves the array alone."""
    from flag4j_gb300 import _lib, synth
    from flag4j_gb300.device import check
    ctx = f4j.default_context()
    m, n, k = 300, 260, 520
    A = synth.scaled(m, k, 4, 11, "row")
    B = synth.scaled(k, n, 4, 12, "col")
    ref, _ = run_gemm(f4j, A, B, mode=mode)
    dA, dB = ctx.from_numpy(A), ctx.from_numpy(B)
    Ch = np.full((m, n), np.nan)
    check(ctx.lib.f4j_host_register(Ch.ctypes.data, Ch.nbytes))
    try:
        wC = ctx.wrap(Ch)
        check(ctx.lib.f4j_dgemm(ctx.handle, m, n, k, dA.handle, 0, dB.handle, 0, wC.handle, _lib.MODES[mode], None))
        ctx.sync()
        assert np.array_equal(Ch, ref)
        wC.free()
        Ch[0, 0] = 1.5  # still the caller's memory
    finally:
        check(ctx.lib.f4j_host_unregister(Ch.ctypes.data))


def test_wrap_rejects_misaligned_and_null(f4j):
    from flag4j_gb300.device import check, IllegalArgumentException
    ctx = f4j.default_context()
    buf = np.zeros(64)
    h = ctypes.c_void_p()
    with pytest.raises(IllegalArgumentException):
        check(ctx.lib.f4j_buf_wrap(ctx.handle, ctypes.c_void_p(buf.ctypes.data + 8), 64, ctypes.byref(h)))
    with pytest.raises(IllegalArgumentException):
        check(ctx.lib.f4j_buf_wrap(ctx.handle, None, 64, ctypes.byref(h)))


@pytest.mark.parametrize("m,n,k,mode,opA,opB,host", [
    # pipelined: A's first row part, B's column parts, the rest of A (parts in 128-row tile rows / columns);
    # no split K, and two tile rows or two tile columns
    (2500, 900, 700, "split", 0, 0, "allocated"),   # 20 x 8 tiles, f4j_host_alloc memory: A 5, 5, 8, 2; B 2 x 4
    (2000, 1300, 600, "split", 0, 1, "registered"),  # 16 x 11 tiles, B stored n x k: A 4, 4, 6, 2; B 2, 3, 3, 3
    (1500, 2000, 300, "split", 0, 0, "pageable"),   # 12 x 16 tiles, ragged last column: A 3, 3, 5, 1; B 4 x 4
    (300, 260, 5000, "split", 0, 1, "registered"),  # 3 x 3 tiles, 79 K blocks (no split K): A 1, 1, 1; B 1, 1, 1
    (130, 200, 4500, "split", 0, 0, "allocated"),   # 2 x 2 tiles, the last row ragged: A 1, 1; B 1, 1
    (3000, 100, 4200, "split", 0, 0, "registered"),  # 24 x 1 tiles, 66 K blocks: A 6, 6, 9, 3; B in one part
    (2200, 90, 4300, "split", 0, 1, "pageable"),    # 18 x 1 tiles, B stored n x k: A 4, 4, 8, 2; B in one part
    (100, 2000, 4200, "split", 0, 0, "registered"),  # 1 x 16 tiles, 66 K blocks: A in one part; B 4 x 4
    (128, 1000, 5000, "split", 0, 1, "allocated"),  # 1 x 8 tiles, B stored n x k: A in one part; B 2 x 4
    # uploaded, multiplied and downloaded in turn
    (1000, 700, 900, "split", 0, 0, "registered"),  # 48 tiles, 15 K blocks: split K
    (300, 260, 520, "split", 0, 0, "pageable"),     # 9 tiles: split K
    (100, 90, 80, "split", 0, 0, "allocated"),      # one tile row
    (3000, 1, 4200, "split", 0, 0, "registered"),   # n = 1: the matrix-vector kernel, as f4j_dgemm
    (600, 500, 400, "split", 1, 0, "registered"),   # op(A) = T
    (500, 300, 200, "plain", 0, 0, "registered"),
    (64, 48, 40, "exact", 0, 1, "allocated"),
])
def test_host_buffer_gemm_matches_device_gemm(f4j, m, n, k, mode, opA, opB, host):
    """f4j_dgemm_host is bitwise f4j_dgemm on the same operands, from registered, pageable or
    f4j_host_alloc host memory, with the same slice count and spread in the report."""
    from flag4j_gb300 import _lib, synth
    from flag4j_gb300.device import check, pinned_empty
    ctx = f4j.default_context()
    A = synth.scaled(m, k, 4, 21, "row") if opA == 0 else synth.scaled(k, m, 4, 21, "col")
    B = synth.scaled(k, n, 4, 22, "col") if opB == 0 else synth.scaled(n, k, 4, 22, "row")
    dA, dB, dC = ctx.from_numpy(A), ctx.from_numpy(B), ctx.alloc(8 * m * n)
    rd = _lib.f4j_report()
    check(ctx.lib.f4j_dgemm(ctx.handle, m, n, k, dA.handle, opA, dB.handle, opB, dC.handle, _lib.MODES[mode],
                            ctypes.byref(rd)))
    ref = dC.to_numpy(np.float64, m * n).reshape(m, n)
    C = np.full((m, n), np.nan)
    if host == "allocated":
        pa, pb, pc = pinned_empty(A.shape), pinned_empty(B.shape), pinned_empty(C.shape)
        pa[...], pb[...], pc[...] = A, B, C
        A, B, C = pa, pb, pc
    arrays = (A, B, C)
    pinned = host == "registered"
    if pinned:
        for a in arrays:
            check(ctx.lib.f4j_host_register(a.ctypes.data, a.nbytes))
    try:
        rep = _lib.f4j_report()
        check(ctx.lib.f4j_dgemm_host(ctx.handle, m, n, k, A.ctypes.data, opA, B.ctypes.data, opB, C.ctypes.data,
                                     _lib.MODES[mode], ctypes.byref(rep)))
        assert np.array_equal(C, ref)
        assert rep.mode_used == rd.mode_used and rep.slices == rd.slices
        if rd.mode_used == _lib.MODE_SPLIT:
            assert rep.slices > 0 and rep.exp_spread == rd.exp_spread
        assert (rep.mode_used == _lib.MODE_SPLIT) == (mode == "split" and n > 1)
    finally:
        if pinned:
            for a in arrays:
                check(ctx.lib.f4j_host_unregister(a.ctypes.data))


@pytest.mark.parametrize("m,n,k,opA,opB,host,poison", [
    # pipelined (B whole, A in row parts; tiles over the 2n-column [Re | Im] concatenation)
    (1000, 600, 5000, 0, 0, "registered", False),  # 8 x 10 tiles, 158 K blocks: A 2, 2, 3, 1
    (2000, 700, 600, 0, 2, "allocated", False),    # 16 x 11 tiles, B stored n x k and conjugated: A 4, 4, 6, 2
    (1000, 600, 5000, 0, 0, "pageable", True),     # a NaN in A's last part: the device path again
    # uploaded, multiplied and downloaded in turn
    (1500, 300, 1000, 0, 1, "pageable", False),    # 60 tiles, 32 K blocks: split K
    (700, 500, 400, 2, 0, "registered", False),    # op(A) = A^H
    (900, 1, 3000, 0, 0, "allocated", False),      # n = 1: the matrix-vector kernel
])
def test_host_buffer_zgemm_matches_device_zgemm(f4j, m, n, k, opA, opB, host, poison):
    """f4j_zgemm_host is bitwise f4j_zgemm on the same interleaved complex operands
    (CMatrix.mult / multTranspose from marshalled host arrays), NaN bits included,
    with the same mode, slice count and spread in the report."""
    from flag4j_gb300 import _lib, synth
    from flag4j_gb300.device import check, pinned_empty
    ctx = f4j.default_context()
    A = (synth.scaled(m, k, 4, 61, "row", cplx=True) if opA == 0 else
         synth.scaled(k, m, 4, 61, "col", cplx=True))
    B = synth.scaled(k, n, 4, 62, "col", cplx=True) if opB == 0 else synth.scaled(n, k, 4, 62, "row", cplx=True)
    if poison:
        A[m - 5, 7] = complex(np.nan, 1.0)
    dA, dB, dC = ctx.from_numpy(A), ctx.from_numpy(B), ctx.alloc(16 * m * n)
    rd = _lib.f4j_report()
    check(ctx.lib.f4j_zgemm(ctx.handle, m, n, k, dA.handle, opA, dB.handle, opB, dC.handle, _lib.MODE_SPLIT,
                            ctypes.byref(rd)))
    ref = dC.to_numpy(np.complex128, m * n).reshape(m, n)
    C = np.zeros((m, n), np.complex128)
    if host == "allocated":
        pa, pb, pc = pinned_empty(A.shape, np.complex128), pinned_empty(B.shape, np.complex128), \
            pinned_empty(C.shape, np.complex128)
        pa[...], pb[...], pc[...] = A, B, C
        A, B, C = pa, pb, pc
    arrays = (A, B, C)
    if host == "registered":
        for a in arrays:
            check(ctx.lib.f4j_host_register(a.ctypes.data, a.nbytes))
    try:
        rep = _lib.f4j_report()
        check(ctx.lib.f4j_zgemm_host(ctx.handle, m, n, k, A.ctypes.data, opA, B.ctypes.data, opB, C.ctypes.data,
                                     _lib.MODE_SPLIT, ctypes.byref(rep)))
        assert np.array_equal(C.view(np.uint64), ref.view(np.uint64))
        assert rep.mode_used == rd.mode_used and rep.slices == rd.slices
        if rd.mode_used == _lib.MODE_SPLIT:
            assert rep.exp_spread == rd.exp_spread
        if poison:
            assert rep.mode_used == _lib.MODE_PLAIN and np.isnan(C[m - 5]).all()
    finally:
        if host == "registered":
            for a in arrays:
                check(ctx.lib.f4j_host_unregister(a.ctypes.data))


@pytest.mark.parametrize("seed", range(16))
def test_host_buffer_gemm_random_shapes_and_parts(f4j, seed, monkeypatch):
    """Seeded random shapes, operand kinds, op(B) and part counts
    (F4J_HOST_PARTS, F4J_HOST_BPARTS): the host-buffer product is bitwise the
    device product, whichever path (pipelined or in turn) the shape takes."""
    from flag4j_gb300 import _lib, synth
    from flag4j_gb300.device import check
    g = np.random.default_rng(1000 + seed)
    cplx = bool(g.integers(0, 2))
    m, n = int(g.integers(1, 2600)), int(g.integers(1, 1800))
    k = int(g.choice([int(g.integers(1, 700)), int(g.integers(4100, 5200))]))  # with and without split K
    opB = int(g.integers(0, 3 if cplx else 2))
    monkeypatch.setenv("F4J_HOST_PARTS", str(int(g.choice([1, 2, 3, 4, 8]))))
    monkeypatch.setenv("F4J_HOST_BPARTS", str(int(g.choice([1, 2, 4, 8]))))
    A = synth.scaled(m, k, 4, 70 + seed, "row", cplx=cplx)
    B = synth.scaled(k, n, 4, 90 + seed, "col", cplx=cplx) if opB == 0 else \
        synth.scaled(n, k, 4, 90 + seed, "row", cplx=cplx)
    ctx = f4j.default_context()
    es, dt = (16, np.complex128) if cplx else (8, np.float64)
    dA, dB, dC = ctx.from_numpy(A), ctx.from_numpy(B), ctx.alloc(es * m * n)
    dev = ctx.lib.f4j_zgemm if cplx else ctx.lib.f4j_dgemm
    host = ctx.lib.f4j_zgemm_host if cplx else ctx.lib.f4j_dgemm_host
    rd = _lib.f4j_report()
    check(dev(ctx.handle, m, n, k, dA.handle, 0, dB.handle, opB, dC.handle, _lib.MODE_SPLIT, ctypes.byref(rd)))
    ref = dC.to_numpy(dt, m * n).reshape(m, n)
    C = np.zeros((m, n), dt)
    rep = _lib.f4j_report()
    check(host(ctx.handle, m, n, k, A.ctypes.data, 0, B.ctypes.data, opB, C.ctypes.data, _lib.MODE_SPLIT,
               ctypes.byref(rep)))
    assert np.array_equal(C.view(np.uint64), ref.view(np.uint64)), (m, n, k, cplx, opB)
    assert rep.mode_used == rd.mode_used and rep.slices == rd.slices


@pytest.mark.parametrize("cp", [False, True])
def test_host_pinning_per_call(f4j, cp):
    """f4j_set_host_pinning: pageable arrays are page-locked for each host-buffer
    call and released after it; the same array passed as A and B (registered
    once, the second registration refused and used as it is) and arrays that
    are already page-locked still give f4j_dgemm's / f4j_zgemm's bits."""
    from flag4j_gb300 import _lib, synth
    from flag4j_gb300.device import check
    ctx = f4j.default_context()
    n = 1536  # 12 x 12 tiles (24 for complex), 24 K blocks: pipelined
    A = synth.scaled(n, n, 4, 31, "row", cplx=cp)
    dt, es = (np.complex128, 16) if cp else (np.float64, 8)
    dev = ctx.lib.f4j_zgemm if cp else ctx.lib.f4j_dgemm
    host = ctx.lib.f4j_zgemm_host if cp else ctx.lib.f4j_dgemm_host
    dA, dC = ctx.from_numpy(A), ctx.alloc(es * n * n)
    check(dev(ctx.handle, n, n, n, dA.handle, 0, dA.handle, 0, dC.handle, _lib.MODE_SPLIT, None))
    ref = dC.to_numpy(dt, n * n).reshape(n, n)
    check(ctx.lib.f4j_set_host_pinning(ctx.handle, 1))
    try:
        for _ in range(2):
            C = np.zeros((n, n), dt)
            check(host(ctx.handle, n, n, n, A.ctypes.data, 0, A.ctypes.data, 0, C.ctypes.data, _lib.MODE_SPLIT, None))
            assert np.array_equal(C, ref)
        # the arrays were released: registering them now succeeds
        check(ctx.lib.f4j_host_register(A.ctypes.data, A.nbytes))
        C = np.zeros((n, n), dt)
        check(host(ctx.handle, n, n, n, A.ctypes.data, 0, A.ctypes.data, 0, C.ctypes.data, _lib.MODE_SPLIT, None))
        assert np.array_equal(C, ref)
        check(ctx.lib.f4j_host_unregister(A.ctypes.data))
    finally:
        check(ctx.lib.f4j_set_host_pinning(ctx.handle, 0))


def test_host_buffer_gemm_nonfinite_parts(f4j, oracle):
    """NaN / Inf in A: every row part falls back to DMMA, which propagates them
    like the reference; finite rows stay within the bound."""
    from flag4j_gb300 import _lib, synth
    from flag4j_gb300.device import check
    ctx = f4j.default_context()
    m, n, k = 700, 300, 256
    A = synth.normal(m, k, 31)
    B = synth.normal(k, n, 32)
    A[5, 7] = np.nan
    A[650, 3] = np.inf
    C = np.zeros((m, n))
    rep = _lib.f4j_report()
    check(ctx.lib.f4j_dgemm_host(ctx.handle, m, n, k, A.ctypes.data, 0, B.ctypes.data, 0, C.ctypes.data,
                                 _lib.MODE_SPLIT, ctypes.byref(rep)))
    assert rep.slices == 0 and rep.mode_used == _lib.MODE_PLAIN
    assert np.isnan(C[5]).all() and not np.isfinite(C[650]).any()
    fin = np.isfinite(A).all(axis=1)
    ref = oracle.dgemm(A[fin], B)
    bound = 2 * k * U * oracle.absgemm(A[fin], B)
    assert np.all(np.abs(C[fin] - ref) <= bound)


@pytest.mark.parametrize("case", ["wider_a_late", "wider_b_late", "nan_late", "inf_first"])
def test_host_buffer_gemm_speculative_slice_count(f4j, case):
    """The pipelined host-buffer product picks its slice count from A's first
    row part and B's first column part (512 rows and 384 columns here).  When
    all of A and B ask for another count, or an operand holds a NaN / Inf, the
    product runs again through the device path: C, the mode used and the slice
    count still equal f4j_dgemm's, NaN and Inf bits included."""
    from flag4j_gb300 import _lib, synth
    from flag4j_gb300.device import check
    ctx = f4j.default_context()
    m, n, k = 2048, 1536, 1024   # 16 x 12 tiles, 16 K blocks: A parts of 4, 4, 6, 2 tile rows, B parts of 3 x 4
    a0, b0 = 512, 384
    A = synth.uniform(m, k, 51)
    B = synth.uniform(k, n, 52)
    g = synth.rng(53)
    if case == "wider_a_late":   # rows past A's first part: elements scaled by 2^-j, j uniform in [0, 24]
        A[a0:] *= np.ldexp(1.0, -g.integers(0, 25, size=(m - a0, k)))
    elif case == "wider_b_late":  # the same for the columns past B's first part
        B[:, b0:] *= np.ldexp(1.0, -g.integers(0, 25, size=(k, n - b0)))
    elif case == "nan_late":
        A[1500, 17] = np.nan
    else:
        A[3, 900] = np.inf

    def device(Ad, Bd):
        mm, nn = Ad.shape[0], Bd.shape[1]
        dA, dB, dC = ctx.from_numpy(Ad), ctx.from_numpy(Bd), ctx.alloc(8 * mm * nn)
        rd = _lib.f4j_report()
        check(ctx.lib.f4j_dgemm(ctx.handle, mm, nn, k, dA.handle, 0, dB.handle, 0, dC.handle, _lib.MODE_SPLIT,
                                ctypes.byref(rd)))
        return dC.to_numpy(np.float64, mm * nn).reshape(mm, nn), rd

    ref, rd = device(A, B)
    C = np.zeros((m, n))
    rep = _lib.f4j_report()
    check(ctx.lib.f4j_dgemm_host(ctx.handle, m, n, k, A.ctypes.data, 0, B.ctypes.data, 0, C.ctypes.data,
                                 _lib.MODE_SPLIT, ctypes.byref(rep)))
    assert np.array_equal(C.view(np.uint64), ref.view(np.uint64))
    assert rep.mode_used == rd.mode_used and rep.slices == rd.slices
    if case.startswith("wider"):
        _, r_first = device(np.ascontiguousarray(A[:a0]), np.ascontiguousarray(B[:, :b0]))
        assert rd.mode_used == _lib.MODE_SPLIT and rd.slices > r_first.slices   # the first pick was too few
        assert rep.exp_spread == rd.exp_spread
    else:
        assert rd.mode_used == _lib.MODE_PLAIN and rd.slices == 0
        assert not np.isfinite(C[1500 if case == "nan_late" else 3]).any()


def test_one_context_shared_by_threads(f4j, oracle):
    """Four threads issue products on one context at once (ctypes releases the GIL,
    so the C calls overlap); every C-ABI call holds the context's lock, and each
    thread's result equals the same product run alone."""
    import threading
    from flag4j_gb300 import _lib, synth
    from flag4j_gb300.device import check
    ctx = f4j.default_context()
    m, n, k = 300, 200, 256
    jobs = [(synth.scaled(m, k, 2, 100 + t, "row"), synth.scaled(k, n, 2, 200 + t, "col")) for t in range(4)]
    refs = [run_gemm(f4j, A, B, mode="split")[0] for A, B in jobs]
    rp, ci, v = synth.csr_poisson(5000, 4000, seed=9)
    x = synth.normal(4000, 1, 10).ravel()
    y_ref = oracle.spmv(rp, ci, v, x)
    results, errors = [None] * 4, []

    def worker(i):
        try:
            A, B = jobs[i]
            dA, dB, dC = ctx.from_numpy(A), ctx.from_numpy(B), ctx.alloc(8 * m * n)
            S = f4j.CsrMatrix((5000, 4000), v, rp, ci)
            for _ in range(10):
                check(ctx.lib.f4j_dgemm(ctx.handle, m, n, k, dA.handle, 0, dB.handle, 0, dC.handle,
                                        _lib.MODE_SPLIT, None))
                assert np.array_equal(S.mult(f4j.Vector(x)).data, y_ref)
                C = np.empty((m, n))
                check(ctx.lib.f4j_dgemm_host(ctx.handle, m, n, k, A.ctypes.data, 0, B.ctypes.data, 0,
                                             C.ctypes.data, _lib.MODE_SPLIT, None))
                assert np.array_equal(C, refs[i])
            results[i] = dC.to_numpy(np.float64, m * n).reshape(m, n)
        except Exception as e:  # reported below
            errors.append(repr(e))

    threads = [threading.Thread(target=worker, args=(i,)) for i in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors, errors
    for i in range(4):
        assert np.array_equal(results[i], refs[i])


@pytest.mark.parametrize("n", [96, 300])
def test_symm_pos_def_product_chain(f4j, oracle, n):
    """RandomDenseTensor.randomSymmPosDefMatrix (RandomDenseTensor.java:649-653) forms
    Q.T().mult(D).mult(Q) from a random diagonal D and orthogonal Q: two chained products whose
    intermediate stays a device handle. Q and D come from a seeded generator here (the reference's
    own generator is not reproducible from its seed)."""
    rng = np.random.default_rng(n)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    D = np.diag(rng.random(n))
    got = f4j.Matrix(Q).T().mult(f4j.Matrix(D), mode="exact").mult(f4j.Matrix(Q), mode="exact").toNumpy()
    ref = oracle.dgemm(oracle.dgemm(np.ascontiguousarray(Q.T), D), Q)
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))
    assert np.all(np.linalg.eigvalsh((got + got.T) / 2) > -1e-12)


@pytest.mark.parametrize("n", [64, 200])
def test_herm_pos_def_product_chain(f4j, oracle, n):
    """RandomDenseTensor.randomHermPosDefMatrix (RandomDenseTensor.java:666-670) forms
    U.H().mult(D).mult(U): a Complex128 x real product (CMatrix.mult(Matrix)) followed by a
    Complex128 product, each bit-identical to the oracle's k-ascending restatement."""
    rng = np.random.default_rng(1000 + n)
    U, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    D = np.diag(rng.random(n))
    UH = np.ascontiguousarray(U.conj().T)
    got = f4j.CMatrix(U).H().mult(f4j.Matrix(D), mode="exact").mult(f4j.CMatrix(U), mode="exact").toNumpy()
    ref = oracle.zgemm(oracle.zgemm(UH, D.astype(np.complex128)), U)
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))
    assert np.max(np.abs(got - got.conj().T)) < 1e-13
