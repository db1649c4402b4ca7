"""Config-file-driven dispatch, the per-result accuracy report, and the
non-square complex product on the GPU.

- F4J_MODE_AUTO follows ./configs/*.properties as Flag4j's dispatchers do
  (src/main/java/org/flag4j/linalg/ops/dispatch/ReDeMatMultDispatcher.java:157-171,
  Cm128DeMatMultDispatcher.java:155-170), plus the gpuGemmMode key.
- The accuracy report's sampled errors equal the oracle's double-double
  evaluation of the same entries (oracle.truth_sampled), and sit next to the
  plain FP64 bound and the plain DMMA product's own error.
- Non-square CMatrix.mult above the small threshold: Flag4j's kernels size the
  result array a.numRows * b.numRows (Cm128DeMatMultKernels.java:46-77), so the
  reference throws there (IllegalArgumentException from the CMatrix
  constructor when b.numRows > b.numCols, ArrayIndexOutOfBoundsException when
  b.numRows < b.numCols); this library returns the product, equal bit for bit
  to the reference's standard kernel (its small-size path, which sizes the
  result correctly).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

M64 = (1 << 64) - 1


def mix64(z):
    z = (z + 0x9E3779B97F4A7C15) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def sample_indices(m, n, samples, seed=0x5EED0F4A6D5EED):
    b = mix64(seed)
    si = np.array([mix64(b ^ (2 * s)) % m for s in range(samples)], np.int64)
    sj = np.array([mix64(b ^ (2 * s + 1)) % n for s in range(samples)], np.int64)
    return si, sj


@pytest.fixture()
def cfg(lib):
    from flag4j_gb300 import configs
    configs.reset()
    yield configs
    configs.reset()


def _dgemm(f4j, A, B, mode, rep=None, cplx=False):
    from flag4j_gb300 import _lib
    from flag4j_gb300.device import check
    ctx = f4j.default_context()
    m, k = A.shape
    n = B.shape[1]
    dA, dB = ctx.from_numpy(A), ctx.from_numpy(B)
    dC = ctx.alloc((16 if cplx else 8) * m * n)
    rep = rep if rep is not None else _lib.f4j_report()
    fn = ctx.lib.f4j_zgemm if cplx else ctx.lib.f4j_dgemm
    check(fn(ctx.handle, m, n, k, dA.handle, 0, dB.handle, 0, dC.handle, _lib.MODES[mode], ctypes.byref(rep)))
    C = dC.to_numpy(np.complex128 if cplx else np.float64, m * n).reshape(m, n)
    return C, rep


def test_auto_follows_the_configuration_files(f4j, oracle, cfg, tmp_path):
    from flag4j_gb300 import _lib, synth
    A, B = synth.uniform(300, 300, 1), synth.uniform(300, 300, 2)
    ref = oracle.dgemm(A, B)
    C, rep = _dgemm(f4j, A, B, "auto")
    assert rep.mode_used == _lib.MODE_SPLIT and rep.ref_kernel == _lib.REF_KERNELS.index("MT_REORD")
    d = tmp_path / "configs"
    d.mkdir()
    (d / "ReDeMatMult.properties").write_text("smallThreshold = 200000\n")
    cfg.load(d)
    C, rep = _dgemm(f4j, A, B, "auto")
    assert rep.mode_used == _lib.MODE_EXACT and np.array_equal(C, ref)   # the reference's bits
    (d / "ReDeMatMult.properties").write_text("gpuGemmMode = plain\n")
    cfg.load(d)
    C, rep = _dgemm(f4j, A, B, "auto")
    assert rep.mode_used == _lib.MODE_PLAIN
    (d / "ReDeMatMult.properties").unlink()
    (d / "GeneralConfigs.properties").write_text("gpuGemmMode = exact\n")
    cfg.load(d)
    Az = A + 1j * synth.uniform(300, 300, 3)
    Bz = B + 1j * synth.uniform(300, 300, 4)
    Cz, rep = _dgemm(f4j, Az, Bz, "auto", cplx=True)
    assert rep.mode_used == _lib.MODE_EXACT and np.array_equal(Cz, oracle.zgemm(Az, Bz))
    # the Python front end passes AUTO through, so Matrix.mult follows the files as well
    assert np.array_equal(f4j.Matrix(A).mult(f4j.Matrix(B)).toNumpy(), ref)


@pytest.mark.parametrize("cplx", [False, True])
def test_accuracy_report_matches_oracle_truth(f4j, oracle, cplx):
    from flag4j_gb300 import _lib, synth
    m, n, k = 700, 600, 900
    A = synth.scaled(m, k, 8, 5, "row", cplx=cplx)
    B = synth.scaled(k, n, 8, 6, "col", cplx=cplx)
    rep = _lib.f4j_report()
    rep.check_samples = 2048
    rep.check_flags = _lib.CHECK_PLAIN
    C, rep = _dgemm(f4j, A, B, "split", rep, cplx=cplx)
    assert rep.mode_used == _lib.MODE_SPLIT and rep.check_samples == 2048
    si, sj = sample_indices(m, n, 2048)
    hi, lo, absref = oracle.truth_sampled(A, B, si, sj)
    c = C[si, sj]
    if cplx:
        er = np.maximum(np.abs((c.real - hi.real) - lo.real), np.abs((c.imag - hi.imag) - lo.imag))
        rr = np.maximum(np.abs((c.real - hi.real) - lo.real) / absref.real,
                        np.abs((c.imag - hi.imag) - lo.imag) / absref.imag)
    else:
        er = np.abs((c - hi) - lo)
        rr = er / absref
    assert rep.max_abs_err == pytest.approx(float(er.max()), rel=1e-6, abs=1e-300)
    assert rep.max_rel_err == pytest.approx(float(rr.max()), rel=1e-6, abs=1e-300)
    assert rep.plain_bound_rel == (2 if cplx else 1) * k * 2.0 ** -53
    assert 0 <= rep.max_rel_err <= rep.plain_bound_rel
    assert 0 <= rep.plain_max_rel_err <= rep.plain_bound_rel
    assert rep.max_rel_err <= rep.plain_max_rel_err   # the split product is the more accurate here


def test_accuracy_report_is_opt_in_and_host_entry_agrees(f4j):
    from flag4j_gb300 import _lib, synth
    from flag4j_gb300.device import check
    A, B = synth.uniform(512, 384, 7), synth.uniform(384, 640, 8)
    C0, rep0 = _dgemm(f4j, A, B, "split")
    assert rep0.max_abs_err == -1 and rep0.plain_max_abs_err == -1 and rep0.check_samples == 0
    rep = _lib.f4j_report()
    rep.check_samples = 1000
    C1, rep1 = _dgemm(f4j, A, B, "split", rep)
    assert np.array_equal(C0, C1) and rep1.max_abs_err >= 0 and rep1.plain_max_abs_err == -1
    ctx = f4j.default_context()
    Ch = np.empty((512, 640))
    reph = _lib.f4j_report()
    reph.check_samples = 1000
    check(ctx.lib.f4j_dgemm_host(ctx.handle, 512, 640, 384, A.ctypes.data, 0, B.ctypes.data, 0, Ch.ctypes.data,
                                 _lib.MODE_SPLIT, ctypes.byref(reph)))
    assert np.array_equal(Ch, C1)
    assert reph.max_abs_err == rep1.max_abs_err and reph.max_rel_err == rep1.max_rel_err


@pytest.mark.parametrize("shape", [(100, 80, 50), (90, 40, 120), (300, 200, 260)])
def test_non_square_complex_product_above_small_threshold(f4j, oracle, shape):
    """Row a7: the reference mis-sizes its result array here and throws; this
    library returns the product: bit-identical to the reference's order in
    EXACT mode, and within 2 (2k) u |A||B| per part in AUTO (the split path
    for the largest shape)."""
    from flag4j_gb300 import _lib, synth
    from conftest import U
    m, k, n = shape
    assert m * k + k * n >= 2450 and k != n
    A = synth.uniform(m, k, 1) + 1j * synth.uniform(m, k, 2)
    B = synth.uniform(k, n, 3) + 1j * synth.uniform(k, n, 4)
    ref = oracle.zgemm(A, B)
    got = f4j.CMatrix(A).mult(f4j.CMatrix(B), mode="exact").toNumpy()
    assert got.shape == (m, n) and np.array_equal(got, ref)
    rep = {}
    auto = f4j.CMatrix(A).mult(f4j.CMatrix(B), report=rep).toNumpy()
    assert auto.shape == (m, n)
    ab_re = np.abs(A.real) @ np.abs(B.real) + np.abs(A.imag) @ np.abs(B.imag)
    ab_im = np.abs(A.real) @ np.abs(B.imag) + np.abs(A.imag) @ np.abs(B.real)
    assert np.all(np.abs(auto.real - ref.real) <= 2 * (2 * k) * U * ab_re)
    assert np.all(np.abs(auto.imag - ref.imag) <= 2 * (2 * k) * U * ab_im)
    if shape == (300, 200, 260):
        assert rep["mode_used"] == _lib.MODE_SPLIT
