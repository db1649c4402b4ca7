"""The no-allocation split GEMM entry point (f4j_dgemm_split_noalloc).

Callers such as engines that own a fixed device-memory pool, or JVM hosts that
only hand over buffers they already hold, cannot allocate device memory; this
entry point takes its scratch from a static array in the library instead.  It must agree with the allocating f4j_dgemm split path
within the same componentwise bound the other tests use, on two calls in a row
(the shared scratch keeps the previous call's contents).  Collected last so a
failure here never hides another test's result.
"""
import ctypes

import numpy as np
import pytest

from conftest import assert_within_bound

pytestmark = pytest.mark.gpu


def _noalloc(f4j, dA, dB, dC, m, n, k, opA=0, opB=0):
    ctx = f4j.default_context()
    s = ctypes.c_int32(0)
    stream = ctx.lib.f4j_get_stream(ctx.handle)  # same stream as the download that follows
    rc = ctx.lib.f4j_dgemm_split_noalloc(m, n, k, ctx.lib.f4j_buf_device_ptr(dA.handle), opA,
                                         ctx.lib.f4j_buf_device_ptr(dB.handle), opB,
                                         ctx.lib.f4j_buf_device_ptr(dC.handle), stream, ctypes.byref(s))
    from flag4j_gb300.device import check
    check(rc)
    check(ctx.lib.f4j_sync(ctx.handle))
    return s.value


def _alloc_path(f4j, dA, dB, dC, m, n, k, opA=0, opB=0):
    from flag4j_gb300 import _lib
    from flag4j_gb300.device import check
    ctx = f4j.default_context()
    check(ctx.lib.f4j_dgemm(ctx.handle, m, n, k, dA.handle, opA, dB.handle, opB, dC.handle, _lib.MODE_SPLIT, None))
    return dC.to_numpy(np.float64, m * n).reshape(m, n)


def test_noalloc_matches_allocating_split_twice(f4j, oracle):
    from flag4j_gb300 import synth
    ctx = f4j.default_context()
    # the allocating path splits K across CTAs for these few-tile shapes (16, 8 and 2 chunks); the
    # no-allocation path runs the same chunks in turn, and the int64 sums make the two bitwise equal
    cases = [(384, 256, 1000, 0, 0, 8), (200, 300, 512, 1, 1, 0), (1024, 1024, 1024, 0, 0, 8)]
    for (m, n, k, opA, opB, phi) in cases:
        As = synth.scaled(m, k, phi, 3, "row") if opA == 0 else synth.scaled(k, m, phi, 3, "col")
        Bs = synth.scaled(k, n, phi, 4, "col") if opB == 0 else synth.scaled(n, k, phi, 4, "row")
        dA, dB = ctx.from_numpy(As), ctx.from_numpy(Bs)
        dC1, dC2 = ctx.alloc(8 * m * n), ctx.alloc(8 * m * n)
        ref_path = _alloc_path(f4j, dA, dB, dC1, m, n, k, opA, opB)
        s = _noalloc(f4j, dA, dB, dC2, m, n, k, opA, opB)
        got = dC2.to_numpy(np.float64, m * n).reshape(m, n)
        assert 2 <= s <= 12
        A = As if opA == 0 else As.T.copy()
        B = Bs if opB == 0 else Bs.T.copy()
        ref = oracle.dgemm(A, B)
        assert_within_bound(got, ref, oracle.absgemm(A, B), k, "noalloc vs oracle")
        assert np.array_equal(got, ref_path), "noalloc vs f4j_dgemm split"


def test_noalloc_size_limit_is_the_documented_formula(f4j, oracle):
    """12 (m + n) roundup(k, 64) + 24 (m + n) + 16384 <= 32 MiB: 1024 x 1024 x 1344 is the
    largest k at m = n = 1024 that fits (and matches f4j_dgemm); 1408 is rejected."""
    from flag4j_gb300 import _lib, synth
    ctx = f4j.default_context()
    limit = 32 << 20
    need = lambda m, n, k: 12 * (m + n) * (-(-k // 64) * 64) + 24 * (m + n) + 16384
    assert need(1024, 1024, 1344) <= limit < need(1024, 1024, 1408)
    big = ctx.alloc(8)
    p = ctx.lib.f4j_buf_device_ptr(big.handle)
    rc = ctx.lib.f4j_dgemm_split_noalloc(1024, 1024, 1408, p, 0, p, 0, p, None, None)
    assert rc == _lib.F4J_ERR_ARG and "static limit" in _lib.last_error()
    m = n = 1024
    k = 1344
    As, Bs = synth.scaled(m, k, 8, 5, "row"), synth.scaled(k, n, 8, 6, "col")
    dA, dB = ctx.from_numpy(As), ctx.from_numpy(Bs)
    dC1, dC2 = ctx.alloc(8 * m * n), ctx.alloc(8 * m * n)
    ref_path = _alloc_path(f4j, dA, dB, dC1, m, n, k)
    assert 2 <= _noalloc(f4j, dA, dB, dC2, m, n, k) <= 12
    assert np.array_equal(dC2.to_numpy(np.float64, m * n).reshape(m, n), ref_path)


def test_noalloc_rejects_nonfinite_then_recovers(f4j):
    from flag4j_gb300 import _lib, synth
    ctx = f4j.default_context()
    A = np.ones((64, 64))
    A[1, 1] = np.inf
    dA, dB, dC = ctx.from_numpy(A), ctx.from_numpy(np.ones((64, 64))), ctx.alloc(8 * 64 * 64)
    rc = ctx.lib.f4j_dgemm_split_noalloc(64, 64, 64, ctx.lib.f4j_buf_device_ptr(dA.handle), 0,
                                         ctx.lib.f4j_buf_device_ptr(dB.handle), 0,
                                         ctx.lib.f4j_buf_device_ptr(dC.handle), None, None)
    assert rc == _lib.F4J_ERR_ARG and "NaN or Inf" in _lib.last_error()
    # the next call clears the shared scratch's flags and computes normally
    As, Bs = synth.uniform(64, 64, 7), synth.uniform(64, 64, 8)
    dA2, dB2 = ctx.from_numpy(As), ctx.from_numpy(Bs)
    ref_path = _alloc_path(f4j, dA2, dB2, ctx.alloc(8 * 64 * 64), 64, 64, 64)
    _noalloc(f4j, dA2, dB2, dC, 64, 64, 64)
    assert np.array_equal(dC.to_numpy(np.float64, 64 * 64).reshape(64, 64), ref_path)
