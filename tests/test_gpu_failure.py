"""Failure detection on the GPU without a fault: a device wait that nothing
completes gives up after its limit, records its code in the context's status
word, and the host reads it at the next f4j_sync as F4J_ERR_TIMEOUT; the
context stays usable afterwards."""
import ctypes
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_context_stays_usable(f4j, oracle):
    from flag4j_gb300 import _lib
    ctx = f4j.default_context()
    lib = ctx.lib
    assert lib.f4j_sync(ctx.handle) == 0
    t0 = time.time()
    assert lib.f4j_selftest_wait(ctx.handle, 20000) == 0  # a 20 ms limit
    rc = lib.f4j_sync(ctx.handle)
    elapsed = time.time() - t0
    assert rc == -6  # F4J_ERR_TIMEOUT
    msg = lib.f4j_last_error().decode()
    assert "gave up" in msg and "99" in msg
    assert 0.015 <= elapsed < 5.0
    # the status was consumed, and products still run on the same context
    assert lib.f4j_sync(ctx.handle) == 0
    A = np.arange(12.0).reshape(3, 4)
    B = np.arange(8.0).reshape(4, 2)
    C = f4j.Matrix(A).mult(f4j.Matrix(B), mode="exact").toNumpy()
    assert np.array_equal(C, oracle.dgemm(A, B))


def test_selftest_limit_is_checked(f4j):
    ctx = f4j.default_context()
    assert ctx.lib.f4j_selftest_wait(ctx.handle, 10) == -1
    assert ctx.lib.f4j_selftest_wait(ctx.handle, 10_000_000) == -1
