"""ctypes front end for the CPU oracle (f4j_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and the benchmark's
CPU-baseline leg as the checker.  The product library never imports this.

``build()`` compiles f4j_oracle.c with gcc -O3 -ffp-contract=off so every
product and sum rounds separately, as the JVM does.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "f4j_oracle.c")
LIB = os.path.join(HERE, "libf4j_oracle.so")
CFLAGS = ["-O3", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread", "-std=c11"]

_lock = threading.Lock()
_lib = None


def _digest():
    """SHA-256 of the source, the flags and the machine: the stamp a reusable build carries."""
    import hashlib
    import platform
    h = hashlib.sha256()
    with open(SRC, "rb") as f:
        h.update(f.read())
    h.update(repr((CFLAGS, platform.machine())).encode())
    return h.hexdigest()


def build(force=False):
    """Compile the oracle shared library (a second or two) unless the stamp
    beside it matches this source, these flags and this machine."""
    stamp = LIB + ".sha256"
    digest = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", *CFLAGS, SRC, "-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    with open(stamp + ".tmp%d" % os.getpid(), "w") as f:
        f.write(digest + "\n")
    os.replace(stamp + ".tmp%d" % os.getpid(), stamp)
    return LIB


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB)
            i64, i32, p = ctypes.c_int64, ctypes.c_int, ctypes.c_void_p
            sig = {
                "orc_dgemm": [i64, i64, i64, p, p, p, i32],
                "orc_dgemm_abt": [i64, i64, i64, p, p, p, i32],
                "orc_dgemv_blocked": [i64, i64, p, p, p, i64],
                "orc_zgemm": [i64, i64, i64, p, p, p, i32],
                "orc_rzgemm": [i64, i64, i64, p, p, p, i32],
                "orc_zrgemm": [i64, i64, i64, p, p, p, i32],
                "orc_spmm_rz": [i64, i64, p, p, p, p, p, i32],
                "orc_zspmm": [i64, i64, p, p, p, p, p, i32],
                "orc_spmv": [i64, p, p, p, p, p, i32],
                "orc_spmm": [i64, i64, p, p, p, p, p, i32],
                "orc_coo_to_csr": [i64, i64, p, p],
                "orc_coo_sort": [i64, p, p, p, p],
                "orc_csr_transpose": [i64, i64, p, p, p, p, p, p, p],
                "orc_sddmm": [i64, i64, p, p, p, p, p],
                "orc_truth_sampled": [i64, p, i64, i32, p, i64, i32, i32, i64, p, p, p, p, p],
                "orc_absgemm": [i64, i64, i64, p, p, p, i32],
                "orc_spgemm_dense": [i64, i64, p, p, p, p, p, p, p],
                "orc_spgemm_csr": [i64, i64, p, p, p, p, p, p, p, p, p],
                "orc_spgemm_dense_z": [i32, i32, i64, i64, p, p, p, p, p, p, p],
                "orc_spgemm_csr_z": [i32, i32, i64, i64, p, p, p, p, p, p, p, p, p],
            }
            for name, args in sig.items():
                f = getattr(L, name)
                f.argtypes = args
                f.restype = None
            L.orc_spgemm_csr.restype = ctypes.c_int64
            L.orc_spgemm_csr_z.restype = ctypes.c_int64
            _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def threads_default():
    return os.cpu_count() or 1


# ------------------------------------------------------------- dense
def dgemm(A, B, threads=1):
    """RealDenseMatMult.reordered order (bit-identical to the Java kernels)."""
    A, B = _f64(A), _f64(B)
    m, k = A.shape
    k2, n = B.shape
    assert k == k2
    C = np.empty((m, n), np.float64)
    lib().orc_dgemm(m, n, k, _p(A), _p(B), _p(C), threads)
    return C


def dgemm_abt(A, Bt, threads=1):
    """RealDenseMatMultTranspose: A @ Bt.T with Bt given n x k."""
    A, Bt = _f64(A), _f64(Bt)
    m, k = A.shape
    n, k2 = Bt.shape
    assert k == k2
    C = np.empty((m, n), np.float64)
    lib().orc_dgemm_abt(m, n, k, _p(A), _p(Bt), _p(C), threads)
    return C


def dgemv_blocked(A, x, block=64):
    A, x = _f64(A), _f64(x)
    m, k = A.shape
    y = np.empty(m, np.float64)
    lib().orc_dgemv_blocked(m, k, _p(A), _p(x), _p(y), block)
    return y


def zgemm(A, B, threads=1):
    """DenseSemiringMatMult over Complex128 (complex128 numpy arrays)."""
    A = np.ascontiguousarray(A, dtype=np.complex128)
    B = np.ascontiguousarray(B, dtype=np.complex128)
    m, k = A.shape
    k2, n = B.shape
    assert k == k2
    C = np.empty((m, n), np.complex128)
    lib().orc_zgemm(m, n, k, _p(A), _p(B), _p(C), threads)
    return C


def rzgemm(A, B, threads=1):
    """Matrix.mult(CMatrix): real A (m x k) times complex B (k x n)."""
    A = _f64(A)
    B = np.ascontiguousarray(B, dtype=np.complex128)
    m, k = A.shape
    assert B.shape[0] == k
    n = B.shape[1]
    C = np.empty((m, n), np.complex128)
    lib().orc_rzgemm(m, n, k, _p(A), _p(B), _p(C), threads)
    return C


def zrgemm(A, B, threads=1):
    """CMatrix.mult(Matrix): complex A (m x k) times real B (k x n)."""
    A = np.ascontiguousarray(A, dtype=np.complex128)
    B = _f64(B)
    m, k = A.shape
    assert B.shape[0] == k
    n = B.shape[1]
    C = np.empty((m, n), np.complex128)
    lib().orc_zrgemm(m, n, k, _p(A), _p(B), _p(C), threads)
    return C


def absgemm(A, B, threads=1):
    A, B = _f64(A), _f64(B)
    m, k = A.shape
    n = B.shape[1]
    C = np.empty((m, n), np.float64)
    lib().orc_absgemm(m, n, k, _p(A), _p(B), _p(C), threads)
    return C


def truth_sampled(A, B, si, sj, opA=0, opB=0):
    """Compensated (Dot2) values of op(A) @ op(B) at (si, sj).

    Returns (hi, lo, absref); complex inputs return complex hi/lo and a complex
    absref whose real/imag parts bound the real/imag components.
    """
    cplx = np.iscomplexobj(A) or np.iscomplexobj(B)
    dt = np.complex128 if cplx else np.float64
    A = np.ascontiguousarray(A, dtype=dt)
    B = np.ascontiguousarray(B, dtype=dt)
    k = A.shape[1] if opA == 0 else A.shape[0]
    si = np.ascontiguousarray(si, dtype=np.int64)
    sj = np.ascontiguousarray(sj, dtype=np.int64)
    ns = len(si)
    hi = np.empty(ns, dt)
    lo = np.empty(ns, dt)
    ab = np.empty(ns, dt)
    lib().orc_truth_sampled(k, _p(A), A.shape[1], opA, _p(B), B.shape[1], opB, int(cplx), ns,
                            _p(si), _p(sj), _p(hi), _p(lo), _p(ab))
    return hi, lo, ab


# ------------------------------------------------------------- sparse
def spmv(rowptr, colidx, vals, x, threads=1):
    rowptr, colidx, vals, x = _i32(rowptr), _i32(colidx), _f64(vals), _f64(x)
    rows = len(rowptr) - 1
    y = np.empty(rows, np.float64)
    lib().orc_spmv(rows, _p(rowptr), _p(colidx), _p(vals), _p(x), _p(y), threads)
    return y


def spmm(rowptr, colidx, vals, X, threads=1):
    rowptr, colidx, vals, X = _i32(rowptr), _i32(colidx), _f64(vals), _f64(X)
    rows = len(rowptr) - 1
    nc = X.shape[1]
    Y = np.empty((rows, nc), np.float64)
    lib().orc_spmm(rows, nc, _p(rowptr), _p(colidx), _p(vals), _p(X), _p(Y), threads)
    return Y


def spgemm_dense(arp, aci, av, brp, bci, bv, n2):
    """CsrMatrix.mult(CsrMatrix): RealCsrMatMult.standard, dense (rows of A) x n2 result."""
    arp, aci, av, brp, bci, bv = _i32(arp), _i32(aci), _f64(av), _i32(brp), _i32(bci), _f64(bv)
    rows = len(arp) - 1
    C = np.empty((rows, n2), np.float64)
    lib().orc_spgemm_dense(rows, n2, _p(arp), _p(aci), _p(av), _p(brp), _p(bci), _p(bv), _p(C))
    return C


def spgemm_csr(arp, aci, av, brp, bci, bv, n2):
    """CsrMatrix.mult2Csr(CsrMatrix): RealCsrMatMult.standardAsSparse -> (rowptr, colidx, vals)."""
    arp, aci, av, brp, bci, bv = _i32(arp), _i32(aci), _f64(av), _i32(brp), _i32(bci), _f64(bv)
    rows = len(arp) - 1
    rp = np.empty(rows + 1, np.int32)
    nnz = lib().orc_spgemm_csr(rows, n2, _p(arp), _p(aci), _p(av), _p(brp), _p(bci), _p(bv), _p(rp), None, None)
    ci, v = np.empty(max(nnz, 1), np.int32), np.empty(max(nnz, 1), np.float64)
    lib().orc_spgemm_csr(rows, n2, _p(arp), _p(aci), _p(av), _p(brp), _p(bci), _p(bv), _p(rp), _p(ci), _p(v))
    return rp, ci[:nnz], v[:nnz]


def _csr_vals(v):
    """(kind, float64 storage): complex values interleaved."""
    v = np.asarray(v)
    if np.iscomplexobj(v):
        return 1, np.ascontiguousarray(v, np.complex128).view(np.float64)
    return 0, _f64(v)


def spgemm_dense_any(arp, aci, av, brp, bci, bv, n2):
    """CSR x CSR with a dense result for any mix of real / complex values (the complex variants
    RealComplexCsrMatMult.standard, SemiringCsrMatMult.standard; real x real as spgemm_dense)."""
    ak, av = _csr_vals(av)
    bk, bv = _csr_vals(bv)
    if not ak and not bk:
        return spgemm_dense(arp, aci, av, brp, bci, bv, n2)
    arp, aci, brp, bci = _i32(arp), _i32(aci), _i32(brp), _i32(bci)
    rows = len(arp) - 1
    C = np.empty((rows, n2), np.complex128)
    lib().orc_spgemm_dense_z(ak, bk, rows, n2, _p(arp), _p(aci), _p(av), _p(brp), _p(bci), _p(bv), _p(C))
    return C


def spgemm_csr_any(arp, aci, av, brp, bci, bv, n2):
    """CSR x CSR with a CSR result for any mix of real / complex values -> (rowptr, colidx, vals)."""
    ak, av = _csr_vals(av)
    bk, bv = _csr_vals(bv)
    if not ak and not bk:
        return spgemm_csr(arp, aci, av, brp, bci, bv, n2)
    arp, aci, brp, bci = _i32(arp), _i32(aci), _i32(brp), _i32(bci)
    rows = len(arp) - 1
    rp = np.empty(rows + 1, np.int32)
    args = (_p(arp), _p(aci), _p(av), _p(brp), _p(bci), _p(bv), _p(rp))
    nnz = lib().orc_spgemm_csr_z(ak, bk, rows, n2, *args, None, None)
    ci, v = np.empty(max(nnz, 1), np.int32), np.empty(max(nnz, 1), np.complex128)
    lib().orc_spgemm_csr_z(ak, bk, rows, n2, *args, _p(ci), _p(v))
    return rp, ci[:nnz], v[:nnz]


def spmm_rz(rowptr, colidx, vals, X, threads=1):
    """CsrMatrix.mult(CMatrix): real CSR times complex dense X (rows of S x ncols)."""
    rowptr, colidx, vals = _i32(rowptr), _i32(colidx), _f64(vals)
    X = np.ascontiguousarray(X, dtype=np.complex128)
    rows = len(rowptr) - 1
    nc = X.shape[1]
    Y = np.empty((rows, nc), np.complex128)
    lib().orc_spmm_rz(rows, nc, _p(rowptr), _p(colidx), _p(vals), _p(X), _p(Y), threads)
    return Y


def zspmm(rowptr, colidx, vals, X, threads=1):
    """CsrCMatrix.mult(CMatrix): complex CSR (complex vals) times complex dense X."""
    rowptr, colidx = _i32(rowptr), _i32(colidx)
    vals = np.ascontiguousarray(vals, dtype=np.complex128)
    X = np.ascontiguousarray(X, dtype=np.complex128)
    rows = len(rowptr) - 1
    nc = X.shape[1]
    Y = np.empty((rows, nc), np.complex128)
    lib().orc_zspmm(rows, nc, _p(rowptr), _p(colidx), _p(vals), _p(X), _p(Y), threads)
    return Y


def coo_to_csr(rows, rowidx):
    rowidx = _i32(rowidx)
    rowptr = np.empty(rows + 1, np.int32)
    lib().orc_coo_to_csr(rows, len(rowidx), _p(rowidx), _p(rowptr))
    return rowptr


def coo_sort(rowidx, colidx, vals):
    r, c, v = _i32(rowidx).copy(), _i32(colidx).copy(), _f64(vals).copy()
    perm = np.empty(len(r), np.int64)
    lib().orc_coo_sort(len(r), _p(r), _p(c), _p(v), _p(perm))
    return r, c, v, perm


def csr_transpose(rows, cols, rowptr, colidx, vals):
    rowptr, colidx, vals = _i32(rowptr), _i32(colidx), _f64(vals)
    nnz = int(rowptr[-1])
    trp = np.empty(cols + 1, np.int32)
    tci = np.empty(nnz, np.int32)
    tv = np.empty(nnz, np.float64)
    perm = np.empty(nnz, np.int32)
    lib().orc_csr_transpose(rows, cols, _p(rowptr), _p(colidx), _p(vals), _p(trp), _p(tci),
                            _p(tv), _p(perm))
    return trp, tci, tv, perm


def sddmm(rowptr, colidx, dC, X):
    rowptr, colidx, dC, X = _i32(rowptr), _i32(colidx), _f64(dC), _f64(X)
    out = np.empty(int(rowptr[-1]), np.float64)
    lib().orc_sddmm(len(rowptr) - 1, dC.shape[1], _p(rowptr), _p(colidx), _p(dC), _p(X), _p(out))
    return out
