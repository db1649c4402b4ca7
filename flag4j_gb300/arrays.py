"""Flag4j's product-path types over the GB300 library.

Mirrors the public surface of the reference types that reach the products
(paths within the Flag4j project):
  Matrix     src/main/java/org/flag4j/arrays/dense/Matrix.java
             (mult :638-640, multTranspose :655-663, mult(Vector) :1406-1407,
              toCoo :1615-1637, toCsr :1645-1647)
  CMatrix    src/main/java/org/flag4j/arrays/dense/CMatrix.java (mult :463-465)
  Vector     src/main/java/org/flag4j/arrays/dense/Vector.java
  CsrMatrix  src/main/java/org/flag4j/arrays/sparse/CsrMatrix.java
             (ctor :175-185, mult(Vector) :1170-1171, T() :1431-1433, mult(Matrix) :1498-1499)
  CooMatrix  src/main/java/org/flag4j/arrays/sparse/CooMatrix.java
             (toCsr :457-470, sortIndices :476-479)
Every product runs on the GPU through libflag4j_cuda.so; host arrays are
uploaded on first use and results stay on the device until read, so chained
products never round-trip through host memory.
"""
import ctypes

import numpy as np

from . import _lib
from .device import (IllegalArgumentException, LinearAlgebraException, check, default_context,
                     gemm_mode)


class Shape(tuple):
    """org.flag4j.arrays.Shape: dims tuple; str() as '(r, c)' (Shape.java:519-526)."""

    def __new__(cls, *dims):
        if len(dims) == 1 and isinstance(dims[0], (tuple, list)):
            dims = tuple(dims[0])
        return super().__new__(cls, tuple(int(d) for d in dims))

    def get(self, i):
        return self[i]

    def getRank(self):
        return len(self)

    def __str__(self):
        return "(" + ", ".join(str(d) for d in self) + ")"

    __repr__ = __str__


def mat_mult_shape_error(s1, s2):
    """ErrorMessages.matMultShapeErrMsg (src/main/java/org/flag4j/util/ErrorMessages.java:52-53)."""
    return LinearAlgebraException("Cannot multiply matrices/vector with shapes %s and %s." % (s1, s2))


def ensure_mat_mult_shapes(s1, s2):
    """ValidateParameters.ensureMatMultShapes (src/main/java/org/flag4j/util/ValidateParameters.java:62-67)."""
    r2 = s2.getRank()
    if s1.getRank() != 2 or (r2 != 2 and r2 != 1) or s1.get(1) != s2.get(0):
        raise mat_mult_shape_error(s1, s2)


def ensure_all_equal(*values):
    """ValidateParameters.ensureAllEqual (ValidateParameters.java:135-139)."""
    for a, b in zip(values, values[1:]):
        if a != b:
            raise IllegalArgumentException(
                "Expecting values to be equal but got: [" + ", ".join(str(v) for v in values) + "]")


def _nan_equal(a, b):
    """RealDenseEquals.tensorEquals: element-wise ==, NaN equal to NaN."""
    return bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


class _Dense:
    """Host/device backed dense array (row-major)."""

    _dtype = np.float64

    def _init_host(self, shape, data):
        self.shape = shape
        self._host = np.ascontiguousarray(data, dtype=self._dtype).reshape(-1)
        self._dev = None
        self._ctx = None

    @classmethod
    def _from_device(cls, shape, buf, ctx):
        obj = cls.__new__(cls)
        obj.shape = shape
        obj._host = None
        obj._dev = buf
        obj._ctx = ctx
        return obj

    def dataLength(self):
        return int(np.prod(self.shape)) if len(self.shape) else 0

    @property
    def data(self):
        if self._host is None:
            self._host = self._dev.to_numpy(self._dtype, self.dataLength())
        return self._host

    def device(self, ctx=None):
        """The device buffer holding this array (uploaded on first use)."""
        ctx = ctx or self._ctx or default_context()
        if self._dev is None or self._ctx is not ctx:
            self._dev = ctx.from_numpy(self._host if self.dataLength() else np.zeros(1, self._dtype))
            self._ctx = ctx
        return self._dev


class Vector(_Dense):
    def __init__(self, entries):
        arr = np.asarray(entries, dtype=np.float64).reshape(-1)
        self._init_host(Shape(arr.size), arr)

    @property
    def size(self):
        return self.shape[0]

    def __eq__(self, other):
        return isinstance(other, Vector) and self.shape == other.shape and _nan_equal(self.data, other.data)

    __hash__ = None


class CVector(_Dense):
    """Complex128 dense vector (interleaved re/im on the device)."""

    _dtype = np.complex128

    def __init__(self, entries):
        arr = np.asarray(entries, dtype=np.complex128).reshape(-1)
        self._init_host(Shape(arr.size), arr)

    @property
    def size(self):
        return self.shape[0]

    def __eq__(self, other):
        return isinstance(other, CVector) and self.shape == other.shape and _nan_equal(self.data, other.data)

    __hash__ = None


class Matrix(_Dense):
    """Real dense matrix: Matrix(double[][]), Matrix(Shape, double...), Matrix(rows, cols)."""

    def __init__(self, *args):
        if len(args) == 1:
            arr = np.asarray(args[0], dtype=np.float64)
            if arr.ndim != 2:
                arr = arr.reshape(len(args[0]), -1)
            self._init_host(Shape(arr.shape), arr)
        elif len(args) == 2 and isinstance(args[0], Shape):
            shape = args[0]
            data = np.asarray(args[1], dtype=np.float64).reshape(-1)
            if data.size != shape.get(0) * shape.get(1):
                raise IllegalArgumentException("data length does not match shape %s" % (shape,))
            self._init_host(shape, data)
        elif len(args) == 2:
            self._init_host(Shape(args[0], args[1]), np.zeros(int(args[0]) * int(args[1])))
        else:
            raise IllegalArgumentException("unsupported Matrix constructor arguments")

    @property
    def numRows(self):
        return self.shape[0]

    @property
    def numCols(self):
        return self.shape[1]

    def toNumpy(self):
        return self.data.reshape(self.shape)

    def T(self):
        return Matrix(self.toNumpy().T.copy())

    def mult(self, b, mode=None, report=None):
        """Matrix.mult(Matrix) / Matrix.mult(Vector) on the GPU."""
        if isinstance(b, Vector):
            ensure_mat_mult_shapes(self.shape, b.shape)
            bm = Matrix._from_device(Shape(b.size, 1), b.device(), b._ctx)
            out = _gemm(self, bm, _lib.OP_N, _lib.OP_N, self.numRows, 1, self.numCols, mode, report)
            return Vector._from_device(Shape(self.numRows), out._dev, out._ctx)
        if isinstance(b, (CMatrix, CVector)):
            # Matrix.mult(CMatrix / CVector) (MatrixMultiplyDispatcher.java:71-200): every variant sums
            # a[i][k] * b[k][j] per real / imaginary part in ascending k, so the product is the real
            # GEMM of this matrix with b's interleaved storage read as a real k x 2n matrix
            vec = isinstance(b, CVector)
            n = 1 if vec else b.numCols
            ensure_mat_mult_shapes(self.shape, Shape(b.size, 1) if vec else b.shape)
            ctx = self._ctx or b._ctx or default_context()
            out = _gemm_bufs(ctx, False, self.numRows, 2 * n, self.numCols, self.device(ctx), _lib.OP_N,
                             b.device(ctx), _lib.OP_N, mode, report)
            return (CVector._from_device(Shape(self.numRows), out, ctx) if vec
                    else CMatrix._from_device(Shape(self.numRows, n), out, ctx))
        ensure_mat_mult_shapes(self.shape, b.shape)
        return _gemm(self, b, _lib.OP_N, _lib.OP_N, self.numRows, b.numCols, self.numCols, mode, report)

    def multTranspose(self, b, mode=None, report=None):
        """Matrix.multTranspose: this * b^T through a transposed operand (no copy)."""
        ensure_all_equal(self.numCols, b.numCols)
        return _gemm(self, b, _lib.OP_N, _lib.OP_T, self.numRows, b.numRows, self.numCols, mode, report)

    def toCoo(self):
        """Matrix.toCoo: nonzeros in row-major order (Matrix.java:1615-1637)."""
        a = self.toNumpy()
        r, c = np.nonzero(a != 0.0)
        return CooMatrix(self.shape, a[r, c], r.astype(np.int32), c.astype(np.int32))

    def toCsr(self):
        return self.toCoo().toCsr()

    def __eq__(self, other):
        return isinstance(other, Matrix) and self.shape == other.shape and _nan_equal(self.data, other.data)

    __hash__ = None


class CMatrix(_Dense):
    """Complex128 dense matrix (interleaved re/im on the device)."""

    _dtype = np.complex128

    def __init__(self, *args):
        if len(args) == 1:
            arr = np.asarray(args[0], dtype=np.complex128)
            self._init_host(Shape(arr.shape), arr)
        elif len(args) == 2 and isinstance(args[0], Shape):
            self._init_host(args[0], np.asarray(args[1], dtype=np.complex128).reshape(-1))
        else:
            raise IllegalArgumentException("unsupported CMatrix constructor arguments")

    @property
    def numRows(self):
        return self.shape[0]

    @property
    def numCols(self):
        return self.shape[1]

    def toNumpy(self):
        return self.data.reshape(self.shape)

    def T(self):
        return CMatrix(self.toNumpy().T.copy())

    def H(self):
        return CMatrix(self.toNumpy().conj().T.copy())

    def toCsr(self):
        """CMatrix.toCsr: the nonzero entries in row-major order as a CsrCMatrix."""
        a = self.toNumpy()
        r, c = np.nonzero(a != 0)
        rp = np.zeros(self.numRows + 1, np.int32)
        np.cumsum(np.bincount(r, minlength=self.numRows), out=rp[1:])
        return CsrCMatrix(self.shape, a[r, c], rp, c.astype(np.int32))

    def mult(self, b, mode=None, report=None):
        """CMatrix.mult(CMatrix / CVector / Matrix / Vector) on the GPU.

        A real operand (CMatrix.mult(Matrix), MatrixMultiplyDispatcher.java:201-260) is promoted to
        complex with zero imaginary parts: each extra product is a signed zero, which leaves every
        k-ascending sum unchanged, so EXACT mode stays bit-identical."""
        vec = isinstance(b, (Vector, CVector))
        if isinstance(b, (Matrix, Vector)):
            arr = b.toNumpy() if isinstance(b, Matrix) else b.data
            b = (CVector if vec else CMatrix)(np.asarray(arr, dtype=np.complex128))
        n = 1 if vec else b.numCols
        ensure_mat_mult_shapes(self.shape, Shape(b.size, 1) if vec else b.shape)
        ctx = self._ctx or b._ctx or default_context()
        out = _gemm_bufs(ctx, True, self.numRows, n, self.numCols, self.device(ctx), _lib.OP_N, b.device(ctx),
                         _lib.OP_N, mode, report)
        return (CVector._from_device(Shape(self.numRows), out, ctx) if vec
                else CMatrix._from_device(Shape(self.numRows, n), out, ctx))

    def multTranspose(self, b, mode=None, report=None):
        """CMatrix.multTranspose (AbstractDenseSemiringMatrix.java:330-334 ->
        DenseSemiringMatMultTranspose, k ascending): this * b^T, b read transposed in place."""
        ensure_all_equal(self.numCols, b.numCols)
        return _gemm(self, b, _lib.OP_N, _lib.OP_T, self.numRows, b.numRows, self.numCols, mode, report)

    def __eq__(self, other):
        return isinstance(other, CMatrix) and self.shape == other.shape and _nan_equal(self.data, other.data)

    __hash__ = None


def _gemm_bufs(ctx, cplx, m, n, k, abuf, opA, bbuf, opB, mode, report):
    """f4j_zgemm / f4j_dgemm on device buffers; returns the new output buffer."""
    out = ctx.alloc(max(m * n * (16 if cplx else 8), 8))
    rep = _lib.f4j_report()
    fn = ctx.lib.f4j_zgemm if cplx else ctx.lib.f4j_dgemm
    md = gemm_mode() if mode is None else _lib.MODES.get(mode, mode)
    check(fn(ctx.handle, m, n, k, abuf.handle, opA, bbuf.handle, opB, out.handle, md, ctypes.byref(rep)))
    if report is not None:
        report.update(rep.as_dict())
    return out


def _gemm(a, b, opA, opB, m, n, k, mode, report):
    ctx = a._ctx or b._ctx or default_context()
    cplx = isinstance(a, CMatrix)
    out = _gemm_bufs(ctx, cplx, m, n, k, a.device(ctx), opA, b.device(ctx), opB, mode, report)
    cls = CMatrix if cplx else Matrix
    return cls._from_device(Shape(m, n), out, ctx)


# ------------------------------------------------------------------ sparse
def validate_csr(shape, nnz, row_pointers, col_indices):
    """SparseValidation.validateCsr (src/main/java/org/flag4j/arrays/sparse/SparseValidation.java:151-206)."""
    rows, cols = shape
    if nnz > rows * cols:
        raise IllegalArgumentException(
            "The number of non-zero entries cannot be greater than the total number of entries in the matrix "
            "but got nnz=%d and totalEntries=%d" % (nnz, rows * cols))
    if len(row_pointers) != rows + 1:
        raise IllegalArgumentException("Expecting rowPointers to have length (numRows + 1)=%d but got "
                                       "rowPointers.length=%d" % (rows + 1, len(row_pointers)))
    if nnz != len(col_indices):
        raise IllegalArgumentException("The number of non-zero entries must match the number of  column indices "
                                       "but got nnz=%d and colIndices.length=%d" % (nnz, len(col_indices)))
    rp = np.asarray(row_pointers, dtype=np.int64)
    if rows:
        # rows are checked in order: negative start first, then decreasing pointers
        bad_rows = np.nonzero((rp[:-1] < 0) | (rp[:-1] > rp[1:]))[0]
        if bad_rows.size:
            i = int(bad_rows[0])
            if rp[i] < 0:
                raise IllegalArgumentException("All rowPointers must be positive but got %d at index %d."
                                               % (rp[i], i))
            raise IllegalArgumentException("rowPointers must be monotonically increasing but got values %d and %d "
                                           "at indices %d and %d." % (rp[i], rp[i + 1], i, i + 1))
        ci = np.asarray(col_indices, dtype=np.int64)
        lo, hi = int(rp[0]), min(int(rp[-1]), len(ci))
        bad = np.nonzero((ci[lo:hi] < 0) | (ci[lo:hi] >= cols))[0]
        if bad.size:
            raise IllegalArgumentException("Invalid column index [%d] encountered for CSR matrix of shape %s"
                                           % (ci[lo + bad[0]], shape))
        seen = int(rp[-1] - rp[0])
        if seen != nnz:
            raise IllegalArgumentException("rowIndices specifies %d elements but nnz=%d. These values must be equal."
                                           % (seen, nnz))


class CsrMatrix:
    """CSR matrix: CsrMatrix(Shape, double[] data, int[] rowPointers, int[] colIndices)."""

    _vdtype = np.float64

    def __init__(self, shape, data, row_pointers, col_indices, validate=True):
        self.shape = Shape(shape)
        self._data = np.ascontiguousarray(data, dtype=self._vdtype).reshape(-1)
        self._rp = np.ascontiguousarray(row_pointers, dtype=np.int32).reshape(-1)
        self._ci = np.ascontiguousarray(col_indices, dtype=np.int32).reshape(-1)
        self.nnz = int(self._data.size)
        if validate:
            validate_csr(self.shape, self.nnz, self._rp, self._ci)
        self._handle = None
        self._bufs = None
        self._ctx = None

    @classmethod
    def _from_handle(cls, shape, nnz, handle, bufs, ctx):
        obj = cls.__new__(cls)
        obj.shape = Shape(shape)
        obj.nnz = int(nnz)
        obj._data = obj._rp = obj._ci = None
        obj._handle = handle
        obj._bufs = bufs
        obj._ctx = ctx
        return obj

    numRows = property(lambda self: self.shape[0])
    numCols = property(lambda self: self.shape[1])

    def _download(self):
        rp, ci, v = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        check(self._ctx.lib.f4j_csr_buffers(self._handle, ctypes.byref(rp), ctypes.byref(ci), ctypes.byref(v)))
        L, h = self._ctx.lib, self._ctx.handle
        self._rp = np.empty(self.numRows + 1, np.int32)
        self._ci = np.empty(self.nnz, np.int32)
        self._data = np.empty(self.nnz, self._vdtype)
        for buf, arr in ((rp, self._rp), (ci, self._ci), (v, self._data)):
            if arr.nbytes:
                check(L.f4j_buf_download(h, buf, arr.ctypes.data, arr.nbytes, 0))

    @property
    def data(self):
        if self._data is None:
            self._download()
        return self._data

    @property
    def rowPointers(self):
        if self._rp is None:
            self._download()
        return self._rp

    @property
    def colIndices(self):
        if self._ci is None:
            self._download()
        return self._ci

    def handle(self, ctx=None):
        """The device f4j_csr handle (uploaded on first use)."""
        ctx = ctx or self._ctx or default_context()
        if self._handle is None or self._ctx is not ctx:
            rp = ctx.from_numpy(self._rp)
            ci = ctx.from_numpy(self._ci if self.nnz else np.zeros(1, np.int32))
            v = ctx.from_numpy(self._data if self.nnz else np.zeros(1, self._vdtype))
            h = ctypes.c_void_p()
            check(ctx.lib.f4j_csr_wrap(ctx.handle, self.numRows, self.numCols, self.nnz, rp.handle, ci.handle,
                                       v.handle, 0, ctypes.byref(h)))
            self._handle, self._bufs, self._ctx = h, (rp, ci, v), ctx
        return self._handle

    def mult(self, b, mode=None, report=None):
        """CsrMatrix.mult(Vector) (IllegalArgumentException on size mismatch) and
        CsrMatrix.mult(Matrix) (LinearAlgebraException on shape mismatch).

        mode "exact" (the default) keeps the reference's rounding: each product and
        each running sum rounded, in storage order.  mode "fma" fuses them
        (fma(v, x, acc), same order), within |y - y_ref| <= 2 k u |S||x|; it applies
        to the real right-hand sides."""
        rep = _lib.f4j_report()
        md = _lib.SPARSE_EXACT if mode is None else _lib.SPARSE_MODES.get(mode, mode)
        if md not in (_lib.SPARSE_EXACT, _lib.SPARSE_FMA):
            raise IllegalArgumentException("unknown sparse mode %r" % (mode,))
        if isinstance(b, Vector):
            ensure_all_equal(self.numCols, b.size)
            ctx = self._ctx or b._ctx or default_context()
            y = ctx.alloc(max(8 * self.numRows, 8))
            check(ctx.lib.f4j_spmv_ex(ctx.handle, self.handle(ctx), b.device(ctx).handle, y.handle, md,
                                      ctypes.byref(rep)))
            out = Vector._from_device(Shape(self.numRows), y, ctx)
        elif isinstance(b, Matrix):
            ensure_mat_mult_shapes(self.shape, b.shape)
            ctx = self._ctx or b._ctx or default_context()
            y = ctx.alloc(max(8 * self.numRows * b.numCols, 8))
            check(ctx.lib.f4j_spmm_ex(ctx.handle, self.handle(ctx), b.device(ctx).handle, b.numCols, y.handle, md,
                                      ctypes.byref(rep)))
            out = Matrix._from_device(Shape(self.numRows, b.numCols), y, ctx)
        elif isinstance(b, (CMatrix, CVector)):
            # CsrMatrix.mult(CMatrix) -> RealFieldDenseCsrMatMult.standard (RealFieldDenseCsrMatMult.java:62-91):
            # y[i][j] += x[col][j] * v per part in storage order, i.e. the real SpMM over b's interleaved
            # storage with 2 * ncols real columns
            vec = isinstance(b, CVector)
            nc = 1 if vec else b.numCols
            if vec:
                ensure_all_equal(self.numCols, b.size)
            else:
                ensure_mat_mult_shapes(self.shape, b.shape)
            ctx = self._ctx or b._ctx or default_context()
            y = ctx.alloc(max(16 * self.numRows * nc, 16))
            check(ctx.lib.f4j_spmm_ex(ctx.handle, self.handle(ctx), b.device(ctx).handle, 2 * nc, y.handle, md,
                                      ctypes.byref(rep)))
            out = (CVector._from_device(Shape(self.numRows), y, ctx) if vec
                   else CMatrix._from_device(Shape(self.numRows, nc), y, ctx))
        elif isinstance(b, CsrMatrix):
            out = self._csr_mult_dense(b, rep)
        else:
            raise NotImplementedError("CsrMatrix.mult(%s) is not on this engine's path" % type(b).__name__)
        if report is not None:
            report.update(rep.as_dict())
        return out

    def _csr_mult_dense(self, b, rep=None):
        """CSR x CSR with a dense result (RealCsrMatMult.standard, RealComplexCsrMatMult.standard,
        SemiringCsrMatMult.standard by the operands' value types), bit-identical."""
        ensure_mat_mult_shapes(self.shape, b.shape)
        ac, bc = isinstance(self, CsrCMatrix), isinstance(b, CsrCMatrix)
        w = 2 if (ac or bc) else 1
        ctx = self._ctx or b._ctx or default_context()
        y = ctx.alloc(max(8 * w * self.numRows * b.numCols, 8))
        check(ctx.lib.f4j_csr_mult_dense_ex(ctx.handle, self.handle(ctx), int(ac), b.handle(ctx), int(bc), y.handle,
                                            ctypes.byref(rep) if rep is not None else None))
        cls = CMatrix if w == 2 else Matrix
        return cls._from_device(Shape(self.numRows, b.numCols), y, ctx)

    def mult2Csr(self, b):
        """CsrMatrix.mult2Csr(CsrMatrix | CsrCMatrix) -> RealCsrMatMult.standardAsSparse
        (RealCsrMatMult.java:92-131) / RealComplexCsrMatMult.standardAsSparse (:133-181); for a
        CsrCMatrix receiver its own variants: the product as CSR, every touched column stored (explicit
        zeros too), bit-identical."""
        if not isinstance(b, CsrMatrix):
            raise NotImplementedError("mult2Csr(%s) is not on this engine's path" % type(b).__name__)
        ensure_mat_mult_shapes(self.shape, b.shape)
        ac, bc = isinstance(self, CsrCMatrix), isinstance(b, CsrCMatrix)
        ctx = self._ctx or b._ctx or default_context()
        h = ctypes.c_void_p()
        check(ctx.lib.f4j_csr_mult_csr_ex(ctx.handle, self.handle(ctx), int(ac), b.handle(ctx), int(bc),
                                          ctypes.byref(h), None))
        nnz = ctypes.c_int64()
        check(ctx.lib.f4j_csr_info(h, None, None, ctypes.byref(nnz)))
        cls = CsrCMatrix if (ac or bc) else CsrMatrix
        return cls._from_handle((self.numRows, b.numCols), nnz.value, h, None, ctx)

    def multTranspose(self, b):
        """CsrMatrix.multTranspose(CsrMatrix) -> RealCsrMatMult.standard(this, b.T()) (CsrMatrix.java:809-810)."""
        if not isinstance(b, CsrMatrix) or isinstance(b, CsrCMatrix) or isinstance(self, CsrCMatrix):
            raise NotImplementedError("CsrMatrix.multTranspose(%s) is not on this engine's path" % type(b).__name__)
        ensure_mat_mult_shapes(self.shape, Shape(b.numCols, b.numRows))
        return self.mult(b.T())

    def multTransposeLeft(self, b):
        """S^T * b without forming S^T (cached transpose permutation)."""
        ensure_mat_mult_shapes(Shape(self.numCols, self.numRows), b.shape)
        ctx = self._ctx or b._ctx or default_context()
        y = ctx.alloc(max(8 * self.numCols * b.numCols, 8))
        check(ctx.lib.f4j_spmm_t(ctx.handle, self.handle(ctx), b.device(ctx).handle, b.numCols, y.handle, None))
        return Matrix._from_device(Shape(self.numCols, b.numCols), y, ctx)

    def T(self):
        """CsrMatrix.T() -> RealCsrOps.transpose, on the GPU."""
        ctx = self._ctx or default_context()
        h = ctypes.c_void_p()
        check(ctx.lib.f4j_csr_transpose(ctx.handle, self.handle(ctx), ctypes.byref(h)))
        return CsrMatrix._from_handle((self.numCols, self.numRows), self.nnz, h, None, ctx)

    def transposePermutation(self):
        ctx = self._ctx or default_context()
        buf = ctx.alloc(max(4 * self.nnz, 8))
        check(ctx.lib.f4j_csr_transpose_perm(ctx.handle, self.handle(ctx), buf.handle))
        return buf.to_numpy(np.int32, self.nnz)

    def toDense(self):
        out = np.zeros(self.shape)
        rp, ci, v = self.rowPointers, self.colIndices, self.data
        for i in range(self.numRows):
            out[i, ci[rp[i]:rp[i + 1]]] = v[rp[i]:rp[i + 1]]
        return Matrix(out)

    def __eq__(self, other):
        """SparseUtils.CSREquals: same shape and same nonzeros (explicit zeros skipped)."""
        if not isinstance(other, CsrMatrix) or self.shape != other.shape:
            return False
        return self.toDense() == other.toDense()

    __hash__ = None

    def close(self):
        if self._handle is not None and self._ctx is not None:
            self._ctx.lib.f4j_csr_free(self._ctx.handle, self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CsrCMatrix(CsrMatrix):
    """Complex CSR matrix: CsrCMatrix(Shape, Complex128[] data, int[] rowPointers, int[] colIndices)."""

    _vdtype = np.complex128

    def mult(self, b, report=None):
        """CsrCMatrix.mult(CMatrix / CVector) -> DenseCsrSemiringMatMult.standard / standardVector
        (DenseCsrSemiringMatMult.java:59-98, :140-160), bit-identical."""
        if isinstance(b, CsrMatrix):
            # CsrCMatrix.mult(CsrMatrix) -> RealComplexCsrMatMult.standard (RealComplexCsrMatMult.java:93-118);
            # CsrCMatrix.mult(CsrCMatrix) -> SemiringCsrMatMult.standard (SemiringCsrMatMult.java:58-87)
            return self._csr_mult_dense(b)
        if not isinstance(b, (CMatrix, CVector)):
            raise NotImplementedError("CsrCMatrix.mult(%s) is not on this engine's path" % type(b).__name__)
        vec = isinstance(b, CVector)
        nc = 1 if vec else b.numCols
        if vec:
            ensure_all_equal(self.numCols, b.size)
        else:
            ensure_mat_mult_shapes(self.shape, b.shape)
        ctx = self._ctx or b._ctx or default_context()
        rep = _lib.f4j_report()
        y = ctx.alloc(max(16 * self.numRows * nc, 16))
        check(ctx.lib.f4j_zspmm(ctx.handle, self.handle(ctx), b.device(ctx).handle, nc, y.handle, ctypes.byref(rep)))
        if report is not None:
            report.update(rep.as_dict())
        return (CVector._from_device(Shape(self.numRows), y, ctx) if vec
                else CMatrix._from_device(Shape(self.numRows, nc), y, ctx))

    def multTransposeLeft(self, b):
        raise NotImplementedError("complex CSR transposes are not on this engine's path")

    def T(self):
        raise NotImplementedError("complex CSR transposes are not on this engine's path")

    def toDense(self):
        out = np.zeros(self.shape, np.complex128)
        rp, ci, v = self.rowPointers, self.colIndices, self.data
        for i in range(self.numRows):
            out[i, ci[rp[i]:rp[i + 1]]] = v[rp[i]:rp[i + 1]]
        return CMatrix(out)

    def __eq__(self, other):
        if not isinstance(other, CsrCMatrix) or self.shape != other.shape:
            return False
        return self.toDense() == other.toDense()

    __hash__ = None


class CooMatrix:
    """COO matrix: CooMatrix(Shape, double[] data, int[] rowIndices, int[] colIndices)."""

    def __init__(self, shape, data, row_indices, col_indices):
        self.shape = Shape(shape)
        self.data = np.ascontiguousarray(data, dtype=np.float64).reshape(-1)
        self.rowIndices = np.ascontiguousarray(row_indices, dtype=np.int32).reshape(-1)
        self.colIndices = np.ascontiguousarray(col_indices, dtype=np.int32).reshape(-1)
        self.nnz = int(self.data.size)
        # SparseValidation.validateCoo (SparseValidation.java:70-98)
        if self.nnz > self.shape[0] * self.shape[1]:
            raise IllegalArgumentException("The number of non-zero entries cannot be greater than the total number "
                                           "of entries in the matrix")
        if self.nnz != self.rowIndices.size or self.nnz != self.colIndices.size:
            raise IllegalArgumentException(
                "The number of non-zero entries must match the number of row and column indices but got nnz=%d, "
                "rowIndices.length=%d, and colIndices.length=%d" % (self.nnz, self.rowIndices.size,
                                                                    self.colIndices.size))

    def _bufs(self, ctx):
        z = lambda a, dt: a if a.size else np.zeros(1, dt)
        return (ctx.from_numpy(z(self.rowIndices, np.int32)), ctx.from_numpy(z(self.colIndices, np.int32)),
                ctx.from_numpy(z(self.data, np.float64)))

    def toCsr(self, ctx=None):
        """CooMatrix.toCsr on the GPU: counts + scan; data/colIndices copied unchanged."""
        ctx = ctx or default_context()
        r, c, v = self._bufs(ctx)
        h = ctypes.c_void_p()
        check(ctx.lib.f4j_csr_from_coo(ctx.handle, self.shape[0], self.shape[1], self.nnz, r.handle, c.handle,
                                       v.handle, ctypes.byref(h)))
        return CsrMatrix._from_handle(self.shape, self.nnz, h, None, ctx)

    def sortIndices(self, ctx=None):
        """CooMatrix.sortIndices: stable lexicographic (row, col) sort, in place."""
        ctx = ctx or default_context()
        r, c, v = self._bufs(ctx)
        check(ctx.lib.f4j_coo_sort(ctx.handle, self.nnz, r.handle, c.handle, v.handle))
        if self.nnz:
            r.download(self.rowIndices)
            c.download(self.colIndices)
            v.download(self.data)
        return self
