"""Matrix Market reader: the host side of "file -> CSR on the device".

A mirror of Flag4j's MatrixMarketReader (src/main/java/org/flag4j/io/
MatrixMarketReader.java) and MatrixMarketHeader (…/io/MatrixMarketHeader.java):
the same supported combinations, the same result types, the same order of the
returned COO entries and the same Flag4jParsingException messages.

- Header: ``%%MatrixMarket matrix <format> <field> <symmetry>`` (case-insensitive
  words; MatrixMarketHeader.parseHeader).
- Comment lines (``%``) may follow the header; blank lines are skipped anywhere
  (MatrixMarketReader.findNextNonemptyLine).
- coordinate real | integer | pattern, general -> CooMatrix sorted
  lexicographically by (row, col), stable (CooDataSorter.sparseSort);
  symmetric -> the off-diagonal entries mirrored after the read entries, then
  the same stable sort; pattern values are 1.0 (MatrixMarketReader.java:369-404).
- coordinate complex, general -> CooCMatrix sorted; symmetric / hermitian ->
  mirrored (conjugated for hermitian), sorted (:412-457).
- array real | integer, general -> Matrix; symmetric -> Matrix from the lower
  triangle; array complex general -> CMatrix; symmetric / hermitian -> CMatrix
  (:255-366).  Array data are column-major.

Indices in the file are 1-based.  ``read_csr`` continues on the GPU:
CooMatrix.toCsr (counts and a scan on the device, data copied unchanged).
"""
import os

import numpy as np

from .arrays import CMatrix, CooMatrix, CsrCMatrix, Matrix, Shape
from .device import IllegalArgumentException, check, default_context

_OBJECTS = ("MATRIX",)
_FORMATS = ("ARRAY", "COORDINATE")
_FIELDS = ("REAL", "INTEGER", "COMPLEX", "PATTERN")
_SYMMETRIES = ("GENERAL", "SYMMETRIC", "HERMITIAN")
_UNSUPPORTED_SYMMETRY = "Unsupported symmetry found in Matrix Market Format file header: %s."


class Flag4jParsingException(RuntimeError):
    """Mirror of org.flag4j.util.exceptions.Flag4jParsingException."""


def _enum(kind, names, token):
    name = token.upper()
    if name not in names:
        # Java's Enum.valueOf
        raise IllegalArgumentException("No enum constant org.flag4j.io.MatrixMarketHeader.%s.%s" % (kind, name))
    return name


def parse_header(line):
    """MatrixMarketHeader.parseHeader (MatrixMarketHeader.java): (object, format, field, symmetry)."""
    tokens = line.split() if line is not None else []
    if not tokens or tokens[0].lower() != "%%matrixmarket":
        raise Flag4jParsingException("Invalid Matrix Market MMFormat file header. Did not find %%MatrixMarket.")
    rest = tokens[1:]
    if len(rest) < 3:
        raise Flag4jParsingException("Invalid Matrix Market file header. Did not specify both <object> and <format>.")
    obj = _enum("MMObject", _OBJECTS, rest[0])
    if len(rest) - 1 != 3:
        raise Flag4jParsingException("Invalid Matrix Market file header. Must specify exactly three qualifiers for a "
                                     "matrix: <format>, <field>, and <symmetry>.")
    return (obj, _enum("MMFormat", _FORMATS, rest[1]), _enum("MMField", _FIELDS, rest[2]),
            _enum("MMSymmetry", _SYMMETRIES, rest[3]))


class CooCMatrix:
    """Complex COO matrix: CooCMatrix(Shape, Complex128[] data, int[] rowIndices, int[] colIndices)."""

    def __init__(self, shape, data, row_indices, col_indices):
        self.shape = Shape(shape)
        self.data = np.ascontiguousarray(data, dtype=np.complex128).reshape(-1)
        self.rowIndices = np.ascontiguousarray(row_indices, dtype=np.int32).reshape(-1)
        self.colIndices = np.ascontiguousarray(col_indices, dtype=np.int32).reshape(-1)
        self.nnz = int(self.data.size)
        if self.nnz != self.rowIndices.size or self.nnz != self.colIndices.size:
            raise IllegalArgumentException(
                "The number of non-zero entries must match the number of row and column indices but got nnz=%d, "
                "rowIndices.length=%d, and colIndices.length=%d" % (self.nnz, self.rowIndices.size,
                                                                    self.colIndices.size))

    def toCsr(self, ctx=None):
        """CooCMatrix.toCsr: row counts and the scan on the GPU (f4j_csr_from_coo on the
        structure), complex data and column indices carried over unchanged."""
        import ctypes
        ctx = ctx or default_context()
        rows = self.shape[0]
        z = lambda a, dt: a if a.size else np.zeros(1, dt)
        r = ctx.from_numpy(z(self.rowIndices, np.int32))
        c = ctx.from_numpy(z(self.colIndices, np.int32))
        v = ctx.from_numpy(np.zeros(max(self.nnz, 1)))
        h = ctypes.c_void_p()
        check(ctx.lib.f4j_csr_from_coo(ctx.handle, rows, self.shape[1], self.nnz, r.handle, c.handle, v.handle,
                                       ctypes.byref(h)))
        rp, ci, vv = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        check(ctx.lib.f4j_csr_buffers(h, ctypes.byref(rp), ctypes.byref(ci), ctypes.byref(vv)))
        rowptr = np.empty(rows + 1, np.int32)
        check(ctx.lib.f4j_buf_download(ctx.handle, rp, rowptr.ctypes.data, rowptr.nbytes, 0))
        check(ctx.lib.f4j_csr_free(ctx.handle, h))
        return CsrCMatrix(self.shape, self.data, rowptr, self.colIndices, validate=False)


class MatrixMarketReader:
    """MatrixMarketReader().read(fileName) -> Matrix | CMatrix | CooMatrix | CooCMatrix."""

    def read(self, file_name):
        return read_matrix_market(file_name)


def _sort_coo(rows, cols, *vals):
    # CooDataSorter.sparseSort: stable lexicographic (row, col)
    order = np.lexsort((cols, rows))
    return (rows[order], cols[order]) + tuple(v[order] for v in vals)


class _Lines:
    """Line cursor with MatrixMarketReader's blank-line skipping and 1-based line numbers."""

    def __init__(self, text):
        self.lines = text.split("\n")
        if self.lines and self.lines[-1] == "":
            self.lines.pop()
        self.i = 0  # index of the current line; line number = i + 1

    def current(self):
        return self.lines[self.i] if self.i < len(self.lines) else None

    def next_nonempty(self):
        self.i += 1
        while self.i < len(self.lines) and self.lines[self.i].strip() == "":
            self.i += 1
        return self.current()

    def data_block(self, count):
        """The next `count` non-empty lines (fewer if the file ends), and the line
        index of each."""
        start = self.i + 1
        chunk = self.lines[start:start + count]
        if len(chunk) == count and all(line.strip() for line in chunk):  # no blank lines: one slice
            self.i = start + count - 1
            return chunk, range(start, start + count)
        out, idx = [], []
        while len(out) < count:
            line = self.next_nonempty()
            if line is None:
                break
            out.append(line)
            idx.append(self.i)
        return out, idx


def _dims(line, expected):
    tokens = line.strip().split()
    if len(tokens) != expected:
        raise Flag4jParsingException("Expected %d values for matrix shape/non-zero data but found %d."
                                     % (expected, len(tokens)))
    return [int(t) for t in tokens]


def _parse_coordinate(cur, field):
    rows, cols, nnz = _dims(cur.current(), 3)
    per = {"PATTERN": 2, "REAL": 3, "INTEGER": 3, "COMPLEX": 4}[field]
    block, idx = cur.data_block(nnz)
    if len(block) < nnz:
        raise Flag4jParsingException("Expecting %d non-zero data for coordinate Format but found %d."
                                     % (nnz, len(block) + 1))
    flat = np.array(" ".join(block).split()) if nnz else np.zeros(0, dtype="U1")
    if flat.size != nnz * per:
        # locate the first line with a different number of values
        for line, li in zip(block, idx):
            n = len(line.split())
            if n > per:
                raise Flag4jParsingException(
                    "Expecting exactly %d values in Matrix Market file for %s coordinate format but found %d on "
                    "line %d." % (per, field, n - per, li + 1))
            if n < per:
                raise Flag4jParsingException("Missing values on line %d of the Matrix Market file." % (li + 1))
    tok = flat.reshape(nnz, per)
    # indices are integers (a non-integer token raises, as Integer.parseInt does)
    r = tok[:, 0].astype(np.int64) - 1
    c = tok[:, 1].astype(np.int64) - 1
    if field == "PATTERN":
        v = np.ones(nnz)
    elif field == "COMPLEX":
        v = tok[:, 2].astype(np.float64) + 1j * tok[:, 3].astype(np.float64)
    else:
        v = tok[:, 2].astype(np.float64)
    if cur.next_nonempty() is not None:
        # the reference reports the column count here
        raise Flag4jParsingException("Found extra non-empty lines at the end of the Matrix Market Format file. "
                                     "The number of  data lines does not match the number of non-zero data "
                                     "specified: %d." % cols)
    return rows, cols, r, c, v


def _parse_array(cur, field, symmetric):
    rows, cols = _dims(cur.current(), 2)
    if symmetric and rows != cols:
        raise Flag4jParsingException("Expecting symmetric matrix to be square but got shape %s." % (Shape(rows, cols),))
    size = rows * (rows + 1) // 2 if symmetric else rows * cols
    block, idx = cur.data_block(size)
    if len(block) < size:
        raise Flag4jParsingException("Expecting %d data in the Matrix Market file but found %d."
                                     % (size, len(block) + 1))
    if field == "COMPLEX":
        vals = np.empty(size, np.complex128)
        for n, line in enumerate(block):
            t = line.split()
            if len(t) > 2:
                raise Flag4jParsingException("Expecting two values for complex data.")
            vals[n] = float(t[0]) + 1j * float(t[1])
    else:
        vals = np.array([float(line) for line in block], dtype=np.float64)
    if cur.next_nonempty() is not None:
        raise Flag4jParsingException("Found extra non-empty lines at the end of the Matrix Market Format file. "
                                     "The number of data lines does not match the number of columns specified: "
                                     "%d." % cols)
    return rows, cols, vals


def read_matrix_market(path):
    """MatrixMarketReader.read: parse the file at `path`."""
    with open(path, "r") as f:
        text = f.read()
    cur = _Lines(text)
    obj, fmt, field, sym = parse_header(cur.current())
    while True:
        line = cur.next_nonempty()
        if line is None or not line.startswith("%"):
            break
    if cur.current() is None:
        raise Flag4jParsingException("No lines found after header of Matrix Market Format file.")

    if fmt == "ARRAY":
        if field in ("REAL", "INTEGER"):
            if sym not in ("GENERAL", "SYMMETRIC"):
                raise Flag4jParsingException(_UNSUPPORTED_SYMMETRY % sym)
        elif field == "COMPLEX":
            pass
        else:
            raise Flag4jParsingException("Unsupported field found in Matrix Market Format file header: %s." % field)
        rows, cols, vals = _parse_array(cur, field, sym != "GENERAL")
        if sym == "GENERAL":
            arr = vals.reshape(cols, rows).T.copy()
        else:
            n = rows
            arr = np.zeros((n, n), vals.dtype)
            u = 0
            for j in range(n):
                for i in range(j, n):
                    v = vals[u]
                    u += 1
                    arr[i, j] = v
                    arr[j, i] = np.conj(v) if (sym == "HERMITIAN" and i != j) else v
        return CMatrix(arr) if field == "COMPLEX" else Matrix(arr)

    # coordinate
    if field in ("REAL", "INTEGER", "PATTERN"):
        if sym not in ("GENERAL", "SYMMETRIC"):
            raise Flag4jParsingException(_UNSUPPORTED_SYMMETRY % sym)
    elif field != "COMPLEX":
        raise Flag4jParsingException("Unsupported field found in Matrix Market Format file header: %s." % field)
    rows, cols, r, c, v = _parse_coordinate(cur, field)
    if sym != "GENERAL":
        if rows != cols:
            what = "Symmetric/Hermitian" if field == "COMPLEX" else "Symmetric"
            raise Flag4jParsingException("%s matrices must be square but got shape %s" % (what, Shape(rows, cols)))
        off = r != c
        mv = v[off]
        if sym == "HERMITIAN":
            mv = np.conj(mv)
        r, c, v = np.concatenate([r, c[off]]), np.concatenate([c, r[off]]), np.concatenate([v, mv])
    r, c, v = _sort_coo(r, c, v)
    shape = Shape(rows, cols)
    if field == "COMPLEX":
        return CooCMatrix(shape, v, r.astype(np.int32), c.astype(np.int32))
    return CooMatrix(shape, v, r.astype(np.int32), c.astype(np.int32))


def read_csr(path, ctx=None):
    """Read a coordinate Matrix Market file and convert it to CSR on the GPU."""
    m = read_matrix_market(path)
    if not isinstance(m, (CooMatrix, CooCMatrix)):
        raise IllegalArgumentException("%s holds a dense (array format) matrix" % os.path.basename(path))
    return m.toCsr(ctx)
