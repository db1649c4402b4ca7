"""Matrix Market reader (host side): known-answer files written by the tests.

The expected results follow MatrixMarketReader's documented semantics
(src/main/java/org/flag4j/io/MatrixMarketReader.java): 1-based indices, stable
(row, col) order for coordinate data, mirrored off-diagonal entries for
symmetric / hermitian matrices, pattern values 1.0, column-major array data,
and the reference's Flag4jParsingException messages.
"""
import numpy as np
import pytest

from flag4j_gb300 import mmio
from flag4j_gb300.arrays import CMatrix, CooMatrix, Matrix
from flag4j_gb300.device import IllegalArgumentException


def write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_coordinate_real_general_sorted_stably(tmp_path):
    # duplicates keep their file order (stable sort); comments and blank lines skipped
    f = write(tmp_path, "a.mtx", "%%MatrixMarket matrix coordinate real general\n% a comment\n%another\n\n"
              "3 4 5\n3 2 7.5\n1 4 -1e-3\n\n2 1 2.0\n1 4 9.0\n1 1 0.25\n")
    m = mmio.read_matrix_market(f)
    assert isinstance(m, CooMatrix) and m.shape == (3, 4)
    assert m.rowIndices.tolist() == [0, 0, 0, 1, 2]
    assert m.colIndices.tolist() == [0, 3, 3, 0, 1]
    assert m.data.tolist() == [0.25, -1e-3, 9.0, 2.0, 7.5]


def test_coordinate_symmetric_and_pattern(tmp_path):
    f = write(tmp_path, "s.mtx", "%%MatrixMarket matrix coordinate real symmetric\n3 3 3\n2 1 4.0\n3 3 1.5\n3 1 -2\n")
    m = mmio.read_matrix_market(f)
    dense = np.zeros((3, 3))
    dense[m.rowIndices, m.colIndices] = m.data
    assert np.array_equal(dense, [[0, 4, -2], [4, 0, 0], [-2, 0, 1.5]])
    assert m.rowIndices.tolist() == [0, 0, 1, 2, 2] and m.colIndices.tolist() == [1, 2, 0, 0, 2]
    f = write(tmp_path, "p.mtx", "%%MatrixMarket matrix coordinate pattern symmetric\n2 2 2\n2 1\n1 1\n")
    m = mmio.read_matrix_market(f)
    assert m.data.tolist() == [1.0, 1.0, 1.0] and m.rowIndices.tolist() == [0, 0, 1]
    f = write(tmp_path, "i.mtx", "%%MatrixMarket MATRIX Coordinate INTEGER General\n2 2 1\n2 2 7\n")
    m = mmio.read_matrix_market(f)
    assert m.data.tolist() == [7.0] and m.rowIndices.tolist() == [1]


def test_coordinate_complex_general_and_hermitian(tmp_path):
    f = write(tmp_path, "c.mtx", "%%MatrixMarket matrix coordinate complex hermitian\n2 2 2\n2 1 1.0 2.0\n1 1 3.0 0\n")
    m = mmio.read_matrix_market(f)
    assert isinstance(m, mmio.CooCMatrix)
    assert m.rowIndices.tolist() == [0, 0, 1] and m.colIndices.tolist() == [0, 1, 0]
    assert m.data.tolist() == [3 + 0j, 1 - 2j, 1 + 2j]
    f = write(tmp_path, "c2.mtx", "%%MatrixMarket matrix coordinate complex symmetric\n2 2 1\n2 1 1.0 2.0\n")
    assert mmio.read_matrix_market(f).data.tolist() == [1 + 2j, 1 + 2j]


def test_array_formats_column_major(tmp_path):
    f = write(tmp_path, "d.mtx", "%%MatrixMarket matrix array real general\n2 3\n1\n2\n3\n4\n5\n6\n")
    m = mmio.read_matrix_market(f)
    assert isinstance(m, Matrix) and np.array_equal(m.toNumpy(), [[1, 3, 5], [2, 4, 6]])
    f = write(tmp_path, "ds.mtx", "%%MatrixMarket matrix array real symmetric\n3 3\n1\n2\n3\n4\n5\n6\n")
    assert np.array_equal(mmio.read_matrix_market(f).toNumpy(), [[1, 2, 3], [2, 4, 5], [3, 5, 6]])
    f = write(tmp_path, "dc.mtx", "%%MatrixMarket matrix array complex hermitian\n2 2\n1 0\n2 3\n4 0\n")
    m = mmio.read_matrix_market(f)
    assert isinstance(m, CMatrix) and np.array_equal(m.toNumpy(), [[1, 2 - 3j], [2 + 3j, 4]])
    f = write(tmp_path, "dg.mtx", "%%MatrixMarket matrix array complex general\n1 2\n1 2\n3 4\n")
    assert np.array_equal(mmio.read_matrix_market(f).toNumpy(), [[1 + 2j, 3 + 4j]])


@pytest.mark.parametrize("text,exc,msg", [
    ("%MatrixMarket matrix coordinate real general\n1 1 0\n", mmio.Flag4jParsingException, "Did not find %%MatrixMarket"),
    ("%%MatrixMarket matrix coordinate\n1 1 0\n", mmio.Flag4jParsingException, "both <object> and <format>"),
    ("%%MatrixMarket matrix coordinate real general extra\n1 1 0\n", mmio.Flag4jParsingException, "exactly three"),
    ("%%MatrixMarket tensor coordinate real general\n1 1 0\n", IllegalArgumentException, "MMObject.TENSOR"),
    ("%%MatrixMarket matrix coordinate real hermitian\n1 1 0\n", mmio.Flag4jParsingException,
     "Unsupported symmetry found in Matrix Market Format file header: HERMITIAN."),
    ("%%MatrixMarket matrix array pattern general\n1 1\n1\n", mmio.Flag4jParsingException,
     "Unsupported field found in Matrix Market Format file header: PATTERN."),
    ("%%MatrixMarket matrix coordinate real general\n% only comments\n", mmio.Flag4jParsingException,
     "No lines found after header"),
    ("%%MatrixMarket matrix coordinate real general\n2 2\n", mmio.Flag4jParsingException,
     "Expected 3 values for matrix shape/non-zero data but found 2."),
    ("%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1.0\n", mmio.Flag4jParsingException,
     "Expecting 2 non-zero data for coordinate Format but found 2."),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 1.0 5\n", mmio.Flag4jParsingException,
     "Expecting exactly 3 values in Matrix Market file for REAL coordinate format but found 1 on line 3."),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 1.0\n2 2 3.0\n", mmio.Flag4jParsingException,
     "Found extra non-empty lines"),
    ("%%MatrixMarket matrix coordinate real symmetric\n2 3 1\n1 1 1.0\n", mmio.Flag4jParsingException,
     "Symmetric matrices must be square"),
    ("%%MatrixMarket matrix array real symmetric\n2 3\n1\n", mmio.Flag4jParsingException,
     "Expecting symmetric matrix to be square"),
    ("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n", mmio.Flag4jParsingException,
     "Expecting 4 data in the Matrix Market file but found 4."),
])
def test_parse_errors(tmp_path, text, exc, msg):
    f = write(tmp_path, "e.mtx", text)
    with pytest.raises(exc, match=msg.replace("(", r"\(").replace(")", r"\)").replace(".", r"\.").replace("%", "%")):
        mmio.read_matrix_market(f)


def test_large_coordinate_file_matches_a_direct_construction(tmp_path):
    # a 2^14-row file written here, read back: the stable-sorted triplets, bit for bit
    from flag4j_gb300 import synth
    rows = 1 << 14
    rp, ci, v = synth.csr_poisson(rows, rows, seed=31)
    r = np.repeat(np.arange(rows), np.diff(rp))
    p = np.random.default_rng(1).permutation(len(v))
    lines = ["%%MatrixMarket matrix coordinate real general", "%d %d %d" % (rows, rows, len(v))]
    lines += ["%d %d %r" % (r[q] + 1, ci[q] + 1, float(v[q])) for q in p]
    f = write(tmp_path, "big.mtx", "\n".join(lines) + "\n")
    m = mmio.read_matrix_market(f)
    assert np.array_equal(m.rowIndices, r) and np.array_equal(m.colIndices, ci) and np.array_equal(m.data, v)


# ------------------------------------------------------------------ the reference's own fixtures
def _golden_mm():
    import json
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "golden", "reference_golden.json")) as fh:
        return json.load(fh)["matrix_market"]


def _drop_zeros(data, rows, cols):
    keep = np.asarray(data) != 0
    return np.asarray(data)[keep], np.asarray(rows)[keep], np.asarray(cols)[keep]


@pytest.mark.parametrize("case", _golden_mm(), ids=lambda c: c["file"].rsplit("/", 1)[-1])
def test_reference_fixture_reads_as_the_reference_expects(case, tmp_path):
    """Each input file of MatrixMarketReadTests (src/test/java/org/flag4j/io/MatrixMarketReadTests.java)
    read by mmio equals the matrix MatrixMarketMatrices.java states for it, under the reference's
    equality: element-wise for Matrix / CMatrix, and for CooMatrix the shape, then the data, row and
    column arrays after dropping stored zeros (RealSparseEquals.cooMatrixEquals,
    src/main/java/org/flag4j/linalg/ops/sparse/coo/real/RealSparseEquals.java:90-102)."""
    f = write(tmp_path, case["file"].rsplit("/", 1)[-1], case["text"])
    got = mmio.read_matrix_market(f)
    exp = case["expected"]
    assert tuple(got.shape) == tuple(exp["shape"])
    if exp["kind"] == "dense":
        assert isinstance(got, Matrix)
        assert np.array_equal(got.toNumpy(), np.array(exp["data"], dtype=np.float64))
    elif exp["kind"] == "cdense":
        assert isinstance(got, CMatrix)
        want = np.array([[complex(re, im) for re, im in row] for row in exp["data"]])
        assert np.array_equal(got.toNumpy(), want)
    else:
        assert isinstance(got, CooMatrix)
        gd, gr, gc = _drop_zeros(got.data, got.rowIndices, got.colIndices)
        ed, er, ec = _drop_zeros(exp["data"], exp["rows"], exp["cols"])
        assert np.array_equal(gd, ed) and np.array_equal(gr, er) and np.array_equal(gc, ec)
