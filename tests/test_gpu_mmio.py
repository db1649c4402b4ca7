"""Matrix Market file -> CSR on the GPU (CooMatrix.toCsr / CooCMatrix.toCsr after the reader).

The structure must equal the oracle's CooMatrix.toCsr restatement of the same
sorted triplets (integer arrays compared exactly), and products on the result
must equal the oracle's loops bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _file(tmp_path, field, rows, cols, r, c, v):
    lines = ["%%%%MatrixMarket matrix coordinate %s general" % field, "%d %d %d" % (rows, cols, len(r))]
    if field == "complex":
        lines += ["%d %d %r %r" % (a + 1, b + 1, float(x.real), float(x.imag)) for a, b, x in zip(r, c, v)]
    else:
        lines += ["%d %d %r" % (a + 1, b + 1, float(x)) for a, b, x in zip(r, c, v)]
    p = tmp_path / ("m_%s.mtx" % field)
    p.write_text("\n".join(lines) + "\n")
    return str(p)


def test_real_file_to_device_csr(f4j, oracle, tmp_path):
    from flag4j_gb300 import mmio, synth
    rows, cols = 1 << 15, 1 << 14
    rp, ci, v = synth.csr_poisson(rows, cols, seed=41)
    r = np.repeat(np.arange(rows), np.diff(rp))
    perm = np.random.default_rng(2).permutation(len(v))
    S = mmio.read_csr(_file(tmp_path, "real", rows, cols, r[perm], ci[perm], v[perm]))
    assert np.array_equal(S.rowPointers, oracle.coo_to_csr(rows, r.astype(np.int32)))
    assert np.array_equal(S.colIndices, ci) and np.array_equal(S.data, v)
    x = np.random.default_rng(3).standard_normal(cols)
    assert np.array_equal(S.mult(f4j.Vector(x)).data, oracle.spmv(rp, ci, v, x))


def test_complex_file_to_device_csr(f4j, oracle, tmp_path):
    from flag4j_gb300 import mmio, synth
    rows, cols = 1 << 13, 1 << 13
    rp, ci, v = synth.csr_poisson(rows, cols, seed=42)
    rng = np.random.default_rng(4)
    vz = v + 1j * rng.standard_normal(len(v))
    r = np.repeat(np.arange(rows), np.diff(rp))
    perm = rng.permutation(len(v))
    S = mmio.read_csr(_file(tmp_path, "complex", rows, cols, r[perm], ci[perm], vz[perm]))
    assert isinstance(S, f4j.CsrCMatrix)
    assert np.array_equal(S.rowPointers, rp) and np.array_equal(S.colIndices, ci) and np.array_equal(S.data, vz)
    X = rng.standard_normal((cols, 4)) + 1j * rng.standard_normal((cols, 4))
    assert np.array_equal(S.mult(f4j.CMatrix(X)).toNumpy(), oracle.zspmm(rp, ci, vz, X))


def _golden_coordinate_cases():
    import json
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "golden", "reference_golden.json")) as fh:
        return [c for c in json.load(fh)["matrix_market"] if c["expected"]["kind"] == "coo"]


@pytest.mark.parametrize("case", _golden_coordinate_cases(), ids=lambda c: c["file"].rsplit("/", 1)[-1])
def test_reference_fixture_to_device_csr(f4j, oracle, case, tmp_path):
    """The reference's coordinate fixtures (MatrixMarketReadTests, src/test/java/org/flag4j/io/
    MatrixMarketReadTests.java:75-146) to CSR on the GPU: row pointers, column indices and values equal
    CooMatrix.toCsr of the expected sorted triplets of MatrixMarketMatrices.java (the oracle's
    restatement), and S x equals the oracle's SpMV on them bit for bit."""
    from flag4j_gb300 import mmio
    p = tmp_path / case["file"].rsplit("/", 1)[-1]
    p.write_text(case["text"])
    S = mmio.read_csr(str(p))
    exp = case["expected"]
    rows, cols = exp["shape"]
    er = np.asarray(exp["rows"], np.int32)
    rp = oracle.coo_to_csr(rows, er)
    assert np.array_equal(S.rowPointers, rp)
    assert np.array_equal(S.colIndices, np.asarray(exp["cols"], np.int32))
    assert np.array_equal(S.data, np.asarray(exp["data"], np.float64))
    x = np.random.default_rng(5).standard_normal(cols)
    assert np.array_equal(S.mult(f4j.Vector(x)).data,
                          oracle.spmv(rp, np.asarray(exp["cols"], np.int32), np.asarray(exp["data"]), x))
