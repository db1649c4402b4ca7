"""Extract Flag4j's known-answer test vectors into JSON fixtures.

Reads the reference's own JUnit sources as text (nothing is executed) and
writes ``reference_golden.json`` next to this script.  Each case records the
Java file, the test method, the line of the assertion that closes it, the
inputs and (where the test states them as literals) the expected output.

Files read (paths within the Flag4j project):
  src/test/java/org/flag4j/linalg/ops/dense/real/MatrixMultiplyTests.java
  src/test/java/org/flag4j/linalg/ops/dense/complex/CMatrixMultiplyTests.java
  src/test/java/org/flag4j/arrays/dense/matrix/MatrixMultTests.java
  src/test/java/org/flag4j/arrays/dense/complex_matrix/CMatrixMultTests.java
  src/test/java/org/flag4j/arrays/dense/matrix/MatrixVectorTests.java
  src/test/java/org/flag4j/arrays/sparse/csr_matrix/RealCsrDenseMatMultTests.java
  src/test/java/org/flag4j/arrays/sparse/csr_matrix/CsrMatrixTransposeTests.java
  src/test/java/org/flag4j/arrays/sparse/csr_matrix/RealCsrCsrMatMultTests.java
  src/test/java/org/flag4j/arrays/sparse/csr_matrix/RealComplexCsrCsrMatMultTests.java

Matrix Market read fixtures ("matrix_market" key): the twelve input files
MatrixMarketReadTests reads (src/test/java/org/flag4j/io/MatrixMarketReadTests.java,
from src/test/data/matrix_market/{array,coordinate}/), each with its text and
the expected result stated in src/test/java/org/flag4j/io/MatrixMarketMatrices.java
(COO expectations sorted as that class's static block does with sortIndices).

Usage:  python tests/golden/make_golden.py /path/to/flag4j
The fixture is committed; the GPU machine never needs the reference tree.
"""
import json
import math
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
T = "src/test/java/org/flag4j/"
FILES = {
    "real_kernels": T + "linalg/ops/dense/real/MatrixMultiplyTests.java",
    "complex_kernels": T + "linalg/ops/dense/complex/CMatrixMultiplyTests.java",
    "matrix_mult": T + "arrays/dense/matrix/MatrixMultTests.java",
    "cmatrix_mult": T + "arrays/dense/complex_matrix/CMatrixMultTests.java",
    "matrix_vector": T + "arrays/dense/matrix/MatrixVectorTests.java",
    "csr_dense": T + "arrays/sparse/csr_matrix/RealCsrDenseMatMultTests.java",
    "csr_transpose": T + "arrays/sparse/csr_matrix/CsrMatrixTransposeTests.java",
    "csr_csr": T + "arrays/sparse/csr_matrix/RealCsrCsrMatMultTests.java",
    "csr_csr_rz": T + "arrays/sparse/csr_matrix/RealComplexCsrCsrMatMultTests.java",
}

# ---------------------------------------------------------------- parsing
NUM = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?[dDfF]?"


def parse_complex_string(s):
    """Complex128(String) literal: 'a+bi', 'a - bi', 'bi', 'a'."""
    t = s.replace(" ", "")
    if not t.endswith("i"):
        return [float(t.rstrip("dD")), 0.0]
    body = t[:-1]
    # split at the last sign that is not part of an exponent and not leading
    cut = None
    for p in range(len(body) - 1, 0, -1):
        if body[p] in "+-" and body[p - 1] not in "eE":
            cut = p
            break
    if cut is None:  # pure imaginary
        return [0.0, float(body) if body not in ("", "+", "-") else float(body + "1")]
    re_part, im_part = body[:cut], body[cut:]
    if im_part in ("+", "-"):
        im_part += "1"
    return [float(re_part), float(im_part)]


class Lit:
    """Tiny evaluator for the array / Complex128 literals used in the tests."""

    def __init__(self, text):
        self.s = text
        self.p = 0

    def ws(self):
        while self.p < len(self.s) and self.s[self.p] in " \t\r\n":
            self.p += 1

    def peek(self, tok):
        self.ws()
        return self.s.startswith(tok, self.p)

    def eat(self, tok):
        self.ws()
        if not self.s.startswith(tok, self.p):
            raise ValueError("expected %r at %r" % (tok, self.s[self.p:self.p + 40]))
        self.p += len(tok)

    def value(self):
        self.ws()
        if self.peek("new double[]") or self.peek("new double[][]") or self.peek("new Complex128[]") \
                or self.peek("new Complex128[][]") or self.peek("new int[]"):
            self.p = self.s.index("{", self.p)
            return self.array()
        if self.peek("{"):
            return self.array()
        if self.peek("new Complex128("):
            self.eat("new Complex128(")
            if self.peek('"'):
                self.eat('"')
                end = self.s.index('"', self.p)
                v = parse_complex_string(self.s[self.p:end])
                self.p = end + 1
                self.eat(")")
                return v
            a = self.scalar()
            b = 0.0
            if self.peek(","):
                self.eat(",")
                b = self.scalar()
            self.eat(")")
            return [a, b]
        if self.peek("Complex128.ZERO"):
            self.eat("Complex128.ZERO")
            return [0.0, 0.0]
        return self.scalar()

    def scalar(self):
        self.ws()
        if self.peek("-Math.PI"):
            self.eat("-Math.PI")
            return -math.pi
        if self.peek("Math.PI"):
            self.eat("Math.PI")
            return math.pi
        m = re.compile(NUM).match(self.s, self.p)
        if not m:
            raise ValueError("bad scalar at %r" % self.s[self.p:self.p + 40])
        self.p = m.end()
        return float(m.group(0).rstrip("dDfF"))

    def array(self):
        self.eat("{")
        out = []
        while True:
            self.ws()
            if self.peek("}"):
                self.eat("}")
                return out
            out.append(self.value())
            self.ws()
            if self.peek(","):
                self.eat(",")


def split_methods(src):
    """Yield (name, body, body_start_line) for each @Test method."""
    for m in re.finditer(r"@Test\s+void\s+(\w+)\s*\(\s*\)\s*\{", src):
        depth, p = 1, m.end()
        while depth:
            c = src[p]
            depth += (c == "{") - (c == "}")
            p += 1
        yield m.group(1), src[m.end():p - 1], src[:m.end()].count("\n") + 1


ASSIGN = re.compile(r"^\s*(\w+)\s*=\s*(new\s+(?:double|Complex128)\[\]|\{|new double\[\]\[\]|"
                    r"new Complex128\[\]\[\])", re.S)


def cases_of(path, rel):
    src = open(path).read()
    out = []
    for name, body, line0 in split_methods(src):
        env = {}
        pos = 0
        for stmt in body.split(";"):
            line = line0 + body[:pos].count("\n")
            pos += len(stmt) + 1
            s = stmt.strip()
            if not s:
                continue
            s = re.sub(r"//[^\n]*", "", s).strip()
            m = ASSIGN.match(s)
            if m:
                env[m.group(1)] = Lit(s[s.index("=") + 1:]).value()
                continue
            call = re.match(r"(assert\w+|build|makeMatrices)\s*\((.*)\)\s*$", s, re.S)
            if call:
                out.append({"file": rel, "method": name, "line": line + s.count("\n"),
                            "call": call.group(1), "args": call.group(2).strip(),
                            "vars": json.loads(json.dumps(env))})
    return out


MM_TESTS = T + "io/MatrixMarketReadTests.java"
MM_MATRICES = T + "io/MatrixMarketMatrices.java"


def mm_expected(src):
    """The expected matrices of MatrixMarketMatrices.java, by field name:
    {"kind": "dense" | "cdense" | "coo", "shape", "data" (dense: rows; coo: values),
    "rows", "cols" (coo: sorted by (row, col), stable, as sortIndices does)}."""
    out = {}
    for m in re.finditer(r"static final (double\[\]\[\]|Complex128\[\]\[\]|CooMatrix|Matrix|CMatrix)\s+(\w+)\s*=", src):
        typ, name = m.group(1), m.group(2)
        p = m.end()
        depth, q = 0, p
        while True:  # the initialiser runs to the ';' at bracket depth 0
            c = src[q]
            depth += (c in "({") - (c in ")}")
            if c == ";" and depth == 0:
                break
            q += 1
        init = src[p:q].strip()
        if typ in ("double[][]", "Complex128[][]"):
            rows = Lit(init).value()
        elif typ in ("Matrix", "CMatrix"):
            inner = init[init.index("(") + 1:init.rindex(")")]
            rows = Lit(inner).value()
        else:  # CooMatrix(new Shape(r, c), new double[]{...}, new int[]{rows}, new int[]{cols})
            shape = [int(v) for v in re.search(r"new Shape\((\d+),\s*(\d+)\)", init).groups()]
            arrays = []
            lit = Lit(init)
            lit.p = init.index("new double[]")
            for _ in range(3):
                arrays.append(lit.value())
                lit.ws()
                if lit.peek(","):
                    lit.eat(",")
            vals, r, c = arrays
            order = sorted(range(len(vals)), key=lambda i: (r[i], c[i]))  # stable, as CooDataSorter
            out[name] = {"kind": "coo", "shape": shape, "data": [vals[i] for i in order],
                         "rows": [int(r[i]) for i in order], "cols": [int(c[i]) for i in order]}
            continue
        cplx = typ.startswith("Complex") or typ == "CMatrix"
        out[name] = {"kind": "cdense" if cplx else "dense", "shape": [len(rows), len(rows[0])], "data": rows}
    return out


def mm_cases(root):
    tests = open(os.path.join(root, MM_TESTS)).read()
    expected = mm_expected(open(os.path.join(root, MM_MATRICES)).read())
    cases = []
    methods = []
    for m in re.finditer(r"@Test\s+void\s+(\w+)\s*\(\s*\)\s*(?:throws\s+\w+\s*)?\{", tests):
        depth, p = 1, m.end()
        while depth:
            depth += (tests[p] == "{") - (tests[p] == "}")
            p += 1
        methods.append((m.group(1), tests[m.end():p - 1], tests[:m.end()].count("\n") + 1))
    for name, body, line0 in methods:
        for m in re.finditer(r'fileName\s*=\s*"\./(src/test/data/matrix_market/[^"]+)";\s*'
                             r'exp\s*=\s*(?:new \w+\()?MatrixMarketMatrices\.(\w+)', body):
            rel = m.group(1)
            with open(os.path.join(root, rel)) as fh:
                text = fh.read()
            cases.append({"file": rel, "method": name, "test_file": MM_TESTS,
                          "line": line0 + body[:m.start()].count("\n"), "expected_name": m.group(2),
                          "expected": expected[m.group(2)], "text": text})
    return cases


def main(root):
    golden = {}
    for key, rel in FILES.items():
        golden[key] = cases_of(os.path.join(root, rel), rel)
    golden["matrix_market"] = mm_cases(root)
    with open(os.path.join(HERE, "reference_golden.json"), "w") as f:
        json.dump(golden, f, indent=1)
    print({k: len(v) for k, v in golden.items()})


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/flag4j (the Flag4j project root)")
    main(sys.argv[1])
