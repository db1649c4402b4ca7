"""Seeded synthetic inputs with the workload shapes and distributions.

Flag4j's own generators cannot stand in (RealGaussian.sample ignores mean and
std, src/main/java/org/flag4j/rng/distributions/RealGaussian.java:85, and the
sparse generator draws from an unseeded global RNG,
src/main/java/org/flag4j/rng/RandomArray.java:169), so inputs come from
numpy's PCG64 with fixed seeds.
"""
import numpy as np


def rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def uniform(m, n, seed):
    """Entries i.i.d. uniform[-1, 1)."""
    return rng(seed).uniform(-1.0, 1.0, size=(m, n))


def normal(m, n, seed):
    return rng(seed).standard_normal(size=(m, n))


def scaled(m, n, phi, seed, per="row", cplx=False):
    """u * 2^e, u ~ uniform[-1, 1), integer e ~ uniform[-phi, phi] per row (A) or per column (B)."""
    g = rng(seed)
    u = g.uniform(-1.0, 1.0, size=(m, n))
    if cplx:
        u = u + 1j * g.uniform(-1.0, 1.0, size=(m, n))
    e = g.integers(-phi, phi + 1, size=(m if per == "row" else n))
    s = np.ldexp(1.0, e)
    return u * (s[:, None] if per == "row" else s[None, :])


def csr_poisson(rows, cols, lam=16.0, lo=1, hi=256, seed=0):
    """Square-ish CSR: row lengths Poisson(lam) clipped to [lo, hi], columns drawn
    uniformly without replacement per row and sorted, values N(0, 1).
    Returns (rowptr int32[rows+1], colidx int32[nnz], vals float64[nnz])."""
    g = rng(seed)
    lens = np.clip(g.poisson(lam, size=rows), lo, min(hi, cols)).astype(np.int64)
    rowptr = np.zeros(rows + 1, np.int64)
    np.cumsum(lens, out=rowptr[1:])
    nnz = int(rowptr[-1])
    row_of = np.repeat(np.arange(rows, dtype=np.int64), lens)
    key = row_of * cols + g.integers(0, cols, size=nnz)
    while True:
        key.sort()
        dup = np.nonzero(key[1:] == key[:-1])[0] + 1
        if dup.size == 0:
            break
        key[dup] = (key[dup] // cols) * cols + g.integers(0, cols, size=dup.size)
    colidx = (key % cols).astype(np.int32)
    vals = g.standard_normal(nnz)
    return rowptr.astype(np.int32), colidx, vals


def coo_shuffled(rowptr, colidx, vals, seed=0):
    """COO triplets of a CSR matrix in a random order (for sort tests)."""
    rows = len(rowptr) - 1
    r = np.repeat(np.arange(rows, dtype=np.int32), np.diff(rowptr))
    p = rng(seed).permutation(len(colidx))
    return r[p], np.asarray(colidx)[p], np.asarray(vals)[p]
