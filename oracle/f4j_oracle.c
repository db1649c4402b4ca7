/*
 * f4j_oracle.c -- CPU oracle for the GB300 product engine.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, the CPU loops
 * that Flag4j (0.1.0-beta) runs for the product path, so that the CUDA
 * library can be checked against the reference's own arithmetic.  Only the
 * tests, the smoke check and the benchmark's CPU-baseline leg load it; the
 * product library never links or calls it.
 *
 * Every function names the reference loop it restates (paths are relative
 * to the Flag4j project root).  Compiled with -O2 -ffp-contract=off
 * -fno-fast-math so that each `a*b` and each `+` is rounded separately,
 * exactly as the JVM does (Java never contracts to FMA).  With that, the
 * restatement is bit-identical to the Java kernels the dispatchers select,
 * which the golden-vector tests pin.
 *
 * Parallel variants split rows into `threads` contiguous chunks of
 * ceil(rows/threads) rows, as ThreadManager.concurrentOperation does
 * (src/main/java/org/flag4j/concurrency/ThreadManager.java:155-169).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* thread helper: ThreadManager.concurrentOperation row chunking        */
/* ------------------------------------------------------------------ */
typedef void (*orc_rows_fn)(void* arg, int64_t r0, int64_t r1);
typedef struct {
    orc_rows_fn fn;
    void* arg;
    int64_t r0, r1;
} orc_task;

static void* orc_task_run(void* p) {
    orc_task* t = (orc_task*)p;
    if (t->r0 < t->r1) t->fn(t->arg, t->r0, t->r1);
    return NULL;
}

static void orc_parallel_rows(int64_t rows, int threads, orc_rows_fn fn, void* arg) {
    if (threads <= 1 || rows < 2) {
        fn(arg, 0, rows);
        return;
    }
    if (threads > 512) threads = 512;
    int64_t chunk = (rows + threads - 1) / threads;
    pthread_t tid[512];
    orc_task task[512];
    int live[512];
    for (int t = 0; t < threads; t++) {
        int64_t r0 = (int64_t)t * chunk;
        int64_t r1 = r0 + chunk < rows ? r0 + chunk : rows;
        task[t].fn = fn;
        task[t].arg = arg;
        task[t].r0 = r0 < rows ? r0 : rows;
        task[t].r1 = r1;
        live[t] = pthread_create(&tid[t], NULL, orc_task_run, &task[t]) == 0;
        if (!live[t]) orc_task_run(&task[t]);
    }
    for (int t = 0; t < threads; t++)
        if (live[t]) pthread_join(tid[t], NULL);
}

/* ------------------------------------------------------------------ */
/* Real dense GEMM                                                      */
/* RealDenseMatMult.reordered / concurrentReordered /                   */
/* blockedReordered / concurrentBlockedReordered                        */
/* (src/main/java/org/flag4j/linalg/ops/dense/real/                     */
/*  RealDenseMatMult.java:284-310, :374-415).  Each dest element        */
/* accumulates a[i,k]*b[k,j] for ascending k, product and sum rounded   */
/* separately, starting from +0.0.  Blocking over j/k does not change   */
/* the per-element order, so one restatement covers all four.          */
/* ------------------------------------------------------------------ */
typedef struct {
    int64_t m, n, k;
    const double *A, *B;
    double* C;
} orc_gemm_args;

static void orc_dgemm_rows(void* p, int64_t r0, int64_t r1) {
    orc_gemm_args* g = (orc_gemm_args*)p;
    const int64_t n = g->n, k = g->k;
    for (int64_t i = r0; i < r1; i++) {
        double* dst = g->C + i * n;
        for (int64_t j = 0; j < n; j++) dst[j] = 0.0;
        const double* arow = g->A + i * k;
        for (int64_t kk = 0; kk < k; kk++) {
            const double av = arow[kk];
            const double* brow = g->B + kk * n;
            for (int64_t j = 0; j < n; j++) {
                double prod = av * brow[j];
                dst[j] = dst[j] + prod;
            }
        }
    }
}

void orc_dgemm(int64_t m, int64_t n, int64_t k, const double* A, const double* B, double* C,
               int threads) {
    orc_gemm_args g = {m, n, k, A, B, C};
    orc_parallel_rows(m, threads, orc_dgemm_rows, &g);
}

/* RealDenseMatMultTranspose.multTranspose* (…/dense/real/
 * RealDenseMatMultTranspose.java:190-233): C = A * B^T with B given as
 * n x k.  `sum` is seeded from dest, so each element is an ascending-k
 * sequential dot. */
static void orc_dgemm_abt_rows(void* p, int64_t r0, int64_t r1) {
    orc_gemm_args* g = (orc_gemm_args*)p;
    const int64_t n = g->n, k = g->k;
    for (int64_t i = r0; i < r1; i++) {
        const double* arow = g->A + i * k;
        for (int64_t j = 0; j < n; j++) {
            const double* brow = g->B + j * k;
            double sum = 0.0;
            for (int64_t kk = 0; kk < k; kk++) {
                double prod = arow[kk] * brow[kk];
                sum = sum + prod;
            }
            g->C[i * n + j] = sum;
        }
    }
}

void orc_dgemm_abt(int64_t m, int64_t n, int64_t k, const double* A, const double* Bt, double* C,
                   int threads) {
    orc_gemm_args g = {m, n, k, A, Bt, C};
    orc_parallel_rows(m, threads, orc_dgemm_abt_rows, &g);
}

/* RealDenseMatMult.blockedVector / concurrentBlockedVector
 * (RealDenseMatMult.java:458-490, :537-569): y[i] accumulates 64-wide
 * partial dots (block size from GeneralConfigs.properties). */
void orc_dgemv_blocked(int64_t m, int64_t k, const double* A, const double* x, double* y,
                       int64_t block) {
    for (int64_t i = 0; i < m; i++) y[i] = 0.0;
    for (int64_t ii = 0; ii < m; ii += block) {
        int64_t ib = ii + block < m ? ii + block : m;
        for (int64_t kk = 0; kk < k; kk += block) {
            int64_t kb = kk + block < k ? kk + block : k;
            for (int64_t i = ii; i < ib; i++) {
                double sum = 0.0;
                for (int64_t q = kk; q < kb; q++) {
                    double prod = A[i * k + q] * x[q];
                    sum = sum + prod;
                }
                y[i] = y[i] + sum;
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* Complex dense GEMM over Complex128                                   */
/* DenseSemiringMatMult.standard/reordered/concurrentBlockedReordered   */
/* (…/dense/semiring_ops/DenseSemiringMatMult.java:54-124, :382-424)    */
/* with Complex128.mult / add (src/main/java/org/flag4j/numbers/        */
/* Complex128.java:336-341, :276-278):                                  */
/*   pr = ar*br - ai*bi ; pi = ar*bi + ai*br ; d = (dr+pr, di+pi)       */
/* Data is interleaved (re, im) pairs, row-major.                       */
/* ------------------------------------------------------------------ */
static void orc_zgemm_rows(void* p, int64_t r0, int64_t r1) {
    orc_gemm_args* g = (orc_gemm_args*)p;
    const int64_t n = g->n, k = g->k;
    for (int64_t i = r0; i < r1; i++) {
        double* dst = g->C + 2 * i * n;
        for (int64_t j = 0; j < 2 * n; j++) dst[j] = 0.0;
        for (int64_t kk = 0; kk < k; kk++) {
            const double ar = g->A[2 * (i * k + kk)];
            const double ai = g->A[2 * (i * k + kk) + 1];
            const double* brow = g->B + 2 * kk * n;
            for (int64_t j = 0; j < n; j++) {
                const double br = brow[2 * j], bi = brow[2 * j + 1];
                double t1 = ar * br, t2 = ai * bi, t3 = ar * bi, t4 = ai * br;
                double pr = t1 - t2;
                double pi = t3 + t4;
                dst[2 * j] = dst[2 * j] + pr;
                dst[2 * j + 1] = dst[2 * j + 1] + pi;
            }
        }
    }
}

void orc_zgemm(int64_t m, int64_t n, int64_t k, const double* A, const double* B, double* C,
               int threads) {
    orc_gemm_args g = {m, n, k, A, B, C};
    orc_parallel_rows(m, threads, orc_zgemm_rows, &g);
}

/* ------------------------------------------------------------------ */
/* Mixed real / complex dense products                                  */
/* RealFieldDenseMatMult.reordered (…/dense/real_field_ops/              */
/* RealFieldDenseMatMult.java:99-135), the order of every variant the   */
/* MatrixMultiplyDispatcher picks for Matrix.mult(CMatrix) (:139-200):  */
/*   dest[i][j] = dest[i][j].add(B[k][j].mult(a[i][k])), k ascending;    */
/* Complex128.mult(double) scales both parts, so each part is a real    */
/* k-ascending no-FMA sum.  CMatrix.mult(Matrix) (:201-260, kernels     */
/* :618-655): dest[i][j] += A[i][k].mult(b[k][j]), the same per part.   */
/* ------------------------------------------------------------------ */
static void orc_rzgemm_rows(void* p, int64_t r0, int64_t r1) {
    orc_gemm_args* g = (orc_gemm_args*)p;  /* A real m x k, B complex k x n */
    const int64_t n = g->n, k = g->k;
    for (int64_t i = r0; i < r1; i++) {
        double* dst = g->C + 2 * i * n;
        for (int64_t j = 0; j < 2 * n; j++) dst[j] = 0.0;
        for (int64_t kk = 0; kk < k; kk++) {
            const double a = g->A[i * k + kk];
            const double* brow = g->B + 2 * kk * n;
            for (int64_t j = 0; j < n; j++) {
                double pr = brow[2 * j] * a, pi = brow[2 * j + 1] * a;
                dst[2 * j] = dst[2 * j] + pr;
                dst[2 * j + 1] = dst[2 * j + 1] + pi;
            }
        }
    }
}

void orc_rzgemm(int64_t m, int64_t n, int64_t k, const double* A, const double* B, double* C, int threads) {
    orc_gemm_args g = {m, n, k, A, B, C};
    orc_parallel_rows(m, threads, orc_rzgemm_rows, &g);
}

static void orc_zrgemm_rows(void* p, int64_t r0, int64_t r1) {
    orc_gemm_args* g = (orc_gemm_args*)p;  /* A complex m x k, B real k x n */
    const int64_t n = g->n, k = g->k;
    for (int64_t i = r0; i < r1; i++) {
        double* dst = g->C + 2 * i * n;
        for (int64_t j = 0; j < 2 * n; j++) dst[j] = 0.0;
        for (int64_t kk = 0; kk < k; kk++) {
            const double ar = g->A[2 * (i * k + kk)], ai = g->A[2 * (i * k + kk) + 1];
            const double* brow = g->B + kk * n;
            for (int64_t j = 0; j < n; j++) {
                double pr = ar * brow[j], pi = ai * brow[j];
                dst[2 * j] = dst[2 * j] + pr;
                dst[2 * j + 1] = dst[2 * j + 1] + pi;
            }
        }
    }
}

void orc_zrgemm(int64_t m, int64_t n, int64_t k, const double* A, const double* B, double* C, int threads) {
    orc_gemm_args g = {m, n, k, A, B, C};
    orc_parallel_rows(m, threads, orc_zrgemm_rows, &g);
}

/* ------------------------------------------------------------------ */
/* CSR x dense                                                          */
/* RealCsrDenseMatMult.standardVector (…/dense_sparse/csr/real/          */
/* RealCsrDenseMatMult.java:172-192): y[i] += v*x[col] in storage order. */
/* RealCsrDenseMatMult.standard (:55-82): Y[i,:] += v*X[col,:] in       */
/* storage order.  Both single-threaded in the reference; the optional  */
/* `threads` split keeps per-row order, so results are unchanged.       */
/* ------------------------------------------------------------------ */
typedef struct {
    int64_t ncols;
    const int32_t *rowptr, *colidx;
    const double *vals, *X;
    double* Y;
} orc_csr_args;

static void orc_spmv_rows(void* p, int64_t r0, int64_t r1) {
    orc_csr_args* a = (orc_csr_args*)p;
    for (int64_t i = r0; i < r1; i++) {
        double acc = 0.0;
        for (int32_t q = a->rowptr[i]; q < a->rowptr[i + 1]; q++) {
            double prod = a->vals[q] * a->X[a->colidx[q]];
            acc = acc + prod;
        }
        a->Y[i] = acc;
    }
}

void orc_spmv(int64_t rows, const int32_t* rowptr, const int32_t* colidx, const double* vals,
              const double* x, double* y, int threads) {
    orc_csr_args a = {1, rowptr, colidx, vals, x, y};
    orc_parallel_rows(rows, threads, orc_spmv_rows, &a);
}

static void orc_spmm_rows(void* p, int64_t r0, int64_t r1) {
    orc_csr_args* a = (orc_csr_args*)p;
    const int64_t nc = a->ncols;
    for (int64_t i = r0; i < r1; i++) {
        double* dst = a->Y + i * nc;
        for (int64_t j = 0; j < nc; j++) dst[j] = 0.0;
        for (int32_t q = a->rowptr[i]; q < a->rowptr[i + 1]; q++) {
            const double v = a->vals[q];
            const double* xr = a->X + (int64_t)a->colidx[q] * nc;
            for (int64_t j = 0; j < nc; j++) {
                double prod = v * xr[j];
                dst[j] = dst[j] + prod;
            }
        }
    }
}

void orc_spmm(int64_t rows, int64_t ncols, const int32_t* rowptr, const int32_t* colidx,
              const double* vals, const double* X, double* Y, int threads) {
    orc_csr_args a = {ncols, rowptr, colidx, vals, X, Y};
    orc_parallel_rows(rows, threads, orc_spmm_rows, &a);
}

/* Real CSR x complex dense: RealFieldDenseCsrMatMult.standard          */
/* (…/dense_sparse/csr/real_field_ops/RealFieldDenseCsrMatMult.java:    */
/* 62-91): Y[i][j] = Y[i][j].add(X[col][j].mult(v)) in storage order.   */
/* Complex CSR x complex dense: DenseCsrSemiringMatMult.standard        */
/* (…/dense_sparse/csr/semiring_ops/DenseCsrSemiringMatMult.java:59-98) */
/* over Complex128: Y[i][j] = Y[i][j].add(X[col][j].mult(v)) with        */
/* Complex128.mult (Complex128.java:336-341) of x = X[col][j] by v:      */
/*   pr = xr*vr - xi*vi ; pi = xr*vi + xi*vr.                            */
/* X, Y interleaved complex; vals interleaved complex for the latter.   */
static void orc_spmm_rz_rows(void* p, int64_t r0, int64_t r1) {
    orc_csr_args* a = (orc_csr_args*)p;
    const int64_t nc = a->ncols;
    for (int64_t i = r0; i < r1; i++) {
        double* dst = a->Y + 2 * i * nc;
        for (int64_t j = 0; j < 2 * nc; j++) dst[j] = 0.0;
        for (int32_t q = a->rowptr[i]; q < a->rowptr[i + 1]; q++) {
            const double v = a->vals[q];
            const double* xr = a->X + 2 * (int64_t)a->colidx[q] * nc;
            for (int64_t j = 0; j < nc; j++) {
                double pr = xr[2 * j] * v, pi = xr[2 * j + 1] * v;
                dst[2 * j] = dst[2 * j] + pr;
                dst[2 * j + 1] = dst[2 * j + 1] + pi;
            }
        }
    }
}

void orc_spmm_rz(int64_t rows, int64_t ncols, const int32_t* rowptr, const int32_t* colidx,
                 const double* vals, const double* X, double* Y, int threads) {
    orc_csr_args a = {ncols, rowptr, colidx, vals, X, Y};
    orc_parallel_rows(rows, threads, orc_spmm_rz_rows, &a);
}

static void orc_zspmm_rows(void* p, int64_t r0, int64_t r1) {
    orc_csr_args* a = (orc_csr_args*)p;
    const int64_t nc = a->ncols;
    for (int64_t i = r0; i < r1; i++) {
        double* dst = a->Y + 2 * i * nc;
        for (int64_t j = 0; j < 2 * nc; j++) dst[j] = 0.0;
        for (int32_t q = a->rowptr[i]; q < a->rowptr[i + 1]; q++) {
            const double vr = a->vals[2 * q], vi = a->vals[2 * q + 1];
            const double* xr = a->X + 2 * (int64_t)a->colidx[q] * nc;
            for (int64_t j = 0; j < nc; j++) {
                const double x_r = xr[2 * j], x_i = xr[2 * j + 1];
                double t1 = x_r * vr, t2 = x_i * vi, t3 = x_r * vi, t4 = x_i * vr;
                double pr = t1 - t2, pi = t3 + t4;
                dst[2 * j] = dst[2 * j] + pr;
                dst[2 * j + 1] = dst[2 * j + 1] + pi;
            }
        }
    }
}

void orc_zspmm(int64_t rows, int64_t ncols, const int32_t* rowptr, const int32_t* colidx,
               const double* vals, const double* X, double* Y, int threads) {
    orc_csr_args a = {ncols, rowptr, colidx, vals, X, Y};
    orc_parallel_rows(rows, threads, orc_zspmm_rows, &a);
}

/* ------------------------------------------------------------------ */
/* Sparse structure                                                     */
/* ------------------------------------------------------------------ */

/* CooMatrix.toCsr (src/main/java/org/flag4j/arrays/sparse/
 * CooMatrix.java:457-470): rowPtr[r+1]++ per entry, inclusive prefix sum.
 * Values and column indices are copied unchanged (input assumed
 * row-sorted). */
void orc_coo_to_csr(int64_t rows, int64_t nnz, const int32_t* rowidx, int32_t* rowptr) {
    for (int64_t i = 0; i <= rows; i++) rowptr[i] = 0;
    for (int64_t q = 0; q < nnz; q++) rowptr[rowidx[q] + 1]++;
    for (int64_t i = 0; i < rows; i++) rowptr[i + 1] += rowptr[i];
}

/* CooMatrix.sortIndices -> CooDataSorter.sparseSort (…/sparse/coo/
 * CooDataSorter.java:176-259): stable sort by row, then stable sort by
 * column inside equal-row runs, i.e. a stable lexicographic (row, col)
 * sort; duplicates keep their input order.  Restated as a stable merge
 * sort of an index permutation.  `perm_out` (may be NULL) receives the
 * source position of each output entry. */
static int orc_key_less(const int32_t* r, const int32_t* c, int64_t a, int64_t b) {
    if (r[a] != r[b]) return r[a] < r[b];
    return c[a] < c[b];
}

/* CSR x CSR, dense result: RealCsrMatMult.standard                      */
/* (src/main/java/org/flag4j/linalg/ops/sparse/csr/real/                  */
/* RealCsrMatMult.java:53-75): destEntries[i*n2 + bCol] += aVal*bVal over */
/* row i's nonzeros in storage order, then the nonzeros of B's row aCol;  */
/* each product and sum rounded (no contraction).                        */
void orc_spgemm_dense(int64_t rows, int64_t n2, const int32_t* arp, const int32_t* aci, const double* av,
                      const int32_t* brp, const int32_t* bci, const double* bv, double* C) {
    for (int64_t i = 0; i < rows * n2; i++) C[i] = 0.0;
    for (int64_t i = 0; i < rows; i++) {
        double* d = C + i * n2;
        for (int32_t q = arp[i]; q < arp[i + 1]; q++) {
            const int32_t k = aci[q];
            const double a = av[q];
            for (int32_t t = brp[k]; t < brp[k + 1]; t++) {
                const double prod = a * bv[t];
                d[bci[t]] = d[bci[t]] + prod;
            }
        }
    }
}

static int orc_cmp_i32(const void* x, const void* y) {
    const int32_t a = *(const int32_t*)x, b = *(const int32_t*)y;
    return (a > b) - (a < b);
}

/* CSR x CSR, CSR result: RealCsrMatMult.standardAsSparse (:92-131).  Per  */
/* row, tempMap.merge(bCol, bVal*aVal, Double::sum) in the same loop order */
/* (:107-118): the first product of a column is stored as is, later ones  */
/* are added to it (old + new); then the row's columns ascending          */
/* (:121-127), every touched column kept.  Fills out_rp (rows + 1) and,   */
/* when out_ci / out_v are non-null, the entries; returns the nnz.        */
int64_t orc_spgemm_csr(int64_t rows, int64_t n2, const int32_t* arp, const int32_t* aci, const double* av,
                       const int32_t* brp, const int32_t* bci, const double* bv, int32_t* out_rp,
                       int32_t* out_ci, double* out_v) {
    double* acc = (double*)calloc(n2 > 0 ? n2 : 1, sizeof(double));
    unsigned char* seen = (unsigned char*)calloc(n2 > 0 ? n2 : 1, 1);
    int32_t* list = (int32_t*)malloc(sizeof(int32_t) * (n2 > 0 ? n2 : 1));
    int64_t nnz = 0;
    out_rp[0] = 0;
    for (int64_t i = 0; i < rows; i++) {
        int64_t nl = 0;
        for (int32_t q = arp[i]; q < arp[i + 1]; q++) {
            const int32_t k = aci[q];
            const double a = av[q];
            for (int32_t t = brp[k]; t < brp[k + 1]; t++) {
                const int32_t j = bci[t];
                const double prod = bv[t] * a;
                if (!seen[j]) {
                    seen[j] = 1;
                    acc[j] = prod;
                    list[nl++] = j;
                } else {
                    acc[j] = acc[j] + prod;
                }
            }
        }
        qsort(list, (size_t)nl, sizeof(int32_t), orc_cmp_i32);
        for (int64_t u = 0; u < nl; u++) {
            const int32_t j = list[u];
            if (out_ci) {
                out_ci[nnz] = j;
                out_v[nnz] = acc[j];
            }
            nnz++;
            seen[j] = 0;
        }
        out_rp[i + 1] = (int32_t)nnz;
    }
    free(acc);
    free(seen);
    free(list);
    return nnz;
}

/* The product one entry of a CSR x CSR product adds, by the operands'     */
/* value kinds (ak / bk 1 = complex, interleaved):                         */
/*   real x real: aVal*bVal (RealCsrMatMult.java:70)                       */
/*   real x complex: bVal.mult(aVal) = (b.re*a, b.im*a)                    */
/*     (RealComplexCsrMatMult.java:78; Complex128.mult(double))            */
/*   complex x real: aVal.mult(bVal) = (a.re*b, a.im*b) (:113)             */
/*   complex x complex: bVal.mult(aVal) (SemiringCsrMatMult.java:81,       */
/*     Complex128.java:336-341): (b.re*a.re - b.im*a.im, b.re*a.im + b.im*a.re) */
static void orc_csr_prod(int ak, int bk, const double* av, int64_t q, const double* bv, int64_t t, double* pr,
                         double* pi) {
    if (!ak && !bk) {
        *pr = av[q] * bv[t];
        *pi = 0.0;
    } else if (!ak) {
        const double a = av[q];
        *pr = bv[2 * t] * a;
        *pi = bv[2 * t + 1] * a;
    } else if (!bk) {
        const double b = bv[t];
        *pr = av[2 * q] * b;
        *pi = av[2 * q + 1] * b;
    } else {
        const double ar = av[2 * q], ai = av[2 * q + 1], br = bv[2 * t], bi = bv[2 * t + 1];
        const double rr = br * ar, ii = bi * ai, ri = br * ai, ir = bi * ar;
        *pr = rr - ii;
        *pi = ri + ir;
    }
}

/* Dense result of the complex variants (RealComplexCsrMatMult.standard,  */
/* :58-83 and :93-118; SemiringCsrMatMult.standard, :58-87): C (rows x n2 */
/* complex, interleaved) starts at Complex128.ZERO and adds each product  */
/* per part in the loop order of orc_spgemm_dense.                        */
void orc_spgemm_dense_z(int ak, int bk, int64_t rows, int64_t n2, const int32_t* arp, const int32_t* aci,
                        const double* av, const int32_t* brp, const int32_t* bci, const double* bv, double* C) {
    for (int64_t i = 0; i < 2 * rows * n2; i++) C[i] = 0.0;
    for (int64_t i = 0; i < rows; i++) {
        double* d = C + 2 * i * n2;
        for (int32_t q = arp[i]; q < arp[i + 1]; q++) {
            const int32_t k = aci[q];
            for (int32_t t = brp[k]; t < brp[k + 1]; t++) {
                double pr, pi;
                orc_csr_prod(ak, bk, av, q, bv, t, &pr, &pi);
                const int64_t j = bci[t];
                d[2 * j] = d[2 * j] + pr;
                d[2 * j + 1] = d[2 * j + 1] + pi;
            }
        }
    }
}

/* CSR result of the complex variants (RealComplexCsrMatMult.standardAs-  */
/* Sparse :133-181 and :190-238; SemiringCsrMatMult.standardToSparse      */
/* :109-158): tempMap.merge(bCol, product, add) per row, columns sorted;  */
/* as orc_spgemm_csr with complex values (out_v interleaved).             */
int64_t orc_spgemm_csr_z(int ak, int bk, int64_t rows, int64_t n2, const int32_t* arp, const int32_t* aci,
                         const double* av, const int32_t* brp, const int32_t* bci, const double* bv,
                         int32_t* out_rp, int32_t* out_ci, double* out_v) {
    double* acc = (double*)calloc(2 * (n2 > 0 ? n2 : 1), sizeof(double));
    unsigned char* seen = (unsigned char*)calloc(n2 > 0 ? n2 : 1, 1);
    int32_t* list = (int32_t*)malloc(sizeof(int32_t) * (n2 > 0 ? n2 : 1));
    int64_t nnz = 0;
    out_rp[0] = 0;
    for (int64_t i = 0; i < rows; i++) {
        int64_t nl = 0;
        for (int32_t q = arp[i]; q < arp[i + 1]; q++) {
            const int32_t k = aci[q];
            for (int32_t t = brp[k]; t < brp[k + 1]; t++) {
                const int32_t j = bci[t];
                double pr, pi;
                orc_csr_prod(ak, bk, av, q, bv, t, &pr, &pi);
                if (!seen[j]) {
                    seen[j] = 1;
                    acc[2 * j] = pr;
                    acc[2 * j + 1] = pi;
                    list[nl++] = j;
                } else {
                    acc[2 * j] = acc[2 * j] + pr;
                    acc[2 * j + 1] = acc[2 * j + 1] + pi;
                }
            }
        }
        qsort(list, (size_t)nl, sizeof(int32_t), orc_cmp_i32);
        for (int64_t u = 0; u < nl; u++) {
            const int32_t j = list[u];
            if (out_ci) {
                out_ci[nnz] = j;
                out_v[2 * nnz] = acc[2 * j];
                out_v[2 * nnz + 1] = acc[2 * j + 1];
            }
            nnz++;
            seen[j] = 0;
        }
        out_rp[i + 1] = (int32_t)nnz;
    }
    free(acc);
    free(seen);
    free(list);
    return nnz;
}


void orc_coo_sort(int64_t nnz, int32_t* rowidx, int32_t* colidx, double* vals, int64_t* perm_out) {
    int64_t* p = (int64_t*)malloc(sizeof(int64_t) * (nnz > 0 ? nnz : 1));
    int64_t* t = (int64_t*)malloc(sizeof(int64_t) * (nnz > 0 ? nnz : 1));
    for (int64_t i = 0; i < nnz; i++) p[i] = i;
    for (int64_t w = 1; w < nnz; w *= 2) {
        for (int64_t lo = 0; lo < nnz; lo += 2 * w) {
            int64_t mid = lo + w < nnz ? lo + w : nnz;
            int64_t hi = lo + 2 * w < nnz ? lo + 2 * w : nnz;
            int64_t a = lo, b = mid, o = lo;
            while (a < mid && b < hi) {
                /* take from the right run only when strictly smaller: stable */
                if (orc_key_less(rowidx, colidx, p[b], p[a])) t[o++] = p[b++];
                else t[o++] = p[a++];
            }
            while (a < mid) t[o++] = p[a++];
            while (b < hi) t[o++] = p[b++];
        }
        int64_t* s = p;
        p = t;
        t = s;
    }
    int32_t* r2 = (int32_t*)malloc(sizeof(int32_t) * (nnz > 0 ? nnz : 1));
    int32_t* c2 = (int32_t*)malloc(sizeof(int32_t) * (nnz > 0 ? nnz : 1));
    double* v2 = (double*)malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
    for (int64_t i = 0; i < nnz; i++) {
        r2[i] = rowidx[p[i]];
        c2[i] = colidx[p[i]];
        if (vals) v2[i] = vals[p[i]];
        if (perm_out) perm_out[i] = p[i];
    }
    memcpy(rowidx, r2, sizeof(int32_t) * nnz);
    memcpy(colidx, c2, sizeof(int32_t) * nnz);
    if (vals) memcpy(vals, v2, sizeof(double) * nnz);
    free(r2);
    free(c2);
    free(v2);
    free(p);
    free(t);
}

/* RealCsrOps.transpose (…/sparse/csr/real/RealCsrOps.java:195-225):
 * counting sort by column; scatter in row order through tempPos[col]++,
 * so output rows (old columns) list old rows ascending.  `perm` (may be
 * NULL) receives, for each output position, the source nnz index: the
 * transpose permutation. */
void orc_csr_transpose(int64_t rows, int64_t cols, const int32_t* rowptr, const int32_t* colidx,
                       const double* vals, int32_t* t_rowptr, int32_t* t_colidx, double* t_vals,
                       int32_t* perm) {
    int64_t nnz = rowptr[rows];
    for (int64_t i = 0; i <= cols; i++) t_rowptr[i] = 0;
    for (int64_t q = 0; q < nnz; q++) t_rowptr[colidx[q] + 1]++;
    for (int64_t i = 1; i <= cols; i++) t_rowptr[i] += t_rowptr[i - 1];
    int32_t* pos = (int32_t*)malloc(sizeof(int32_t) * (cols + 1));
    memcpy(pos, t_rowptr, sizeof(int32_t) * (cols + 1));
    for (int64_t r = 0; r < rows; r++) {
        for (int32_t q = rowptr[r]; q < rowptr[r + 1]; q++) {
            int32_t c = colidx[q];
            int32_t d = pos[c]++;
            if (t_vals) t_vals[d] = vals[q];
            t_colidx[d] = (int32_t)r;
            if (perm) perm[d] = q;
        }
    }
    free(pos);
}

/* SDDMM on S's pattern (no reference function; formula restatement):
 * out[q] = sum_j dC[row(q), j] * X[col(q), j], ascending j. */
void orc_sddmm(int64_t rows, int64_t ncols, const int32_t* rowptr, const int32_t* colidx,
               const double* dC, const double* X, double* out) {
    for (int64_t i = 0; i < rows; i++) {
        for (int32_t q = rowptr[i]; q < rowptr[i + 1]; q++) {
            const double* a = dC + i * ncols;
            const double* b = X + (int64_t)colidx[q] * ncols;
            double s = 0.0;
            for (int64_t j = 0; j < ncols; j++) {
                double prod = a[j] * b[j];
                s = s + prod;
            }
            out[q] = s;
        }
    }
}

/* ------------------------------------------------------------------ */
/* FP64 "truth": compensated dot (Ogita, Rump, Oishi, "Accurate sum     */
/* and dot product", SIAM J. Sci. Comput. 26(6), 2005, Algorithm Dot2): */
/* TwoProduct through fma, TwoSum (Knuth), result as hi+lo.  Evaluated  */
/* at sampled (i, j) of C = op(A)*op(B) with general strides, real or   */
/* complex.  `absref` receives sum |a||b| (the componentwise bound's     */
/* |A||B| term; for complex the sum of |ar br|+|ai bi| (+) terms).       */
/* ------------------------------------------------------------------ */
static inline void two_sum(double a, double b, double* s, double* e) {
    double x = a + b;
    double z = x - a;
    *e = (a - (x - z)) + (b - z);
    *s = x;
}

static inline void dd_add_prod(double a, double b, double* hi, double* lo) {
    double p = a * b;
    double pe = fma(a, b, -p);
    double s, e;
    two_sum(*hi, p, &s, &e);
    *hi = s;
    *lo = *lo + (e + pe);
}

/* element (r, c) of op(X) for a row-major matrix X with leading dim ld:
 * op 0: X[r, c]; op 1 (transpose): X[c, r]; op 2 (conj transpose). */
static inline void ld_elem(const double* X, int64_t ld, int op, int cplx, int64_t r, int64_t c,
                           double* re, double* im) {
    int64_t idx = (op == 0) ? r * ld + c : c * ld + r;
    if (cplx) {
        *re = X[2 * idx];
        *im = (op == 2) ? -X[2 * idx + 1] : X[2 * idx + 1];
    } else {
        *re = X[idx];
        *im = 0.0;
    }
}

void orc_truth_sampled(int64_t k, const double* A, int64_t lda, int opA, const double* B,
                       int64_t ldb, int opB, int cplx, int64_t nsamp, const int64_t* si,
                       const int64_t* sj, double* out_hi, double* out_lo, double* absref) {
    for (int64_t s = 0; s < nsamp; s++) {
        int64_t i = si[s], j = sj[s];
        double rh = 0, rl = 0, ih = 0, il = 0, ab = 0, abi = 0;
        for (int64_t q = 0; q < k; q++) {
            double ar, ai, br, bi;
            ld_elem(A, lda, opA, cplx, i, q, &ar, &ai);
            ld_elem(B, ldb, opB, cplx, q, j, &br, &bi);
            dd_add_prod(ar, br, &rh, &rl);
            ab += fabs(ar * br);
            if (cplx) {
                dd_add_prod(-ai, bi, &rh, &rl);
                dd_add_prod(ar, bi, &ih, &il);
                dd_add_prod(ai, br, &ih, &il);
                ab += fabs(ai * bi);
                abi += fabs(ar * bi) + fabs(ai * br);
            }
        }
        if (cplx) {
            out_hi[2 * s] = rh;
            out_lo[2 * s] = rl;
            out_hi[2 * s + 1] = ih;
            out_lo[2 * s + 1] = il;
            absref[2 * s] = ab;
            absref[2 * s + 1] = abi;
        } else {
            out_hi[s] = rh;
            out_lo[s] = rl;
            absref[s] = ab;
        }
    }
}

/* Componentwise |A||B| for all of C (real, op N/N), used by the parity
 * bound |C - C_ref| <= 2 k u |A||B| at sizes the CPU finishes quickly. */
static void orc_absgemm_rows(void* p, int64_t r0, int64_t r1) {
    orc_gemm_args* g = (orc_gemm_args*)p;
    const int64_t n = g->n, k = g->k;
    for (int64_t i = r0; i < r1; i++) {
        double* dst = g->C + i * n;
        for (int64_t j = 0; j < n; j++) dst[j] = 0.0;
        for (int64_t kk = 0; kk < k; kk++) {
            const double av = fabs(g->A[i * k + kk]);
            const double* brow = g->B + kk * n;
            for (int64_t j = 0; j < n; j++) dst[j] += av * fabs(brow[j]);
        }
    }
}

void orc_absgemm(int64_t m, int64_t n, int64_t k, const double* A, const double* B, double* C,
                 int threads) {
    orc_gemm_args g = {m, n, k, A, B, C};
    orc_parallel_rows(m, threads, orc_absgemm_rows, &g);
}
