// f4j_sparse.cu -- CSR products and sparse structure on sm_103a.
//
// Products follow the reference loops' per-element order exactly (storage
// order over a row's nonzeros, product and sum rounded separately), so the
// results are bit-identical to Flag4j:
//   SpMV  RealCsrDenseMatMult.standardVector
//         (src/main/java/org/flag4j/linalg/ops/dense_sparse/csr/real/RealCsrDenseMatMult.java:172-192)
//   SpMM  RealCsrDenseMatMult.standard (same file :55-82)
//   S^T X RealCsrOps.transpose + standard (…/sparse/csr/real/RealCsrOps.java:195-225)
//   S1 S2 RealCsrMatMult, RealComplexCsrMatMult, SemiringCsrMatMult (CSR x CSR)
// SpMV / SpMM also have an opt-in FMA mode (fused multiply-add in storage
// order, within 2 k u |S||X|); SDDMM (the sparse adjoint's dS) has no
// reference counterpart and meets the same bound.
// Structure (COO->CSR, stable COO sort, transpose permutation) is integer
// work done with histograms, scans, a row-bucketed sort and a stable LSD
// radix sort.
#include <vector>

#include "f4j_internal.cuh"
#include "f4j_ptx.cuh"

namespace {

// ------------------------------------------------------------------ SpMV
// Load-balanced lanes.  A warp owns rpw consecutive rows [w0, w1) with
// nonzeros [E0, E1).  Lane l owns the rows whose first nonzero lies in
// [E0 + ceil(l * span / 32), E0 + ceil((l + 1) * span / 32)), span = E1 - E0:
// consecutive rows holding about span / 32 nonzeros, found by a lower-bound
// search on the row pointers.  Rows of different lengths therefore share the
// warp's work evenly (a lane per row made every warp wait for its longest
// row: about 1.75 add steps per nonzero at Poisson(16) lengths).  Each lane
// walks its contiguous nonzeros 8 at a time, from a multiple of 8: column
// indices and values with 32-byte loads, one L2 sector each (VEC; a group's
// loads stay inside the arrays, entries outside the lane's range are loaded
// and ignored; two 16-byte loads per sector reached L2 about twice), the 8
// gathers of x in flight together, then the products and the running sum in
// storage order,
// storing y at each row end.  Each product and each sum is rounded as
// RealCsrDenseMatMult.standardVector rounds them (acc starts at +0.0), so y is
// bit-identical.  GB300's FP64 pipe (2 lane-operations per clock per SM, two
// per nonzero) bounds the exact mode; the random 8-byte gathers of x (one L2
// sector each) come next.  No shared memory, so L1 keeps its full size for
// the gathers.
// FUSED (the opt-in FMA mode) accumulates fma(v, x, acc) in the same order,
// one FP64 instruction per nonzero, within the reference's componentwise bound.
constexpr int SPMV_RPW_MAX = 256;  // rows per warp for large matrices
constexpr int SPMV_BLOCK = 256;

// Blocks per SM: 5 for the exact mode (48 registers, no spills), 4 for FMA
// (whose 48-register build spills).
template <bool FUSED>
struct SpmvOcc {
    static constexpr int BLOCKS = FUSED ? 4 : 5;
};

// 32-byte read-only loads (one sector): 8 column indices, 4 values.  The
// address must be 32-byte aligned.
__device__ __forceinline__ void ld_nc_v8_b32(const int* p, int (&c)[8]) {
    asm volatile("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(c[0]), "=r"(c[1]), "=r"(c[2]), "=r"(c[3]), "=r"(c[4]), "=r"(c[5]), "=r"(c[6]), "=r"(c[7])
                 : "l"(p));
}
__device__ __forceinline__ void ld_nc_v4_f64(const double* p, double& a, double& b, double& c, double& d) {
    asm volatile("ld.global.nc.v4.f64 {%0,%1,%2,%3}, [%4];" : "=d"(a), "=d"(b), "=d"(c), "=d"(d) : "l"(p));
}

template <bool FUSED, bool VEC>
__global__ void __launch_bounds__(SPMV_BLOCK, SpmvOcc<FUSED>::BLOCKS)
    k_spmv(int64_t rows, int64_t nnz, int rpw, const int* __restrict__ rowptr, const int* __restrict__ colidx,
           const double* __restrict__ vals, const double* __restrict__ x, double* __restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * SPMV_BLOCK + threadIdx.x) >> 5;
    const int64_t w0 = warp * rpw;
    if (w0 >= rows) return;
    const int64_t w1 = w0 + rpw < rows ? w0 + rpw : rows;
    const int64_t E0 = __ldg(rowptr + w0), span = (int64_t)__ldg(rowptr + w1) - E0;
    // first row whose first nonzero is at or after this lane's target
    const int64_t target = E0 + (span * lane + 31) / 32;
    int64_t lo = w0, hi = w1;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if ((int64_t)__ldg(rowptr + mid) >= target) hi = mid;
        else lo = mid + 1;
    }
    const int64_t a = lo;
    int64_t b = __shfl_down_sync(0xffffffffu, a, 1);
    if (lane == 31) b = w1;
    if (a >= b) return;
    const int qs = __ldg(rowptr + a), qe = __ldg(rowptr + b);
    // rend: end of row r; rnext: end of row r + 1, loaded one row ahead so that
    // a row end never waits for a load on the running sum's chain
    int64_t r = a;
    int rend = __ldg(rowptr + a + 1);
    int rnext = a + 1 < b ? __ldg(rowptr + a + 2) : qe;
    double acc = 0.0;
    while (rend == qs) {  // empty rows before the lane's first nonzero
        y[r] = 0.0;
        if (++r == b) return;
        rend = rnext;
        rnext = r + 1 < b ? __ldg(rowptr + r + 2) : qe;
    }
    for (int qb = VEC ? (qs & ~7) : qs; qb < qe; qb += 8) {
        int c[8];
        double v[8];
        if (VEC && (int64_t)qb + 8 <= nnz) {
            // qb is a multiple of 8: one 32-byte sector of indices, two of values
            ld_nc_v8_b32(colidx + qb, c);
            ld_nc_v4_f64(vals + qb, v[0], v[1], v[2], v[3]);
            ld_nc_v4_f64(vals + qb + 4, v[4], v[5], v[6], v[7]);
        } else {
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const bool ok = qb + u < qe;
                c[u] = ok ? __ldg(colidx + qb + u) : 0;
                v[u] = ok ? __ldg(vals + qb + u) : 0.0;
            }
        }
        double xv[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int q = qb + u;
            xv[u] = (q >= qs && q < qe) ? __ldg(x + c[u]) : 0.0;
        }
        if (!FUSED) {
#pragma unroll
            for (int u = 0; u < 8; u++) v[u] = __dmul_rn(v[u], xv[u]);
        }
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int q = qb + u;
            if (q < qs || q >= qe) continue;
            acc = FUSED ? __fma_rn(v[u], xv[u], acc) : __dadd_rn(acc, v[u]);
            while (q + 1 == rend) {  // row r ends here (and any empty rows after it)
                y[r] = acc;
                acc = 0.0;
                if (++r == b) break;
                rend = rnext;
                rnext = r + 1 < b ? __ldg(rowptr + r + 2) : qe;
            }
        }
    }
}

// ------------------------------------------------------------------ SpMM
// A group of G lanes owns one row; each lane owns 2 adjacent columns
// (128-bit loads of X rows) and sums over the row's nonzeros in storage order.
// For S^T products the same kernel reads values through the transpose
// permutation and row indices from the cached S^T structure.
// FUSED (the opt-in FMA mode): one fma(v, x, acc) per nonzero and column, in
// storage order; within the reference's componentwise bound.  Its FP64 work
// is half the exact mode's, so the X gathers' latency decides its speed: it
// runs 8 blocks per SM (32 registers) to keep more of them in flight; the
// exact mode runs 6 (40 registers), its best balance of loads in flight per
// warp against warps.
template <bool VEC2, bool PERM, bool FUSED = false>
__global__ void __launch_bounds__(256, FUSED ? 8 : 6)
    k_spmm(int64_t rows, int64_t ncols, int G, const int* __restrict__ rowptr, const int* __restrict__ colidx,
           const double* __restrict__ vals, const int* __restrict__ perm, const double* __restrict__ X,
           double* __restrict__ Y) {
    const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const int lane = threadIdx.x % G;
    const int64_t row = gid;
    if (row >= rows) return;
    const int q0 = rowptr[row], q1 = rowptr[row + 1];
    constexpr int W = VEC2 ? 2 : 1;
    for (int64_t cbase = (int64_t)lane * W; cbase < ncols; cbase += (int64_t)G * W) {
        double a0 = 0.0, a1 = 0.0;
        int q = q0;
        constexpr int UN = 8;  // nonzeros whose X rows are in flight together
        for (; q + UN <= q1; q += UN) {
            int c[UN];
            double v[UN];
#pragma unroll
            for (int u = 0; u < UN; u++) {
                c[u] = __ldg(&colidx[q + u]);
                v[u] = PERM ? __ldg(&vals[__ldg(&perm[q + u])]) : __ldg(&vals[q + u]);
            }
            if (VEC2) {
                double2 xv[UN];
#pragma unroll
                for (int u = 0; u < UN; u++) xv[u] = __ldg(reinterpret_cast<const double2*>(X + (int64_t)c[u] * ncols + cbase));
#pragma unroll
                for (int u = 0; u < UN; u++) {
                    if (FUSED) {
                        a0 = __fma_rn(v[u], xv[u].x, a0);
                        a1 = __fma_rn(v[u], xv[u].y, a1);
                    } else {
                        a0 = __dadd_rn(a0, __dmul_rn(v[u], xv[u].x));
                        a1 = __dadd_rn(a1, __dmul_rn(v[u], xv[u].y));
                    }
                }
            } else {
                double xv[UN];
#pragma unroll
                for (int u = 0; u < UN; u++) xv[u] = __ldg(X + (int64_t)c[u] * ncols + cbase);
#pragma unroll
                for (int u = 0; u < UN; u++) a0 = FUSED ? __fma_rn(v[u], xv[u], a0) : __dadd_rn(a0, __dmul_rn(v[u], xv[u]));
            }
        }
        for (; q < q1; q++) {
            const int c = __ldg(&colidx[q]);
            const double v = PERM ? __ldg(&vals[__ldg(&perm[q])]) : __ldg(&vals[q]);
            if (VEC2) {
                const double2 xv = __ldg(reinterpret_cast<const double2*>(X + (int64_t)c * ncols + cbase));
                a0 = FUSED ? __fma_rn(v, xv.x, a0) : __dadd_rn(a0, __dmul_rn(v, xv.x));
                a1 = FUSED ? __fma_rn(v, xv.y, a1) : __dadd_rn(a1, __dmul_rn(v, xv.y));
            } else {
                const double xe = __ldg(X + (int64_t)c * ncols + cbase);
                a0 = FUSED ? __fma_rn(v, xe, a0) : __dadd_rn(a0, __dmul_rn(v, xe));
            }
        }
        if (VEC2) *reinterpret_cast<double2*>(Y + row * ncols + cbase) = make_double2(a0, a1);
        else Y[row * ncols + cbase] = a0;
    }
}

// Complex CSR x complex dense (CsrCMatrix.mult(CMatrix) ->
// DenseCsrSemiringMatMult.standard, src/main/java/org/flag4j/linalg/ops/
// dense_sparse/csr/semiring_ops/DenseCsrSemiringMatMult.java:59-98): a group
// of G lanes owns one row, a lane one complex column; per nonzero in storage
// order y += x * v with Complex128.mult's rounding (Complex128.java:336-341):
// pr = xr*vr - xi*vi, pi = xr*vi + xi*vr, each product and sum rounded.
__global__ void __launch_bounds__(256)
    k_zspmm(int64_t rows, int64_t ncols, int G, const int* __restrict__ rowptr, const int* __restrict__ colidx,
            const double2* __restrict__ vals, const double2* __restrict__ X, double2* __restrict__ Y) {
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const int lane = threadIdx.x % G;
    if (row >= rows) return;
    const int q0 = rowptr[row], q1 = rowptr[row + 1];
    for (int64_t c0 = lane; c0 < ncols; c0 += G) {
        double ar = 0.0, ai = 0.0;
        int q = q0;
        constexpr int UN = 8;  // nonzeros whose X entries are in flight together
        for (; q + UN <= q1; q += UN) {
            double2 v[UN], x[UN];
#pragma unroll
            for (int u = 0; u < UN; u++) {
                v[u] = __ldg(&vals[q + u]);
                x[u] = __ldg(&X[(int64_t)__ldg(&colidx[q + u]) * ncols + c0]);
            }
#pragma unroll
            for (int u = 0; u < UN; u++) {
                const double pr = __dsub_rn(__dmul_rn(x[u].x, v[u].x), __dmul_rn(x[u].y, v[u].y));
                const double pi = __dadd_rn(__dmul_rn(x[u].x, v[u].y), __dmul_rn(x[u].y, v[u].x));
                ar = __dadd_rn(ar, pr);
                ai = __dadd_rn(ai, pi);
            }
        }
        for (; q < q1; q++) {
            const double2 v = __ldg(&vals[q]);
            const double2 x = __ldg(&X[(int64_t)__ldg(&colidx[q]) * ncols + c0]);
            const double pr = __dsub_rn(__dmul_rn(x.x, v.x), __dmul_rn(x.y, v.y));
            const double pi = __dadd_rn(__dmul_rn(x.x, v.y), __dmul_rn(x.y, v.x));
            ar = __dadd_rn(ar, pr);
            ai = __dadd_rn(ai, pi);
        }
        Y[row * ncols + c0] = make_double2(ar, ai);
    }
}

// ------------------------------------------------------------------ SDDMM
// Warp per row of S; half-warps take alternate nonzeros; a lane owns 4
// columns of each 64-column pass (sequential), then a 16-lane tree sum.
__global__ void __launch_bounds__(256)
    k_sddmm(int64_t rows, int64_t ncols, const int* __restrict__ rowptr, const int* __restrict__ colidx,
            const double* __restrict__ A, const double* __restrict__ B, double* __restrict__ out) {
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x % 32, half = lane / 16, l16 = lane % 16;
    if (row >= rows) return;
    const int q0 = rowptr[row], q1 = rowptr[row + 1];
    const double* arow = A + row * ncols;
    for (int qb = q0; qb < q1; qb += 2) {
        const int q = qb + half;
        double s = 0.0;
        if (q < q1) {
            const double* brow = B + (int64_t)__ldg(&colidx[q]) * ncols;
            for (int64_t c0 = 0; c0 < ncols; c0 += 64) {
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const int64_t c = c0 + l16 * 4 + u;
                    if (c < ncols) s = fma(__ldg(&arow[c]), __ldg(&brow[c]), s);
                }
            }
        }
        for (int off = 8; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (q < q1 && l16 == 0) out[q] = s;
    }
}

// SDDMM with 64 columns, flat over the nonzeros: a block takes 64 consecutive
// nonzeros whatever their rows, a group of 4 lanes one nonzero.  The block's
// distinct rows of A (rows are sorted, so equal rows are adjacent) are staged
// in shared memory once, so a lane holds only its 16 values of the row of B
// in registers (60 registers and 4 blocks per SM, against 74 and about 20
// warps per SM with A in registers too).  Lane l4 of a group owns the
// 16-byte pairs l4, l4 + 4, ..., l4 + 28 of the 64 columns: the group's four
// lanes read 64 contiguous bytes per step from shared memory and from B, and
// the padded row stride (33 pairs) puts neighbouring rows in other banks.
// 16 FMAs and a 2-step tree sum per lane: 18 FP64 warp instructions per 8
// nonzeros.  The B loads are issued first, so they are in flight while the
// block stages A.  rowidx: the row of each nonzero.
constexpr int SD_NNZ = 64;        // nonzeros per block (256 threads)
constexpr int SD_PAIRS = 33;      // padded row stride of the staged rows, in 16-byte pairs
__global__ void __launch_bounds__(256, 4)
    k_sddmm64s(int64_t nnz, const int* __restrict__ rowidx, const int* __restrict__ colidx,
               const double* __restrict__ A, const double* __restrict__ B, double* __restrict__ out) {
    __shared__ double2 sA[SD_NNZ * SD_PAIRS];
    __shared__ int slot[SD_NNZ], srow[SD_NNZ], s_nrows;
    const int64_t q0 = (int64_t)blockIdx.x * SD_NNZ;
    const int tid = threadIdx.x, g = tid >> 2, l4 = tid & 3;
    const int64_t q = q0 + g;
    double2 b[8];
    if (q < nnz) {
        const double2* brow = reinterpret_cast<const double2*>(B + (int64_t)__ldg(&colidx[q]) * 64) + l4;
#pragma unroll
        for (int u = 0; u < 8; u++) b[u] = __ldg(brow + 4 * u);
    } else {
#pragma unroll
        for (int u = 0; u < 8; u++) b[u] = make_double2(0.0, 0.0);
    }
    if (tid < 32) {  // warp 0: slots of the block's nonzeros (two per lane) and the distinct rows
        int r[2];
        bool head[2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int t = tid + 32 * h;
            const int64_t qq = q0 + t;
            r[h] = qq < nnz ? __ldg(&rowidx[qq]) : -1;
            head[h] = qq < nnz && (t == 0 || __ldg(&rowidx[qq - 1]) != r[h]);
        }
        const unsigned b0 = __ballot_sync(0xffffffffu, head[0]), b1 = __ballot_sync(0xffffffffu, head[1]);
        const unsigned below = (1u << tid) - 1u;
        const int n0 = __popc(b0);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int t = tid + 32 * h;
            const int idx = (h ? n0 + __popc(b1 & below) : __popc(b0 & below)) + (head[h] ? 1 : 0) - 1;
            slot[t] = idx;
            if (head[h]) srow[idx] = r[h];
        }
        if (tid == 0) s_nrows = n0 + __popc(b1);
    }
    __syncthreads();
    const int nrows = s_nrows;
    for (int i = tid; i < nrows * 32; i += 256) {
        const int rr = i >> 5, pr = i & 31;
        sA[rr * SD_PAIRS + pr] = __ldg(reinterpret_cast<const double2*>(A + (int64_t)srow[rr] * 64) + pr);
    }
    __syncthreads();
    double s = 0.0;
    if (q < nnz) {
        const double2* arow = sA + slot[g] * SD_PAIRS + l4;
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const double2 a = arow[4 * u];
            s = fma(a.y, b[u].y, fma(a.x, b[u].x, s));
        }
    }
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    if (q < nnz && l4 == 0) out[q] = s;
}

// ------------------------------------------------------------------ structure
__global__ void k_count(int64_t n, const int* __restrict__ idx, int* __restrict__ counts_plus1) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&counts_plus1[idx[i] + 1], 1);
}

// COO -> CSR row count with the row range check of SparseValidation.validateCoo:
// one count per in-range row index in counts_plus1[r + 1], and the first
// position of an out-of-range one in *first_bad.  Lanes of a warp holding the
// same row add together (COO input is usually row-sorted, so a warp's 32
// entries fall in a few rows).
__global__ void k_count_rows_checked(int64_t n, const int* __restrict__ idx, int64_t limit,
                                     int* __restrict__ counts_plus1, int* __restrict__ first_bad) {
    const int lane = threadIdx.x & 31;
    const int64_t stride = ((int64_t)gridDim.x * blockDim.x) & ~(int64_t)31;
    for (int64_t base = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~(int64_t)31; base < n; base += stride) {
        const int64_t i = base + lane;
        const bool in = i < n;
        const int v = in ? idx[i] : -1;
        const bool ok = in && v >= 0 && v < limit;
        if (in && !ok) atomicMin(first_bad, (int)i);
        const unsigned peers = __match_any_sync(0xffffffffu, ok ? v : -1);
        if (ok && lane == __ffs(peers) - 1) atomicAdd(&counts_plus1[v + 1], __popc(peers));
    }
}

// Copy of COO column indices into the CSR with the column range check:
// the first offending position in *first_bad.  VEC: 16-byte loads and stores.
template <bool VEC>
__global__ void k_copy_cols_checked(int64_t n, const int* __restrict__ src, int64_t limit, int* __restrict__ dst,
                                    int* __restrict__ first_bad) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    int64_t done = 0;
    if (VEC) {
        const int64_t n4 = n / 4;
        for (int64_t j = t; j < n4; j += stride) {
            const int4 v = reinterpret_cast<const int4*>(src)[j];
            const int e[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int q = 0; q < 4; q++)
                if (e[q] < 0 || e[q] >= limit) atomicMin(first_bad, (int)(4 * j + q));
            reinterpret_cast<int4*>(dst)[j] = v;
        }
        done = 4 * n4;
    }
    for (int64_t i = done + t; i < n; i += stride) {
        const int v = src[i];
        if (v < 0 || v >= limit) atomicMin(first_bad, (int)i);
        dst[i] = v;
    }
}

// SparseValidation.validateCsr checks (src/main/java/org/flag4j/arrays/sparse/SparseValidation.java:151-206):
// first row with negative start or decreasing pointers, first bad column.
__global__ void k_validate_csr(int64_t rows, int64_t cols, int64_t nnz, const int* __restrict__ rowptr,
                               const int* __restrict__ colidx, int* __restrict__ bad_row,
                               int* __restrict__ bad_col) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x) {
        int s = rowptr[i], e = rowptr[i + 1];
        if (s < 0 || s > e) {
            atomicMin(bad_row, (int)i);
            continue;
        }
        for (int q = s; q < e && q < nnz; q++) {
            int c = colidx[q];
            if (c < 0 || c >= cols) {
                atomicMin(bad_col, q);
                break;
            }
        }
    }
}

__global__ void k_expand_rows(int64_t rows, const int* __restrict__ rowptr, int* __restrict__ rowidx) {
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x % 32;
    if (row >= rows) return;
    for (int q = rowptr[row] + lane; q < rowptr[row + 1]; q += 32) rowidx[q] = (int)row;
}

__global__ void k_iota(int64_t n, int* __restrict__ v) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] = (int)i;
}

// keys[i] = src[perm ? perm[i] : i], with the sign bit flipped when `flip`
// (so unsigned order is signed int order)
__global__ void k_flip_copy(int64_t n, const int* __restrict__ perm, const int* __restrict__ src, bool flip,
                            unsigned* __restrict__ keys) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) keys[i] = (unsigned)src[perm ? perm[i] : i] ^ (flip ? 0x80000000u : 0u);
}

template <typename T>
__global__ void k_gather(int64_t n, const int* __restrict__ perm, const T* __restrict__ src, T* __restrict__ dst) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[perm[i]];
}

// ---------------- inclusive scan (int32), 1024 threads x 4 items per block
constexpr int SCAN_T = 1024, SCAN_IPT = 4, SCAN_TILE = SCAN_T * SCAN_IPT;

__device__ __forceinline__ int block_scan_incl(int v, int* sh) {
    const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
    for (int off = 1; off < 32; off <<= 1) {
        int o = __shfl_up_sync(0xffffffffu, v, off);
        if (lane >= off) v += o;
    }
    if (lane == 31) sh[warp] = v;
    __syncthreads();
    if (warp == 0) {
        int w = sh[lane];
        for (int off = 1; off < 32; off <<= 1) {
            int o = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += o;
        }
        sh[lane] = w;
    }
    __syncthreads();
    if (warp > 0) v += sh[warp - 1];
    __syncthreads();
    return v;
}

__global__ void __launch_bounds__(SCAN_T) k_scan_tiles(int64_t n, int* __restrict__ data, int* __restrict__ sums) {
    __shared__ int sh[32];
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_IPT;
    int v[SCAN_IPT];
    int t = 0;
#pragma unroll
    for (int i = 0; i < SCAN_IPT; i++) {
        v[i] = (base + i < n) ? data[base + i] : 0;
        t += v[i];
    }
    int incl = block_scan_incl(t, sh);
    int run = incl - t;
#pragma unroll
    for (int i = 0; i < SCAN_IPT; i++) {
        run += v[i];
        if (base + i < n) data[base + i] = run;
    }
    if (threadIdx.x == SCAN_T - 1) sums[blockIdx.x] = incl;
}

__global__ void k_scan_add(int64_t n, int* __restrict__ data, const int* __restrict__ sums) {
    if (blockIdx.x == 0) return;
    const int add = sums[blockIdx.x - 1];
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    for (int i = threadIdx.x; i < SCAN_TILE; i += blockDim.x)
        if (base + i < n) data[base + i] += add;
}

// ---------------- stable LSD radix sort of (key, value) pairs, 8-bit digits
constexpr int RS_T = 256, RS_SUB = 16, RS_TILE = RS_T * RS_SUB;  // 4096 items per block

__global__ void __launch_bounds__(RS_T) k_radix_hist(int64_t n, const unsigned* __restrict__ keys, int shift,
                                                     int* __restrict__ hist, int nblocks) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * RS_TILE;
    for (int i = threadIdx.x; i < RS_TILE; i += RS_T)
        if (base + i < n) atomicAdd(&h[(keys[base + i] >> shift) & 255], 1);
    __syncthreads();
    hist[(int64_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// hist holds inclusive scan over [digit][block]; block b's start for digit d
// is incl[d*nb + b] - count.  Items are ranked stably: sub-tile order, then
// warp order, then lane order.
__global__ void __launch_bounds__(RS_T) k_radix_scatter(int64_t n, const unsigned* __restrict__ keys_in,
                                                        const int* __restrict__ vals_in, int shift,
                                                        const int* __restrict__ incl, const int* __restrict__ cnt,
                                                        int nblocks, unsigned* __restrict__ keys_out,
                                                        int* __restrict__ vals_out) {
    __shared__ int run[256];       // running output position per digit
    __shared__ int wcount[8][256];  // per-warp digit counts of the current sub-tile
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    {
        const int64_t idx = (int64_t)threadIdx.x * nblocks + blockIdx.x;
        run[threadIdx.x] = incl[idx] - cnt[idx];
    }
    const int64_t base = (int64_t)blockIdx.x * RS_TILE;
    for (int sub = 0; sub < RS_SUB; sub++) {
        for (int w = 0; w < 8; w++) wcount[w][threadIdx.x] = 0;
        __syncthreads();
        const int64_t i = base + (int64_t)sub * RS_T + threadIdx.x;
        const bool valid = i < n;
        unsigned key = valid ? keys_in[i] : 0u;
        int val = valid ? vals_in[i] : 0;
        int d = valid ? (int)((key >> shift) & 255) : 256 + lane;  // invalid lanes get unique dummies
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int rank_in_warp = __popc(peers & ((1u << lane) - 1));
        if (valid && rank_in_warp == 0) wcount[warp][d] = __popc(peers);
        __syncthreads();
        int pos = 0;
        if (valid) {
            int before = 0;
            for (int w = 0; w < warp; w++) before += wcount[w][d];
            pos = run[d] + before + rank_in_warp;
        }
        __syncthreads();
        {
            int tot = 0;
            for (int w = 0; w < 8; w++) tot += wcount[w][threadIdx.x];
            run[threadIdx.x] += tot;
        }
        if (valid) {
            keys_out[pos] = key;
            vals_out[pos] = val;
        }
        __syncthreads();
    }
}

// ---------------- COO sort by (row, col), stable
// Sorting by (row, col) stably is sorting by the unique key (row, col, input
// index).  The triplets are bucketed by row through per-row atomic cursors
// (which leaves each row's order arbitrary), then each row's segment is
// sorted by (col, input index), packed as one 64-bit key, in registers (rows
// of up to 32 entries, a warp per row) or in shared memory (bitonic, up to
// SEG_CAP entries, a block per row).  The values follow through the input
// index.  Longer rows, and negative indices, take the radix path.
constexpr int SEG_CAP = 4096;

__global__ void k_coo_minmax(int64_t n, const int* __restrict__ r, const int* __restrict__ c, int* __restrict__ mm) {
    int lo = INT32_MAX, hr = INT32_MIN, hc = INT32_MIN;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int a = __ldg(&r[i]), b = __ldg(&c[i]);
        lo = min(lo, min(a, b));
        hr = max(hr, a);
        hc = max(hc, b);
    }
    for (int o = 16; o; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hr = max(hr, __shfl_xor_sync(0xffffffffu, hr, o));
        hc = max(hc, __shfl_xor_sync(0xffffffffu, hc, o));
    }
    if (threadIdx.x % 32 == 0) {
        atomicMin(&mm[0], lo);
        atomicMax(&mm[1], hr);
        atomicMax(&mm[2], hc);
    }
}

__global__ void k_count_rows(int64_t n, const int* __restrict__ r, int* __restrict__ cnt) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&cnt[__ldg(&r[i])], 1);
}

__global__ void k_max_int(int64_t n, const int* __restrict__ v, int* __restrict__ out) {
    int m = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = max(m, __ldg(&v[i]));
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x % 32 == 0) atomicMax(out, m);
}

// rp: exclusive row offsets (rows + 1); cur: per-row cursors, zeroed
__global__ void k_coo_bucket(int64_t n, const int* __restrict__ r, const int* __restrict__ c,
                             const int* __restrict__ rp, int* __restrict__ cur, unsigned long long* __restrict__ key) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int row = __ldg(&r[i]);
        const int pos = __ldg(&rp[row]) + atomicAdd(&cur[row], 1);
        key[pos] = ((unsigned long long)(unsigned)__ldg(&c[i]) << 32) | (unsigned)i;
    }
}

// writes one sorted entry: row, column, and the value of its input index
__device__ __forceinline__ void coo_emit(int64_t pos, int row, unsigned long long k, int* __restrict__ ro,
                                         int* __restrict__ co, const double* __restrict__ vin,
                                         double* __restrict__ vo, int* __restrict__ po) {
    ro[pos] = row;
    co[pos] = (int)(k >> 32);
    if (vo) vo[pos] = __ldg(&vin[(unsigned)k]);
    if (po) po[pos] = (int)(unsigned)k;
}

// a warp per row; rows of up to 64 entries are ranked in registers, two keys
// per lane (keys are unique, so the ranks are a permutation), longer ones are
// listed for k_coo_seg_block (nlong[0] counts them; nlong[3] is the longest row)
__global__ void k_coo_seg_warp(int64_t rows, const int* __restrict__ rp, const unsigned long long* __restrict__ key,
                               int* __restrict__ ro, int* __restrict__ co, const double* __restrict__ vin,
                               double* __restrict__ vo, int* __restrict__ po, int* __restrict__ longlist,
                               int* __restrict__ nlong) {
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x % 32;
    // nlong[3]: the longest row; beyond SEG_CAP the host sorts by radix from
    // the untouched input instead
    if (row >= rows || nlong[3] > SEG_CAP) return;
    const int q0 = __ldg(&rp[row]), len = __ldg(&rp[row + 1]) - q0;
    if (len > 64) {
        if (lane == 0) longlist[atomicAdd(nlong, 1)] = (int)row;
        return;
    }
    const unsigned long long k0 = lane < len ? key[q0 + lane] : ~0ull;
    const unsigned long long k1 = lane + 32 < len ? key[q0 + 32 + lane] : ~0ull;
    const int n0 = len < 32 ? len : 32, n1 = len - n0;
    int r0 = 0, r1 = 0;
    for (int j = 0; j < n0; j++) {
        const unsigned long long x = __shfl_sync(0xffffffffu, k0, j);
        r0 += x < k0;
        r1 += x < k1;
    }
    for (int j = 0; j < n1; j++) {
        const unsigned long long x = __shfl_sync(0xffffffffu, k1, j);
        r0 += x < k0;
        r1 += x < k1;
    }
    if (lane < len) coo_emit(q0 + r0, (int)row, k0, ro, co, vin, vo, po);
    if (lane + 32 < len) coo_emit(q0 + r1, (int)row, k1, ro, co, vin, vo, po);
}

// a block per listed row (65 .. pmax entries, pmax a power of two up to
// SEG_CAP): bitonic sort in shared memory (pmax keys)
__global__ void __launch_bounds__(512) k_coo_seg_block(const int* __restrict__ longlist, const int* __restrict__ nlong,
                                                       const int* __restrict__ rp,
                                                       const unsigned long long* __restrict__ key,
                                                       int* __restrict__ ro, int* __restrict__ co,
                                                       const double* __restrict__ vin, double* __restrict__ vo,
                                                       int* __restrict__ po) {
    extern __shared__ unsigned long long sk[];
    const int nl = *nlong;
    for (int b = blockIdx.x; b < nl; b += gridDim.x) {
        const int row = longlist[b];
        const int q0 = rp[row], len = rp[row + 1] - q0;
        int P = 64;
        while (P < len) P <<= 1;
        for (int i = threadIdx.x; i < P; i += blockDim.x) sk[i] = i < len ? key[q0 + i] : ~0ull;
        __syncthreads();
        for (int size = 2; size <= P; size <<= 1) {
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int t = threadIdx.x; t < P / 2; t += blockDim.x) {
                    const int lo = 2 * t - (t & (stride - 1));
                    const int hi = lo + stride;
                    const bool up = (lo & size) == 0;
                    const unsigned long long a = sk[lo], c = sk[hi];
                    if ((a > c) == up) {
                        sk[lo] = c;
                        sk[hi] = a;
                    }
                }
                __syncthreads();
            }
        }
        for (int i = threadIdx.x; i < len; i += blockDim.x) coo_emit(q0 + i, row, sk[i], ro, co, vin, vo, po);
        __syncthreads();
    }
}

// ---------------- CSR x CSR (RealCsrMatMult, src/main/java/org/flag4j/linalg/
// ops/sparse/csr/real/RealCsrMatMult.java)
// Dense result (standard, :53-75): a warp per row i of A walks the row's
// nonzeros in storage order; for each, the lanes add a * B[k, :] into the
// dense row i of C (zeroed), each product and sum rounded.  A row of B holds
// distinct columns, so the lanes of one step touch distinct entries; the
// __syncwarp orders successive steps.
template <int AK, int BK>
__device__ __forceinline__ double2 spgemm_prod(const double* __restrict__ av, int64_t q,
                                               const double* __restrict__ bv, int64_t t) {
    // the product each variant adds: real b*a; bVal.mult(aVal) with a real
    // (RealComplexCsrMatMult.java:78) or complex a (SemiringCsrMatMult.java:81,
    // Complex128.java:336-341: b.re a.re - b.im a.im, b.re a.im + b.im a.re);
    // aVal.mult(bVal) with b real (RealComplexCsrMatMult.java:113)
    if (!AK && !BK) return make_double2(__dmul_rn(__ldg(&av[q]), __ldg(&bv[t])), 0.0);
    if (!AK) {
        const double a = __ldg(&av[q]);
        const double2 b = __ldg(reinterpret_cast<const double2*>(bv) + t);
        return make_double2(__dmul_rn(b.x, a), __dmul_rn(b.y, a));
    }
    const double2 a = __ldg(reinterpret_cast<const double2*>(av) + q);
    if (!BK) {
        const double b = __ldg(&bv[t]);
        return make_double2(__dmul_rn(a.x, b), __dmul_rn(a.y, b));
    }
    const double2 b = __ldg(reinterpret_cast<const double2*>(bv) + t);
    return make_double2(__dsub_rn(__dmul_rn(b.x, a.x), __dmul_rn(b.y, a.y)),
                        __dadd_rn(__dmul_rn(b.x, a.y), __dmul_rn(b.y, a.x)));
}

// AK / BK: 1 when A's / B's values are complex (interleaved); C is complex
// (interleaved) when either is.
template <int AK, int BK>
__global__ void k_spgemm_dense(int64_t rows, int64_t n2, const int* __restrict__ arp, const int* __restrict__ aci,
                               const double* __restrict__ av, const int* __restrict__ brp,
                               const int* __restrict__ bci, const double* __restrict__ bv, double* __restrict__ C) {
    constexpr int W = (AK || BK) ? 2 : 1;
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x % 32;
    if (row >= rows) return;
    double* Cr = C + row * n2 * W;
    const int q1 = __ldg(&arp[row + 1]);
    for (int q = __ldg(&arp[row]); q < q1; q++) {
        const int k = __ldg(&aci[q]);
        const int t1 = __ldg(&brp[k + 1]);
        for (int t = __ldg(&brp[k]) + lane; t < t1; t += 32) {
            const int64_t j = __ldg(&bci[t]);
            const double2 p = spgemm_prod<AK, BK>(av, q, bv, t);
            Cr[W * j] = __dadd_rn(Cr[W * j], p.x);
            if (W == 2) Cr[W * j + 1] = __dadd_rn(Cr[W * j + 1], p.y);
        }
        __syncwarp();
    }
}

// CSR result (standardAsSparse, :92-131), expand-sort-compress: every product
// b * a is written out in the reference's loop order (rows of A, a row's
// nonzeros, then the nonzeros of B's row), stably sorted by (row, column),
// and each run of one (row, column) summed in order starting from its first
// product, as HashMap.merge(col, b * a, Double::sum) does.
__global__ void k_spgemm_len(int64_t annz, const int* __restrict__ aci, const int* __restrict__ brp,
                             int* __restrict__ len, unsigned long long* __restrict__ total) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long l = 0;
    if (q < annz) {
        const int k = __ldg(&aci[q]);
        l = (unsigned long long)(__ldg(&brp[k + 1]) - __ldg(&brp[k]));
        len[q] = (int)l;
    }
    for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if (threadIdx.x % 32 == 0 && l) atomicAdd(total, l);
}

// off: inclusive scan of the expansion lengths, one per nonzero of A; ev
// holds W values per product (interleaved when complex)
template <int AK, int BK>
__global__ void k_spgemm_expand(int64_t rows, const int* __restrict__ arp, const int* __restrict__ aci,
                                const double* __restrict__ av, const int* __restrict__ brp,
                                const int* __restrict__ bci, const double* __restrict__ bv,
                                const int* __restrict__ off, int* __restrict__ er, int* __restrict__ ec,
                                double* __restrict__ ev) {
    constexpr int W = (AK || BK) ? 2 : 1;
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x % 32;
    if (row >= rows) return;
    const int q1 = __ldg(&arp[row + 1]);
    for (int q = __ldg(&arp[row]); q < q1; q++) {
        const int k = __ldg(&aci[q]);
        const int t0 = __ldg(&brp[k]), t1 = __ldg(&brp[k + 1]);
        const int64_t base = (int64_t)(q ? __ldg(&off[q - 1]) : 0) - t0;
        for (int t = t0 + lane; t < t1; t += 32) {
            er[base + t] = (int)row;
            ec[base + t] = __ldg(&bci[t]);
            const double2 p = spgemm_prod<AK, BK>(av, q, bv, t);
            ev[W * (base + t)] = p.x;
            if (W == 2) ev[W * (base + t) + 1] = p.y;
        }
    }
}

// complex products gathered into sorted order: dst[i] = src[perm[i]]
__global__ void k_gather_z(int64_t n, const int* __restrict__ perm, const double2* __restrict__ src,
                           double2* __restrict__ dst) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[perm[i]];
}

// fs: inclusive scan of the run-start flags of the sorted expansion
__global__ void k_run_flags(int64_t n, const int* __restrict__ r, const int* __restrict__ c, int* __restrict__ f) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) f[e] = (e == 0 || r[e] != r[e - 1] || c[e] != c[e - 1]) ? 1 : 0;
}

__global__ void k_run_starts(int64_t n, const int* __restrict__ fs, int* __restrict__ starts) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n && (e == 0 || fs[e] != fs[e - 1])) starts[fs[e] - 1] = (int)e;
}

template <int W>
__global__ void k_run_sum(int64_t runs, int64_t n, const int* __restrict__ starts, const int* __restrict__ r,
                          const int* __restrict__ c, const double* __restrict__ v, int* __restrict__ oc,
                          double* __restrict__ ov, int* __restrict__ rowcnt) {
    const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= runs) return;
    const int s0 = starts[u];
    const int64_t s1 = u + 1 < runs ? starts[u + 1] : n;
    double acc0 = v[W * (int64_t)s0], acc1 = W == 2 ? v[W * (int64_t)s0 + 1] : 0.0;
    for (int64_t e = s0 + 1; e < s1; e++) {
        acc0 = __dadd_rn(acc0, v[W * e]);
        if (W == 2) acc1 = __dadd_rn(acc1, v[W * e + 1]);
    }
    oc[u] = c[s0];
    ov[W * u] = acc0;
    if (W == 2) ov[W * u + 1] = acc1;
    atomicAdd(&rowcnt[r[s0]], 1);
}

}  // namespace

// ------------------------------------------------------------------ host helpers
static int grid1(int64_t n, int t = 256) {
    int64_t b = (n + t - 1) / t;
    if (b < 1) b = 1;
    if (b > 1 << 20) b = 1 << 20;
    return (int)b;
}

// In-place inclusive scan of int32 data[n] (recursive over tile sums).
static int scan_inclusive(f4j_ctx* ctx, int* data, int64_t n) {
    if (n <= 0) return F4J_OK;
    const int64_t tiles = f4j_cdiv(n, SCAN_TILE);
    int* sums = nullptr;
    int rc = f4j_dev_alloc(ctx, (size_t)tiles * sizeof(int), (void**)&sums);
    if (rc) return rc;
    k_scan_tiles<<<(unsigned)tiles, SCAN_T, 0, ctx->stream>>>(n, data, sums);
    F4J_LAUNCHED(ctx);
    if (tiles > 1) {
        rc = scan_inclusive(ctx, sums, tiles);
        if (rc) {
            f4j_dev_free(ctx, sums);
            return rc;
        }
        k_scan_add<<<(unsigned)tiles, 256, 0, ctx->stream>>>(n, data, sums);
        F4J_LAUNCHED(ctx);
    }
    f4j_dev_free(ctx, sums);
    return F4J_OK;
}

// Stable sort of (keys, vals) by the low `bits` bits of keys; result in place.
static int radix_sort_pairs(f4j_ctx* ctx, unsigned* keys, int* vals, int64_t n, int bits) {
    if (n <= 1 || bits <= 0) return F4J_OK;
    const int nb = (int)f4j_cdiv(n, RS_TILE);
    unsigned* k2 = nullptr;
    int* v2 = nullptr;
    int *hist = nullptr, *cnt = nullptr;
    int rc = f4j_dev_alloc(ctx, (size_t)n * 4, (void**)&k2);
    if (!rc) rc = f4j_dev_alloc(ctx, (size_t)n * 4, (void**)&v2);
    if (!rc) rc = f4j_dev_alloc(ctx, (size_t)256 * nb * 4, (void**)&hist);
    if (!rc) rc = f4j_dev_alloc(ctx, (size_t)256 * nb * 4, (void**)&cnt);
    unsigned *ka = keys, *kb = k2;
    int *va = vals, *vb = v2;
    for (int shift = 0; !rc && shift < bits; shift += 8) {
        k_radix_hist<<<nb, RS_T, 0, ctx->stream>>>(n, ka, shift, hist, nb);
        F4J_LAUNCHED(ctx);
        cudaMemcpyAsync(cnt, hist, (size_t)256 * nb * 4, cudaMemcpyDeviceToDevice, ctx->stream);
        rc = scan_inclusive(ctx, hist, (int64_t)256 * nb);
        if (rc) break;
        k_radix_scatter<<<nb, RS_T, 0, ctx->stream>>>(n, ka, va, shift, hist, cnt, nb, kb, vb);
        F4J_LAUNCHED(ctx);
        unsigned* tk = ka; ka = kb; kb = tk;
        int* tv = va; va = vb; vb = tv;
    }
    if (!rc && ka != keys) {
        cudaMemcpyAsync(keys, ka, (size_t)n * 4, cudaMemcpyDeviceToDevice, ctx->stream);
        cudaMemcpyAsync(vals, va, (size_t)n * 4, cudaMemcpyDeviceToDevice, ctx->stream);
    }
    f4j_dev_free(ctx, k2);
    f4j_dev_free(ctx, v2);
    f4j_dev_free(ctx, hist);
    f4j_dev_free(ctx, cnt);
    return rc;
}

static int bits_for(int64_t maxval) {
    int b = 0;
    while (b < 31 && (1ll << b) <= maxval) b++;
    return b;
}

// Builds the cached transpose structure of S (RealCsrOps.transpose order).
static int ensure_transpose(f4j_ctx* ctx, f4j_csr S) {
    if (S->t_perm) return F4J_OK;
    const int64_t nnz = S->nnz, rows = S->rows, cols = S->cols;
    int *trp = nullptr, *perm = nullptr, *trow = nullptr;
    unsigned* keys = nullptr;
    int* rowidx = nullptr;
    int rc = f4j_dev_alloc(ctx, (size_t)(cols + 1) * 4, (void**)&trp);
    if (!rc) rc = f4j_dev_alloc(ctx, (size_t)nnz * 4, (void**)&perm);
    if (!rc) rc = f4j_dev_alloc(ctx, (size_t)nnz * 4, (void**)&trow);
    if (!rc) rc = f4j_dev_alloc(ctx, (size_t)nnz * 4, (void**)&keys);
    if (!rc) rc = f4j_dev_alloc(ctx, (size_t)nnz * 4, (void**)&rowidx);
    if (rc) goto fail;
    // pointers of S^T: column counts, inclusive scan (as RealCsrOps.transpose :203-211)
    F4J_CUDA(cudaMemsetAsync(trp, 0, (size_t)(cols + 1) * 4, ctx->stream));
    if (nnz) {
        k_count<<<grid1(nnz), 256, 0, ctx->stream>>>(nnz, (const int*)S->colidx->ptr, trp);
        F4J_LAUNCHED(ctx);
        rc = scan_inclusive(ctx, trp + 1, cols);
        if (rc) goto fail;
        // stable order by column == scatter in storage order (:216-222)
        F4J_CUDA(cudaMemcpyAsync(keys, S->colidx->ptr, (size_t)nnz * 4, cudaMemcpyDeviceToDevice, ctx->stream));
        k_iota<<<grid1(nnz), 256, 0, ctx->stream>>>(nnz, perm);
        F4J_LAUNCHED(ctx);
        rc = radix_sort_pairs(ctx, keys, perm, nnz, bits_for(cols - 1));
        if (rc) goto fail;
        k_expand_rows<<<grid1(rows * 32), 256, 0, ctx->stream>>>(rows, (const int*)S->rowptr->ptr, rowidx);
        F4J_LAUNCHED(ctx);
        k_gather<int><<<grid1(nnz), 256, 0, ctx->stream>>>(nnz, perm, rowidx, trow);
        F4J_LAUNCHED(ctx);
    }
    f4j_dev_free(ctx, keys);
    f4j_dev_free(ctx, rowidx);
    S->t_rowptr = trp;
    S->t_perm = perm;
    S->t_rowidx = trow;
    return F4J_OK;
fail:
    f4j_dev_free(ctx, trp);
    f4j_dev_free(ctx, perm);
    f4j_dev_free(ctx, trow);
    f4j_dev_free(ctx, keys);
    f4j_dev_free(ctx, rowidx);
    return rc;
}

// Row of each nonzero, cached in the handle.
static int ensure_rowidx(f4j_ctx* ctx, f4j_csr S) {
    if (S->rowidx || S->nnz == 0) return F4J_OK;
    int* ri = nullptr;
    int rc = f4j_dev_alloc(ctx, (size_t)S->nnz * 4, (void**)&ri);
    if (rc) return rc;
    k_expand_rows<<<grid1(S->rows * 32), 256, 0, ctx->stream>>>(S->rows, (const int*)S->rowptr->ptr, ri);
    F4J_LAUNCHED(ctx);
    S->rowidx = ri;
    return F4J_OK;
}

static int launch_spmm(f4j_ctx* ctx, int64_t rows, int64_t ncols, const int* rp, const int* ci, const double* v,
                       const int* perm, const double* X, double* Y, bool fused = false) {
    if (rows == 0 || ncols == 0) return F4J_OK;
    // one row per warp from 17 columns on (the FP64 instructions of a warp then
    // never wait on a second row of another length); 128-bit X loads only
    // where a warp of 2-column lanes is still needed for the width
    const bool vec2 = ncols > 32 && (ncols % 2 == 0) && f4j_aligned16(X) && f4j_aligned16(Y);
    const int64_t per_lane = vec2 ? 2 : 1;
    int G = 1;
    while (G < 32 && G * per_lane < ncols) G *= 2;
    const int64_t threads = rows * G;
    const unsigned blocks = (unsigned)f4j_cdiv(threads, 256);
    f4j_prof_begin(ctx);
    if (fused) {
        // the FMA mode (products with no reference order to keep): no transpose variant
        if (vec2) k_spmm<true, false, true><<<blocks, 256, 0, ctx->stream>>>(rows, ncols, G, rp, ci, v, perm, X, Y);
        else k_spmm<false, false, true><<<blocks, 256, 0, ctx->stream>>>(rows, ncols, G, rp, ci, v, perm, X, Y);
    } else if (vec2) {
        if (perm) k_spmm<true, true><<<blocks, 256, 0, ctx->stream>>>(rows, ncols, G, rp, ci, v, perm, X, Y);
        else k_spmm<true, false><<<blocks, 256, 0, ctx->stream>>>(rows, ncols, G, rp, ci, v, perm, X, Y);
    } else {
        if (perm) k_spmm<false, true><<<blocks, 256, 0, ctx->stream>>>(rows, ncols, G, rp, ci, v, perm, X, Y);
        else k_spmm<false, false><<<blocks, 256, 0, ctx->stream>>>(rows, ncols, G, rp, ci, v, perm, X, Y);
    }
    f4j_prof_end(ctx);
    F4J_LAUNCHED(ctx);
    return F4J_OK;
}

// ------------------------------------------------------------------ C ABI
extern "C" int f4j_csr_wrap(f4j_ctx* ctx, int64_t rows, int64_t cols, int64_t nnz, f4j_buf rowptr, f4j_buf colidx,
                            f4j_buf vals, int validate, f4j_csr* out) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (!out) return f4j_fail(F4J_ERR_ARG, "null output pointer");
    *out = nullptr;
    if (!rowptr || !colidx || !vals) return f4j_fail(F4J_ERR_ARG, "null CSR buffer");
    if (rows < 0 || cols < 0 || nnz < 0) return f4j_fail(F4J_ERR_ARG, "negative CSR size");
    if (rows > INT32_MAX || cols > INT32_MAX || nnz > INT32_MAX)
        return f4j_fail(F4J_ERR_ARG, "CSR sizes exceed Flag4j's int range");
    if ((int64_t)rows * cols < nnz)
        return f4j_fail(F4J_ERR_CSR,
                        "The number of non-zero entries cannot be greater than the total number of entries in the "
                        "matrix but got nnz=%lld and totalEntries=%lld",
                        (long long)nnz, (long long)(rows * cols));
    if (rowptr->bytes < (size_t)(rows + 1) * 4)
        return f4j_fail(F4J_ERR_CSR, "Expecting rowPointers to have length (numRows + 1)=%lld", (long long)(rows + 1));
    if (colidx->bytes < (size_t)nnz * 4 || vals->bytes < (size_t)nnz * 8)
        return f4j_fail(F4J_ERR_CSR, "column index / value buffers shorter than nnz=%lld", (long long)nnz);
    if (!f4j_aligned(rowptr->ptr, 4) || !f4j_aligned(colidx->ptr, 4) || !f4j_aligned(vals->ptr, 8))
        return f4j_fail(F4J_ERR_ARG, "CSR buffers must be aligned to their element size");
    F4J_CUDA(cudaSetDevice(ctx->device));
    if (validate) {
        void* ws;
        int rc = f4j_workspace(ctx, 2, 64, &ws);
        if (rc) return rc;
        int h[4] = {INT32_MAX, INT32_MAX, 0, 0};
        F4J_CUDA(cudaMemcpyAsync(ws, h, 8, cudaMemcpyHostToDevice, ctx->stream));
        if (rows) {
            k_validate_csr<<<grid1(rows), 256, 0, ctx->stream>>>(rows, cols, nnz, (const int*)rowptr->ptr,
                                                                 (const int*)colidx->ptr, (int*)ws, (int*)ws + 1);
            F4J_LAUNCHED(ctx);
        }
        int first_last[2] = {0, 0};
        F4J_CUDA(cudaMemcpyAsync(h, ws, 8, cudaMemcpyDeviceToHost, ctx->stream));
        F4J_CUDA(cudaMemcpyAsync(&first_last[0], rowptr->ptr, 4, cudaMemcpyDeviceToHost, ctx->stream));
        F4J_CUDA(cudaMemcpyAsync(&first_last[1], (int*)rowptr->ptr + rows, 4, cudaMemcpyDeviceToHost, ctx->stream));
        F4J_CUDA(cudaStreamSynchronize(ctx->stream));
        if (h[0] != INT32_MAX) {
            int p[2];
            cudaMemcpy(p, (int*)rowptr->ptr + h[0], 8, cudaMemcpyDeviceToHost);
            if (p[0] < 0)
                return f4j_fail(F4J_ERR_CSR, "All rowPointers must be positive but got %d at index %d.", p[0], h[0]);
            return f4j_fail(F4J_ERR_CSR,
                            "rowPointers must be monotonically increasing but got values %d and %d at indices %d "
                            "and %d.",
                            p[0], p[1], h[0], h[0] + 1);
        }
        if (h[1] != INT32_MAX) {
            int c = 0;
            cudaMemcpy(&c, (int*)colidx->ptr + h[1], 4, cudaMemcpyDeviceToHost);
            return f4j_fail(F4J_ERR_CSR, "Invalid column index [%d] encountered for CSR matrix of shape (%lld, %lld)", c,
                            (long long)rows, (long long)cols);
        }
        if ((int64_t)first_last[1] - first_last[0] != nnz)
            return f4j_fail(F4J_ERR_CSR, "rowIndices specifies %lld elements but nnz=%lld. These values must be equal.",
                            (long long)((int64_t)first_last[1] - first_last[0]), (long long)nnz);
    }
    *out = new f4j_csr_s{rows, cols, nnz, rowptr, colidx, vals, false, nullptr, nullptr, nullptr, nullptr};
    return F4J_OK;
}

extern "C" int f4j_csr_free(f4j_ctx* ctx, f4j_csr S) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (!S) return F4J_OK;
    F4J_CUDA(cudaStreamSynchronize(ctx->stream));
    cudaFree(S->t_rowptr);
    cudaFree(S->t_perm);
    cudaFree(S->t_rowidx);
    cudaFree(S->rowidx);
    if (S->owns) {
        f4j_buf_free(ctx, S->rowptr);
        f4j_buf_free(ctx, S->colidx);
        f4j_buf_free(ctx, S->vals);
    }
    delete S;
    return F4J_OK;
}

extern "C" int f4j_csr_info(f4j_csr S, int64_t* rows, int64_t* cols, int64_t* nnz) {
    if (!S) return f4j_fail(F4J_ERR_ARG, "null CSR handle");
    if (rows) *rows = S->rows;
    if (cols) *cols = S->cols;
    if (nnz) *nnz = S->nnz;
    return F4J_OK;
}

extern "C" int f4j_csr_buffers(f4j_csr S, f4j_buf* rowptr, f4j_buf* colidx, f4j_buf* vals) {
    if (!S) return f4j_fail(F4J_ERR_ARG, "null CSR handle");
    if (rowptr) *rowptr = S->rowptr;
    if (colidx) *colidx = S->colidx;
    if (vals) *vals = S->vals;
    return F4J_OK;
}

static int alloc_owned_csr(f4j_ctx* ctx, int64_t rows, int64_t cols, int64_t nnz, f4j_csr* out, int vw = 1) {
    f4j_buf rp = nullptr, ci = nullptr, v = nullptr;
    int rc = f4j_buf_alloc_pooled(ctx, (size_t)(rows + 1) * 4, &rp);
    if (!rc) rc = f4j_buf_alloc_pooled(ctx, (size_t)nnz * 4, &ci);
    if (!rc) rc = f4j_buf_alloc_pooled(ctx, (size_t)nnz * 8 * vw, &v);
    if (rc) {
        f4j_buf_free(ctx, rp);
        f4j_buf_free(ctx, ci);
        f4j_buf_free(ctx, v);
        return rc;
    }
    *out = new f4j_csr_s{rows, cols, nnz, rp, ci, v, true, nullptr, nullptr, nullptr, nullptr};
    return F4J_OK;
}

extern "C" int f4j_csr_from_coo(f4j_ctx* ctx, int64_t rows, int64_t cols, int64_t nnz, f4j_buf rowidx, f4j_buf colidx,
                                f4j_buf vals, f4j_csr* out) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (!out) return f4j_fail(F4J_ERR_ARG, "null output pointer");
    *out = nullptr;
    if (!rowidx || !colidx || !vals) return f4j_fail(F4J_ERR_ARG, "null COO buffer");
    if (rows < 0 || cols < 0 || nnz < 0 || rows > INT32_MAX || cols > INT32_MAX || nnz > INT32_MAX)
        return f4j_fail(F4J_ERR_ARG, "bad COO sizes");
    if (rowidx->bytes < (size_t)nnz * 4 || colidx->bytes < (size_t)nnz * 4 || vals->bytes < (size_t)nnz * 8)
        return f4j_fail(F4J_ERR_CSR,
                        "The number of non-zero entries must match the number of row and column indices");
    if ((int64_t)rows * cols < nnz)
        return f4j_fail(F4J_ERR_CSR, "The number of non-zero entries cannot be greater than the total number of entries");
    F4J_CUDA(cudaSetDevice(ctx->device));
    // SparseValidation.validateCoo (…/SparseValidation.java:70-98): indices in
    // range, checked by the count and the column copy themselves; the handle is
    // returned only after both checks have passed (one wait, at the end)
    void* ws;
    int rc = f4j_workspace(ctx, 2, 64, &ws);
    if (rc) return rc;
    int h[2] = {INT32_MAX, INT32_MAX};
    F4J_CUDA(cudaMemcpyAsync(ws, h, 8, cudaMemcpyHostToDevice, ctx->stream));
    f4j_csr S;
    rc = alloc_owned_csr(ctx, rows, cols, nnz, &S);
    if (rc) return rc;
    int* rp = (int*)S->rowptr->ptr;
    // CooMatrix.toCsr (…/CooMatrix.java:457-470): count per row into rp[r+1],
    // inclusive scan; column indices and values copied unchanged
    F4J_CUDA(cudaMemsetAsync(rp, 0, (size_t)(rows + 1) * 4, ctx->stream));
    if (nnz) {
        k_count_rows_checked<<<grid1(nnz), 256, 0, ctx->stream>>>(nnz, (const int*)rowidx->ptr, rows, rp, (int*)ws);
        F4J_LAUNCHED(ctx);
        const bool vec = ((reinterpret_cast<uintptr_t>(colidx->ptr) | reinterpret_cast<uintptr_t>(S->colidx->ptr)) &
                          15) == 0;
        if (vec)
            k_copy_cols_checked<true><<<grid1(f4j_cdiv(nnz, 4)), 256, 0, ctx->stream>>>(
                nnz, (const int*)colidx->ptr, cols, (int*)S->colidx->ptr, (int*)ws + 1);
        else
            k_copy_cols_checked<false><<<grid1(nnz), 256, 0, ctx->stream>>>(
                nnz, (const int*)colidx->ptr, cols, (int*)S->colidx->ptr, (int*)ws + 1);
        F4J_LAUNCHED(ctx);
    }
    rc = scan_inclusive(ctx, rp + 1, rows);
    if (rc) {
        f4j_csr_free(ctx, S);
        return rc;
    }
    F4J_CUDA(cudaMemcpyAsync(S->vals->ptr, vals->ptr, (size_t)nnz * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    F4J_CUDA(cudaMemcpyAsync(h, ws, 8, cudaMemcpyDeviceToHost, ctx->stream));
    F4J_CUDA(cudaStreamSynchronize(ctx->stream));
    if (h[0] != INT32_MAX || h[1] != INT32_MAX) {
        f4j_csr_free(ctx, S);
        int at = h[0] < h[1] ? h[0] : h[1];
        int rc2[2];
        cudaMemcpy(&rc2[0], (int*)rowidx->ptr + at, 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(&rc2[1], (int*)colidx->ptr + at, 4, cudaMemcpyDeviceToHost);
        return f4j_fail(F4J_ERR_CSR, "Invalid index [%d, %d] encountered for COO matrix of shape (%lld, %lld)", rc2[0],
                        rc2[1], (long long)rows, (long long)cols);
    }
    *out = S;
    return F4J_OK;
}

// Radix path of f4j_coo_sort: stable LSD by column, then by row, over the
// keys' significant bits (all 32 with a sign flip when an index is negative,
// so negative indices order first as the reference's int comparison has them).
static int coo_sort_radix(f4j_ctx* ctx, int64_t nnz, int* rowidx, int* colidx, double* vals, int rbits, int cbits,
                          bool flip, int* perm_out) {
    unsigned* keys = nullptr;
    int *perm = nullptr, *tmp = nullptr;
    double* vtmp = nullptr;
    int rc = f4j_dev_alloc(ctx, (size_t)nnz * 4, (void**)&keys);
    if (!rc) rc = f4j_dev_alloc(ctx, (size_t)nnz * 4, (void**)&perm);
    if (!rc) rc = f4j_dev_alloc(ctx, (size_t)nnz * 4, (void**)&tmp);
    if (!rc && vals) rc = f4j_dev_alloc(ctx, (size_t)nnz * 8, (void**)&vtmp);
    if (!rc) {
        k_iota<<<grid1(nnz), 256, 0, ctx->stream>>>(nnz, perm);
        k_flip_copy<<<grid1(nnz), 256, 0, ctx->stream>>>(nnz, nullptr, colidx, flip, keys);
        ctx->launches += 2;
        rc = radix_sort_pairs(ctx, keys, perm, nnz, cbits);
    }
    if (!rc) {
        k_flip_copy<<<grid1(nnz), 256, 0, ctx->stream>>>(nnz, perm, rowidx, flip, keys);
        ctx->launches++;
        rc = radix_sort_pairs(ctx, keys, perm, nnz, rbits);
    }
    if (!rc) {
        k_gather<int><<<grid1(nnz), 256, 0, ctx->stream>>>(nnz, perm, rowidx, tmp);
        cudaMemcpyAsync(rowidx, tmp, (size_t)nnz * 4, cudaMemcpyDeviceToDevice, ctx->stream);
        k_gather<int><<<grid1(nnz), 256, 0, ctx->stream>>>(nnz, perm, colidx, tmp);
        cudaMemcpyAsync(colidx, tmp, (size_t)nnz * 4, cudaMemcpyDeviceToDevice, ctx->stream);
        if (vals) {
            k_gather<double><<<grid1(nnz), 256, 0, ctx->stream>>>(nnz, perm, vals, vtmp);
            cudaMemcpyAsync(vals, vtmp, (size_t)nnz * 8, cudaMemcpyDeviceToDevice, ctx->stream);
        }
        ctx->launches += vals ? 3 : 2;
        if (perm_out) cudaMemcpyAsync(perm_out, perm, (size_t)nnz * 4, cudaMemcpyDeviceToDevice, ctx->stream);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = f4j_cuda_fail(e, "coo sort");
    }
    f4j_dev_free(ctx, keys);
    f4j_dev_free(ctx, perm);
    f4j_dev_free(ctx, tmp);
    f4j_dev_free(ctx, vtmp);
    return rc;
}

// Stable sort of n device triplets by (row, col), in place (v may be null);
// perm_out (may be null) receives the input index of every sorted position.
static int coo_sort_dev(f4j_ctx* ctx, int64_t nnz, int* r, int* c, double* v, int* perm_out = nullptr) {
    if (nnz <= 1) {
        if (nnz == 1 && perm_out) F4J_CUDA(cudaMemsetAsync(perm_out, 0, 4, ctx->stream));
        return F4J_OK;
    }
    const unsigned red_grid = (unsigned)std::min<int64_t>(grid1(nnz), (int64_t)ctx->sm_count * 8);

    // index range: mm = {min of rows and columns, max row, max column, longest row}
    int* mm = nullptr;
    int rc = f4j_dev_alloc(ctx, 16, (void**)&mm);
    if (rc) return rc;
    const int mm0[4] = {INT32_MAX, INT32_MIN, INT32_MIN, 0};
    F4J_CUDA(cudaMemcpyAsync(mm, mm0, 16, cudaMemcpyHostToDevice, ctx->stream));
    k_coo_minmax<<<red_grid, 256, 0, ctx->stream>>>(nnz, r, c, mm);
    ctx->launches++;
    int hm[4];
    F4J_CUDA(cudaMemcpyAsync(hm, mm, 16, cudaMemcpyDeviceToHost, ctx->stream));
    F4J_CUDA(cudaStreamSynchronize(ctx->stream));
    if (hm[0] < 0) {
        f4j_dev_free(ctx, mm);
        return coo_sort_radix(ctx, nnz, r, c, v, 32, 32, true, perm_out);
    }
    const int64_t rows = (int64_t)hm[1] + 1;
    if (rows > 4 * nnz + 4096) {  // row offsets would outweigh the triplets
        f4j_dev_free(ctx, mm);
        int rb = 0, cb = 0;
        while (rb < 31 && (1ll << rb) <= hm[1]) rb++;
        while (cb < 31 && (1ll << cb) <= hm[2]) cb++;
        return coo_sort_radix(ctx, nnz, r, c, v, rb, cb, false, perm_out);
    }

    // row offsets and the longest row
    int *rp = nullptr, *cur = nullptr;
    rc = f4j_dev_alloc(ctx, (size_t)(rows + 1) * 4, (void**)&rp);
    if (!rc) rc = f4j_dev_alloc(ctx, (size_t)rows * 4, (void**)&cur);
    if (!rc) {
        F4J_CUDA(cudaMemsetAsync(rp, 0, (size_t)(rows + 1) * 4, ctx->stream));
        k_count_rows<<<red_grid, 256, 0, ctx->stream>>>(nnz, r, rp + 1);
        k_max_int<<<(unsigned)std::min<int64_t>(grid1(rows), (int64_t)ctx->sm_count * 8), 256, 0, ctx->stream>>>(
            rows, rp + 1, mm + 3);
        ctx->launches += 2;
        rc = scan_inclusive(ctx, rp + 1, rows);
    }
    // buckets and the warp segment sort are queued before the host reads the
    // longest row, so the GPU never waits on the host between them; the warp
    // kernel leaves the input untouched when a row exceeds SEG_CAP
    unsigned long long* key = nullptr;
    double* vin = nullptr;
    int* longlist = nullptr;
    const int64_t maxlong = std::min<int64_t>(rows, nnz / 65 + 1);
    if (!rc) rc = f4j_dev_alloc(ctx, (size_t)nnz * 8, (void**)&key);
    if (!rc && v) rc = f4j_dev_alloc(ctx, (size_t)nnz * 8, (void**)&vin);
    if (!rc) rc = f4j_dev_alloc(ctx, (size_t)maxlong * 4, (void**)&longlist);
    if (!rc) {
        F4J_CUDA(cudaMemsetAsync(cur, 0, (size_t)rows * 4, ctx->stream));
        F4J_CUDA(cudaMemsetAsync(mm, 0, 4, ctx->stream));  // mm[0]: count of listed long rows
        if (v) F4J_CUDA(cudaMemcpyAsync(vin, v, (size_t)nnz * 8, cudaMemcpyDeviceToDevice, ctx->stream));
        k_coo_bucket<<<red_grid, 256, 0, ctx->stream>>>(nnz, r, c, rp, cur, key);
        k_coo_seg_warp<<<(unsigned)f4j_cdiv(rows * 32, 256), 256, 0, ctx->stream>>>(rows, rp, key, r, c, vin, v,
                                                                                   perm_out, longlist, mm);
        ctx->launches += 2;
        F4J_CUDA(cudaMemcpyAsync(&hm[3], mm + 3, 4, cudaMemcpyDeviceToHost, ctx->stream));
        F4J_CUDA(cudaStreamSynchronize(ctx->stream));
        if (hm[3] > SEG_CAP) {
            f4j_dev_free(ctx, key);
            f4j_dev_free(ctx, vin);
            f4j_dev_free(ctx, longlist);
            f4j_dev_free(ctx, rp);
            f4j_dev_free(ctx, cur);
            f4j_dev_free(ctx, mm);
            int rb = 0, cb = 0;
            while (rb < 31 && (1ll << rb) <= hm[1]) rb++;
            while (cb < 31 && (1ll << cb) <= hm[2]) cb++;
            return coo_sort_radix(ctx, nnz, r, c, v, rb, cb, false, perm_out);
        }
        if (hm[3] > 64) {
            // block path sized to the longest row: pmax keys of shared memory, pmax / 2 threads
            int pmax = 128;
            while (pmax < hm[3]) pmax <<= 1;
            const int bthreads = pmax / 2 < 512 ? pmax / 2 : 512;
            const unsigned bgrid = (unsigned)std::min<int64_t>(maxlong, (int64_t)ctx->sm_count * 32);
            k_coo_seg_block<<<bgrid, bthreads, (size_t)pmax * 8, ctx->stream>>>(longlist, mm, rp, key, r, c, vin, v,
                                                                                perm_out);
            ctx->launches++;
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = f4j_cuda_fail(e, "coo sort");
    }
    f4j_dev_free(ctx, key);
    f4j_dev_free(ctx, vin);
    f4j_dev_free(ctx, longlist);
    f4j_dev_free(ctx, rp);
    f4j_dev_free(ctx, cur);
    f4j_dev_free(ctx, mm);
    return rc;
}

extern "C" int f4j_coo_sort(f4j_ctx* ctx, int64_t nnz, f4j_buf rowidx, f4j_buf colidx, f4j_buf vals) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (!rowidx || !colidx) return f4j_fail(F4J_ERR_ARG, "null COO buffer");
    if (nnz < 0 || nnz > INT32_MAX) return f4j_fail(F4J_ERR_ARG, "bad nnz");
    if (rowidx->bytes < (size_t)nnz * 4 || colidx->bytes < (size_t)nnz * 4 || (vals && vals->bytes < (size_t)nnz * 8))
        return f4j_fail(F4J_ERR_ARG, "COO buffers shorter than nnz");
    if (nnz <= 1) return F4J_OK;
    F4J_CUDA(cudaSetDevice(ctx->device));
    return coo_sort_dev(ctx, nnz, (int*)rowidx->ptr, (int*)colidx->ptr, vals ? (double*)vals->ptr : nullptr);
}

// ------------------------------------------------------------------ CSR x CSR
// The value kinds of A and B select the variant: real x real (RealCsrMatMult),
// real x complex and complex x real (RealComplexCsrMatMult), complex x complex
// (SemiringCsrMatMult over Complex128).
static int check_csr_values(f4j_csr S, int cplx) {
    if (cplx && (S->vals->bytes < (size_t)S->nnz * 16 || !f4j_aligned16(S->vals->ptr)))
        return f4j_fail(F4J_ERR_ARG, "complex CSR values need 16 * nnz bytes, 16-byte aligned");
    return F4J_OK;
}

template <int AK, int BK>
static void launch_spgemm_dense(f4j_ctx* ctx, f4j_csr A, f4j_csr B, double* C) {
    k_spgemm_dense<AK, BK><<<(unsigned)f4j_cdiv(A->rows * 32, 256), 256, 0, ctx->stream>>>(
        A->rows, B->cols, (const int*)A->rowptr->ptr, (const int*)A->colidx->ptr, (const double*)A->vals->ptr,
        (const int*)B->rowptr->ptr, (const int*)B->colidx->ptr, (const double*)B->vals->ptr, C);
}

extern "C" int f4j_csr_mult_dense_ex(f4j_ctx* ctx, f4j_csr A, int a_complex, f4j_csr B, int b_complex, f4j_buf C,
                                     f4j_report* rep) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (!A || !B || !C) return f4j_fail(F4J_ERR_ARG, "null argument");
    if (A->cols != B->rows) return f4j_shape_error(A->rows, A->cols, B->rows, B->cols);
    int rc = check_csr_values(A, a_complex);
    if (!rc) rc = check_csr_values(B, b_complex);
    if (rc) return rc;
    const int W = (a_complex || b_complex) ? 2 : 1;
    if (C->bytes < (size_t)(A->rows * B->cols) * 8 * W) return f4j_fail(F4J_ERR_ARG, "C buffer too small");
    F4J_CUDA(cudaSetDevice(ctx->device));
    int64_t l0 = ctx->launches;
    if (A->rows * B->cols > 0) {
        F4J_CUDA(cudaMemsetAsync(C->ptr, 0, (size_t)(A->rows * B->cols) * 8 * W, ctx->stream));
        double* Cp = (double*)C->ptr;
        f4j_prof_begin(ctx);
        if (a_complex && b_complex) launch_spgemm_dense<1, 1>(ctx, A, B, Cp);
        else if (a_complex) launch_spgemm_dense<1, 0>(ctx, A, B, Cp);
        else if (b_complex) launch_spgemm_dense<0, 1>(ctx, A, B, Cp);
        else launch_spgemm_dense<0, 0>(ctx, A, B, Cp);
        f4j_prof_end(ctx);
        F4J_LAUNCHED(ctx);
    }
    if (rep) {
        *rep = f4j_report{};
        rep->launches = (int32_t)(ctx->launches - l0);
    }
    return F4J_OK;
}

extern "C" int f4j_csr_mult_dense(f4j_ctx* ctx, f4j_csr A, f4j_csr B, f4j_buf C, f4j_report* rep) {
    F4J_LOCK(ctx);
    return f4j_csr_mult_dense_ex(ctx, A, 0, B, 0, C, rep);
}

template <int AK, int BK>
static void launch_spgemm_expand(f4j_ctx* ctx, f4j_csr A, f4j_csr B, const int* off, int* er, int* ec, double* ev) {
    k_spgemm_expand<AK, BK><<<(unsigned)f4j_cdiv(A->rows * 32, 256), 256, 0, ctx->stream>>>(
        A->rows, (const int*)A->rowptr->ptr, (const int*)A->colidx->ptr, (const double*)A->vals->ptr,
        (const int*)B->rowptr->ptr, (const int*)B->colidx->ptr, (const double*)B->vals->ptr, off, er, ec, ev);
}

extern "C" int f4j_csr_mult_csr_ex(f4j_ctx* ctx, f4j_csr A, int a_complex, f4j_csr B, int b_complex, f4j_csr* out,
                                   f4j_report* rep) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (!A || !B || !out) return f4j_fail(F4J_ERR_ARG, "null argument");
    *out = nullptr;
    if (A->cols != B->rows) return f4j_shape_error(A->rows, A->cols, B->rows, B->cols);
    int rc = check_csr_values(A, a_complex);
    if (!rc) rc = check_csr_values(B, b_complex);
    if (rc) return rc;
    const int W = (a_complex || b_complex) ? 2 : 1;
    F4J_CUDA(cudaSetDevice(ctx->device));
    int64_t l0 = ctx->launches;
    const int64_t annz = A->nnz, rows = A->rows;
    const int* aci = (const int*)A->colidx->ptr;
    const int* brp = (const int*)B->rowptr->ptr;

    // expansion size
    int* len = nullptr;
    unsigned long long* total = nullptr;
    unsigned long long E = 0;
    rc = f4j_dev_alloc(ctx, (size_t)(annz > 0 ? annz : 1) * 4, (void**)&len);
    if (!rc) rc = f4j_dev_alloc(ctx, 8, (void**)&total);
    if (!rc && annz > 0) {
        F4J_CUDA(cudaMemsetAsync(total, 0, 8, ctx->stream));
        k_spgemm_len<<<(unsigned)f4j_cdiv(annz, 256), 256, 0, ctx->stream>>>(annz, aci, brp, len, total);
        ctx->launches++;
        F4J_CUDA(cudaMemcpyAsync(&E, total, 8, cudaMemcpyDeviceToHost, ctx->stream));
        F4J_CUDA(cudaStreamSynchronize(ctx->stream));
        if (E > (unsigned long long)INT32_MAX)
            rc = f4j_fail(F4J_ERR_UNSUPPORTED, "CSR product expands to %llu products, over 2^31 - 1", E);
    }
    int *er = nullptr, *ec = nullptr, *fs = nullptr, *starts = nullptr, *perm = nullptr;
    double *ev = nullptr, *evs = nullptr;
    int64_t runs = 0;
    if (!rc && E > 0) {
        rc = scan_inclusive(ctx, len, annz);
        if (!rc) rc = f4j_dev_alloc(ctx, E * 4, (void**)&er);
        if (!rc) rc = f4j_dev_alloc(ctx, E * 4, (void**)&ec);
        if (!rc) rc = f4j_dev_alloc(ctx, E * 8 * W, (void**)&ev);
        if (!rc) {
            if (a_complex && b_complex) launch_spgemm_expand<1, 1>(ctx, A, B, len, er, ec, ev);
            else if (a_complex) launch_spgemm_expand<1, 0>(ctx, A, B, len, er, ec, ev);
            else if (b_complex) launch_spgemm_expand<0, 1>(ctx, A, B, len, er, ec, ev);
            else launch_spgemm_expand<0, 0>(ctx, A, B, len, er, ec, ev);
            ctx->launches++;
            if (W == 1) {
                rc = coo_sort_dev(ctx, (int64_t)E, er, ec, ev);
            } else {
                // complex products follow the sort through its permutation
                rc = f4j_dev_alloc(ctx, E * 4, (void**)&perm);
                if (!rc) rc = coo_sort_dev(ctx, (int64_t)E, er, ec, nullptr, perm);
                if (!rc) rc = f4j_dev_alloc(ctx, E * 16, (void**)&evs);
                if (!rc) {
                    k_gather_z<<<(unsigned)f4j_cdiv(E, 256), 256, 0, ctx->stream>>>(
                        (int64_t)E, perm, (const double2*)ev, (double2*)evs);
                    ctx->launches++;
                    double* t = ev;
                    ev = evs;
                    evs = t;
                }
            }
        }
        if (!rc) rc = f4j_dev_alloc(ctx, E * 4, (void**)&fs);
        if (!rc) {
            k_run_flags<<<(unsigned)f4j_cdiv(E, 256), 256, 0, ctx->stream>>>((int64_t)E, er, ec, fs);
            ctx->launches++;
            rc = scan_inclusive(ctx, fs, (int64_t)E);
        }
        if (!rc) {
            int last = 0;
            F4J_CUDA(cudaMemcpyAsync(&last, fs + E - 1, 4, cudaMemcpyDeviceToHost, ctx->stream));
            F4J_CUDA(cudaStreamSynchronize(ctx->stream));
            runs = last;
            rc = f4j_dev_alloc(ctx, (size_t)runs * 4, (void**)&starts);
        }
        if (!rc) {
            k_run_starts<<<(unsigned)f4j_cdiv(E, 256), 256, 0, ctx->stream>>>((int64_t)E, fs, starts);
            ctx->launches++;
        }
    }
    f4j_csr T = nullptr;
    if (!rc) rc = alloc_owned_csr(ctx, rows, B->cols, runs, &T, W);
    if (!rc) {
        int* trp = (int*)T->rowptr->ptr;
        F4J_CUDA(cudaMemsetAsync(trp, 0, (size_t)(rows + 1) * 4, ctx->stream));
        if (runs > 0) {
            const unsigned g = (unsigned)f4j_cdiv(runs, 256);
            if (W == 2)
                k_run_sum<2><<<g, 256, 0, ctx->stream>>>(runs, (int64_t)E, starts, er, ec, ev, (int*)T->colidx->ptr,
                                                         (double*)T->vals->ptr, trp + 1);
            else
                k_run_sum<1><<<g, 256, 0, ctx->stream>>>(runs, (int64_t)E, starts, er, ec, ev, (int*)T->colidx->ptr,
                                                         (double*)T->vals->ptr, trp + 1);
            ctx->launches++;
            rc = scan_inclusive(ctx, trp + 1, rows);
        }
        cudaError_t e = cudaGetLastError();
        if (!rc && e != cudaSuccess) rc = f4j_cuda_fail(e, "CSR x CSR");
    }
    f4j_dev_free(ctx, len);
    f4j_dev_free(ctx, total);
    f4j_dev_free(ctx, er);
    f4j_dev_free(ctx, ec);
    f4j_dev_free(ctx, ev);
    f4j_dev_free(ctx, evs);
    f4j_dev_free(ctx, perm);
    f4j_dev_free(ctx, fs);
    f4j_dev_free(ctx, starts);
    if (rc) {
        if (T) f4j_csr_free(ctx, T);
        return rc;
    }
    *out = T;
    if (rep) {
        *rep = f4j_report{};
        rep->launches = (int32_t)(ctx->launches - l0);
    }
    return F4J_OK;
}

extern "C" int f4j_csr_mult_csr(f4j_ctx* ctx, f4j_csr A, f4j_csr B, f4j_csr* out, f4j_report* rep) {
    F4J_LOCK(ctx);
    return f4j_csr_mult_csr_ex(ctx, A, 0, B, 0, out, rep);
}

extern "C" int f4j_csr_transpose(f4j_ctx* ctx, f4j_csr S, f4j_csr* out) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (!S || !out) return f4j_fail(F4J_ERR_ARG, "null argument");
    F4J_CUDA(cudaSetDevice(ctx->device));
    int rc = ensure_transpose(ctx, S);
    if (rc) return rc;
    f4j_csr T;
    rc = alloc_owned_csr(ctx, S->cols, S->rows, S->nnz, &T);
    if (rc) return rc;
    F4J_CUDA(cudaMemcpyAsync(T->rowptr->ptr, S->t_rowptr, (size_t)(S->cols + 1) * 4, cudaMemcpyDeviceToDevice,
                             ctx->stream));
    F4J_CUDA(cudaMemcpyAsync(T->colidx->ptr, S->t_rowidx, (size_t)S->nnz * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    if (S->nnz) {
        k_gather<double><<<grid1(S->nnz), 256, 0, ctx->stream>>>(S->nnz, (const int*)S->t_perm,
                                                                 (const double*)S->vals->ptr, (double*)T->vals->ptr);
        F4J_LAUNCHED(ctx);
    }
    *out = T;
    return F4J_OK;
}

extern "C" int f4j_csr_transpose_perm(f4j_ctx* ctx, f4j_csr S, f4j_buf perm_out) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (!S || !perm_out) return f4j_fail(F4J_ERR_ARG, "null argument");
    if (perm_out->bytes < (size_t)S->nnz * 4) return f4j_fail(F4J_ERR_ARG, "perm buffer too small");
    F4J_CUDA(cudaSetDevice(ctx->device));
    int rc = ensure_transpose(ctx, S);
    if (rc) return rc;
    F4J_CUDA(cudaMemcpyAsync(perm_out->ptr, S->t_perm, (size_t)S->nnz * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    return F4J_OK;
}

extern "C" int f4j_spmv_ex(f4j_ctx* ctx, f4j_csr S, f4j_buf x, f4j_buf y, int mode, f4j_report* rep) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (mode != F4J_SPARSE_EXACT && mode != F4J_SPARSE_FMA) return f4j_fail(F4J_ERR_ARG, "unknown sparse mode %d", mode);
    if (!S || !x || !y) return f4j_fail(F4J_ERR_ARG, "null argument");
    if (x->bytes < (size_t)S->cols * 8)
        return f4j_fail(F4J_ERR_ARG, "Expecting values to be equal but got: [%lld, %lld]", (long long)S->cols,
                        (long long)(x->bytes / 8));
    if (y->bytes < (size_t)S->rows * 8) return f4j_fail(F4J_ERR_ARG, "y buffer too small");
    if (!f4j_aligned(x->ptr, 8) || !f4j_aligned(y->ptr, 8)) return f4j_fail(F4J_ERR_ARG, "x and y must be 8-byte aligned");
    F4J_CUDA(cudaSetDevice(ctx->device));
    int64_t l0 = ctx->launches;
    if (S->rows) {
        // rows per warp: as many as fill every SM's resident blocks of 8 warps
        // once (173 exact / 216 FMA at 2^20 rows), so the SMs finish together;
        // more rows per warp balance the lanes better, up to 256; at least 32
        const int bps = mode == F4J_SPARSE_FMA ? SpmvOcc<true>::BLOCKS : SpmvOcc<false>::BLOCKS;
        const int64_t slots = (int64_t)ctx->sm_count * bps * (SPMV_BLOCK / 32);
        int64_t rpw64 = f4j_cdiv(S->rows, slots);
        const int rpw = (int)(rpw64 < 32 ? 32 : (rpw64 > SPMV_RPW_MAX ? SPMV_RPW_MAX : rpw64));
        const unsigned blocks = (unsigned)f4j_cdiv(f4j_cdiv(S->rows, rpw), SPMV_BLOCK / 32);
        const bool fused = mode == F4J_SPARSE_FMA;
        // 32-byte loads of column indices and values when both arrays start 32-byte aligned
        const bool vec = f4j_aligned(S->colidx->ptr, 32) && f4j_aligned(S->vals->ptr, 32);
        auto kern = fused ? (vec ? k_spmv<true, true> : k_spmv<true, false>)
                          : (vec ? k_spmv<false, true> : k_spmv<false, false>);
        f4j_prof_begin(ctx);
        kern<<<blocks, SPMV_BLOCK, 0, ctx->stream>>>(S->rows, S->nnz, rpw, (const int*)S->rowptr->ptr,
                                                     (const int*)S->colidx->ptr, (const double*)S->vals->ptr,
                                                     (const double*)x->ptr, (double*)y->ptr);
        f4j_prof_end(ctx);
        F4J_LAUNCHED(ctx);
    }
    if (rep) {
        *rep = f4j_report{};
        rep->flops = 2.0 * S->nnz;
        rep->bytes = 12.0 * S->nnz + 4.0 * (S->rows + 1) + 8.0 * S->cols + 8.0 * S->rows;
        rep->launches = (int32_t)(ctx->launches - l0);
    }
    return F4J_OK;
}

extern "C" int f4j_spmv(f4j_ctx* ctx, f4j_csr S, f4j_buf x, f4j_buf y, f4j_report* rep) {
    F4J_LOCK(ctx);
    return f4j_spmv_ex(ctx, S, x, y, F4J_SPARSE_EXACT, rep);
}

extern "C" int f4j_spmm_ex(f4j_ctx* ctx, f4j_csr S, f4j_buf X, int64_t ncols, f4j_buf Y, int mode,
                           f4j_report* rep) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (mode != F4J_SPARSE_EXACT && mode != F4J_SPARSE_FMA) return f4j_fail(F4J_ERR_ARG, "unknown sparse mode %d", mode);
    if (!S || !X || !Y) return f4j_fail(F4J_ERR_ARG, "null argument");
    if (ncols < 0) return f4j_fail(F4J_ERR_ARG, "negative column count");
    if (X->bytes < (size_t)S->cols * ncols * 8) return f4j_fail(F4J_ERR_ARG, "X buffer too small");
    if (Y->bytes < (size_t)S->rows * ncols * 8) return f4j_fail(F4J_ERR_ARG, "Y buffer too small");
    if (!f4j_aligned(X->ptr, 8) || !f4j_aligned(Y->ptr, 8)) return f4j_fail(F4J_ERR_ARG, "X and Y must be 8-byte aligned");
    F4J_CUDA(cudaSetDevice(ctx->device));
    int64_t l0 = ctx->launches;
    int rc = launch_spmm(ctx, S->rows, ncols, (const int*)S->rowptr->ptr, (const int*)S->colidx->ptr,
                         (const double*)S->vals->ptr, nullptr, (const double*)X->ptr, (double*)Y->ptr,
                         mode == F4J_SPARSE_FMA);
    if (rc) return rc;
    if (rep) {
        *rep = f4j_report{};
        rep->flops = 2.0 * S->nnz * ncols;
        rep->bytes = 12.0 * S->nnz + 4.0 * (S->rows + 1) + 8.0 * ncols * (S->cols + S->rows);
        rep->launches = (int32_t)(ctx->launches - l0);
    }
    return F4J_OK;
}

extern "C" int f4j_spmm(f4j_ctx* ctx, f4j_csr S, f4j_buf X, int64_t ncols, f4j_buf Y, f4j_report* rep) {
    F4J_LOCK(ctx);
    return f4j_spmm_ex(ctx, S, X, ncols, Y, F4J_SPARSE_EXACT, rep);
}

extern "C" int f4j_zspmm(f4j_ctx* ctx, f4j_csr S, f4j_buf X, int64_t ncols, f4j_buf Y, f4j_report* rep) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (!S || !X || !Y) return f4j_fail(F4J_ERR_ARG, "null argument");
    if (ncols < 0) return f4j_fail(F4J_ERR_ARG, "negative column count");
    if (S->vals->bytes < (size_t)S->nnz * 16)
        return f4j_fail(F4J_ERR_ARG, "complex CSR values need 16 bytes per nonzero (nnz=%lld)", (long long)S->nnz);
    if (X->bytes < (size_t)S->cols * ncols * 16) return f4j_fail(F4J_ERR_ARG, "X buffer too small");
    if (Y->bytes < (size_t)S->rows * ncols * 16) return f4j_fail(F4J_ERR_ARG, "Y buffer too small");
    if (!f4j_aligned16(S->vals->ptr) || !f4j_aligned16(X->ptr) || !f4j_aligned16(Y->ptr))
        return f4j_fail(F4J_ERR_ARG, "complex buffers must be 16-byte aligned");
    F4J_CUDA(cudaSetDevice(ctx->device));
    int64_t l0 = ctx->launches;
    if (S->rows && ncols) {
        int G = 1;
        while (G < 32 && G < ncols) G *= 2;
        f4j_prof_begin(ctx);
        k_zspmm<<<(unsigned)f4j_cdiv(S->rows * G, 256), 256, 0, ctx->stream>>>(
            S->rows, ncols, G, (const int*)S->rowptr->ptr, (const int*)S->colidx->ptr, (const double2*)S->vals->ptr,
            (const double2*)X->ptr, (double2*)Y->ptr);
        f4j_prof_end(ctx);
        F4J_LAUNCHED(ctx);
    }
    if (rep) {
        *rep = f4j_report{};
        rep->flops = 8.0 * S->nnz * ncols;
        rep->bytes = 20.0 * S->nnz + 4.0 * (S->rows + 1) + 16.0 * ncols * (S->cols + S->rows);
        rep->launches = (int32_t)(ctx->launches - l0);
    }
    return F4J_OK;
}

extern "C" int f4j_spmm_t(f4j_ctx* ctx, f4j_csr S, f4j_buf dC, int64_t ncols, f4j_buf dX, f4j_report* rep) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (!S || !dC || !dX) return f4j_fail(F4J_ERR_ARG, "null argument");
    if (ncols < 0) return f4j_fail(F4J_ERR_ARG, "negative column count");
    if (dC->bytes < (size_t)S->rows * ncols * 8) return f4j_fail(F4J_ERR_ARG, "dC buffer too small");
    if (dX->bytes < (size_t)S->cols * ncols * 8) return f4j_fail(F4J_ERR_ARG, "dX buffer too small");
    F4J_CUDA(cudaSetDevice(ctx->device));
    int64_t l0 = ctx->launches;
    int rc = ensure_transpose(ctx, S);
    if (rc) return rc;
    rc = launch_spmm(ctx, S->cols, ncols, (const int*)S->t_rowptr, (const int*)S->t_rowidx,
                     (const double*)S->vals->ptr, (const int*)S->t_perm, (const double*)dC->ptr, (double*)dX->ptr);
    if (rc) return rc;
    if (rep) {
        *rep = f4j_report{};
        rep->flops = 2.0 * S->nnz * ncols;
        rep->bytes = 16.0 * S->nnz + 4.0 * (S->cols + 1) + 8.0 * ncols * (S->cols + S->rows);
        rep->launches = (int32_t)(ctx->launches - l0);
    }
    return F4J_OK;
}

extern "C" int f4j_sddmm(f4j_ctx* ctx, f4j_csr S, f4j_buf A, f4j_buf B, int64_t ncols, f4j_buf out,
                         f4j_report* rep) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (!S || !A || !B || !out) return f4j_fail(F4J_ERR_ARG, "null argument");
    if (ncols < 0) return f4j_fail(F4J_ERR_ARG, "negative column count");
    if (A->bytes < (size_t)S->rows * ncols * 8) return f4j_fail(F4J_ERR_ARG, "A buffer too small");
    if (B->bytes < (size_t)S->cols * ncols * 8) return f4j_fail(F4J_ERR_ARG, "B buffer too small");
    if (out->bytes < (size_t)S->nnz * 8) return f4j_fail(F4J_ERR_ARG, "output buffer too small");
    F4J_CUDA(cudaSetDevice(ctx->device));
    int64_t l0 = ctx->launches;
    if (S->rows && S->nnz) {
        f4j_prof_begin(ctx);
        if (ncols == 64 && ((reinterpret_cast<uintptr_t>(A->ptr) | reinterpret_cast<uintptr_t>(B->ptr)) & 15) == 0) {
            int rc = ensure_rowidx(ctx, S);
            if (rc) return rc;
            k_sddmm64s<<<(unsigned)f4j_cdiv(S->nnz, SD_NNZ), 256, 0, ctx->stream>>>(
                S->nnz, (const int*)S->rowidx, (const int*)S->colidx->ptr, (const double*)A->ptr,
                (const double*)B->ptr, (double*)out->ptr);
        } else
            k_sddmm<<<(unsigned)f4j_cdiv(S->rows * 32, 256), 256, 0, ctx->stream>>>(
                S->rows, ncols, (const int*)S->rowptr->ptr, (const int*)S->colidx->ptr, (const double*)A->ptr,
                (const double*)B->ptr, (double*)out->ptr);
        f4j_prof_end(ctx);
        F4J_LAUNCHED(ctx);
    }
    if (rep) {
        *rep = f4j_report{};
        rep->flops = 2.0 * S->nnz * ncols;
        rep->bytes = 12.0 * S->nnz + 4.0 * (S->rows + 1) + 8.0 * ncols * (S->rows + S->cols);
        rep->launches = (int32_t)(ctx->launches - l0);
    }
    return F4J_OK;
}
