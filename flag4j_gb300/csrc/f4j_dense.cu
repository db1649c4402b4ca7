// f4j_dense.cu -- FP64 dense GEMM kernels for sm_103a.
//
//  * k_gemm_exact: Flag4j's own arithmetic order (RealDenseMatMult.reordered,
//    src/main/java/org/flag4j/linalg/ops/dense/real/RealDenseMatMult.java:284-310;
//    complex: DenseSemiringMatMult.java:382-424 with Complex128.java:276-341).
//    Every output accumulates k-ascending with separately rounded products and
//    sums (no FMA), so results are bit-identical to the reference.
//  * k_gemm_dmma: FP64 tensor-core GEMM (mma.sync m16n8k4 f64), operand tiles
//    fed by TMA into shared memory through an mbarrier ring, one producer warp
//    and four consumer warps.  Complex runs the four real products on the
//    interleaved tiles (Cr = Ar Br - Ai Bi, Ci = Ar Bi + Ai Br).
//    Transposed / conjugated operands use transposed TMA boxes; nothing is
//    materialised.
//  * k_gemv_rows / k_gemv_cols: matrix-vector products (n == 1) in the fast
//    modes, FP64 FMA dot products reading A once.
//  * k_gemm_check: double-double (Dot2) evaluation of sampled entries.
#include <cstring>

#include "f4j_internal.cuh"
#include "f4j_ptx.cuh"

namespace {

// element (r, c) of op(X), X row-major with leading dimension ld (in elements).
template <bool CPLX>
__device__ __forceinline__ void ld_op(const double* __restrict__ X, int64_t ld, int op, int64_t r,
                                      int64_t c, double& re, double& im) {
    int64_t idx = (op == F4J_OP_N) ? r * ld + c : c * ld + r;
    if (CPLX) {
        re = X[2 * idx];
        im = X[2 * idx + 1];
        if (op == F4J_OP_C) im = -im;
    } else {
        re = X[idx];
        im = 0.0;
    }
}

// ------------------------------------------------------------------ EXACT
constexpr int EX_BM = 64, EX_BN = 64, EX_BK = 16, EX_T = 256;  // 16x16 threads, 4x4 each

template <bool CPLX>
__global__ void __launch_bounds__(EX_T) k_gemm_exact(int64_t m, int64_t n, int64_t k,
                                                     const double* __restrict__ A, int64_t lda, int opA,
                                                     const double* __restrict__ B, int64_t ldb, int opB,
                                                     double* __restrict__ C) {
    __shared__ double sAr[EX_BK][EX_BM + 1], sBr[EX_BK][EX_BN + 1];
    __shared__ double sAi[CPLX ? EX_BK : 1][EX_BM + 1], sBi[CPLX ? EX_BK : 1][EX_BN + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int64_t m0 = (int64_t)blockIdx.y * EX_BM, n0 = (int64_t)blockIdx.x * EX_BN;
    double cr[4][4], ci[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) cr[i][j] = ci[i][j] = 0.0;

    for (int64_t k0 = 0; k0 < k; k0 += EX_BK) {
        for (int e = threadIdx.x; e < EX_BK * EX_BM; e += EX_T) {
            int kk = e / EX_BM, r = e % EX_BM;
            double re = 0, im = 0;
            if (m0 + r < m && k0 + kk < k) ld_op<CPLX>(A, lda, opA, m0 + r, k0 + kk, re, im);
            sAr[kk][r] = re;
            if (CPLX) sAi[kk][r] = im;
        }
        for (int e = threadIdx.x; e < EX_BK * EX_BN; e += EX_T) {
            int kk = e / EX_BN, c = e % EX_BN;
            double re = 0, im = 0;
            if (n0 + c < n && k0 + kk < k) ld_op<CPLX>(B, ldb, opB, k0 + kk, n0 + c, re, im);
            sBr[kk][c] = re;
            if (CPLX) sBi[kk][c] = im;
        }
        __syncthreads();
        const int kmax = (int)((k - k0) < EX_BK ? (k - k0) : EX_BK);
        for (int kk = 0; kk < kmax; kk++) {
            double ar[4], br[4], ai[4], bi[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                ar[i] = sAr[kk][ty + 16 * i];
                br[i] = sBr[kk][tx + 16 * i];
                if (CPLX) {
                    ai[i] = sAi[kk][ty + 16 * i];
                    bi[i] = sBi[kk][tx + 16 * i];
                }
            }
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    if (CPLX) {
                        double pr = __dsub_rn(__dmul_rn(ar[i], br[j]), __dmul_rn(ai[i], bi[j]));
                        double pi = __dadd_rn(__dmul_rn(ar[i], bi[j]), __dmul_rn(ai[i], br[j]));
                        cr[i][j] = __dadd_rn(cr[i][j], pr);
                        ci[i][j] = __dadd_rn(ci[i][j], pi);
                    } else {
                        cr[i][j] = __dadd_rn(cr[i][j], __dmul_rn(ar[i], br[j]));
                    }
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            int64_t r = m0 + ty + 16 * i, c = n0 + tx + 16 * j;
            if (r < m && c < n) {
                if (CPLX) {
                    C[2 * (r * n + c)] = cr[i][j];
                    C[2 * (r * n + c) + 1] = ci[i][j];
                } else {
                    C[r * n + c] = cr[i][j];
                }
            }
        }
}

// ------------------------------------------------------------------ DMMA
// CTA tile 64 x 64, K step 16 (real) per stage, 4 stages.  Warp 0 produces,
// warps 1..4 consume; each consumer owns a 32 x 32 quadrant = 2 x 4 tiles of
// m16n8, k4 per mma.
constexpr int DM_BM = 64, DM_BN = 64, DM_BK = 16, DM_ST = 4, DM_THREADS = 160;

struct DmmaParams {
    int64_t m, n, k;
    const double* A;
    const double* B;
    double* C;
    int64_t lda, ldb;  // leading dims of the stored matrices, in elements
    int opA, opB;
    int use_tma;
    int* status;
    const int* gate;  // compute only when null or *gate != 0
    int tiles_n, ntiles;
};

__device__ __forceinline__ void dmma_16x8x4(double (&d)[4], double a0, double a1, double b0) {
    asm volatile(
        "mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0, %1, %2, %3}, {%4, %5}, {%6}, {%0, %1, %2, %3};"
        : "+d"(d[0]), "+d"(d[1]), "+d"(d[2]), "+d"(d[3])
        : "d"(a0), "d"(a1), "d"(b0));
}

// Shared-memory tile geometry (in doubles).  A tile holds op(A)[m0:m0+BM,
// k0:k0+BK]; stored as [BM][W*BK] when opA == N (W = 2 for complex) or as
// [BK][W*BM] when transposed.  Likewise B as [BK][W*BN] (N) or [BN][W*BK].
template <bool CPLX>
struct DmTile {
    static constexpr int W = CPLX ? 2 : 1;
    static constexpr int A_ELEMS = DM_BM * DM_BK * W;
    static constexpr int B_ELEMS = DM_BN * DM_BK * W;
    static constexpr int STAGE_BYTES = (A_ELEMS + B_ELEMS) * 8;
};

template <bool CPLX>
__device__ __forceinline__ void sm_a(const double* s, int opA, int r, int kk, double& re, double& im) {
    constexpr int W = CPLX ? 2 : 1;
    int idx = (opA == F4J_OP_N) ? (r * DM_BK + kk) : (kk * DM_BM + r);
    re = s[W * idx];
    im = CPLX ? s[W * idx + 1] : 0.0;
    if (CPLX && opA == F4J_OP_C) im = -im;
}

template <bool CPLX>
__device__ __forceinline__ void sm_b(const double* s, int opB, int kk, int c, double& re, double& im) {
    constexpr int W = CPLX ? 2 : 1;
    int idx = (opB == F4J_OP_N) ? (kk * DM_BN + c) : (c * DM_BK + kk);
    re = s[W * idx];
    im = CPLX ? s[W * idx + 1] : 0.0;
    if (CPLX && opB == F4J_OP_C) im = -im;
}

template <bool CPLX>
__global__ void __launch_bounds__(DM_THREADS, 1)
    k_gemm_dmma(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                DmmaParams p) {
    using G = DmTile<CPLX>;
    constexpr int W = G::W;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    double* sA = reinterpret_cast<double*>(smem_raw);
    double* sB = sA + DM_ST * G::A_ELEMS;
    __shared__ __align__(8) uint64_t full[DM_ST], empty[DM_ST];
    __shared__ int abort_flag;

    if (p.gate && *(volatile const int*)p.gate == 0) return;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int nk = (int)((p.k + DM_BK - 1) / DM_BK);

    if (threadIdx.x == 0) {
        for (int s = 0; s < DM_ST; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 4);
        }
        abort_flag = 0;
        fence_barrier_init();
    }
    __syncthreads();

    if (warp == 0) {
        // ---------------- producer (persistent over tiles; the stage counter
        // `it` runs on across tiles so barrier phases stay in step)
        int it = 0;
        for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
        const int64_t m0 = (int64_t)(tile / p.tiles_n) * DM_BM, n0 = (int64_t)(tile % p.tiles_n) * DM_BN;
        for (int kt = 0; kt < nk; kt++, it++) {
            const int s = it % DM_ST;
            const uint32_t ph = (it / DM_ST) & 1;
            if (it >= DM_ST) {
                bool ok = true;
                if (lane == 0) ok = mbar_wait(&empty[s], ph ^ 1, p.status, 1);
                ok = __shfl_sync(0xffffffffu, ok, 0);
                if (!ok || *(volatile int*)&abort_flag) {
                    abort_flag = 1;
                    break;
                }
            }
            const int64_t k0 = (int64_t)kt * DM_BK;
            double* a = sA + s * G::A_ELEMS;
            double* b = sB + s * G::B_ELEMS;
            if (p.use_tma) {
                if (lane == 0) {
                    mbar_arrive_expect_tx(&full[s], G::STAGE_BYTES);
                    if (p.opA == F4J_OP_N) tma_load_2d(a, &tmA, &full[s], (int)(W * k0), (int)m0);
                    else tma_load_2d(a, &tmA, &full[s], (int)(W * m0), (int)k0);
                    if (p.opB == F4J_OP_N) tma_load_2d(b, &tmB, &full[s], (int)(W * n0), (int)k0);
                    else tma_load_2d(b, &tmB, &full[s], (int)(W * k0), (int)n0);
                }
            } else {
                // Plain loads for leading dimensions TMA cannot describe (odd real k / n).
                for (int e = lane; e < DM_BM * DM_BK * W; e += 32) {
                    int outer, inner;
                    double v = 0.0;
                    if (p.opA == F4J_OP_N) {
                        outer = e / (DM_BK * W); inner = e % (DM_BK * W);
                        int64_t gr = m0 + outer, gc = W * k0 + inner;
                        if (gr < p.m && gc < W * p.k) v = p.A[gr * W * p.lda + gc];
                    } else {
                        outer = e / (DM_BM * W); inner = e % (DM_BM * W);
                        int64_t gr = k0 + outer, gc = W * m0 + inner;
                        if (gr < p.k && gc < W * p.m) v = p.A[gr * W * p.lda + gc];
                    }
                    a[e] = v;
                }
                for (int e = lane; e < DM_BN * DM_BK * W; e += 32) {
                    int outer, inner;
                    double v = 0.0;
                    if (p.opB == F4J_OP_N) {
                        outer = e / (DM_BN * W); inner = e % (DM_BN * W);
                        int64_t gr = k0 + outer, gc = W * n0 + inner;
                        if (gr < p.k && gc < W * p.n) v = p.B[gr * W * p.ldb + gc];
                    } else {
                        outer = e / (DM_BK * W); inner = e % (DM_BK * W);
                        int64_t gr = n0 + outer, gc = W * k0 + inner;
                        if (gr < p.n && gc < W * p.k) v = p.B[gr * W * p.ldb + gc];
                    }
                    b[e] = v;
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(&full[s]);
            }
        }
        if (*(volatile int*)&abort_flag) break;
        }  // tile loop
        // Drain: wait (bounded) for the last copies in flight before exiting.
        if (lane == 0 && p.use_tma) {
            for (int q = (it > DM_ST ? it - DM_ST : 0); q < it; q++)
                mbar_wait(&full[q % DM_ST], (q / DM_ST) & 1, nullptr, 0);
        }
        return;
    }

    // ---------------- consumers (warps 1..4)
    const int cw = warp - 1;
    const int wm = (cw / 2) * 32, wn = (cw % 2) * 32;
    const int g = lane >> 2, t = lane & 3;
    int it = 0;
    for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
    const int64_t m0 = (int64_t)(tile / p.tiles_n) * DM_BM, n0 = (int64_t)(tile % p.tiles_n) * DM_BN;
    double accr[2][4][4], acci[CPLX ? 2 : 1][4][4];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int q = 0; q < 4; q++) {
                accr[i][j][q] = 0.0;
                if (CPLX) acci[i][j][q] = 0.0;
            }

    for (int kt = 0; kt < nk; kt++, it++) {
        const int s = it % DM_ST;
        const uint32_t ph = (it / DM_ST) & 1;
        bool ok = true;
        if (lane == 0) ok = mbar_wait(&full[s], ph, p.status, 2);
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok || *(volatile int*)&abort_flag) {
            abort_flag = 1;
            break;
        }
        const double* a = sA + s * G::A_ELEMS;
        const double* b = sB + s * G::B_ELEMS;
#pragma unroll
        for (int k4 = 0; k4 < DM_BK; k4 += 4) {
            double ar[2][2], ai[2][2], br[4], bi[4];
#pragma unroll
            for (int i = 0; i < 2; i++) {
                sm_a<CPLX>(a, p.opA, wm + 16 * i + g, k4 + t, ar[i][0], ai[i][0]);
                sm_a<CPLX>(a, p.opA, wm + 16 * i + g + 8, k4 + t, ar[i][1], ai[i][1]);
            }
#pragma unroll
            for (int j = 0; j < 4; j++) sm_b<CPLX>(b, p.opB, k4 + t, wn + 8 * j + g, br[j], bi[j]);
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    dmma_16x8x4(accr[i][j], ar[i][0], ar[i][1], br[j]);
                    if (CPLX) {
                        dmma_16x8x4(accr[i][j], -ai[i][0], -ai[i][1], bi[j]);
                        dmma_16x8x4(acci[i][j], ar[i][0], ar[i][1], bi[j]);
                        dmma_16x8x4(acci[i][j], ai[i][0], ai[i][1], br[j]);
                    }
                }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
    }
    if (*(volatile int*)&abort_flag) return;

#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int64_t r = m0 + wm + 16 * i + g + (q >= 2 ? 8 : 0);
                const int64_t c = n0 + wn + 8 * j + 2 * t + (q & 1);
                if (r < p.m && c < p.n) {
                    if (CPLX) {
                        p.C[2 * (r * p.n + c)] = accr[i][j][q];
                        p.C[2 * (r * p.n + c) + 1] = acci[i][j][q];
                    } else {
                        p.C[r * p.n + c] = accr[i][j][q];
                    }
                }
            }
    }  // tile loop
}

// ------------------------------------------------------------------ check
struct DD {
    double hi, lo;
};

__device__ __forceinline__ void dd_add(DD& a, double b) {
    double s = a.hi + b;
    double z = s - a.hi;
    double e = (a.hi - (s - z)) + (b - z);
    a.hi = s;
    a.lo += e;
}

__device__ __forceinline__ void dd_add_prod(DD& a, double x, double y) {
    double p = x * y;
    double pe = fma(x, y, -p);
    dd_add(a, p);
    a.lo += pe;
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

template <bool CPLX>
__global__ void k_gemm_check(int64_t m, int64_t n, int64_t k, const double* __restrict__ A, int64_t lda,
                             int opA, const double* __restrict__ B, int64_t ldb, int opB,
                             const double* __restrict__ C, int64_t samples, uint64_t seed,
                             unsigned long long* out) {
    const int64_t s = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x % 32;
    if (s >= samples) return;
    const uint64_t base = mix64(seed);  // every seed bit reaches the samples
    const int64_t i = (int64_t)(mix64(base ^ (2 * s)) % (uint64_t)m);
    const int64_t j = (int64_t)(mix64(base ^ (2 * s + 1)) % (uint64_t)n);
    DD re{0, 0}, im{0, 0};
    double absr = 0, absi = 0;
    for (int64_t q = lane; q < k; q += 32) {
        double ar, ai, br, bi;
        ld_op<CPLX>(A, lda, opA, i, q, ar, ai);
        ld_op<CPLX>(B, ldb, opB, q, j, br, bi);
        dd_add_prod(re, ar, br);
        absr += fabs(ar * br);
        if (CPLX) {
            dd_add_prod(re, -ai, bi);
            dd_add_prod(im, ar, bi);
            dd_add_prod(im, ai, br);
            absr += fabs(ai * bi);
            absi += fabs(ar * bi) + fabs(ai * br);
        }
    }
    for (int off = 16; off; off >>= 1) {
        DD o{__shfl_xor_sync(0xffffffffu, re.hi, off), __shfl_xor_sync(0xffffffffu, re.lo, off)};
        dd_add(re, o.hi);
        re.lo += o.lo;
        absr += __shfl_xor_sync(0xffffffffu, absr, off);
        if (CPLX) {
            DD oi{__shfl_xor_sync(0xffffffffu, im.hi, off), __shfl_xor_sync(0xffffffffu, im.lo, off)};
            dd_add(im, oi.hi);
            im.lo += oi.lo;
            absi += __shfl_xor_sync(0xffffffffu, absi, off);
        }
    }
    if (lane == 0) {
        double cr = CPLX ? C[2 * (i * n + j)] : C[i * n + j];
        double er = fabs((cr - re.hi) - re.lo);
        double rr = absr > 0 ? er / absr : (er > 0 ? INFINITY : 0.0);
        double ea = er, ra = rr;
        if (CPLX) {
            double ci = C[2 * (i * n + j) + 1];
            double ei = fabs((ci - im.hi) - im.lo);
            double ri = absi > 0 ? ei / absi : (ei > 0 ? INFINITY : 0.0);
            ea = fmax(ea, ei);
            ra = fmax(ra, ri);
        }
        if (ea != ea) ea = INFINITY;
        if (ra != ra) ra = INFINITY;
        atomicMax(&out[0], (unsigned long long)__double_as_longlong(ea));
        atomicMax(&out[1], (unsigned long long)__double_as_longlong(ra));
    }
}

// ------------------------------------------------------------------ GEMV
// y = op(A) x (n == 1) for the non-exact modes: FP64 FMA dot products, error
// within k u |A||x| (the plain DMMA path's class).  W = 2 for interleaved
// complex; sa / sx = -1 conjugate A / x (an exact sign flip).
// op(A) = N: A stored m x k, a warp per row, lanes stride the row, warp sum.
template <bool CPLX>
__global__ void __launch_bounds__(256) k_gemv_rows(int64_t m, int64_t k, const double* __restrict__ A,
                                                   const double* __restrict__ x, double sx, double* __restrict__ y) {
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x % 32;
    if (row >= m) return;
    double re = 0.0, im = 0.0;
    if (!CPLX) {
        // four independent chains, their eight loads issued together: the
        // FP64 pipe (2 lanes per clock per SM) bounds this kernel, and two
        // chains per warp left it waiting on loads
        const double* a = A + row * k;
        double r1 = 0.0, r2 = 0.0, r3 = 0.0;
        int64_t j = lane;
        for (; j + 96 < k; j += 128) {
            const double a0 = __ldg(&a[j]), a1 = __ldg(&a[j + 32]), a2 = __ldg(&a[j + 64]), a3 = __ldg(&a[j + 96]);
            const double x0 = __ldg(&x[j]), x1 = __ldg(&x[j + 32]), x2 = __ldg(&x[j + 64]), x3 = __ldg(&x[j + 96]);
            re = fma(a0, x0, re);
            r1 = fma(a1, x1, r1);
            r2 = fma(a2, x2, r2);
            r3 = fma(a3, x3, r3);
        }
        for (; j < k; j += 32) re = fma(__ldg(&a[j]), __ldg(&x[j]), re);
        re = (re + r1) + (r2 + r3);
    } else {
        const double2* a = reinterpret_cast<const double2*>(A) + row * k;
        const double2* xv = reinterpret_cast<const double2*>(x);
        for (int64_t j = lane; j < k; j += 32) {
            const double2 av = __ldg(&a[j]), xx = __ldg(&xv[j]);
            const double xi = sx * xx.y;
            re = fma(av.x, xx.x, re);
            re = fma(-av.y, xi, re);
            im = fma(av.x, xi, im);
            im = fma(av.y, xx.x, im);
        }
    }
    for (int o = 16; o; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        if (CPLX) im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if (lane == 0) {
        if (CPLX) {
            y[2 * row] = re;
            y[2 * row + 1] = im;
        } else {
            y[row] = re;
        }
    }
}

// op(A) = T / C: A stored k x m; a thread per output element and K chunk
// (coalesced along the stored rows), partial sums part[chunk][m * W].
template <bool CPLX>
__global__ void __launch_bounds__(256) k_gemv_cols(int64_t m, int64_t k, int64_t kchunk, const double* __restrict__ A,
                                                   double sa, const double* __restrict__ x, double sx,
                                                   double* __restrict__ part) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int64_t k0 = (int64_t)blockIdx.y * kchunk, k1 = k0 + kchunk < k ? k0 + kchunk : k;
    if (!CPLX) {
        double s = 0.0;
        for (int64_t kk = k0; kk < k1; kk++) s = fma(__ldg(&A[kk * m + i]), __ldg(&x[kk]), s);
        part[blockIdx.y * m + i] = s;
    } else {
        const double2* a = reinterpret_cast<const double2*>(A);
        const double2* xv = reinterpret_cast<const double2*>(x);
        double re = 0.0, im = 0.0;
        for (int64_t kk = k0; kk < k1; kk++) {
            const double2 av = __ldg(&a[kk * m + i]), xx = __ldg(&xv[kk]);
            const double ai = sa * av.y, xi = sx * xx.y;
            re = fma(av.x, xx.x, re);
            re = fma(-ai, xi, re);
            im = fma(av.x, xi, im);
            im = fma(ai, xx.x, im);
        }
        part[(blockIdx.y * m + i) * 2] = re;
        part[(blockIdx.y * m + i) * 2 + 1] = im;
    }
}

__global__ void k_gemv_sum(int64_t len, int64_t nchunk, const double* __restrict__ part, double* __restrict__ y) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= len) return;
    double s = 0.0;
    for (int64_t c = 0; c < nchunk; c++) s += part[c * len + i];
    y[i] = s;
}

}  // namespace

// ------------------------------------------------------------------ host side
int f4j_gemm_exact(f4j_ctx* ctx, bool cplx, int64_t m, int64_t n, int64_t k, const double* A, int opA,
                   const double* B, int opB, double* C) {
    int64_t lda = (opA == F4J_OP_N) ? k : m;
    int64_t ldb = (opB == F4J_OP_N) ? n : k;
    dim3 grid((unsigned)f4j_cdiv(n, EX_BN), (unsigned)f4j_cdiv(m, EX_BM));
    if (grid.y > 65535) return f4j_fail(F4J_ERR_ARG, "m too large for the exact kernel grid");
    f4j_prof_begin(ctx);
    if (cplx)
        k_gemm_exact<true><<<grid, EX_T, 0, ctx->stream>>>(m, n, k, A, lda, opA, B, ldb, opB, C);
    else
        k_gemm_exact<false><<<grid, EX_T, 0, ctx->stream>>>(m, n, k, A, lda, opA, B, ldb, opB, C);
    f4j_prof_end(ctx);
    F4J_LAUNCHED(ctx);
    return F4J_OK;
}

static int make_map_2d(CUtensorMap* map, const void* base, uint64_t inner, uint64_t outer, uint32_t box_inner,
                       uint32_t box_outer) {
    f4j_encode_tiled_fn enc = f4j_encode_fn();
    if (!enc) return f4j_fail(F4J_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {inner * 8};
    cuuint32_t box[2] = {box_inner, box_outer};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<void*>(base), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return f4j_fail(F4J_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return F4J_OK;
}

int f4j_gemm_dmma(f4j_ctx* ctx, bool cplx, int64_t m, int64_t n, int64_t k, const double* A, int opA,
                  const double* B, int opB, double* C, const int* gate) {
    const int W = cplx ? 2 : 1;
    DmmaParams p{};
    p.m = m; p.n = n; p.k = k; p.A = A; p.B = B; p.C = C;
    p.opA = opA; p.opB = opB;
    p.lda = (opA == F4J_OP_N) ? k : m;
    p.ldb = (opB == F4J_OP_N) ? n : k;
    p.status = ctx->d_status + F4J_ST_TIMEOUT;
    p.gate = gate;
    p.tiles_n = (int)f4j_cdiv(n, DM_BN);
    const int64_t ntiles = f4j_cdiv(n, DM_BN) * f4j_cdiv(m, DM_BM);
    if (ntiles > INT32_MAX) return f4j_fail(F4J_ERR_ARG, "DMMA GEMM too large");
    p.ntiles = (int)ntiles;
    // TMA needs 16-byte aligned bases and row strides.
    p.use_tma = f4j_aligned16(A) && f4j_aligned16(B) && ((p.lda * 8 * W) % 16 == 0) &&
                ((p.ldb * 8 * W) % 16 == 0) && f4j_encode_fn() != nullptr;
    CUtensorMap ta{}, tb{};
    if (p.use_tma) {
        int rc;
        if (opA == F4J_OP_N) rc = make_map_2d(&ta, A, W * k, m, W * DM_BK, DM_BM);
        else rc = make_map_2d(&ta, A, W * m, k, W * DM_BM, DM_BK);
        if (rc) return rc;
        if (opB == F4J_OP_N) rc = make_map_2d(&tb, B, W * n, k, W * DM_BN, DM_BK);
        else rc = make_map_2d(&tb, B, W * k, n, W * DM_BK, DM_BN);
        if (rc) return rc;
    }
    size_t smem = (size_t)DM_ST * (cplx ? DmTile<true>::STAGE_BYTES : DmTile<false>::STAGE_BYTES);
    // persistent: as many CTAs as fit at once (shared memory bound), each
    // walking tiles grid-stride
    const int per_sm = (int)((200 * 1024) / (smem + 2048)) > 0 ? (int)((200 * 1024) / (smem + 2048)) : 1;
    const int64_t cap = (int64_t)ctx->sm_count * per_sm;
    const unsigned grid = (unsigned)(ntiles < cap ? ntiles : cap);
    if (cplx) {
        F4J_CUDA(cudaFuncSetAttribute(k_gemm_dmma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        f4j_prof_begin(ctx);
        k_gemm_dmma<true><<<grid, DM_THREADS, smem, ctx->stream>>>(ta, tb, p);
    } else {
        F4J_CUDA(cudaFuncSetAttribute(k_gemm_dmma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        f4j_prof_begin(ctx);
        k_gemm_dmma<false><<<grid, DM_THREADS, smem, ctx->stream>>>(ta, tb, p);
    }
    f4j_prof_end(ctx);
    F4J_LAUNCHED(ctx);
    return F4J_OK;
}

int f4j_check_sampled(f4j_ctx* ctx, bool cplx, int64_t m, int64_t n, int64_t k, const double* A, int opA,
                      const double* B, int opB, const double* C, int64_t samples, uint64_t seed, double* max_abs,
                      double* max_rel) {
    if (!cplx) {
        if (opA == F4J_OP_C) opA = F4J_OP_T;
        if (opB == F4J_OP_C) opB = F4J_OP_T;
    }
    const int64_t lda = (opA == F4J_OP_N) ? k : m;
    const int64_t ldb = (opB == F4J_OP_N) ? n : k;
    void* ws = nullptr;
    int rc = f4j_dev_alloc(ctx, 16, &ws);
    if (rc) return rc;
    F4J_CUDA(cudaMemsetAsync(ws, 0, 16, ctx->stream));
    const unsigned blocks = (unsigned)f4j_cdiv(samples, 4);
    if (cplx)
        k_gemm_check<true><<<blocks, 128, 0, ctx->stream>>>(m, n, k, A, lda, opA, B, ldb, opB, C, samples, seed,
                                                             (unsigned long long*)ws);
    else
        k_gemm_check<false><<<blocks, 128, 0, ctx->stream>>>(m, n, k, A, lda, opA, B, ldb, opB, C, samples, seed,
                                                              (unsigned long long*)ws);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    unsigned long long h[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, ws, 16, cudaMemcpyDeviceToHost, ctx->stream);
    f4j_dev_free(ctx, ws);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return f4j_cuda_fail(e, "sampled accuracy check");
    memcpy(max_abs, &h[0], 8);
    memcpy(max_rel, &h[1], 8);
    return F4J_OK;
}

extern "C" int f4j_gemm_check(f4j_ctx* ctx, int cplx, int64_t m, int64_t n, int64_t k, f4j_buf A, int opA,
                              f4j_buf B, int opB, f4j_buf C, int64_t samples, uint64_t seed,
                              double* max_abs, double* max_rel) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (!A || !B || !C || !max_abs || !max_rel) return f4j_fail(F4J_ERR_ARG, "null argument");
    if (m <= 0 || n <= 0 || k < 0 || samples <= 0) return f4j_fail(F4J_ERR_ARG, "bad sizes");
    size_t es = cplx ? 16 : 8;
    if ((size_t)m * k * es > A->bytes || (size_t)k * n * es > B->bytes || (size_t)m * n * es > C->bytes)
        return f4j_fail(F4J_ERR_ARG, "buffer too small");
    F4J_CUDA(cudaSetDevice(ctx->device));
    return f4j_check_sampled(ctx, cplx != 0, m, n, k, (const double*)A->ptr, opA, (const double*)B->ptr, opB,
                             (const double*)C->ptr, samples, seed, max_abs, max_rel);
}

int f4j_gemv(f4j_ctx* ctx, bool cplx, int64_t m, int64_t k, const double* A, int opA, const double* x, bool conj_x,
             double* y) {
    const double sx = conj_x ? -1.0 : 1.0;
    if (opA == F4J_OP_N) {
        const unsigned blocks = (unsigned)f4j_cdiv(m * 32, 256);
        f4j_prof_begin(ctx);
        if (cplx) k_gemv_rows<true><<<blocks, 256, 0, ctx->stream>>>(m, k, A, x, sx, y);
        else k_gemv_rows<false><<<blocks, 256, 0, ctx->stream>>>(m, k, A, x, sx, y);
        f4j_prof_end(ctx);
        F4J_LAUNCHED(ctx);
        return F4J_OK;
    }
    // K split so that about 2048 threads per SM are busy; partials summed in chunk order
    int64_t nchunk = f4j_cdiv((int64_t)ctx->sm_count * 2048, m);
    if (nchunk > k) nchunk = k;
    if (nchunk > 65535) nchunk = 65535;
    if (nchunk < 1) nchunk = 1;
    const int64_t kchunk = f4j_cdiv(k, nchunk);
    nchunk = f4j_cdiv(k, kchunk);
    const int64_t len = m * (cplx ? 2 : 1);
    double* part = nullptr;
    int rc = f4j_dev_alloc(ctx, (size_t)(nchunk * len) * 8, (void**)&part);
    if (rc) return rc;
    const double sa = (opA == F4J_OP_C) ? -1.0 : 1.0;
    const dim3 grid((unsigned)f4j_cdiv(m, 256), (unsigned)nchunk);
    f4j_prof_begin(ctx);
    if (cplx) k_gemv_cols<true><<<grid, 256, 0, ctx->stream>>>(m, k, kchunk, A, sa, x, sx, part);
    else k_gemv_cols<false><<<grid, 256, 0, ctx->stream>>>(m, k, kchunk, A, sa, x, sx, part);
    k_gemv_sum<<<(unsigned)f4j_cdiv(len, 256), 256, 0, ctx->stream>>>(len, nchunk, part, y);
    f4j_prof_end(ctx);
    ctx->launches += 2;
    f4j_dev_free(ctx, part);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? F4J_OK : f4j_cuda_fail(e, "gemv");
}
