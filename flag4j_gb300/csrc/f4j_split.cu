// f4j_split.cu -- FP64-accurate split-precision GEMM on tcgen05 FP8 tensor cores.
//
// Scheme (Ozaki-style error-free slicing):
//  1. k_stats_*: per row of op(A) and per column of op(B), the power-of-two
//     bound 2^e > max|x| and the exponent spread (bits between the largest and
//     the mean element exponent).  The host picks the slice count s from the
//     spread.
//  2. k_split: every element becomes a fixed-point integer Y = round(x 2^(F-e))
//     (F = 4 + 5(s-1) bits, pure integer arithmetic on the IEEE bits), cut
//     into s balanced digits d_1 in [-16,16], d_2..d_s in [-16,15]; each digit
//     is exactly representable in E4M3.  Slices are written K-major
//     (rows x Kp bytes), one plane per slice.
//  3. k_split_gemm: for each output tile, the products A_i B_j with
//     i + j <= s + 1 run as tcgen05.mma kind::f8f6f4 with FP32 accumulation in
//     TMEM.  Products of one "round" share a weight; a round is sized so that
//     its sum of |d_a d_b| <= 2^24, so the FP32 accumulator holds the exact
//     integer.  Epilogue warps read each round from TMEM, convert to int64 and
//     add it (shifted by the round weight) into 64-bit fixed-point registers;
//     the only FP64 work is the final int64 -> double and the 2^(e_i + e_j)
//     scale.
// Complex: op(A)_cat = [Re op(A) | Im op(A)], op(B)_cat = [[Re, Im], [-Im, Re]]
// so one real product of size m x 2n x 2k gives [Cr | Ci] (the four real
// products of Complex128.mult, src/main/java/org/flag4j/numbers/Complex128.java:336-341).
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "f4j_internal.cuh"
#include "f4j_ptx.cuh"

namespace {

constexpr int S_MAX = 12;          // at most 12 slices: F = 4 + 55 = 59 bits keeps Y < 2^62 in int64
constexpr int BM = 128, BN = 128;  // output tile
constexpr int BKB = 64;            // K bytes per tile load (one 64-byte swizzle row; two K = 32 MMAs)
// Ring geometry (compile-time): operand tiles per stage (2w + band - 1 for w
// A slices per group) and stages in the shared-memory ring.
#ifndef F4J_SPLIT_STAGE_TILES
#define F4J_SPLIT_STAGE_TILES 9
#endif
#ifndef F4J_SPLIT_NSTAGE
#define F4J_SPLIT_NSTAGE 3
#endif
constexpr int STAGE_TILES = F4J_SPLIT_STAGE_TILES;
constexpr int NSTAGE = F4J_SPLIT_NSTAGE;
constexpr int RING = STAGE_TILES * NSTAGE;
constexpr int NBUF = 4;            // TMEM accumulator buffers of BN columns (= levels per band)
constexpr int TILE_BYTES = BM * BKB;  // 8 KB per operand tile
static_assert(BKB == 64, "umma_f8_k64 issues the two K = 32 steps of one 64-byte K block");
// Epilogue warps (compile-time, 8 or 16): each owns one TMEM lane quarter and
// BN / (EPI_WARPS / 4) columns of the tile.
#ifndef F4J_SPLIT_EPI_WARPS
#define F4J_SPLIT_EPI_WARPS 8
#endif
constexpr int EPI_WARPS = F4J_SPLIT_EPI_WARPS;
static_assert(EPI_WARPS == 8 || EPI_WARPS == 16, "8 or 16 epilogue warps");
constexpr int EPI_COLS = BN / (EPI_WARPS / 4);
constexpr int GEMM_THREADS = 64 + 32 * EPI_WARPS;  // warp 0 TMA, warp 1 MMA, warps 2.. epilogue
constexpr int MAX_ROUNDS = 16, MAX_GROUPS = 64, MAX_LOADS = 512, MAX_OPS = 96;

// One round: the products A_i B_j of weight level t = i + j over one K chunk,
// accumulated in one TMEM buffer.
struct Round {
    uint8_t level;   // t = i + j
    uint8_t i0, i1;  // A slices i0..i1-1 (1-based), B slice t - i
    int8_t shift;    // left shift of this round's integer into the fixed-point accumulator
    uint8_t buf;     // TMEM buffer: level - t0 of its band
    uint8_t pad[3];
};

// A band is up to NBUF adjacent levels t0..t1, level t in TMEM buffer t - t0
// (columns (t - t0) * BN ...).  Its products are computed by groups, one per
// chunk of w consecutive A slices i: per K block a group loads A_i for its i
// and every B_j with t0 <= i + j <= t1 (one ring stage of at most STAGE_TILES
// tiles, B tiles in ascending j) and issues each of those products into its
// level's buffer, so a loaded tile feeds up to NBUF products.  Two products
// A_i B_j, A_i B_{j+1} of an even and the next odd buffer run as one N = 256
// MMA: B_j and B_{j+1} are adjacent in shared memory and their buffers
// adjacent in TMEM.  Consecutive groups of a band keep accumulating into the
// same buffers, which the epilogue zeroes after reading them.
struct Load {
    uint8_t which;  // 0: A slice tile, 1: B slice tile
    uint8_t slice;  // 0-based slice plane
};
struct Op {
    uint32_t a_off, b_off;  // A / B tile offsets in the stage, in 16-byte units (descriptor address field)
    uint32_t dcol;          // TMEM column of the first product's buffer
    uint32_t idesc;         // instruction descriptor: N = 256 (B tiles b, b+1 into buffers dcol / BN and
                            // the next) or N = 128
};
struct Group {
    int16_t r0, nr;        // rounds [r0, r0 + nr)
    int16_t load0, nload;  // load list (per K block)
    int16_t op0, nop;      // MMA list (per K block)
    int32_t flags;         // GF_CONT_IN: keeps accumulating into the previous group's
                           // buffers; GF_CONT_OUT: its rounds continue in the next group;
                           // bits 8-11: buffers first used in the band by this group (the
                           // epilogue must have drained them before its MMAs); bits 12-15:
                           // buffers last used in the band by this group (complete after it)
};
constexpr int GF_CONT_IN = 1, GF_CONT_OUT = 2, GF_ACQ_SHIFT = 8, GF_REL_SHIFT = 12;

// Decided on the device from the exponent statistics (k_plan), so a split
// GEMM never waits for the host between its kernels.  The group / round
// program covers one K chunk; the slice GEMM runs it once per chunk.
struct SplitPlan {
    int s;          // slices per operand
    int nrounds;    // rounds per K chunk
    int ubits;      // fixed-point unit exponent: value = acc * 2^(ubits + ea + eb)
    int nonfinite;  // a NaN/Inf was seen (or no plan fits): the split stands down
    float spread;   // measured exponent spread (bits)
    int ngroups;    // groups per K chunk
    int nkb;        // K blocks of BKB bytes
    int kcb;        // K blocks per chunk
    Round rounds[MAX_ROUNDS];
    Group groups[MAX_GROUPS];
    Load loads[MAX_LOADS];
    Op ops[MAX_OPS];
};

struct SplitGemmParams {
    int M, N, Kp;           // cat sizes; Kp multiple of BKB
    int cplx;               // 1: C interleaved complex, N = 2n
    int n_out;              // n (complex output columns) or N
    const int* ea;          // [M]
    const int* eb;          // [N]
    double* C;
    int* status;
    const SplitPlan* plan;
    int tm0, tm1;           // the launch covers tile rows [tm0, tm1) of C
    int tn0, tn1;           // and tile columns [tn0, tn1)
    long long* wpart;       // split K: per-chunk int64 sums [nchunks][M][N] (null: whole tiles)
};

// ------------------------------------------------------------------ stats
__device__ __forceinline__ void stat_elem(double x, unsigned long long& mx, long long& esum, int& cnt, int& bad) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
    int E = (int)(b >> 52);
    if (E == 2047) bad = 1;
    if (b > mx) mx = b;
    if (b) {
        esum += (E ? E : 1) - 1023;
        cnt++;
    }
}

// One warp per stored row: stats of stored rows (block blk covers rows 8 blk .. 8 blk + 7).
__device__ __forceinline__ void stats_rows_body(const double* __restrict__ X, int64_t rows, int64_t cols, int cplx,
                                                int64_t blk, unsigned long long* __restrict__ mx_out,
                                                long long* __restrict__ esum_out, int* __restrict__ cnt_out,
                                                int* __restrict__ bad_out) {
    int64_t r = blk * (blockDim.x / 32) + threadIdx.x / 32;
    int lane = threadIdx.x % 32;
    if (r >= rows) return;
    unsigned long long mx = 0;
    long long es = 0;
    int cnt = 0, bad = 0;
    int64_t w = cplx ? 2 * cols : cols;
    const double* row = X + r * w;
    for (int64_t c = lane; c < w; c += 32) stat_elem(row[c], mx, es, cnt, bad);
    for (int off = 16; off; off >>= 1) {
        unsigned long long o = __shfl_xor_sync(0xffffffffu, mx, off);
        mx = o > mx ? o : mx;
        es += __shfl_xor_sync(0xffffffffu, es, off);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
        bad |= __shfl_xor_sync(0xffffffffu, bad, off);
    }
    if (lane == 0) {
        mx_out[r] = mx;
        esum_out[r] = es;
        cnt_out[r] = cnt;
        if (bad) atomicExch(bad_out, 1);
    }
}

__global__ void k_stats_rows(const double* __restrict__ X, int64_t rows, int64_t cols, int cplx,
                             unsigned long long* __restrict__ mx_out, long long* __restrict__ esum_out,
                             int* __restrict__ cnt_out, int* __restrict__ bad_out) {
    stats_rows_body(X, rows, cols, cplx, blockIdx.x, mx_out, esum_out, cnt_out, bad_out);
}

// Thread per stored column, block (bx, by) over chunks of `chunk` rows: stats
// of stored columns (cols of them, rows ld elements apart).
__device__ __forceinline__ void stats_cols_body(const double* __restrict__ X, int64_t rows, int64_t cols, int64_t ld,
                                                int cplx, int chunk, int64_t bx, int64_t by,
                                                unsigned long long* __restrict__ mx_out,
                                                long long* __restrict__ esum_out, int* __restrict__ cnt_out,
                                                int* __restrict__ bad_out) {
    int64_t c = bx * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    int64_t r0 = by * chunk, r1 = r0 + chunk < rows ? r0 + chunk : rows;
    unsigned long long mx = 0;
    long long es = 0;
    int cnt = 0, bad = 0;
    for (int64_t r = r0; r < r1; r++) {
        if (cplx) {
            stat_elem(X[2 * (r * ld + c)], mx, es, cnt, bad);
            stat_elem(X[2 * (r * ld + c) + 1], mx, es, cnt, bad);
        } else {
            stat_elem(X[r * ld + c], mx, es, cnt, bad);
        }
    }
    if (mx) atomicMax(&mx_out[c], mx);
    if (cnt) {
        atomicAdd((unsigned long long*)&esum_out[c], (unsigned long long)es);
        atomicAdd(&cnt_out[c], cnt);
    }
    if (bad) atomicExch(bad_out, 1);
}

__global__ void k_stats_cols(const double* __restrict__ X, int64_t rows, int64_t cols, int64_t ld, int cplx,
                             int chunk, unsigned long long* __restrict__ mx_out, long long* __restrict__ esum_out,
                             int* __restrict__ cnt_out, int* __restrict__ bad_out) {
    stats_cols_body(X, rows, cols, ld, cplx, chunk, blockIdx.x, blockIdx.y, mx_out, esum_out, cnt_out, bad_out);
}

// Exponent bound e (max|x| < 2^e) of target t, and its spread (x256).
__device__ __forceinline__ int finalize_target(int64_t t, int64_t targets, int dup,
                                               const unsigned long long* __restrict__ mx,
                                               const long long* __restrict__ esum, const int* __restrict__ cnt,
                                               int* __restrict__ e_out) {
    int sp = 0;
    if (t < targets) {
        unsigned long long b = mx[t];
        int e = 0;
        if (b) {
            // max|x| < 2^e, tight: for a subnormal maximum (E = 0) from its
            // highest mantissa bit, so a row of subnormals keeps all its bits
            // in the fixed-point form instead of being rounded at 2^(-1022 - F)
            int E = (int)(b >> 52);
            e = E ? E - 1022 : (63 - __clzll((long long)b)) - 1073;
            double mean = (double)esum[t] / (double)cnt[t];
            double s = (double)(e - 1) - mean;
            sp = s > 0 ? (int)(s * 256.0 + 0.5) : 0;
        }
        e_out[t] = e;
        if (dup) e_out[t + targets] = e;
    }
    for (int off = 16; off; off >>= 1) {
        int o = __shfl_xor_sync(0xffffffffu, sp, off);
        sp = o > sp ? o : sp;
    }
    return sp;
}

// Exponent bound e (max|x| < 2^e) per target, spread (x256, max-reduced).
__global__ void k_stats_finalize(int64_t targets, int dup, const unsigned long long* __restrict__ mx,
                                 const long long* __restrict__ esum, const int* __restrict__ cnt,
                                 int* __restrict__ e_out, int* __restrict__ spread_x256) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int sp = finalize_target(t, targets, dup, mx, esum, cnt, e_out);
    if ((threadIdx.x & 31) == 0 && sp) atomicMax(spread_x256, sp);
}

// ------------------------------------------------------------------ plan
// Slice count from the measured exponent spreads sa, sb of op(A)'s rows and
// op(B)'s columns (bits between the largest element exponent and the mean
// exponent, maximised over rows / columns) and the length k of the sums (2k
// for a complex product's concatenated K).  Error model, fitted on GB300 to
// the largest sampled error |C - C_true| / sum|a||b| (double-double truth) of
// split products with F = 4 + 5(s - 1) fraction bits:
//   err(F) ~ 2.2e-16 * 2^(49 - F) * 2^(0.81 (sa + sb - 2.12)) * (k / 8192)^-0.36
// (uniform and N(0,1) operands, k from 256 to 65536, s from 8 to 11; the
// dropped slice products of level s + 2 dominate it).  The plain FP64 DMMA
// product's error on the same scale measured 3.2e-16 .. 4.8e-16 over the same
// range; s is the smallest count whose modelled error is at most 0.8 x 3.2e-16:
//   F >= 51.74 + 0.81 (sa + sb) - 0.36 log2 k.
// A second floor, F >= 54 + max(sa, sb) - floor(log2 k), keeps short sums
// within the componentwise bound 2 k u |A||B|.
__host__ __device__ inline int slices_for(double sa, double sb, int64_t k, int64_t klen) {
    sa = sa > 0 ? sa : 0.0;
    sb = sb > 0 ? sb : 0.0;
    int lk = 0;
    while (lk < 62 && (2ll << lk) <= k) lk++;  // floor(log2 k)
    const double lklen = log2((double)(klen > 1 ? klen : 1));
    const double need = fmax(51.74 + 0.81 * (sa + sb) - 0.36 * lklen, 54.0 + fmax(sa, sb) - (double)lk);
    int s = 1 + (int)ceil((need - 4.0) / 5.0);
    return s < 2 ? 2 : (s > S_MAX ? S_MAX : s);
}

// Round program: a round accumulates the pairs of one level over one K chunk
// in FP32, exact as long as pairs * kchunk * 16 * 16 <= 2^24; a level has at
// most s pairs, so the chunk is the largest power-of-two number of K blocks
// with s * kchunk * 256 <= 2^24.  The fixed-point unit keeps the worst-case
// accumulator below 2^62.  Levels 2..s+1 are cut into bands of `band`
// (<= NBUF) levels, the lowest band taking the remainder; each band's A-slice range is cut into chunks of
// w = (STAGE_TILES - band + 1) / 2 slices, one group each, so a group loads
// at most 2w + band - 1 <= STAGE_TILES tiles per K block.  Returns the
// number of rounds per chunk, or -1 if a table would overflow.  kcb_cap > 0
// bounds the chunk (split K for products with few output tiles).
__host__ __device__ inline int plan_build(int s, int64_t Kp, int64_t klen_cat, SplitPlan* P, int band = NBUF,
                                          int kcb_cap = 0) {
    if (band < 1) band = 1;
    if (band > NBUF) band = NBUF;
    const int w = (STAGE_TILES - band + 1) / 2;
    const int64_t nkb = Kp / BKB;
    int64_t kcb = 1;
    while (2 * kcb <= nkb && (int64_t)s * (2 * kcb) * BKB * 256 <= (1ll << 24) && (kcb_cap <= 0 || 2 * kcb <= kcb_cap))
        kcb *= 2;
    P->nkb = (int)nkb;
    P->kcb = (int)kcb;
    int kbits = 0;
    while (kbits < 62 && (1ll << kbits) < (klen_cat > 0 ? klen_cat : 1)) kbits++;  // ceil(log2 k)
    int D = kbits + 9 + 5 * (s - 1) - 62;
    if (D < 0) D = 0;
    P->ubits = -(8 + 5 * (s - 1)) + D;
    int nr = 0, ng = 0, nl = 0, no = 0;
    // the lowest band takes the remainder (low levels have the fewest
    // products); bands run from the highest levels down, so a tile starts
    // with its longest band and the epilogue's final stores of the previous
    // tile overlap that band's MMAs
    const int first = s % band ? s % band : band;
    const int nbands = 1 + (s - first) / band;
    for (int bi = nbands - 1; bi >= 0; bi--) {
        const int t0 = bi == 0 ? 2 : 2 + first + (bi - 1) * band;
        const int t1 = bi == 0 ? 1 + first : t0 + band - 1;
        if (nr + (t1 - t0 + 1) > MAX_ROUNDS) return -1;
        const int r0 = nr;
        for (int t = t0; t <= t1; t++) {
            Round rd;
            rd.level = (uint8_t)t;
            rd.i0 = (uint8_t)(t - s > 1 ? t - s : 1);
            rd.i1 = (uint8_t)((t - 1 < s ? t - 1 : s) + 1);
            rd.shift = (int8_t)(5 * (s + 1 - t) - D);
            rd.buf = (uint8_t)(t - t0);
            rd.pad[0] = rd.pad[1] = rd.pad[2] = 0;
            P->rounds[nr++] = rd;
        }
        // A slices with a partner in the band
        const int ilo = t0 - s > 1 ? t0 - s : 1, ihi = t1 - 1 < s ? t1 - 1 : s;
        const int gband = ng;  // the band's first group
        for (int c0 = ilo; c0 <= ihi; c0 += w) {
            const int c1 = c0 + w - 1 < ihi ? c0 + w - 1 : ihi;
            const int jlo = t0 - c1 > 1 ? t0 - c1 : 1, jhi = t1 - c0 < s ? t1 - c0 : s;
            const int na = c1 - c0 + 1, nb = jhi - jlo + 1;
            if (ng >= MAX_GROUPS || nl + na + nb > MAX_LOADS || no + na * (t1 - t0 + 1) > MAX_OPS) return -1;
            if (na + nb > STAGE_TILES) return -1;
            Group g;
            g.r0 = (int16_t)r0;
            g.nr = (int16_t)(t1 - t0 + 1);
            g.load0 = (int16_t)nl;
            g.nload = (int16_t)(na + nb);
            g.op0 = (int16_t)no;
            g.flags = (c0 > ilo ? GF_CONT_IN : 0) | (c1 < ihi ? GF_CONT_OUT : 0);
            for (int i = c0; i <= c1; i++) {
                P->loads[nl].which = 0;
                P->loads[nl].slice = (uint8_t)(i - 1);
                nl++;
            }
            for (int j = jlo; j <= jhi; j++) {
                P->loads[nl].which = 1;
                P->loads[nl].slice = (uint8_t)(j - 1);
                nl++;
            }
            for (int i = c0; i <= c1; i++) {
                // levels of this i with a B partner: t in [ta, tb]
                const int ta = i + 1 > t0 ? i + 1 : t0, tb = i + s < t1 ? i + s : t1;
                for (int t = ta; t <= tb;) {
                    const bool wide = ((t - t0) % 2 == 0) && t + 1 <= tb;
                    if (no >= MAX_OPS) return -1;
                    Op op;
                    op.a_off = (uint32_t)((i - c0) * (TILE_BYTES >> 4));
                    op.b_off = (uint32_t)((na + (t - i) - jlo) * (TILE_BYTES >> 4));
                    op.dcol = (uint32_t)((t - t0) * BN);
                    op.idesc = umma_idesc_e4m3_f32(BM, wide ? 2 * BN : BN);
                    P->ops[no++] = op;
                    t += wide ? 2 : 1;
                }
            }
            g.nop = (int16_t)(no - g.op0);
            P->groups[ng++] = g;
        }
        // each buffer is acquired by the first group of the band that uses it and
        // released by the last one (a buffer no group uses: first / last group)
        const uint32_t all = (1u << (t1 - t0 + 1)) - 1u;
        uint32_t seen = 0, later = 0;
        for (int q = gband; q < ng; q++) {
            uint32_t m = 0;
            for (int o = P->groups[q].op0; o < P->groups[q].op0 + P->groups[q].nop; o++)
                m |= (P->ops[o].idesc == umma_idesc_e4m3_f32(BM, 2 * BN) ? 3u : 1u) << (P->ops[o].dcol / BN);
            P->groups[q].flags |= (int32_t)((m & ~seen) << GF_ACQ_SHIFT);
            seen |= m;
            P->groups[q].flags |= (int32_t)(m << 16);  // scratch: this group's use mask
        }
        for (int q = ng - 1; q >= gband; q--) {
            const uint32_t m = ((uint32_t)P->groups[q].flags >> 16) & 15u;
            P->groups[q].flags &= 0xFFFF;
            P->groups[q].flags |= (int32_t)((m & ~later) << GF_REL_SHIFT);
            later |= m;
        }
        P->groups[gband].flags |= (int32_t)((all & ~seen) << GF_ACQ_SHIFT);
        P->groups[ng - 1].flags |= (int32_t)((all & ~seen) << GF_REL_SHIFT);
    }
    P->ngroups = ng;
    return nr;
}

// One thread: slice count and the group / round / MMA program from the
// statistics.  misc: [0] non-finite flag, [1] spread of A x256, [2] of B.
__global__ void k_plan(const int* __restrict__ misc, int64_t k, int64_t Kp, int64_t klen_cat, int s_req,
                       int band, int kcb_cap, SplitPlan* __restrict__ plan) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double spread = (misc[1] > misc[2] ? misc[1] : misc[2]) / 256.0;
    int s = s_req > 0 ? (s_req > S_MAX ? S_MAX : (s_req < 2 ? 2 : s_req))
                      : slices_for(misc[1] / 256.0, misc[2] / 256.0, k, klen_cat);
    int n = plan_build(s, Kp, klen_cat, plan, band, kcb_cap);
    plan->s = s;
    plan->nrounds = n < 0 ? 0 : n;
    plan->spread = (float)spread;
    // a plan that does not fit is treated like a non-finite input (plain path)
    plan->nonfinite = (misc[0] != 0 || n < 0) ? 1 : 0;
}

// The plan of every slice count s = 2..S_MAX (block s - 2, one thread each):
// tab[s] for a context's plan table.  nrounds < 0 marks a plan that does not fit.
__global__ void k_plan_table(int64_t Kp, int64_t klen_cat, int band, int kcb_cap, SplitPlan* __restrict__ tab) {
    if (threadIdx.x != 0) return;
    const int s = 2 + (int)blockIdx.x;
    SplitPlan* P = &tab[s];
    const int n = plan_build(s, Kp, klen_cat, P, band, kcb_cap);
    P->s = s;
    P->nrounds = n;
}

// One block of 128 threads: k_plan's result from a plan table (the slice count
// from the statistics, that plan copied, the header filled in).
__global__ void k_plan_pick(const int* __restrict__ misc, int64_t k, int64_t klen_cat, int s_req,
                            const SplitPlan* __restrict__ tab, SplitPlan* __restrict__ plan) {
    if (blockIdx.x != 0) return;
    const double spread = (misc[1] > misc[2] ? misc[1] : misc[2]) / 256.0;
    const int s = s_req > 0 ? (s_req > S_MAX ? S_MAX : (s_req < 2 ? 2 : s_req))
                            : slices_for(misc[1] / 256.0, misc[2] / 256.0, k, klen_cat);
    const uint4* src = reinterpret_cast<const uint4*>(&tab[s]);
    uint4* dst = reinterpret_cast<uint4*>(plan);
#pragma unroll 4
    for (int i = threadIdx.x; i < (int)(sizeof(SplitPlan) / 16); i += blockDim.x) dst[i] = src[i];
    __syncthreads();
    if (threadIdx.x == 0) {
        const int n = tab[s].nrounds;
        plan->s = s;
        plan->nrounds = n < 0 ? 0 : n;
        plan->spread = (float)spread;
        plan->nonfinite = (misc[0] != 0 || n < 0) ? 1 : 0;
    }
}

// Both operands' exponent bounds and spreads, then the plan, in one launch:
// blocks [0, cdiv(ta, 256)) finalise op(A)'s targets, the rest op(B)'s (dupb:
// the complex B_cat's targets appear twice).  Each block counts itself done
// on misc[4] (zeroed with misc before the statistics); the block that counts
// last has seen every spread and picks the plan as k_plan_pick does.  No
// block waits for another.
__global__ void __launch_bounds__(256) k_finalize_pick(int64_t ta, int64_t tb, int dupb,
                                                       const unsigned long long* __restrict__ mxa,
                                                       const long long* __restrict__ esa,
                                                       const int* __restrict__ cna,
                                                       const unsigned long long* __restrict__ mxb,
                                                       const long long* __restrict__ esb,
                                                       const int* __restrict__ cnb, int* __restrict__ ea,
                                                       int* __restrict__ eb, int* misc, int64_t k,
                                                       int64_t klen_cat, int s_req,
                                                       const SplitPlan* __restrict__ tab,
                                                       SplitPlan* __restrict__ plan) {
    const int64_t nba = (ta + 255) / 256;
    const bool is_b = (int64_t)blockIdx.x >= nba;
    const int64_t t = ((int64_t)blockIdx.x - (is_b ? nba : 0)) * 256 + threadIdx.x;
    const int sp = is_b ? finalize_target(t, tb, dupb, mxb, esb, cnb, eb)
                        : finalize_target(t, ta, 0, mxa, esa, cna, ea);
    if ((threadIdx.x & 31) == 0 && sp) atomicMax(&misc[is_b ? 2 : 1], sp);
    __shared__ int last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(&misc[4], 1) == (int)gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // every block's spreads are in; read them past L1
    const int sa = atomicAdd(&misc[1], 0), sb = atomicAdd(&misc[2], 0), bad = atomicAdd(&misc[0], 0);
    const double spread = (sa > sb ? sa : sb) / 256.0;
    const int s = s_req > 0 ? (s_req > S_MAX ? S_MAX : (s_req < 2 ? 2 : s_req))
                            : slices_for(sa / 256.0, sb / 256.0, k, klen_cat);
    const uint4* src = reinterpret_cast<const uint4*>(&tab[s]);
    uint4* dst = reinterpret_cast<uint4*>(plan);
    for (int i = threadIdx.x; i < (int)(sizeof(SplitPlan) / 16); i += blockDim.x) dst[i] = src[i];
    __syncthreads();
    if (threadIdx.x == 0) {
        const int n = tab[s].nrounds;
        plan->s = s;
        plan->nrounds = n < 0 ? 0 : n;
        plan->spread = (float)spread;
        plan->nonfinite = (bad != 0 || n < 0) ? 1 : 0;
    }
}

// One thread, after every statistic of both operands is in: misc[5] = 1 when
// the slice count those statistics give differs from the one `plan` was
// picked with (from part of op(A)), or an operand holds a NaN / Inf, or the
// plan stood down; 0 when the product sliced with `plan` is the one k_plan
// would have planned.
__global__ void k_spec_check(int* __restrict__ misc, int64_t k, int64_t klen_cat, int s_req,
                             const SplitPlan* __restrict__ plan) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int s = s_req > 0 ? (s_req > S_MAX ? S_MAX : (s_req < 2 ? 2 : s_req))
                            : slices_for(misc[1] / 256.0, misc[2] / 256.0, k, klen_cat);
    misc[5] = (s != plan->s || misc[0] != 0 || plan->nonfinite) ? 1 : 0;
}

// ------------------------------------------------------------------ split

// Exact float of an integer |d| < 2^22: d added to the bit pattern of 1.5 * 2^23.
__device__ __forceinline__ float float_of_small_int(int d) {
    return __int_as_float(0x4B400000 + d) - 12582912.0f;
}

// Eight small integers (exact in E4M3) as E4M3 bytes, stored as 8 bytes.
__device__ __forceinline__ void store_e4m3x8(uint8_t* dst, const float (&f)[8]) {
    uint32_t w[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
        uint16_t h;
        // the first source operand goes to the upper byte
        asm("cvt.rn.satfinite.e4m3x2.f32 %0, %1, %2;" : "=h"(h) : "f"(f[2 * u + 1]), "f"(f[2 * u]));
        w[u] = h;
    }
    *reinterpret_cast<uint2*>(dst) = make_uint2(w[0] | (w[1] << 16), w[2] | (w[3] << 16));
}

// Fixed-point integer of x relative to 2^e with F fractional bits:
// round(|x| 2^(F - e)) with the sign of x; |result| <= 2^F.
__device__ __forceinline__ long long fixed_of(double x, int e, int F) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    bool neg = b >> 63;
    int E = (int)((b >> 52) & 0x7FF);
    unsigned long long M = b & 0xFFFFFFFFFFFFFull;
    if (E) M |= 1ull << 52;
    else E = 1;
    int sh = (E - 1075) - e + F;
    unsigned long long Y;
    if (M == 0) Y = 0;
    else if (sh >= 0) Y = M << sh;
    else if (sh <= -64) Y = 0;
    else {
        int rs = -sh;
        Y = (rs >= 54) ? 0 : ((M + (1ull << (rs - 1))) >> rs);
    }
    return neg ? -(long long)Y : (long long)Y;
}

// The s balanced base-32 digits of eight fixed-point integers Y = H 2^30 + L
// (0 <= L < 2^30) as E4M3 bytes: digit p (0 = most significant) of element j
// to base[p * plane + j].
__device__ __forceinline__ void store_digits8(int (&L)[8], int (&H)[8], int s, uint8_t* base, int64_t plane) {
    // balanced base-32 digits from the least significant slice (p = s - 1) up
#pragma unroll
    for (int c = 0; c < S_MAX - 1; c++) {
        if (c >= s - 1) break;
        float f[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            // with t = x + 16 the balanced digit is (t & 31) - 16 and the
            // rest (x - digit) / 32 is t >> 5; the -16 is folded into the
            // float conversion's constant
            int t;
            if (c < 6) {
                t = L[j] + 16;
                L[j] = t >> 5;
                if (c == 5) H[j] += L[j];  // carry out of the low 30 bits: 0 or 1
            } else {
                t = H[j] + 16;
                H[j] = t >> 5;
            }
            f[j] = float_of_small_int((t & 31) - 16);
        }
        store_e4m3x8(base + (int64_t)(s - 1 - c) * plane, f);
    }
    // the most significant digit is what remains
    float f[8];
#pragma unroll
    for (int j = 0; j < 8; j++)
        f[j] = float_of_small_int(s - 1 < 6 ? L[j] + H[j] * (1 << (30 - 5 * (s - 1))) : H[j]);
    store_e4m3x8(base, f);
}

constexpr int SP_TR = 32, SP_TQ = 64;  // tile: 32 target rows x 64 k-indices

// Writes slices of one operand.  Output plane p (0-based slice) is
// rows_out x Kp bytes at out + p * rows_out * Kp.
//   transposed == 0: target row r = stored row, q = stored column
//   transposed == 1: target row r = stored column, q = stored row
//   role 0 (A_cat): complex value (re, im) -> out[r][q] = re, out[r][Kh+q] = im
//   role 1 (B_cat^T): -> out[r][q] = re, out[r][Kh+q] = -im,
//                        out[n+r][q] = im, out[n+r][Kh+q] = re
// CPLX is the operand's kind (the imaginary parts' staging exists only then).
template <bool CPLX>
__device__ __forceinline__ void split_body(const double* __restrict__ X, int64_t srows, int64_t scols,
                                           int transposed, int conj, int role, int64_t targets,
                                           int64_t klen, int64_t Kh, int64_t Kp, int64_t rows_out,
                                           const int* __restrict__ e_t, const SplitPlan* __restrict__ plan,
                                           uint8_t* __restrict__ out, int64_t bx, int by0, int by_step) {
    __shared__ double sre[SP_TR][SP_TQ + 1];
    __shared__ double sim[CPLX ? SP_TR : 1][SP_TQ + 1];
    if (plan->nonfinite) return;  // the same for every thread of the block
    const int s = plan->s;
    const int64_t q0 = bx * SP_TQ;
    // tile rows by0, by0 + by_step, ... (more than grid.y's limit of 65535
    // when there are over 2 M targets): the bound is the same for the whole
    // block, and every thread meets both barriers of every tile
    for (int by = by0; (int64_t)by * SP_TR < targets; by += by_step) {
        const int64_t r0 = (int64_t)by * SP_TR;
        // ---- stage the tile (zeros outside the matrix)
        for (int e = threadIdx.x; e < SP_TR * SP_TQ; e += 256) {
            int rr, qq;
            if (!transposed) { rr = e / SP_TQ; qq = e % SP_TQ; }
            else { qq = e / SP_TR; rr = e % SP_TR; }
            int64_t r = r0 + rr, q = q0 + qq;
            double re = 0, im = 0;
            if (r < targets && q < klen) {
                int64_t idx = transposed ? (q * scols + r) : (r * scols + q);
                if constexpr (CPLX) {
                    re = X[2 * idx];
                    im = X[2 * idx + 1];
                    if (conj) im = -im;
                } else {
                    re = X[idx];
                }
            }
            sre[rr][qq] = re;
            if constexpr (CPLX) sim[rr][qq] = im;
        }
        __syncthreads();
        // ---- each thread: one target row, 8 consecutive q
        const int rr = threadIdx.x / 8, qs = (threadIdx.x % 8) * 8;
        const int64_t r = r0 + rr;
        if (r < targets) {
            const int e = e_t[r];
            const int F = 4 + 5 * (s - 1);
            const int nparts = CPLX ? (role == 0 ? 2 : 4) : 1;
            for (int part = 0; part < nparts; part++) {
                // part: 0 -> (row r, col q) ; 1 -> (row r, col Kh+q) ; 2 -> (row n+r, col q) ; 3 -> (row n+r, col Kh+q)
                // Y = H * 2^30 + L with 0 <= L < 2^30: the low six digits come from L,
                // the rest from H (plus the carry out of L), all in 32-bit arithmetic
                int L[8], H[8];
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    double v;
                    const double a = sre[rr][qs + j];
                    double b = 0.0;
                    if constexpr (CPLX) b = sim[rr][qs + j];
                    if (role == 0) v = (part == 0) ? a : b;
                    else v = (part == 0) ? a : (part == 1) ? -b : (part == 2) ? b : a;
                    const long long y = fixed_of(v, e, F);
                    L[j] = (int)(y & 0x3FFFFFFFll);
                    H[j] = (int)(y >> 30);
                }
                const int64_t orow = (part >= 2) ? (targets + r) : r;
                const int64_t ocol = ((part & 1) ? Kh : 0) + q0 + qs;
                store_digits8(L, H, s, out + orow * Kp + ocol, rows_out * Kp);
            }
        }
        __syncthreads();  // the next tile's staging overwrites sre / sim
    }
}

// k_split's body for real targets stored as rows (transposed = 0), without
// staging: thread (rr, qs) of the 32 x 64 tile reads its 8 consecutive
// elements of row r0 + rr straight from global memory (the 8 threads of a row
// together read its 512 contiguous bytes) and writes the same bytes the
// staged body does.
__device__ __forceinline__ void split_rows_body(const double* __restrict__ X, int64_t scols, int64_t targets,
                                                int64_t klen, int64_t Kp, int64_t rows_out,
                                                const int* __restrict__ e_t, const SplitPlan* __restrict__ plan,
                                                uint8_t* __restrict__ out, int64_t bx, int by0, int by_step) {
    if (plan->nonfinite) return;
    const int s = plan->s;
    const int64_t q0 = bx * SP_TQ + (threadIdx.x % 8) * 8;
    for (int by = by0; (int64_t)by * SP_TR < targets; by += by_step) {  // tile rows, as in split_body
        const int64_t r = (int64_t)by * SP_TR + threadIdx.x / 8;
        if (r >= targets) continue;
        const double* row = X + r * scols;
        const int e = e_t[r];
        const int F = 4 + 5 * (s - 1);
        int L[8], H[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const double v = q0 + j < klen ? __ldg(row + q0 + j) : 0.0;
            const long long y = fixed_of(v, e, F);
            L[j] = (int)(y & 0x3FFFFFFFll);
            H[j] = (int)(y >> 30);
        }
        store_digits8(L, H, s, out + r * Kp + q0, rows_out * Kp);
    }
}

// Real operands: 17 KB of staging and at most 32 registers, so 8 blocks (64
// warps) fit an SM and hide the staging loads; complex: 34 KB and 60
// registers (tighter caps spill), 4 blocks.
template <bool CPLX>
__global__ void __launch_bounds__(256, CPLX ? 4 : 8) k_split(const double* __restrict__ X, int64_t srows,
                                                             int64_t scols, int transposed, int conj, int role,
                                                             int64_t targets, int64_t klen, int64_t Kh, int64_t Kp,
                                                             int64_t rows_out, const int* __restrict__ e_t,
                                                             const SplitPlan* __restrict__ plan,
                                                             uint8_t* __restrict__ out) {
    if (!CPLX && !transposed)
        split_rows_body(X, scols, targets, klen, Kp, rows_out, e_t, plan, out, blockIdx.x, blockIdx.y, gridDim.y);
    else
        split_body<CPLX>(X, srows, scols, transposed, conj, role, targets, klen, Kh, Kp, rows_out, e_t, plan, out,
                         blockIdx.x, blockIdx.y, gridDim.y);
}

// One operand of k_split_pair (the arguments k_split takes for it).
struct SplitOperand {
    const double* X;
    int64_t srows, scols;
    int transposed, conj, role;
    int64_t targets, rows_out;
    const int* e_t;
    uint8_t* out;
};

// Both operands' slice planes in one launch: blockIdx.z = 0 slices op(A), 1
// op(B)_cat^T; blocks past an operand's targets return at once.
template <bool CPLX>
__global__ void __launch_bounds__(256, CPLX ? 6 : 8) k_split_pair(const SplitOperand a, const SplitOperand b,
                                                                  int64_t klen, int64_t Kh, int64_t Kp,
                                                                  const SplitPlan* __restrict__ plan) {
    // one inlined copy of the body per operand, each reading its own kernel
    // parameters directly (selecting the operand first kept every field in
    // registers: 60 registers against 35, and fewer blocks per SM)
    if (blockIdx.z == 0) {
        if ((int64_t)blockIdx.y * SP_TR >= a.targets) return;
        if (!CPLX && !a.transposed)  // rows of a real operand: no staging
            split_rows_body(a.X, a.scols, a.targets, klen, Kp, a.rows_out, a.e_t, plan, a.out, blockIdx.x,
                            blockIdx.y, gridDim.y);
        else
            split_body<CPLX>(a.X, a.srows, a.scols, a.transposed, a.conj, a.role, a.targets, klen, Kh, Kp,
                             a.rows_out, a.e_t, plan, a.out, blockIdx.x, blockIdx.y, gridDim.y);
    } else {
        if ((int64_t)blockIdx.y * SP_TR >= b.targets) return;
        if (!CPLX && !b.transposed)  // rows of a real operand: no staging
            split_rows_body(b.X, b.scols, b.targets, klen, Kp, b.rows_out, b.e_t, plan, b.out, blockIdx.x,
                            blockIdx.y, gridDim.y);
        else
            split_body<CPLX>(b.X, b.srows, b.scols, b.transposed, b.conj, b.role, b.targets, klen, Kh, Kp,
                             b.rows_out, b.e_t, plan, b.out, blockIdx.x, blockIdx.y, gridDim.y);
    }
}

// ------------------------------------------------------------------ GEMM
// Development tracing (built only with -DF4J_TRACE): per-role cycle counts of
// the slice GEMM's barrier waits, summed over CTAs, read by f4j_debug_trace.
#ifdef F4J_TRACE
__device__ unsigned long long g_f4j_trace[8];
#define F4J_T_BEGIN() const long long f4j_t0 = clock64()
#define F4J_T_ADD(acc) (acc) += (unsigned long long)(clock64() - f4j_t0)
#else
#define F4J_T_BEGIN() ((void)0)
#define F4J_T_ADD(acc) ((void)0)
#endif

// v * 2^X without a libm call; two in-range factors when X leaves the normal range.
__device__ __forceinline__ double scale_pow2(double v, int X) {
    if (X >= -1022 && X <= 1023) return v * __longlong_as_double((long long)(X + 1023) << 52);
    int X1 = X / 2, X2 = X - X1;
    X1 = X1 < -1022 ? -1022 : (X1 > 1023 ? 1023 : X1);
    X2 = X2 < -1022 ? -1022 : (X2 > 1023 ? 1023 : X2);
    return (v * __longlong_as_double((long long)(X1 + 1023) << 52)) * __longlong_as_double((long long)(X2 + 1023) << 52);
}

// Output tile order: bands of TILE_GROUP_M tile rows, column-major inside a
// band, so the CTAs running at the same time (consecutive tile indices) form a
// TILE_GROUP_M x ~(grid / TILE_GROUP_M) block: each B slice tile they load is
// shared by up to TILE_GROUP_M of them in L2, each A slice tile by the rest.
#ifndef F4J_SPLIT_GROUP_M
#define F4J_SPLIT_GROUP_M 8
#endif
constexpr int TILE_GROUP_M = F4J_SPLIT_GROUP_M;
__device__ __forceinline__ void tile_origin(int tile, int tiles_m, int tiles_n, int& m0, int& n0) {
    const int per_group = TILE_GROUP_M * tiles_n;
    const int g = tile / per_group, first = g * TILE_GROUP_M;
    const int gm = tiles_m - first < TILE_GROUP_M ? tiles_m - first : TILE_GROUP_M;
    const int r = tile - g * per_group;
    m0 = (first + r % gm) * BM;
    n0 = (r / gm) * BN;
}

// One CTA per SM: the register file is shared by GEMM_THREADS threads.  With
// 8 epilogue warps (320 threads) three warps share two of the four SM
// sub-partitions, which caps a thread at 168 registers; the epilogue keeps 64
// int64 accumulators and reads TMEM 16 columns at a time to stay inside it.
// (16 epilogue warps cap a thread at 96 registers and measured 5 % slower.)
__global__ void __launch_bounds__(GEMM_THREADS, 1)
    k_split_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                 const __grid_constant__ SplitGemmParams p) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte alignment for the swizzled TMA tiles
    unsigned char* smem = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    unsigned char* sT = smem;  // RING operand tiles of 8 KB
    __shared__ __align__(8) uint64_t full[NSTAGE], empty[NSTAGE], accfull[NBUF], accempty[NBUF], mma_done;
    __shared__ uint32_t tmem_base_slot;
    __shared__ int abort_flag;

    const SplitPlan* __restrict__ plan = p.plan;
    if (plan->nonfinite) return;  // the gated plain path computes this product
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int nrounds = plan->nrounds;
    // persistent: CTA b takes tiles b, b + grid, ...; see tile_origin for the order
    const int tiles_n = p.tn1 - p.tn0, tiles_m = p.tm1 - p.tm0;
    const int ntiles = tiles_n * tiles_m;

    const int ngroups = plan->ngroups;
    if (threadIdx.x == 0) {
        for (int i = 0; i < NSTAGE; i++) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < NBUF; i++) {
            mbar_init(&accfull[i], 1);
            mbar_init(&accempty[i], EPI_WARPS);
        }
        mbar_init(&mma_done, 1);
        abort_flag = 0;
        fence_barrier_init();
    }
    if (warp == 1) {
        tmem_alloc(&tmem_base_slot, NBUF * BN);
        tmem_relinquish();
    }
    if (warp == 0 && lane == 0) {
        prefetch_tmap(&tmA);
        prefetch_tmap(&tmB);
    }
    // stage the plan (a few KB) in shared memory: the MMA-issuing thread
    // never waits on a global load between MMAs
    static_assert(sizeof(SplitPlan) % 16 == 0, "plan copied in 16-byte words");
    SplitPlan* sp = reinterpret_cast<SplitPlan*>(smem + RING * TILE_BYTES);
    for (int i = threadIdx.x; i < (int)(sizeof(SplitPlan) / 16); i += blockDim.x)
        reinterpret_cast<uint4*>(sp)[i] = reinterpret_cast<const uint4*>(plan)[i];
    const Group* gp = sp->groups;
    const Load* ldp = sp->loads;
    // per ring slot, the ops with absolute descriptor low words and TMEM addresses
    Op* opx = reinterpret_cast<Op*>(reinterpret_cast<unsigned char*>(sp) + sizeof(SplitPlan));
    const int nkb = plan->nkb, kcb = plan->kcb, nchunks = (nkb + kcb - 1) / kcb;
    // split K (p.wpart): a unit is one K chunk of one tile; else a whole tile
    const bool ksplit = p.wpart != nullptr;
    const int nunits = ksplit ? ntiles * nchunks : ntiles;
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_slot;
    {
        const int nops = ngroups > 0 ? gp[ngroups - 1].op0 + gp[ngroups - 1].nop : 0;
        const uint32_t lo0 = (uint32_t)umma_desc_sw64(sT);
        for (int i = threadIdx.x; i < NSTAGE * nops; i += blockDim.x) {
            const int st = i / nops, o = i % nops;
            const Op O = sp->ops[o];
            const uint32_t slot = lo0 + (uint32_t)(st * STAGE_TILES * (TILE_BYTES >> 4));
            opx[st * MAX_OPS + o] = Op{slot + O.a_off, slot + O.b_off, tmem + O.dcol, O.idesc};
        }
    }
    if (warp >= 2) {
        // every MMA accumulates: the buffers start at zero (and are zeroed
        // again by the epilogue after each read)
        const int q = warp % 4, h = (warp - 2) / 4;
#pragma unroll
        for (int b = 0; b < NBUF; b++)
#pragma unroll
            for (int c = 0; c < EPI_COLS; c += 32) tmem_zero32(tmem + ((uint32_t)(32 * q) << 16) + b * BN + h * EPI_COLS + c);
        tmem_st_wait();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();

    if (warp == 0) {
        // ---------------- TMA producer: one stage per K block of a group.  The
        // whole warp issues a stage: lane 0 waits for the slot and arms its
        // barrier, then lane l copies the stage's tile l (issuing the loads from
        // one thread was measured to limit the ring's fill rate).
        {
#ifdef F4J_TRACE
            unsigned long long tr_wait = 0;
            const long long tr_start = clock64();
#endif
            int st = 0;  // stages issued, carried across tiles
            bool ok = true;
            for (int u = blockIdx.x; u < nunits && ok; u += gridDim.x) {
                const int tile = ksplit ? u / nchunks : u;
                const int kc0 = ksplit ? (u % nchunks) * kcb : 0, kc1 = ksplit ? kc0 + kcb : nkb;
                int m0, n0;
                tile_origin(tile, tiles_m, tiles_n, m0, n0);
                m0 += p.tm0 * BM;
                n0 += p.tn0 * BN;
                for (int kc = kc0; kc < kc1 && kc < nkb && ok; kc += kcb) {
                    const int kend = kc + kcb < nkb ? kc + kcb : nkb;
                    for (int g = 0; g < ngroups && ok; g++) {
                        const Group G = gp[g];
                        // this lane's tile of every stage of the group
                        Load L{};
                        if (lane < G.nload) L = ldp[G.load0 + lane];
                        const CUtensorMap* map = L.which ? &tmB : &tmA;
                        const int row0 = L.which ? n0 : m0;
                        for (int kb = kc; kb < kend; kb++, st++) {
                            const int s = st % NSTAGE;
                            if (lane == 0) {
                                if (st >= NSTAGE) {
                                    F4J_T_BEGIN();
                                    ok = mbar_wait(&empty[s], ((st / NSTAGE) & 1) ^ 1, p.status, 11) &&
                                         !*(volatile int*)&abort_flag;
                                    F4J_T_ADD(tr_wait);
                                }
                                if (ok) mbar_arrive_expect_tx(&full[s], G.nload * TILE_BYTES);
                                else abort_flag = 1;
                            }
                            ok = __shfl_sync(0xffffffffu, ok, 0);
                            if (!ok) break;
                            if (lane < G.nload)
                                tma_load_3d(sT + (s * STAGE_TILES + lane) * TILE_BYTES, map, &full[s], kb * BKB, row0,
                                            L.slice);
                        }
                    }
                }
            }
#ifdef F4J_TRACE
            if (lane == 0) {
                atomicAdd(&g_f4j_trace[4], (unsigned long long)(clock64() - tr_start));
                atomicAdd(&g_f4j_trace[5], tr_wait);
            }
#endif
            // drain the copies still in flight (bounded)
            if (lane == 0)
                for (int q = st > NSTAGE ? st - NSTAGE : 0; q < st; q++)
                    mbar_wait(&full[q % NSTAGE], (q / NSTAGE) & 1, nullptr, 0);
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer (one thread)
        if (lane == 0) {
#ifdef F4J_TRACE
            unsigned long long tr_wait = 0, tr_acc = 0, tr_ops = 0;
            const long long tr_start = clock64();
#endif
            // smem descriptors differ only in the start-address field, the low 14
            // bits of the low word (shared memory < 256 KB, so the op tables'
            // precomputed low words never carry into the rest)
            const uint32_t desc_hi = (uint32_t)(umma_desc_sw64(sT) >> 32);
            int st = 0;             // stages consumed, carried across tiles
            uint32_t used = 0;      // bit b: buffer b has been filled before
            uint32_t drained = 0;   // bit b: parity of the next accempty[b] phase to wait for
            for (int u = blockIdx.x; u < nunits && !*(volatile int*)&abort_flag; u += gridDim.x) {
                const int kc0 = ksplit ? (u % nchunks) * kcb : 0, kc1 = ksplit ? kc0 + kcb : nkb;
                for (int kc = kc0; kc < kc1 && kc < nkb && !*(volatile int*)&abort_flag; kc += kcb) {
                    const int kend = kc + kcb < nkb ? kc + kcb : nkb;
                    for (int g = 0; g < ngroups && !*(volatile int*)&abort_flag; g++) {
                        const Group G = gp[g];
                        const uint32_t acq = ((uint32_t)G.flags >> GF_ACQ_SHIFT) & 15u;
                        const uint32_t rel = ((uint32_t)G.flags >> GF_REL_SHIFT) & 15u;
                        if (acq & used) {
                            // buffers this group is first in its band to use must have
                            // been read (and zeroed) by the epilogue
                            uint32_t wq = acq & used;
                            while (wq) {
                                const int b = __ffs(wq) - 1;
                                wq &= wq - 1;
                                F4J_T_BEGIN();
                                const bool okw = mbar_wait(&accempty[b], (drained >> b) & 1, p.status, 12);
                                F4J_T_ADD(tr_acc);
                                drained ^= 1u << b;
                                if (!okw) abort_flag = 1;
                            }
                            tc_fence_after();
                        }
                        const Op* ops = opx + G.op0;
                        for (int kb = kc; kb < kend; kb++, st++) {
                            const int s = st % NSTAGE;
                            F4J_T_BEGIN();
                            const bool okw = mbar_wait(&full[s], (st / NSTAGE) & 1, p.status, 13);
                            F4J_T_ADD(tr_wait);
                            if (!okw) {
                                abort_flag = 1;
                                break;
                            }
                            tc_fence_after();
                            const Op* so = ops + s * MAX_OPS;
#pragma unroll 2
                            for (int o = 0; o < G.nop; o++) {
                                const Op O = so[o];
                                // K = 64: two K = 32 MMAs, the second 32 bytes on in the swizzled rows
                                umma_f8_k64(O.dcol, O.a_off, O.b_off, desc_hi, O.idesc);
#ifdef F4J_TRACE
                                tr_ops++;
#endif
                            }
                            umma_commit(&empty[s]);
                        }
                        if (rel) {
                            // buffers whose level is complete: to the epilogue
                            for (uint32_t wr = rel; wr; wr &= wr - 1) umma_commit(&accfull[__ffs(wr) - 1]);
                            used |= rel;
                        }
                    }
                }
            }
#ifdef F4J_TRACE
            atomicAdd(&g_f4j_trace[0], (unsigned long long)(clock64() - tr_start));
            atomicAdd(&g_f4j_trace[1], tr_wait);
            atomicAdd(&g_f4j_trace[2], tr_acc);
            atomicAdd(&g_f4j_trace[3], tr_ops);
#endif
            umma_commit(&mma_done);
            mbar_wait(&mma_done, 0, p.status, 14);
        }
    } else {
        // ---------------- epilogue warps
        const int q = warp % 4;          // TMEM lane quarter this warp may access
        const int h = (warp - 2) / 4;    // column slice of the tile: columns h * EPI_COLS ...
        const int ubits = plan->ubits;
        uint32_t filled = 0;  // bit b: parity of the next accfull[b] phase to wait for
#ifdef F4J_TRACE
        unsigned long long tr_wait = 0;
        const long long tr_start = clock64();
#endif
        for (int u = blockIdx.x; u < nunits; u += gridDim.x) {
        const int tile = ksplit ? u / nchunks : u;
        int m0, n0;
        tile_origin(tile, tiles_m, tiles_n, m0, n0);
        m0 += p.tm0 * BM;
        n0 += p.tn0 * BN;
        const int row = m0 + 32 * q + lane;
        long long acc[EPI_COLS];
#pragma unroll
        for (int c = 0; c < EPI_COLS; c++) acc[c] = 0;
        bool ok = true;
        // the round program repeats once per K chunk; the rounds of a band
        // complete together, in round order
        for (int rr = 0; rr < (ksplit ? 1 : nchunks) * nrounds; rr++) {
            const Round R = sp->rounds[rr % nrounds];
            const int buf = R.buf;
            bool w = true;
            {
                F4J_T_BEGIN();
                if (lane == 0) w = mbar_wait(&accfull[buf], (filled >> buf) & 1, p.status, 15);
                F4J_T_ADD(tr_wait);
            }
            filled ^= 1u << buf;
            w = __shfl_sync(0xffffffffu, w, 0);
            if (!w || *(volatile int*)&abort_flag) {
                ok = false;
                abort_flag = 1;
                break;
            }
            tc_fence_after();
            const int sh = R.shift;
            const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + buf * BN + h * EPI_COLS;
#pragma unroll
            for (int part = 0; part < EPI_COLS / 16; part++) {
                uint32_t v[16];
                tmem_ld16(taddr + part * 16, v);
                tmem_ld_wait();
#pragma unroll
                for (int c = 0; c < 16; c++) {
                    // rounds are sized so |value| <= 2^24: an int32 holds it exactly
                    long long x = (long long)__float2int_rn(__uint_as_float(v[c]));
                    if (sh >= 0) acc[part * 16 + c] += x << sh;
                    else acc[part * 16 + c] += (x + (1ll << (-sh - 1))) >> (-sh);
                }
            }
#pragma unroll
            for (int c = 0; c < EPI_COLS; c += 32) tmem_zero32(taddr + c);
            tmem_st_wait();
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&accempty[buf]);
        }
        if (!ok) break;
        if (ksplit) {
            // the chunk's exact sums; k_split_fixup adds the chunks and scales
            if (row < p.M) {
                long long* dst = p.wpart + ((int64_t)(u % nchunks) * p.M + row) * p.N;
#pragma unroll
                for (int c = 0; c < EPI_COLS; c += 2) {
                    const int col = n0 + h * EPI_COLS + c;
                    if (col + 1 < p.N && ((reinterpret_cast<uintptr_t>(dst + col) & 15) == 0)) {
                        *reinterpret_cast<longlong2*>(dst + col) = make_longlong2(acc[c], acc[c + 1]);
                    } else {
                        if (col < p.N) dst[col] = acc[c];
                        if (col + 1 < p.N) dst[col + 1] = acc[c + 1];
                    }
                }
            }
        } else if (row < p.M) {
            const int ea = p.ea[row];
#pragma unroll
            for (int c = 0; c < EPI_COLS; c += 2) {
                const int col = n0 + h * EPI_COLS + c;
                double v0 = 0, v1 = 0;
                if (col < p.N) v0 = scale_pow2((double)acc[c], ubits + ea + p.eb[col]);
                if (col + 1 < p.N) v1 = scale_pow2((double)acc[c + 1], ubits + ea + p.eb[col + 1]);
                if (!p.cplx) {
                    double* dst = p.C + (int64_t)row * p.N + col;
                    if (col + 1 < p.N && ((reinterpret_cast<uintptr_t>(dst) & 15) == 0)) {
                        *reinterpret_cast<double2*>(dst) = make_double2(v0, v1);
                    } else {
                        if (col < p.N) dst[0] = v0;
                        if (col + 1 < p.N) dst[1] = v1;
                    }
                } else {
                    for (int u = 0; u < 2; u++) {
                        const int cc = col + u;
                        if (cc >= p.N) break;
                        const double v = u ? v1 : v0;
                        const int jn = cc < p.n_out ? cc : cc - p.n_out;
                        p.C[2 * ((int64_t)row * p.n_out + jn) + (cc < p.n_out ? 0 : 1)] = v;
                    }
                }
            }
        }
        }  // tile loop
#ifdef F4J_TRACE
        if (warp == 2 && lane == 0) {
            atomicAdd(&g_f4j_trace[6], (unsigned long long)(clock64() - tr_start));
            atomicAdd(&g_f4j_trace[7], tr_wait);
        }
#endif
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, NBUF * BN);
    }
}

// Split K: each C entry is the sum of its tile's chunk sums (exact in int64,
// so equal to one CTA accumulating the chunks in turn), converted and scaled as
// the slice GEMM's epilogue does.
__global__ void __launch_bounds__(256) k_split_fixup(const __grid_constant__ SplitGemmParams p, int nchunks) {
    if (p.plan->nonfinite) return;  // the gated plain path computes this product
    const int64_t mn = (int64_t)p.M * p.N;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= mn) return;
    const int row = (int)(idx / p.N), col = (int)(idx % p.N);
    long long acc = 0;
    for (int c = 0; c < nchunks; c++) acc += p.wpart[(int64_t)c * mn + idx];
    const double v = scale_pow2((double)acc, p.plan->ubits + p.ea[row] + p.eb[col]);
    if (!p.cplx) {
        p.C[idx] = v;
    } else {
        const int jn = col < p.n_out ? col : col - p.n_out;
        p.C[2 * ((int64_t)row * p.n_out + jn) + (col < p.n_out ? 0 : 1)] = v;
    }
}

}  // namespace

// ------------------------------------------------------------------ host side
static int make_slice_map(CUtensorMap* map, const void* base, uint64_t Kp, uint64_t rows, uint64_t planes) {
    f4j_encode_tiled_fn enc = f4j_encode_fn();
    if (!enc) return f4j_fail(F4J_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[3] = {Kp, rows, planes};
    cuuint64_t strides[2] = {Kp, Kp * rows};
    cuuint32_t box[3] = {BKB, BM, 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 3, const_cast<void*>(base), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return f4j_fail(F4J_ERR_CUDA, "cuTensorMapEncodeTiled (slices) failed (%d)", (int)r);
    return F4J_OK;
}

// Slice-count override from the environment (F4J_SPLIT_SLICES), 0 = from spread.
static int env_slices() {
    const char* env = getenv("F4J_SPLIT_SLICES");
    return (env && atoi(env) > 0) ? atoi(env) : 0;
}

// Row parts of A (F4J_HOST_PARTS) and column parts of B (F4J_HOST_BPARTS) of a
// host-buffer split product, 1..F4J_HOST_PARTS_MAX each.
static int env_host_parts(const char* name, int dflt) {
    const char* e = getenv(name);
    const int v = e ? atoi(e) : dflt;
    return v < 1 ? 1 : (v > F4J_HOST_PARTS_MAX ? F4J_HOST_PARTS_MAX : v);
}

// Levels per band in the slice GEMM's schedule (F4J_SPLIT_BAND, 1..4; default 4).
static int env_band() {
    const char* env = getenv("F4J_SPLIT_BAND");
    const int b = env ? atoi(env) : 0;
    return (b >= 1 && b <= NBUF) ? b : NBUF;
}

static size_t al1k(size_t x) { return (x + 1023) & ~size_t(1023); }

// grid.y of a slicing launch over `targets` rows of slices: one block row per
// 32 targets, at most 65535 (the kernels then loop over the remaining tile rows)
static unsigned slice_grid_y(int64_t targets) {
    const int64_t t = f4j_cdiv(targets, SP_TR);
    return (unsigned)(t < 65535 ? (t > 0 ? t : 1) : 65535);
}

// Asynchronous split GEMM: statistics -> device plan -> slicing -> slice GEMM,
// all queued on the context stream with no host synchronisation.  *gate
// receives the device flag that is non-zero when the plan stood down (NaN/Inf
// input); the caller then runs the gated plain kernel.  With a report the
// call waits for the plan to fill in slices / spread.
// Everything of one split GEMM but the slice GEMM launch: statistics, plan,
// slicing, tensor maps and kernel parameters (the launch covers all tile rows
// until split_launch narrows it).
struct SplitLaunch {
    CUtensorMap ta, tb;
    SplitGemmParams prm;
    int tiles_m, tiles_n;
    int kchunks;  // split K: chunks per tile, each a work unit (0: whole tiles)
};

// Split K for products with few output tiles.  The K chunk (a power of two of
// K blocks) minimising waves x (chunk + 1) over SPLIT_UNITS work units is a
// function of the shape alone, so every path that plans this product (device,
// host buffers, no-allocation) gets the same chunks and the same bits; split
// or not, a tile's int64 sum over its chunks is the same number.  Only for
// K <= 64 blocks, where the chunk the FP32 exactness budget allows is the
// largest power of two <= the block count for every slice count.  Returns the
// chunk cap for the planner (0: none) and, in *nchunks, the chunk count when
// the product runs split (0 otherwise).
static_assert(S_MAX * 64 * BKB * 256 <= (1 << 24), "64-block chunks fit the FP32 budget for every slice count");
constexpr int64_t SPLIT_UNITS = 152;
static int split_kcb_cap(int64_t tiles, int64_t nkb, int* nchunks) {
    *nchunks = 0;
    if (tiles >= SPLIT_UNITS || nkb < 2 || nkb > 64) return 0;
    int64_t nat = 1;
    while (2 * nat <= nkb) nat *= 2;
    int64_t best = nat, best_cost = INT64_MAX;
    for (int64_t kcb = nat; kcb >= 1; kcb /= 2) {
        const int64_t cost = f4j_cdiv(tiles * f4j_cdiv(nkb, kcb), SPLIT_UNITS) * (kcb + 1);
        if (cost < best_cost) {
            best_cost = cost;
            best = kcb;
        }
    }
    const int64_t nch = f4j_cdiv(nkb, best);
    if (nch >= 2) *nchunks = (int)nch;
    return (int)best;
}

// Column statistics of a stored rows x cols operand whose rows are ld elements
// apart.  Row chunks of 256, halved (down to 16) while the grid has fewer than
// four blocks per SM: a 1024-wide operand otherwise runs as 16 blocks.  The
// chunk count stays within grid.y.
static void launch_stats_cols(const double* X, int64_t rows, int64_t cols, int64_t ld, int cplx, int sm_count,
                              unsigned long long* mx, long long* es, int* cn, int* bad, cudaStream_t st) {
    const int64_t bx = f4j_cdiv(cols, 256);
    int64_t chunk = 256;
    while (chunk > 16 && bx * f4j_cdiv(rows, chunk) < 4 * (int64_t)sm_count) chunk /= 2;
    while (f4j_cdiv(rows, chunk) > 65535) chunk *= 2;
    k_stats_cols<<<dim3((unsigned)bx, (unsigned)f4j_cdiv(rows, chunk)), 256, 0, st>>>(X, rows, cols, ld, cplx,
                                                                                      (int)chunk, mx, es, cn, bad);
}

// Offsets in the small workspace of one split GEMM (M rows of op(A), n
// columns of op(B), N = n or 2n slice rows of B_cat^T): per-target statistics
// and exponents, the flag words, the plan.  Everything before `plan` starts at
// zero for each product (one memset).
struct SmallLayout {
    size_t mxa, esa, cna, mxb, esb, cnb, ea, eb, misc, plan, total;
};
static SmallLayout small_layout(int64_t M, int64_t n, int64_t N) {
    SmallLayout L;
    L.mxa = 0;
    L.esa = L.mxa + al1k(M * 8);
    L.cna = L.esa + al1k(M * 8);
    L.mxb = L.cna + al1k(M * 4);
    L.esb = L.mxb + al1k(n * 8);
    L.cnb = L.esb + al1k(n * 8);
    L.ea = L.cnb + al1k(n * 4);
    L.eb = L.ea + al1k(M * 4);
    L.misc = L.eb + al1k(N * 4);
    L.plan = L.misc + 1024;
    L.total = L.plan + al1k(sizeof(SplitPlan));
    return L;
}

// The context's table of plans for every slice count (k_plan_table), queued
// for a rebuild on the context stream when its key (K, summed length, band,
// K-chunk cap) changes; the one-thread build of a plan takes ~10 us.
static int plan_table(f4j_ctx* ctx, int64_t Kp, int64_t klen_cat, int kcb_cap, SplitPlan** out) {
    const int t = ctx->ws_base ? 1 : 0;
    const long long key[4] = {(long long)Kp, (long long)klen_cat, (long long)env_band(), (long long)kcb_cap};
    if (!ctx->plan_tab[t]) {
        F4J_CUDA(cudaMalloc(&ctx->plan_tab[t], (size_t)(S_MAX + 1) * sizeof(SplitPlan)));
        ctx->plan_valid[t] = false;
    }
    SplitPlan* tab = (SplitPlan*)ctx->plan_tab[t];
    if (!ctx->plan_valid[t] || memcmp(key, ctx->plan_key[t], sizeof key) != 0) {
        k_plan_table<<<S_MAX - 1, 32, 0, ctx->stream>>>(Kp, klen_cat, (int)key[2], kcb_cap, tab);
        F4J_LAUNCHED(ctx);
        memcpy(ctx->plan_key[t], key, sizeof key);
        ctx->plan_valid[t] = true;
    }
    *out = tab;
    return F4J_OK;
}

static int split_prepare(f4j_ctx* ctx, bool cplx, int64_t m, int64_t n, int64_t k, const double* A, int opA,
                         const double* B, int opB, double* C, int slices_req, SplitLaunch* L) {
    const int64_t M = m, N = cplx ? 2 * n : n;
    const int64_t Kh = f4j_cdiv(k, BKB) * BKB;  // K of one real part, padded to whole stages
    const int64_t Kp = cplx ? 2 * Kh : Kh;      // cat K: [re | im], zero padded in between
    const int64_t klen_cat = cplx ? 2 * k : k;
    if (M > INT32_MAX || N > INT32_MAX || Kp > INT32_MAX) return f4j_fail(F4J_ERR_ARG, "split GEMM too large");

    // ---- small workspace (slot 1): statistics, exponents, plan
    const SmallLayout Lo = small_layout(M, n, N);
    // ---- bulk workspace (slot 0): S_MAX slice planes per operand
    const size_t plane_a = (size_t)M * Kp, plane_b = (size_t)N * Kp;
    void *ws1, *ws0;
    int rc = f4j_workspace(ctx, ctx->ws_base + 1, Lo.total, &ws1);
    if (rc) return rc;
    int kchunks = 0;
    const int kcb_cap = split_kcb_cap(f4j_cdiv(M, BM) * f4j_cdiv(N, BN), Kp / BKB, &kchunks);
    const size_t wpart_bytes = kchunks ? (size_t)kchunks * M * N * 8 : 0;  // split K: chunk sums
    rc = f4j_workspace(ctx, ctx->ws_base, al1k(plane_a * S_MAX) + al1k(plane_b * S_MAX) + wpart_bytes, &ws0);
    if (rc) return rc;
    char* w = (char*)ws1;
    unsigned long long* mxa = (unsigned long long*)(w + Lo.mxa);
    long long* esa = (long long*)(w + Lo.esa);
    int* cna = (int*)(w + Lo.cna);
    unsigned long long* mxb = (unsigned long long*)(w + Lo.mxb);
    long long* esb = (long long*)(w + Lo.esb);
    int* cnb = (int*)(w + Lo.cnb);
    int* ea = (int*)(w + Lo.ea);
    int* eb = (int*)(w + Lo.eb);
    int* misc = (int*)(w + Lo.misc);  // [0] non-finite seen, [1] spread A x256, [2] spread B x256
    SplitPlan* plan = (SplitPlan*)(w + Lo.plan);
    uint8_t* slA = (uint8_t*)ws0;
    uint8_t* slB = slA + al1k(plane_a * S_MAX);

    // statistics accumulate with atomics and misc holds flags and the block
    // counter of k_finalize_pick: one clear of everything up to the plan
    F4J_CUDA(cudaMemsetAsync(w, 0, Lo.plan, ctx->stream));

    const bool a_rows = (opA == F4J_OP_N);  // targets of A (rows of op(A)) are stored rows
    const bool b_rows = (opB != F4J_OP_N);  // targets of B (columns of op(B)) are stored rows
    f4j_prof_begin(ctx, F4J_PROF_PREP);
    // statistics, one launch per operand (one launch for both measured 233 us
    // against 91 + 85 us at 8192^3, and the same at 1024^3)
    if (a_rows) {
        k_stats_rows<<<(unsigned)f4j_cdiv(M, 8), 256, 0, ctx->stream>>>(A, M, k, cplx, mxa, esa, cna, misc);
    } else {
        launch_stats_cols(A, k, M, M, cplx, ctx->sm_count, mxa, esa, cna, misc, ctx->stream);
    }
    F4J_LAUNCHED(ctx);
    if (b_rows) {
        k_stats_rows<<<(unsigned)f4j_cdiv(n, 8), 256, 0, ctx->stream>>>(B, n, k, cplx, mxb, esb, cnb, misc);
    } else {
        launch_stats_cols(B, k, n, n, cplx, ctx->sm_count, mxb, esb, cnb, misc, ctx->stream);
    }
    F4J_LAUNCHED(ctx);
    {   // exponents, spreads and the plan in one launch: the plan comes from the
        // context's table of plans for every slice count, rebuilt when the key
        // changes (the one-thread build takes ~10 us)
        SplitPlan* tab = nullptr;
        rc = plan_table(ctx, Kp, klen_cat, kcb_cap, &tab);
        if (rc) return rc;
        const unsigned blocks = (unsigned)(f4j_cdiv(M, 256) + f4j_cdiv(n, 256));
        k_finalize_pick<<<blocks, 256, 0, ctx->stream>>>(M, n, cplx ? 1 : 0, mxa, esa, cna, mxb, esb, cnb, ea, eb,
                                                         misc, k, klen_cat,
                                                         slices_req > 0 ? slices_req : env_slices(), tab, plan);
        F4J_LAUNCHED(ctx);
    }
    {   // both operands' slice planes in one launch.  A: targets = rows of op(A),
        // stored m x k (N) or k x m (T/C); B: targets = columns of op(B), stored
        // k x n (N, transposed read) or n x k (T/C)
        const SplitOperand sa{A, a_rows ? M : k, a_rows ? k : M, a_rows ? 0 : 1, opA == F4J_OP_C ? 1 : 0, 0, M, M,
                              ea, slA};
        const SplitOperand sb{B, b_rows ? n : k, b_rows ? k : n, b_rows ? 0 : 1, opB == F4J_OP_C ? 1 : 0, 1, n, N,
                              eb, slB};
        const unsigned gy = slice_grid_y(M > n ? M : n);
        auto pair = cplx ? k_split_pair<true> : k_split_pair<false>;
        pair<<<dim3((unsigned)(Kh / SP_TQ), gy, 2), 256, 0, ctx->stream>>>(sa, sb, k, Kh, Kp, plan);
        F4J_LAUNCHED(ctx);
    }
    f4j_prof_end(ctx);

    rc = make_slice_map(&L->ta, slA, Kp, M, S_MAX);
    if (rc) return rc;
    rc = make_slice_map(&L->tb, slB, Kp, N, S_MAX);
    if (rc) return rc;

    SplitGemmParams& prm = L->prm;
    prm = SplitGemmParams{};
    prm.M = (int)M;
    prm.N = (int)N;
    prm.Kp = (int)Kp;
    prm.cplx = cplx ? 1 : 0;
    prm.n_out = (int)n;
    prm.ea = ea;
    prm.eb = eb;
    prm.C = C;
    prm.status = ctx->d_status + F4J_ST_TIMEOUT;
    prm.plan = plan;
    prm.tm0 = 0;
    prm.tm1 = (int)f4j_cdiv(M, BM);
    prm.tn0 = 0;
    prm.tn1 = (int)f4j_cdiv(N, BN);
    prm.wpart = kchunks ? reinterpret_cast<long long*>(slB + al1k(plane_b * S_MAX)) : nullptr;
    L->tiles_m = prm.tm1;
    L->tiles_n = (int)f4j_cdiv(N, BN);
    L->kchunks = kchunks;
    return F4J_OK;
}

// The slice GEMM over tile rows [tm0, tm1) and tile columns [tn0, tn1) of C
// on `stream` (tn1 < 0: every tile column).
static int split_launch(f4j_ctx* ctx, const SplitLaunch& L, cudaStream_t stream, int tm0, int tm1, int tn0 = 0,
                        int tn1 = -1) {
    SplitGemmParams prm = L.prm;
    prm.tm0 = tm0;
    prm.tm1 = tm1;
    prm.tn0 = tn0;
    prm.tn1 = tn1 < 0 ? L.tiles_n : tn1;
    const size_t smem = (size_t)RING * TILE_BYTES + 1024 + sizeof(SplitPlan) + (size_t)NSTAGE * MAX_OPS * sizeof(Op);
    cudaError_t e = cudaFuncSetAttribute(k_split_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return f4j_cuda_fail(e, "cudaFuncSetAttribute(k_split_gemm)");
    const bool ksplit = prm.wpart != nullptr;
    if (ksplit && (tm0 != 0 || tm1 != L.tiles_m || prm.tn0 != 0 || prm.tn1 != L.tiles_n))
        return f4j_fail(F4J_ERR_ARG, "split-K slice GEMM over part of C");
    if (tm0 < 0 || tm1 > L.tiles_m || tm0 >= tm1 || prm.tn0 < 0 || prm.tn1 > L.tiles_n || prm.tn0 >= prm.tn1)
        return f4j_fail(F4J_ERR_ARG, "slice GEMM tile range [%d, %d) x [%d, %d) outside %d x %d", tm0, tm1, prm.tn0,
                        prm.tn1, L.tiles_m, L.tiles_n);
    const int64_t nunits = (int64_t)(prm.tn1 - prm.tn0) * (tm1 - tm0) * (ksplit ? L.kchunks : 1);
    const unsigned grid = (unsigned)(nunits < ctx->sm_count ? nunits : ctx->sm_count);
    const cudaStream_t saved = ctx->stream;
    ctx->stream = stream;
    f4j_prof_begin(ctx);
    k_split_gemm<<<grid, GEMM_THREADS, smem, stream>>>(L.ta, L.tb, prm);
    if (ksplit) {
        k_split_fixup<<<(unsigned)f4j_cdiv((int64_t)prm.M * prm.N, 256), 256, 0, stream>>>(prm, L.kchunks);
        ctx->launches++;
    }
    f4j_prof_end(ctx);
    ctx->stream = saved;
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        cudaFuncAttributes fa{};
        cudaFuncGetAttributes(&fa, k_split_gemm);
        return f4j_fail(F4J_ERR_CUDA,
                        "k_split_gemm launch: %s (regs %d, max threads %d, static smem %zu, local %zu, "
                        "max dyn smem %d, requested dyn smem %zu, params %zu B)",
                        cudaGetErrorString(e), fa.numRegs, fa.maxThreadsPerBlock, fa.sharedSizeBytes,
                        fa.localSizeBytes, fa.maxDynamicSharedSizeBytes, smem, sizeof(SplitGemmParams));
    }
    ctx->launches++;
    return F4J_OK;
}

// Plan header (s, nrounds, ubits, nonfinite, spread) into a report.
static int split_report(f4j_ctx* ctx, const SplitPlan* plan, f4j_report* rep) {
    int hp[5];
    F4J_CUDA(cudaMemcpyAsync(hp, plan, sizeof hp, cudaMemcpyDeviceToHost, ctx->stream));
    F4J_CUDA(cudaStreamSynchronize(ctx->stream));
    float spread;
    memcpy(&spread, &hp[4], 4);
    rep->slices = hp[0];
    rep->frac_bits = 4 + 5 * (hp[0] - 1);
    rep->exp_spread = spread;
    if (hp[3]) rep->slices = 0;
    return F4J_OK;
}

int f4j_gemm_split(f4j_ctx* ctx, bool cplx, int64_t m, int64_t n, int64_t k, const double* A, int opA,
                   const double* B, int opB, double* C, int slices_req, f4j_report* rep, const int** gate) {
    *gate = nullptr;
    SplitLaunch L;
    int rc = split_prepare(ctx, cplx, m, n, k, A, opA, B, opB, C, slices_req, &L);
    if (rc) return rc;
    rc = split_launch(ctx, L, ctx->stream, 0, L.tiles_m);
    if (rc) return rc;
    *gate = &L.prm.plan->nonfinite;
    if (rep) return split_report(ctx, L.prm.plan, rep);
    return F4J_OK;
}

// ------------------------------------------------------------------ host buffers
// Row parts of A for a pipelined host-buffer product, in tile rows: part p
// is [bound[p], bound[p + 1]), 1 <= parts <= min(tiles_m, F4J_HOST_PARTS_MAX).
// One part is all of A.  Otherwise the first part has up to 8 tile rows (a
// quarter of A when that is less), the second as many, the last 1/8 of the
// tile rows and the rest is cut into equal middle parts; every part keeps at
// least one tile row.
static void host_part_bounds(int tiles_m, int parts, int* bound) {
    bound[0] = 0;
    bound[1] = tiles_m;
    if (parts < 2) return;
    const int a0 = tiles_m / 4 < 1 ? 1 : (tiles_m / 4 > 8 ? 8 : tiles_m / 4);
    const int last = tiles_m / 8 < 1 ? 1 : tiles_m / 8;
    bound[parts] = tiles_m;
    bound[1] = a0;
    if (parts >= 3) bound[parts - 1] = tiles_m - last;
    if (parts >= 4) bound[2] = 2 * a0;
    for (int p = 3; p < parts - 1; p++)
        bound[p] = bound[2] + (int)((int64_t)(bound[parts - 1] - bound[2]) * (p - 2) / (parts - 3));
    for (int p = 1; p < parts; p++) {  // keep every part non-empty
        const int lo = bound[p - 1] + 1, hi = tiles_m - (parts - p);
        bound[p] = bound[p] < lo ? lo : (bound[p] > hi ? hi : bound[p]);
    }
}

// The split product C = A op(B) from host memory with its uploads pipelined
// (f4j_dgemm_host / f4j_zgemm_host, op(A) = N).  The uploads go back to back
// on their own stream: A's first row part, then B in column parts (complex: B
// whole, since a column part of B lands in both halves of the [Re | Im]
// concatenation), then the rest of A in row parts.  Each part's statistics and slicing run on the context stream as
// soon as it is up; each column part of B is then multiplied by A's first
// rows, and each later row part of A by all of B.  Every product is one launch
// on its own stream, its block of C going down behind it.  The slice count
// cannot wait for all of A and B, so it is picked from A's first rows and B's
// first columns (k_plan_pick on the spreads so far).  Once every statistic is
// in, k_spec_check compares it with the count all of A and B give: *recompute
// is set when they differ, or when an operand holds a NaN / Inf, and the
// caller then runs the ordinary path.  When the counts agree, every exponent,
// slice, plan and tile sum is the ordinary path's, and so is every bit of C.
// Waits for everything it queued before returning; *spread_out receives the
// spread all of A and B give.
//
// Part sizes.  A's first part has up to 8 tile rows (all of A in one part
// when parts == 1): its product with one of
// F4J_HOST_BPARTS = 4 column parts of B takes about as long as the next column
// part's upload (both scale with K and the part's width; measured at 8192^3:
// 0.67 ms of product on 128 SMs per 0.75 ms of upload).  B's column parts go up
// as 2D copies: 4 parts of an 8192-column B (16 KB rows) move 180 GB/s, 8
// parts (8 KB rows) only 106 GB/s.  A's second part is as small as its first,
// so that products follow soon after B's upload ends; the last part is 1/8 of
// the tile rows, so that little of C's download follows the last product; the
// rest is in equal middle parts.  A part's statistics and slicing cannot run
// beside a slice GEMM (its CTA fills two of an SM's four register files and
// all but ~1 KB of its shared memory), so they wait for SMs whenever the
// products before them hold every SM; these sizes keep that wait short.
static int host_split_pipelined(f4j_ctx* ctx, bool cplx, int64_t m, int64_t n, int64_t k, const double* A,
                                const double* B, int opB, double* C, double* dA, double* dB, double* dC, int parts,
                                int bparts, bool* recompute, const SplitPlan** plan_out, float* spread_out) {
    *recompute = false;
    // complex: the [Re | Im] concatenation of the ordinary path (2n slice rows
    // of B, K of 2 Kh), interleaved (re, im) doubles in host and device memory
    const int64_t M = m, N = cplx ? 2 * n : n;
    const int64_t Kh = f4j_cdiv(k, BKB) * BKB;  // K of one part, padded to whole K blocks
    const int64_t Kp = cplx ? 2 * Kh : Kh;
    const int64_t klen_cat = cplx ? 2 * k : k;
    const int64_t w2 = cplx ? 2 : 1;  // doubles per element
    if (M > INT32_MAX || N > INT32_MAX || Kp > INT32_MAX) return f4j_fail(F4J_ERR_ARG, "host-buffer split GEMM too large");
    const SmallLayout Lo = small_layout(M, n, N);
    void *ws1, *ws0;
    int rc = f4j_workspace(ctx, ctx->ws_base + 1, Lo.total, &ws1);
    if (rc) return rc;
    const size_t plane_a = (size_t)M * Kp, plane_b = (size_t)N * Kp;
    rc = f4j_workspace(ctx, ctx->ws_base, al1k(plane_a * S_MAX) + al1k(plane_b * S_MAX), &ws0);
    if (rc) return rc;
    char* w = (char*)ws1;
    unsigned long long* mxa = (unsigned long long*)(w + Lo.mxa);
    long long* esa = (long long*)(w + Lo.esa);
    int* cna = (int*)(w + Lo.cna);
    unsigned long long* mxb = (unsigned long long*)(w + Lo.mxb);
    long long* esb = (long long*)(w + Lo.esb);
    int* cnb = (int*)(w + Lo.cnb);
    int* ea = (int*)(w + Lo.ea);
    int* eb = (int*)(w + Lo.eb);
    int* misc = (int*)(w + Lo.misc);  // [0] non-finite, [1] spread of A so far, [2] of B, [5] the check
    SplitPlan* plan = (SplitPlan*)(w + Lo.plan);
    uint8_t* slA = (uint8_t*)ws0;
    uint8_t* slB = slA + al1k(plane_a * S_MAX);
    const bool b_rows = opB != F4J_OP_N;  // columns of op(B) are stored rows of B (n x k)
    const int conjb = cplx && opB == F4J_OP_C ? 1 : 0;
    const auto split_k = cplx ? k_split<true> : k_split<false>;
    const int s_req = env_slices();
    // the same K-chunk cap the ordinary path plans with (no split K here)
    int kchunks = 0;
    const int kcb_cap = split_kcb_cap(f4j_cdiv(M, BM) * f4j_cdiv(N, BN), Kp / BKB, &kchunks);
    if (kchunks) return f4j_fail(F4J_ERR_ARG, "split-K product in parts");
    const cudaStream_t st = ctx->stream;

    SplitLaunch L;
    rc = make_slice_map(&L.ta, slA, Kp, M, S_MAX);
    if (rc) return rc;
    rc = make_slice_map(&L.tb, slB, Kp, N, S_MAX);
    if (rc) return rc;
    SplitGemmParams& prm = L.prm;
    prm = SplitGemmParams{};
    prm.M = (int)M;
    prm.N = (int)N;
    prm.Kp = (int)Kp;
    prm.cplx = cplx ? 1 : 0;
    prm.n_out = (int)n;
    prm.ea = ea;
    prm.eb = eb;
    prm.C = dC;
    prm.status = ctx->d_status + F4J_ST_TIMEOUT;
    prm.plan = plan;
    prm.wpart = nullptr;
    L.tiles_m = (int)f4j_cdiv(M, BM);
    L.tiles_n = (int)f4j_cdiv(N, BN);
    L.kchunks = 0;
    prm.tm0 = 0;
    prm.tm1 = L.tiles_m;
    prm.tn0 = 0;
    prm.tn1 = L.tiles_n;

    // A's row parts and B's column parts, in tile rows / columns
    const int tiles_m = L.tiles_m, tiles_n = L.tiles_n;
    if (parts < 1 || parts > tiles_m || parts > F4J_HOST_PARTS_MAX)
        return f4j_fail(F4J_ERR_ARG, "%d row parts of %d tile rows", parts, tiles_m);
    int bound[F4J_HOST_PARTS_MAX + 1];
    host_part_bounds(tiles_m, parts, bound);
    // complex: B whole (its column parts would fall on both halves of the
    // concatenation)
    const int qb = cplx ? 1 : (bparts < tiles_n ? bparts : tiles_n);
    int cbound[F4J_HOST_PARTS_MAX + 1];
    for (int j = 0; j <= qb; j++) cbound[j] = (int)((int64_t)tiles_n * j / qb);

    // everything is queued by `queue`; whatever it returns, every stream that
    // holds queued work is waited for before this function returns, so no
    // copy still reads A or B, or writes C, after an error
    int launched = 0;
    auto queue = [&]() -> int {
        F4J_CUDA(cudaMemsetAsync(w, 0, Lo.plan, st));
        SplitPlan* tab = nullptr;
        rc = plan_table(ctx, Kp, klen_cat, kcb_cap, &tab);
        if (rc) return rc;

        // Every upload goes up back to back on the upload stream, in the order the
        // parts are used (A's first rows, B's column parts, the rest of A); the
        // kernels of part u wait on its event up_ev[u] on the context stream.
        const cudaStream_t up = ctx->up_stream;
        F4J_CUDA(cudaEventRecord(ctx->up_start, st));
        F4J_CUDA(cudaStreamWaitEvent(up, ctx->up_start, 0));
        {
            int u = 0;
            const int64_t r1 = (int64_t)bound[1] * BM < m ? (int64_t)bound[1] * BM : m;
            F4J_CUDA(cudaMemcpyAsync(dA, A, (size_t)r1 * k * 8 * w2, cudaMemcpyHostToDevice, up));
            F4J_CUDA(cudaEventRecord(ctx->up_ev[u++], up));
            for (int j = 0; j < qb; j++) {
                const int64_t c0 = (int64_t)cbound[j] * BN;
                const int64_t c1 = (int64_t)cbound[j + 1] * BN < n ? (int64_t)cbound[j + 1] * BN : n;
                if (b_rows)  // stored rows [c0, c1) of B (n x k)
                    F4J_CUDA(cudaMemcpyAsync(dB + c0 * k * w2, B + c0 * k * w2, (size_t)(c1 - c0) * k * 8 * w2,
                                             cudaMemcpyHostToDevice, up));
                else         // stored columns [c0, c1) of B (k x n)
                    F4J_CUDA(cudaMemcpy2DAsync(dB + c0 * w2, (size_t)n * 8 * w2, B + c0 * w2, (size_t)n * 8 * w2,
                                               (size_t)(c1 - c0) * 8 * w2, (size_t)k, cudaMemcpyHostToDevice, up));
                F4J_CUDA(cudaEventRecord(ctx->up_ev[u++], up));
            }
            for (int p = 1; p < parts; p++) {
                const int64_t r0 = (int64_t)bound[p] * BM;
                const int64_t re = (int64_t)bound[p + 1] * BM < m ? (int64_t)bound[p + 1] * BM : m;
                F4J_CUDA(cudaMemcpyAsync(dA + r0 * k * w2, A + r0 * k * w2, (size_t)(re - r0) * k * 8 * w2,
                                         cudaMemcpyHostToDevice, up));
                F4J_CUDA(cudaEventRecord(ctx->up_ev[u++], up));
            }
        }

        // one row part of A (upload u): statistics, exponents (spread into misc[1])
        auto a_part_stats = [&](int u, int64_t r0, int64_t rows) -> int {
            F4J_CUDA(cudaStreamWaitEvent(st, ctx->up_ev[u], 0));
            k_stats_rows<<<(unsigned)f4j_cdiv(rows, 8), 256, 0, st>>>(dA + r0 * k * w2, rows, k, cplx ? 1 : 0,
                                                                      mxa + r0, esa + r0, cna + r0, misc);
            F4J_LAUNCHED(ctx);
            k_stats_finalize<<<(unsigned)f4j_cdiv(rows, 256), 256, 0, st>>>(rows, 0, mxa + r0, esa + r0, cna + r0,
                                                                             ea + r0, misc + 1);
            F4J_LAUNCHED(ctx);
            return F4J_OK;
        };
        // its slice planes: target t of the part is row r0 + t
        auto a_part_split = [&](int64_t r0, int64_t rows) -> int {
            split_k<<<dim3((unsigned)(Kh / SP_TQ), slice_grid_y(rows)), 256, 0, st>>>(
                dA + r0 * k * w2, rows, k, 0, 0, 0, rows, k, Kh, Kp, M, ea + r0, plan, slA + r0 * Kp);
            F4J_LAUNCHED(ctx);
            return F4J_OK;
        };
        // launch `id`: its stream waits for the slicing queued so far, runs the
        // slice GEMM over tile rows [tm0, tm1) x tile columns [tn0, tn1), and
        // downloads that block of C
        auto product = [&](int id, int tm0, int tm1, int tn0, int tn1) -> int {
            F4J_CUDA(cudaEventRecord(ctx->part_prep_ev[id], st));
            const cudaStream_t ps = ctx->part_stream[id];
            F4J_CUDA(cudaStreamWaitEvent(ps, ctx->part_prep_ev[id], 0));
            launched = id + 1;
            int r = split_launch(ctx, L, ps, tm0, tm1, tn0, tn1);
            if (r) return r;
            const int64_t r0 = (int64_t)tm0 * BM, r1 = (int64_t)tm1 * BM < m ? (int64_t)tm1 * BM : m;
            const int64_t c0 = (int64_t)tn0 * BN, c1 = (int64_t)tn1 * BN < n ? (int64_t)tn1 * BN : n;
            F4J_CUDA(cudaMemcpy2DAsync(C + (r0 * n + c0) * w2, (size_t)n * 8 * w2, dC + (r0 * n + c0) * w2,
                                       (size_t)n * 8 * w2, (size_t)(c1 - c0) * 8 * w2, (size_t)(r1 - r0),
                                       cudaMemcpyDeviceToHost, ps));
            F4J_CUDA(cudaEventRecord(ctx->part_ev[id], ps));
            return F4J_OK;
        };

        // A's first rows, then B's column parts, each multiplied by those rows
        const int64_t a0_rows = (int64_t)bound[1] * BM < m ? (int64_t)bound[1] * BM : m;
        rc = a_part_stats(0, 0, a0_rows);
        for (int j = 0; j < qb && !rc; j++) {
            const int64_t c0 = (int64_t)cbound[j] * BN;
            const int64_t c1 = (int64_t)cbound[j + 1] * BN < n ? (int64_t)cbound[j + 1] * BN : n;
            const int64_t cw = c1 - c0;
            F4J_CUDA(cudaStreamWaitEvent(st, ctx->up_ev[1 + j], 0));
            if (b_rows) {  // stored rows [c0, c1) of B (n x k)
                k_stats_rows<<<(unsigned)f4j_cdiv(cw, 8), 256, 0, st>>>(dB + c0 * k * w2, cw, k, cplx ? 1 : 0,
                                                                        mxb + c0, esb + c0, cnb + c0, misc);
            } else {       // stored columns [c0, c1) of B (k x n)
                launch_stats_cols(dB + c0 * w2, k, cw, n, cplx ? 1 : 0, ctx->sm_count, mxb + c0, esb + c0, cnb + c0,
                                  misc, st);
            }
            F4J_LAUNCHED(ctx);
            // complex (B whole): each target's exponent also for its row in B_cat^T's second half
            k_stats_finalize<<<(unsigned)f4j_cdiv(cw, 256), 256, 0, st>>>(cw, cplx ? 1 : 0, mxb + c0, esb + c0,
                                                                           cnb + c0, eb + c0, misc + 2);
            F4J_LAUNCHED(ctx);
            if (j == 0) {  // the plan from A's first rows and B's first columns, then those rows' slices
                k_plan_pick<<<1, 128, 0, st>>>(misc, k, klen_cat, s_req, tab, plan);
                F4J_LAUNCHED(ctx);
                rc = a_part_split(0, a0_rows);
                if (rc) break;
            }
            split_k<<<dim3((unsigned)(Kh / SP_TQ), slice_grid_y(cw)), 256, 0, st>>>(
                b_rows ? dB + c0 * k * w2 : dB + c0 * w2, b_rows ? cw : k, b_rows ? k : n, b_rows ? 0 : 1, conjb, 1,
                cw, k, Kh, Kp, N, eb + c0, plan, slB + c0 * Kp);
            F4J_LAUNCHED(ctx);
            rc = product(j, 0, bound[1], cbound[j], cbound[j + 1]);
        }
        // the rest of A, each row part multiplied by all of B
        for (int p = 1; p < parts && !rc; p++) {
            const int64_t r0 = (int64_t)bound[p] * BM;
            const int64_t r1 = (int64_t)bound[p + 1] * BM < m ? (int64_t)bound[p + 1] * BM : m;
            rc = a_part_stats(qb + p, r0, r1 - r0);
            if (!rc) rc = a_part_split(r0, r1 - r0);
            if (!rc) rc = product(qb + p - 1, bound[p], bound[p + 1], 0, tiles_n);
        }
        return rc;
    };
    rc = queue();
    int hm[6] = {0, 0, 0, 0, 0, 0};
    if (!rc) {
        k_spec_check<<<1, 32, 0, st>>>(misc, k, klen_cat, s_req, plan);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) {
            ctx->launches++;
            e = cudaMemcpyAsync(hm, misc, sizeof hm, cudaMemcpyDeviceToHost, st);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = f4j_cuda_fail(e, "slice count check of a host-buffer product");
    } else {
        cudaStreamSynchronize(st);
    }
    {
        cudaError_t e = cudaStreamSynchronize(ctx->up_stream);
        if (e != cudaSuccess && !rc) rc = f4j_cuda_fail(e, "upload of a host-buffer product");
    }
    for (int i = 0; i < launched; i++) {
        cudaError_t e = cudaStreamSynchronize(ctx->part_stream[i]);
        if (e != cudaSuccess && !rc) rc = f4j_cuda_fail(e, "part of a host-buffer product");
    }
    if (rc) return rc;
    *recompute = hm[5] != 0;
    *plan_out = plan;
    *spread_out = (float)((hm[1] > hm[2] ? hm[1] : hm[2]) / 256.0);
    return F4J_OK;
}

// C = op(A) op(B) from and to host memory (pinned for full copy speed).  A
// split product with op(A) = N, n > 1, no split K and at least two tile rows
// (or, real, two tile columns) runs pipelined (host_split_pipelined): A's
// first rows up (all of A when it has one tile row), then B (real: in
// F4J_HOST_BPARTS column parts; complex: whole), then the rest of A in row
// parts (F4J_HOST_PARTS in all), each part sliced and multiplied on its own
// stream as soon as it arrives and its block of C downloaded behind its
// product.  In the rare case that all of A and B ask for another slice count
// than their first parts did (or an operand holds a NaN / Inf), the product
// runs again through the ordinary path on the operands already on the device.
// Either way C equals f4j_dgemm's (f4j_zgemm's) bit for bit.  Other products
// upload, multiply and download in turn.  Returns when C is in host memory.
// f4j_dgemm_host (cplx false) and f4j_zgemm_host (cplx true): the same
// pipeline for both; complex operands and C are interleaved (re, im) doubles.
static int gemm_host(f4j_ctx* ctx, bool cplx, int64_t m, int64_t n, int64_t k, const double* A, int opA,
                     const double* B, int opB, double* C, int mode, f4j_report* rep) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (!A || !B || !C) return f4j_fail(F4J_ERR_ARG, "null host pointer");
    if (m < 0 || n < 0 || k < 0) return f4j_fail(F4J_ERR_ARG, "negative dimension");
    if (m > INT32_MAX || n > INT32_MAX || k > INT32_MAX)
        return f4j_fail(F4J_ERR_ARG, "dimension exceeds Flag4j's int range");
    if (opA < F4J_OP_N || opA > F4J_OP_C || opB < F4J_OP_N || opB > F4J_OP_C) return f4j_fail(F4J_ERR_ARG, "bad op");
    if (mode < F4J_MODE_PLAIN || mode > F4J_MODE_EXACT) return f4j_fail(F4J_ERR_ARG, "bad mode %d", mode);
    F4J_CUDA(cudaSetDevice(ctx->device));
    if (rep && rep->check_samples < 0) return f4j_fail(F4J_ERR_ARG, "negative check_samples");
    const int check_samples = rep ? rep->check_samples : 0, check_flags = rep ? rep->check_flags : 0;
    if (rep) {
        *rep = f4j_report{};
        rep->max_abs_err = rep->max_rel_err = rep->plain_max_abs_err = rep->plain_max_rel_err = -1.0;
    }
    if (m == 0 || n == 0) return F4J_OK;
    if (!cplx && opA == F4J_OP_C) opA = F4J_OP_T;  // conjugation is the identity for real data
    if (!cplx && opB == F4J_OP_C) opB = F4J_OP_T;
    const size_t es = cplx ? 16 : 8;  // bytes per element
    const size_t ab = (size_t)m * k * es, bb = (size_t)k * n * es, cb = (size_t)m * n * es;
    // With host pinning on, the caller's arrays are page-locked for this call
    // and released on every way out (after the context's streams have
    // drained).  An array that is already page-locked, or that cannot be
    // registered (e.g. it shares a page with one that is), is used as it is.
    struct HostPins {
        f4j_ctx* ctx;
        void* p[3];
        int n = 0;
        ~HostPins() {
            if (!n) return;
            cudaStreamSynchronize(ctx->stream);
            for (int i = 0; i < n; i++) cudaHostUnregister(p[i]);
            cudaGetLastError();
        }
    } pins{ctx, {nullptr, nullptr, nullptr}};
    if (ctx->host_pin) {
        void* const ptrs[3] = {(void*)A, (void*)B, (void*)C};
        const size_t bytes[3] = {ab, bb, cb};
        for (int i = 0; i < 3; i++) {
            if (!bytes[i]) continue;
            if (cudaHostRegister(ptrs[i], bytes[i], cudaHostRegisterDefault) == cudaSuccess) pins.p[pins.n++] = ptrs[i];
            else cudaGetLastError();  // stays pageable; clear the error so later launch checks do not see it
        }
    }
    void *dA, *dB, *dC;
    int rc = f4j_workspace(ctx, 3, ab, &dA);
    if (!rc) rc = f4j_workspace(ctx, 6, bb, &dB);
    if (!rc) rc = f4j_workspace(ctx, 7, cb, &dC);
    if (rc) return rc;
    // n == 1 runs the device path's matrix-vector kernel
    const bool split = k > 0 && n > 1 && f4j_resolve_mode(cplx, m, n, k, mode) == F4J_MODE_SPLIT;
    const int tiles_m = (int)f4j_cdiv(m, BM);
    const int want = env_host_parts("F4J_HOST_PARTS", F4J_HOST_PARTS);
    const int parts = tiles_m < want ? tiles_m : want;
    const int bparts = env_host_parts("F4J_HOST_BPARTS", F4J_HOST_BPARTS);
    const int64_t ncat = cplx ? 2 * n : n;  // slice rows of B (the [Re | Im] concatenation when complex)
    const int tiles_n = (int)f4j_cdiv(ncat, BN);
    // pipelined when A has two row parts or B two column parts (real only)
    const bool piped = parts >= 2 || (!cplx && bparts >= 2 && tiles_n >= 2);
    int kchunks = 0;
    split_kcb_cap(tiles_m * (int64_t)tiles_n, (cplx ? 2 : 1) * f4j_cdiv(k, BKB), &kchunks);
    if (!split || opA != F4J_OP_N || !piped || kchunks) {  // split K runs as one launch
        if (ab) F4J_CUDA(cudaMemcpyAsync(dA, A, ab, cudaMemcpyHostToDevice, ctx->stream));
        if (bb) F4J_CUDA(cudaMemcpyAsync(dB, B, bb, cudaMemcpyHostToDevice, ctx->stream));
        rc = f4j_gemm_impl(ctx, cplx, m, n, k, (const double*)dA, opA, (const double*)dB, opB, (double*)dC, mode,
                           rep);
        if (rc) return rc;
        F4J_CUDA(cudaMemcpyAsync(C, dC, cb, cudaMemcpyDeviceToHost, ctx->stream));
        F4J_CUDA(cudaStreamSynchronize(ctx->stream));
        return f4j_report_accuracy(ctx, cplx, m, n, k, (const double*)dA, opA, (const double*)dB, opB,
                                   (const double*)dC, check_samples, check_flags, rep);
    }
    if (!ctx->parts_init) {
        for (int i = 0; i < F4J_HOST_STREAMS; i++) {
            F4J_CUDA(cudaStreamCreateWithFlags(&ctx->part_stream[i], cudaStreamNonBlocking));
            F4J_CUDA(cudaEventCreateWithFlags(&ctx->part_ev[i], cudaEventDisableTiming));
            F4J_CUDA(cudaEventCreateWithFlags(&ctx->part_prep_ev[i], cudaEventDisableTiming));
            F4J_CUDA(cudaEventCreateWithFlags(&ctx->up_ev[i], cudaEventDisableTiming));
        }
        F4J_CUDA(cudaStreamCreateWithFlags(&ctx->up_stream, cudaStreamNonBlocking));
        F4J_CUDA(cudaEventCreateWithFlags(&ctx->up_start, cudaEventDisableTiming));
        ctx->parts_init = true;
    }
    const int64_t l0 = ctx->launches;
    bool recompute = false;
    const SplitPlan* plan = nullptr;
    float spread = 0.0f;
    rc = host_split_pipelined(ctx, cplx, m, n, k, A, B, opB, C, (double*)dA, (double*)dB, (double*)dC, parts, bparts,
                              &recompute, &plan, &spread);
    if (rc) return rc;
    if (recompute) {
        // all of A and B ask for another slice count than their first parts
        // did, or an operand holds a NaN / Inf: the product again through the
        // ordinary path on the operands now on the device, and all of C down
        rc = f4j_gemm_impl(ctx, cplx, m, n, k, (const double*)dA, F4J_OP_N, (const double*)dB, opB, (double*)dC,
                           mode, rep);
        if (rc) return rc;
        F4J_CUDA(cudaMemcpyAsync(C, dC, cb, cudaMemcpyDeviceToHost, ctx->stream));
        F4J_CUDA(cudaStreamSynchronize(ctx->stream));
    } else if (rep) {
        rep->flops = (cplx ? 8.0 : 2.0) * (double)m * (double)n * (double)k;
        rep->mode_used = F4J_MODE_SPLIT;
        rc = split_report(ctx, plan, rep);
        if (rc) return rc;
        rep->exp_spread = spread;
    }
    if (rep) rep->launches = (int32_t)(ctx->launches - l0);
    return f4j_report_accuracy(ctx, cplx, m, n, k, (const double*)dA, F4J_OP_N, (const double*)dB, opB,
                               (const double*)dC, check_samples, check_flags, rep);
}

extern "C" int f4j_dgemm_host(f4j_ctx* ctx, int64_t m, int64_t n, int64_t k, const double* A, int opA,
                              const double* B, int opB, double* C, int mode, f4j_report* rep) {
    return gemm_host(ctx, false, m, n, k, A, opA, B, opB, C, mode, rep);
}

extern "C" int f4j_set_host_pinning(f4j_ctx* ctx, int on) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    ctx->host_pin = on != 0;
    return F4J_OK;
}

extern "C" int f4j_zgemm_host(f4j_ctx* ctx, int64_t m, int64_t n, int64_t k, const double* A, int opA,
                              const double* B, int opB, double* C, int mode, f4j_report* rep) {
    return gemm_host(ctx, true, m, n, k, A, opA, B, opB, C, mode, rep);
}

// ------------------------------------------------------------------ no-allocation variant
// Some callers cannot allocate device memory: engines that hand out a fixed
// memory pool and forbid cudaMalloc after start-up, and JVM or other runtime
// hosts that only pass in buffers they already own.  f4j_dgemm_split_noalloc
// serves them: it runs the same split GEMM as f4j_dgemm(..., F4J_MODE_SPLIT,
// ...) but takes its scratch (exponent statistics, the plan and the FP8 slice
// planes) from the file-scope array below, so it calls no allocator at all.
//
// The array holds F4J_NOALLOC_SCRATCH_BYTES on every GPU that loads this
// library, until the process exits.  It is shared by every call on a device and
// keeps the last call's contents; each call clears what must start at zero.
// Calls whose GPU work overlaps (e.g. on two streams) race on it.
//
// A call needs at most F4J_NOALLOC_NEED(m, n, Kp) bytes of it (Kp = k rounded
// up to 64): 12 slice planes of (m + n) x Kp bytes, 24 bytes of statistics and
// exponents per row of op(A) and column of op(B), and under 16 KiB for the
// plan, the status words and the 1 KiB roundings of each part.  The call is
// rejected exactly when that formula exceeds the array.
#define F4J_NOALLOC_SCRATCH_BYTES (32u << 20)
#define F4J_NOALLOC_NEED(m, n, Kp) \
    ((size_t)12 * (size_t)((m) + (n)) * (size_t)(Kp) + (size_t)24 * (size_t)((m) + (n)) + (size_t)16384)
static_assert(sizeof(SplitPlan) <= 4096, "the no-allocation bound's fixed part counts the plan as at most 4 KiB");
static __device__ __align__(256) unsigned char g_f4j_noalloc_scratch[F4J_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[256];  // device address of the array, per device

// Device address of the scratch array on the current device; the first call
// on a device looks it up (cudaGetSymbolAddress) with that device current.
static int noalloc_scratch(void** out) {
    int dev = 0;
    F4J_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) return f4j_fail(F4J_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_f4j_noalloc_scratch);
        if (e != cudaSuccess || !p) return f4j_cuda_fail(e, "cudaGetSymbolAddress(no-allocation scratch)");
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return F4J_OK;
}

extern "C" int f4j_dgemm_split_noalloc(int64_t m, int64_t n, int64_t k, const double* A, int opA, const double* B,
                                       int opB, double* C, void* stream, int32_t* slices_out) {
    if (slices_out) *slices_out = 0;
    if (!A || !B || !C) return f4j_fail(F4J_ERR_ARG, "null matrix pointer");
    if (m < 0 || n < 0 || k < 0) return f4j_fail(F4J_ERR_ARG, "negative dimension");
    if (m > INT32_MAX || n > INT32_MAX || k > INT32_MAX)
        return f4j_fail(F4J_ERR_ARG, "dimension exceeds Flag4j's int range");
    if (opA == F4J_OP_C) opA = F4J_OP_T;
    if (opB == F4J_OP_C) opB = F4J_OP_T;
    if (opA < 0 || opA > F4J_OP_T || opB < 0 || opB > F4J_OP_T) return f4j_fail(F4J_ERR_ARG, "bad op");
    cudaStream_t st = (cudaStream_t)stream;
    if (m == 0 || n == 0) return F4J_OK;
    if (k == 0) {
        F4J_CUDA(cudaMemsetAsync(C, 0, (size_t)m * n * 8, st));
        return F4J_OK;
    }
    const int64_t M = m, N = n;
    const int64_t Kp = f4j_cdiv(k, BKB) * BKB;
    if (F4J_NOALLOC_NEED(M, N, Kp) > F4J_NOALLOC_SCRATCH_BYTES)
        return f4j_fail(F4J_ERR_ARG,
                        "f4j_dgemm_split_noalloc: m=%lld n=%lld k=%lld needs %zu bytes of scratch "
                        "(12*(m+n)*roundup(k,64) + 24*(m+n) + 16384), more than the %u-byte static limit; "
                        "use f4j_dgemm",
                        (long long)m, (long long)n, (long long)k, F4J_NOALLOC_NEED(M, N, Kp),
                        F4J_NOALLOC_SCRATCH_BYTES);
    const size_t off_mxa = 0, off_esa = off_mxa + al1k(M * 8), off_cna = off_esa + al1k(M * 8);
    const size_t off_mxb = off_cna + al1k(M * 4), off_esb = off_mxb + al1k(N * 8), off_cnb = off_esb + al1k(N * 8);
    const size_t off_ea = off_cnb + al1k(N * 4), off_eb = off_ea + al1k(M * 4);
    const size_t off_misc = off_eb + al1k(N * 4);
    const size_t off_plan = off_misc + 1024;
    const size_t off_sl = off_plan + al1k(sizeof(SplitPlan));
    if (off_sl + al1k((size_t)M * Kp * S_MAX) + al1k((size_t)N * Kp * S_MAX) > F4J_NOALLOC_NEED(M, N, Kp))
        return f4j_fail(F4J_ERR_UNSUPPORTED, "f4j_dgemm_split_noalloc: scratch layout exceeds its stated bound");
    void* base;
    int rc = noalloc_scratch(&base);
    if (rc) return rc;
    int dev = 0, sms = 0;
    F4J_CUDA(cudaGetDevice(&dev));
    F4J_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    char* w = (char*)base;
    unsigned long long* mxa = (unsigned long long*)(w + off_mxa);
    long long* esa = (long long*)(w + off_esa);
    int* cna = (int*)(w + off_cna);
    unsigned long long* mxb = (unsigned long long*)(w + off_mxb);
    long long* esb = (long long*)(w + off_esb);
    int* cnb = (int*)(w + off_cnb);
    int* ea = (int*)(w + off_ea);
    int* eb = (int*)(w + off_eb);
    int* misc = (int*)(w + off_misc);  // [0] non-finite input, [1..2] spreads, [8] wait status
    SplitPlan* plan = (SplitPlan*)(w + off_plan);
    // statistics accumulate with atomics and the status word must read 0
    F4J_CUDA(cudaMemsetAsync(w, 0, off_ea, st));
    F4J_CUDA(cudaMemsetAsync(w + off_misc, 0, 1024, st));

    const bool a_rows = (opA == F4J_OP_N), b_rows = (opB != F4J_OP_N);
    if (a_rows) k_stats_rows<<<(unsigned)f4j_cdiv(M, 8), 256, 0, st>>>(A, M, k, 0, mxa, esa, cna, misc);
    else launch_stats_cols(A, k, M, M, 0, sms, mxa, esa, cna, misc, st);
    if (b_rows) k_stats_rows<<<(unsigned)f4j_cdiv(N, 8), 256, 0, st>>>(B, N, k, 0, mxb, esb, cnb, misc);
    else launch_stats_cols(B, k, N, N, 0, sms, mxb, esb, cnb, misc, st);
    k_stats_finalize<<<(unsigned)f4j_cdiv(M, 256), 256, 0, st>>>(M, 0, mxa, esa, cna, ea, misc + 1);
    k_stats_finalize<<<(unsigned)f4j_cdiv(N, 256), 256, 0, st>>>(N, 0, mxb, esb, cnb, eb, misc + 2);
    int kchunks_na = 0;  // the same chunks as f4j_dgemm plans for this shape, run in turn
    const int kcb_cap = split_kcb_cap(f4j_cdiv(M, BM) * f4j_cdiv(N, BN), Kp / BKB, &kchunks_na);
    k_plan<<<1, 32, 0, st>>>(misc, k, Kp, k, env_slices(), env_band(), kcb_cap, plan);
    F4J_CUDA(cudaGetLastError());
    // The slicing and slice GEMM kernels read the plan's verdict on the device
    // and return at once for a NaN/Inf operand or a plan that does not fit.
    uint8_t* slA = (uint8_t*)(w + off_sl);
    uint8_t* slB = slA + al1k((size_t)M * Kp * S_MAX);
    k_split<false><<<dim3((unsigned)(Kp / SP_TQ), slice_grid_y(M)), 256, 0, st>>>(
        A, a_rows ? M : k, a_rows ? k : M, a_rows ? 0 : 1, 0, 0, M, k, Kp, Kp, M, ea, plan, slA);
    k_split<false><<<dim3((unsigned)(Kp / SP_TQ), slice_grid_y(N)), 256, 0, st>>>(
        B, b_rows ? N : k, b_rows ? k : N, b_rows ? 0 : 1, 0, 1, N, k, Kp, Kp, N, eb, plan, slB);
    F4J_CUDA(cudaGetLastError());
    CUtensorMap ta{}, tb{};
    rc = make_slice_map(&ta, slA, Kp, M, S_MAX);
    if (rc) return rc;
    rc = make_slice_map(&tb, slB, Kp, N, S_MAX);
    if (rc) return rc;
    SplitGemmParams prm{};
    prm.M = (int)M;
    prm.N = (int)N;
    prm.Kp = (int)Kp;
    prm.cplx = 0;
    prm.n_out = (int)N;
    prm.ea = ea;
    prm.eb = eb;
    prm.C = C;
    prm.status = misc + 8;
    prm.plan = plan;
    prm.tm0 = 0;
    prm.tm1 = (int)f4j_cdiv(M, BM);
    prm.tn0 = 0;
    prm.tn1 = (int)f4j_cdiv(N, BN);
    const size_t smem = (size_t)RING * TILE_BYTES + 1024 + sizeof(SplitPlan) + (size_t)NSTAGE * MAX_OPS * sizeof(Op);
    F4J_CUDA(cudaFuncSetAttribute(k_split_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t ntiles = f4j_cdiv(N, BN) * f4j_cdiv(M, BM);
    const unsigned grid = (unsigned)(ntiles < sms ? ntiles : sms);
    k_split_gemm<<<grid, GEMM_THREADS, smem, st>>>(ta, tb, prm);
    F4J_CUDA(cudaGetLastError());
    // One wait, after all the work: the plan header (s, nrounds, ubits,
    // nonfinite), the input flag and the slice GEMM's wait status.
    int hp[4], hm[9];
    F4J_CUDA(cudaMemcpyAsync(hp, plan, sizeof hp, cudaMemcpyDeviceToHost, st));
    F4J_CUDA(cudaMemcpyAsync(hm, misc, sizeof hm, cudaMemcpyDeviceToHost, st));
    F4J_CUDA(cudaStreamSynchronize(st));
    if (hm[8])
        return f4j_fail(F4J_ERR_TIMEOUT,
                        "f4j_dgemm_split_noalloc: a device-side wait gave up (code %d); C is incomplete", hm[8]);
    if (hm[0])
        return f4j_fail(F4J_ERR_ARG,
                        "f4j_dgemm_split_noalloc: NaN or Inf in an operand; C is not written; use f4j_dgemm (AUTO)");
    if (hp[3])
        return f4j_fail(F4J_ERR_UNSUPPORTED,
                        "f4j_dgemm_split_noalloc: no split plan fits this shape; C is not written; use f4j_dgemm");
    if (slices_out) *slices_out = hp[0];
    return F4J_OK;
}

#ifdef F4J_TRACE
// Development build only: returns and clears the slice GEMM's trace counters
// (cycles summed over CTAs): [0] MMA thread total, [1] its full-barrier
// waits, [2] its accumulator-buffer waits, [3] MMA ops issued, [4] producer
// total, [5] producer slot waits, [6] epilogue total, [7] epilogue waits.
extern "C" int f4j_debug_trace(unsigned long long* out8) {
    F4J_CUDA(cudaDeviceSynchronize());
    F4J_CUDA(cudaMemcpyFromSymbol(out8, g_f4j_trace, 8 * sizeof(unsigned long long)));
    unsigned long long z[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    F4J_CUDA(cudaMemcpyToSymbol(g_f4j_trace, z, sizeof z));
    return F4J_OK;
}
#endif
