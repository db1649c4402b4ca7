// f4j_internal.cuh -- shared declarations of libflag4j_cuda.so (not installed).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <mutex>
#include <cstdio>
#include <string>

#include "../../include/flag4j_cuda.h"

struct f4j_buf_s {
    void* ptr;
    size_t bytes;
    bool owned;   // false for f4j_buf_wrap handles
    bool pooled;  // from the stream-ordered pool (library-made results): freed on the context stream
};

// A library-made result buffer from the stream-ordered pool, ordered on the
// context stream (what the library returns inside handles, e.g. CSR results).
int f4j_buf_alloc_pooled(f4j_ctx* ctx, size_t bytes, f4j_buf* out);

struct f4j_csr_s {
    int64_t rows, cols, nnz;
    f4j_buf rowptr, colidx, vals;
    bool owns;  // true when the handle frees its three buffers
    // Cached transpose structure, built on first f4j_spmm_t / transpose use:
    //   t_rowptr int32[cols+1], t_perm int32[nnz] (source nnz of each S^T slot),
    //   t_rowidx int32[nnz] (row of S for each S^T slot, i.e. S^T's colidx).
    void* t_rowptr;
    void* t_perm;
    void* t_rowidx;
    // Row of each nonzero (int32[nnz]), built on first use by f4j_sddmm.
    void* rowidx;
};

// Parts of a host-buffer split GEMM (a part's upload and slicing overlap the
// earlier parts' products, its download the later ones'): A in F4J_HOST_PARTS
// row parts and B in F4J_HOST_BPARTS column parts by default, each up to
// F4J_HOST_PARTS_MAX through the environment variables of the same names.
// Every part's product is one launch on a stream of its own.
#define F4J_HOST_PARTS 4
#define F4J_HOST_BPARTS 4
#define F4J_HOST_PARTS_MAX 8
#define F4J_HOST_STREAMS (2 * F4J_HOST_PARTS_MAX)

struct f4j_ctx {
    std::recursive_mutex mu;  // held by every C-ABI call on this context (F4J_LOCK)
    int device;
    int sm_count;
    cudaStream_t stream;
    bool own_stream;
    void* ws[8];       // grow-only workspaces (slot ws_base + 0: split bulk, ws_base + 1: split
    size_t ws_bytes[8];  // small/stats; 2: sparse; 4-5: the second product of an adjoint;
                         // 3, 6, 7: A, B, C of f4j_dgemm_host)
    int ws_base;       // first split workspace slot (0, or 4 while an adjoint's second product is queued)
    cudaStream_t aux_stream;  // second stream of an adjoint (created on first use)
    cudaEvent_t ev_fork, ev_join;
    // Streams of the row parts of a host-buffer GEMM (f4j_dgemm_host), created
    // on first use, with an event per part for its slices being ready
    // (part_prep_ev, on the context stream) and its download done (part_ev).
    cudaStream_t part_stream[F4J_HOST_STREAMS];
    cudaEvent_t part_ev[F4J_HOST_STREAMS], part_prep_ev[F4J_HOST_STREAMS];
    // The uploads of a pipelined host-buffer GEMM, back to back on their own
    // stream, with an event per uploaded part and one the stream starts behind.
    cudaStream_t up_stream;
    cudaEvent_t up_ev[F4J_HOST_STREAMS], up_start;
    // Split GEMM plans for every slice count, per workspace base (0 / 4), built
    // when the key (Kp, K length, band, chunk cap) changes.
    void* plan_tab[2];
    long long plan_key[2][4];
    bool plan_valid[2];
    bool parts_init;
    bool host_pin;     // host-buffer products page-lock their arrays per call (f4j_set_host_pinning)
    int* d_status;     // device status words (bounded-wait timeouts, validation)
    cudaEvent_t ev[16];
    bool ev_init[16];
    int64_t launches;
    // Opt-in profiling: CUDA events around product kernels, tagged
    // F4J_PROF_MAIN (the product kernel) or F4J_PROF_PREP (statistics,
    // slicing, structure preparation).
    bool prof;
    int prof_n;
    cudaEvent_t prof_ev[2 * 512];
    int prof_tag[512];
    bool prof_init;
};

enum { F4J_PROF_MAIN = 0, F4J_PROF_PREP = 1 };

// Bracket a kernel with profiling events (no-ops unless profiling is on).
void f4j_prof_begin(f4j_ctx* ctx, int tag = F4J_PROF_MAIN);
void f4j_prof_end(f4j_ctx* ctx);

// ---------------------------------------------------------------- errors
int f4j_fail(int code, const char* fmt, ...);
int f4j_cuda_fail(cudaError_t e, const char* what);

#define F4J_CUDA(call)                                              \
    do {                                                            \
        cudaError_t e__ = (call);                                   \
        if (e__ != cudaSuccess) return f4j_cuda_fail(e__, #call);   \
    } while (0)

// After a kernel launch: record it and surface launch errors.
#define F4J_LAUNCHED(ctx)                                                    \
    do {                                                                     \
        (ctx)->launches++;                                                   \
        cudaError_t e__ = cudaGetLastError();                                \
        if (e__ != cudaSuccess) return f4j_cuda_fail(e__, "kernel launch");  \
    } while (0)

#define F4J_CHECK_CTX(ctx) \
    do { if (!(ctx)) return f4j_fail(F4J_ERR_ARG, "null context"); } while (0)

// First statement of every C-ABI entry that takes a context: the null check,
// then the context's lock until the entry returns (entries that call other
// entries take it again: the mutex is recursive).  Calls from several threads
// on one context therefore run one at a time, in a consistent state.
#define F4J_LOCK(ctx) \
    if (!(ctx)) return f4j_fail(F4J_ERR_ARG, "null context"); \
    std::lock_guard<std::recursive_mutex> f4j_ctx_lock_((ctx)->mu)

// Workspace slot of at least `bytes` (stream-ordered reuse; growing syncs the
// stream and discards the slot's previous contents).
int f4j_workspace(f4j_ctx* ctx, int slot, size_t bytes, void** out);
// Device allocation helpers (stream-ordered pool).
int f4j_dev_alloc(f4j_ctx* ctx, size_t bytes, void** out);
void f4j_dev_free(f4j_ctx* ctx, void* p);
// Reads and clears status word `idx` (synchronises the stream).
int f4j_status_take(f4j_ctx* ctx, int idx, int* value);

// Shape error text of Flag4j's ErrorMessages.matMultShapeErrMsg
// (src/main/java/org/flag4j/util/ErrorMessages.java:52-53, :162-164).
int f4j_shape_error(int64_t r1, int64_t c1, int64_t r2, int64_t c2);

// Status word slots.
enum { F4J_ST_TIMEOUT = 0, F4J_ST_CSR_ROW = 1, F4J_ST_CSR_COL = 2, F4J_ST_NONFINITE = 3,
       F4J_ST_CSR_NEG = 4, F4J_ST_COO_ROW = 5, F4J_ST_COO_COL = 6, F4J_ST_WORDS = 16 };

// TMA descriptor encode (driver entry point, no libcuda link).
typedef CUresult (*f4j_encode_tiled_fn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                        const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                        const cuuint32_t*, CUtensorMapInterleave,
                                        CUtensorMapSwizzle, CUtensorMapL2promotion,
                                        CUtensorMapFloatOOBfill);
f4j_encode_tiled_fn f4j_encode_fn();

static inline int64_t f4j_cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }
static inline bool f4j_aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }
static inline bool f4j_aligned(const void* p, uintptr_t n) { return (reinterpret_cast<uintptr_t>(p) % n) == 0; }

// The mode a dense product runs in: F4J_MODE_AUTO resolved by the dispatcher
// configuration (f4j_config.cu); other modes unchanged.
int f4j_resolve_mode(bool cplx, int64_t m, int64_t n, int64_t k, int mode);

// Fills a dense product's report with its accuracy fields (check_samples,
// check_flags as the caller set them; see f4j_report).
int f4j_report_accuracy(f4j_ctx* ctx, bool cplx, int64_t m, int64_t n, int64_t k, const double* A, int opA,
                        const double* B, int opB, const double* C, int samples, int flags, f4j_report* rep);

// Internal GEMM entry points shared by the dense front ends.
// `gate_out` (may be null): for a split product, the device word of its plan
// that flags a NaN/Inf stand-down; the plan's header (s, nrounds, ubits,
// nonfinite, spread) ends at that word, so a caller can read it after a sync.
int f4j_gemm_impl(f4j_ctx* ctx, bool cplx, int64_t m, int64_t n, int64_t k, const double* A,
                  int opA, const double* B, int opB, double* C, int mode, f4j_report* rep,
                  const int** gate_out = nullptr);
// `gate` (device int, may be null): the DMMA kernel computes only when *gate
// is non-zero -- the split path's NaN/Inf fallback, decided on the device.
// y = op(A) x with FP64 FMA dot products (n == 1 in the non-exact modes); x
// conjugated when conj_x.  A, x, y interleaved when cplx.
int f4j_gemv(f4j_ctx* ctx, bool cplx, int64_t m, int64_t k, const double* A, int opA, const double* x, bool conj_x,
             double* y);
int f4j_gemm_dmma(f4j_ctx* ctx, bool cplx, int64_t m, int64_t n, int64_t k, const double* A,
                  int opA, const double* B, int opB, double* C, const int* gate = nullptr);
// Sampled accuracy of C = op(A) op(B): `samples` seeded entries evaluated in
// double-double (Dot2) on the GPU; max |C - C_true| and max |C - C_true| /
// sum|a||b| (synchronises the stream).
int f4j_check_sampled(f4j_ctx* ctx, bool cplx, int64_t m, int64_t n, int64_t k, const double* A, int opA,
                      const double* B, int opB, const double* C, int64_t samples, uint64_t seed, double* max_abs,
                      double* max_rel);
int f4j_gemm_exact(f4j_ctx* ctx, bool cplx, int64_t m, int64_t n, int64_t k, const double* A,
                   int opA, const double* B, int opB, double* C);
int f4j_gemm_split(f4j_ctx* ctx, bool cplx, int64_t m, int64_t n, int64_t k, const double* A,
                   int opA, const double* B, int opB, double* C, int slices_req,
                   f4j_report* rep, const int** gate);
