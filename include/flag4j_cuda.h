/*
 * flag4j_cuda.h -- C ABI of libflag4j_cuda.so, the GB300 (sm_103a) engine for
 * Flag4j's product path: dense real / complex GEMM and CSR x dense products.
 *
 * Flag4j has no native layer; the seam this library replaces is the Java
 * method + dispatcher pair for each product.  Each entry point below names the
 * reference interface it stands in for (paths within the Flag4j project).
 *
 * Conventions
 *  - Every function returns an int status: F4J_OK (0) or a negative F4J_ERR_*.
 *    f4j_last_error() gives a thread-local message for the last failure on the
 *    calling thread.  Shape errors carry Flag4j's own wording
 *    ("Cannot multiply matrices/vector with shapes (m, k) and (k2, n).").
 *  - Matrices are row-major float64; complex matrices are interleaved
 *    (re, im) float64 pairs, i.e. Flag4j's Complex128[] marshalled to double[2n].
 *  - Operands live in device buffers (f4j_buf) so forward operands can be kept
 *    on the GPU across calls.  Inputs are never modified; outputs are written.
 *  - All work of a context runs in order on that context's CUDA stream; calls
 *    return once the work is queued (use f4j_sync or a download to wait).
 *    Separate contexts are independent.  A context may be shared by threads:
 *    every call on it holds the context's lock until it returns, so calls
 *    from several threads run one at a time (the reference's dispatcher
 *    cache, BiTensorOpDispatcher.java:68-84, is not thread-safe; this layer is).
 *  - No CPU fallback: every product runs as CUDA kernels on the context's GPU.
 */
#ifndef FLAG4J_CUDA_H
#define FLAG4J_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define F4J_OK 0
#define F4J_ERR_ARG (-1)         /* bad argument -> IllegalArgumentException          */
#define F4J_ERR_SHAPE (-2)       /* shape mismatch -> LinearAlgebraException           */
#define F4J_ERR_CSR (-3)         /* invalid CSR/COO -> IllegalArgumentException        */
#define F4J_ERR_OOM (-4)         /* device allocation failed                           */
#define F4J_ERR_CUDA (-5)        /* CUDA runtime / launch error -> Flag4jDeviceException */
#define F4J_ERR_TIMEOUT (-6)     /* a bounded device-side wait gave up                 */
#define F4J_ERR_UNSUPPORTED (-7) /* configuration not supported on this device        */
#define F4J_SELFTEST_WAIT_CODE 99 /* status code of f4j_selftest_wait's expired wait  */

/* ---- operand transforms and GEMM modes ---------------------------------- */
#define F4J_OP_N 0 /* op(X) = X                        */
#define F4J_OP_T 1 /* op(X) = X^T                      */
#define F4J_OP_C 2 /* op(X) = X^H (complex only; = T for real) */

#define F4J_MODE_PLAIN 0 /* FP64 DMMA tensor-core GEMM (mma.sync f64)                   */
#define F4J_MODE_SPLIT 1 /* FP64-accurate split GEMM: FP8 slices on tcgen05, exact FP32 */
#define F4J_MODE_AUTO 2  /* the dispatcher configuration's choice (f4j_config_load): EXACT
                            below smallThreshold entries or 2^24 flops; otherwise
                            gpuGemmMode, by default SPLIT for finite inputs and PLAIN
                            when a NaN/Inf is present                                   */
#define F4J_MODE_EXACT 3 /* Flag4j's own order: k-ascending, no FMA -> bit-identical     */

typedef struct f4j_ctx f4j_ctx;
typedef struct f4j_buf_s* f4j_buf;
typedef struct f4j_csr_s* f4j_csr;

/* Optional per-call report (pass NULL to skip).  Zero it before the call; the
 * call fills the outputs.  Accuracy report (f4j_dgemm, f4j_zgemm,
 * f4j_dgemm_host; no counterpart in Flag4j): with check_samples > 0 the call
 * also evaluates that many seeded entries of its result in double-double
 * (compensated Dot2) on the GPU and reports the largest error, next to the
 * componentwise bound a plain FP64 product guarantees on the same scale; with
 * F4J_CHECK_PLAIN in check_flags it also runs the plain DMMA product into
 * scratch memory and reports that product's error on the same entries.  The
 * check costs one extra kernel and a wait (plus the plain product when asked);
 * without it the call is unchanged. */
#define F4J_CHECK_PLAIN 1
/* Entry s (0-based) of a check is C[i][j] with b = mix(F4J_CHECK_SEED),
 * i = mix(b ^ 2s) mod m, j = mix(b ^ (2s + 1)) mod n, mix the splitmix64
 * finaliser (f4j_gemm_check samples the same way with its own seed). */
#define F4J_CHECK_SEED 0x5EED0F4A6D5EEDull
typedef struct f4j_report {
    int32_t mode_used;        /* F4J_MODE_* that actually ran                             */
    int32_t slices;           /* SPLIT: slice count s per operand                         */
    int32_t launches;         /* kernels this call launched                               */
    int32_t frac_bits;        /* SPLIT: fixed-point bits kept per element (4 + 5(s-1))    */
    double flops;             /* algorithmic flops: 2mnk real, 8mnk complex, 2*nnz*cols   */
    double bytes;             /* algorithmic (compulsory) bytes of sparse products        */
    double exp_spread;        /* SPLIT: measured exponent spread of the operands (bits)   */
    int32_t check_samples;    /* in: entries of C to check (0: no accuracy report)        */
    int32_t check_flags;      /* in: F4J_CHECK_PLAIN                                      */
    double max_abs_err;       /* out: max |C - C_true| over the checked entries           */
    double max_rel_err;       /* out: max |C - C_true| / sum_k |a||b| over the same        */
    double plain_bound_rel;   /* out: k u (real) or 2k u (complex, per part): the bound a  */
                              /*      plain FP64 product guarantees, on max_rel_err's scale */
    double plain_max_abs_err; /* out: the plain DMMA product's max_abs_err (F4J_CHECK_PLAIN; else -1) */
    double plain_max_rel_err; /* out: the plain DMMA product's max_rel_err (F4J_CHECK_PLAIN; else -1) */
    int32_t ref_kernel;       /* out: F4J_REF_* kernel Flag4j's dispatcher runs for these shapes */
    int32_t reserved;
} f4j_report;

/* ---- dispatcher configuration (./configs/*.properties) ------------------- */
/* Flag4j's dense-product dispatchers read java.util.Properties files from
 * ./configs at class initialisation and fall back to defaults when a file is
 * absent:
 *   ReDeMatMult.properties    ReDeMatMultDispatchConfigs
 *     (src/main/java/org/flag4j/linalg/ops/dispatch/configs/ReDeMatMultDispatchConfigs.java:52-121)
 *   CmDeMatMult.properties    Cm128DeMatMultDispatchConfigs (same directory, :52-108)
 *   GeneralConfigs.properties Configurations
 *     (src/main/java/org/flag4j/concurrency/Configurations.java:65-88)
 * This library reads the same files, keys, defaults and number syntax
 * (Integer.parseInt / Double.parseDouble), plus the key
 *   gpuGemmMode = auto | split | plain | exact
 * (GeneralConfigs.properties for both dispatchers; ReDeMatMult.properties /
 * CmDeMatMult.properties override it per dispatcher).  F4J_MODE_AUTO then
 * resolves as the reference's dispatch() does first
 * (ReDeMatMultDispatcher.java:157-171, Cm128DeMatMultDispatcher.java:155-170):
 *   dataLength(A) + dataLength(B) < smallThreshold   -> F4J_MODE_EXACT
 *   otherwise, products of at most 2^24 flops        -> F4J_MODE_EXACT
 *   otherwise gpuGemmMode (auto: SPLIT, with PLAIN for NaN/Inf operands).
 * The files are read on the first AUTO product from ./configs relative to the
 * working directory (a malformed file there leaves the defaults), or when
 * f4j_config_load is called. */
typedef struct f4j_dispatch_config {
    double cache_size;                       /* cacheSize (the reference's shape-cache size)      */
    double aspect_threshold;                 /* aspectThreshold                                    */
    int32_t small_threshold;                 /* smallThreshold: entries of A plus B                */
    int32_t square_mt_standard_threshold;    /* squareMtStandardThreshold                          */
    int32_t square_mt_reordered_threshold;   /* squareMtReorderedThreshold                         */
    int32_t wide_mt_reordered_threshold;     /* wideMtReorderedThreshold                           */
    int32_t square_sequential_vec_threshold; /* squareSequentialVecThreshold (real only)           */
    int32_t min_dim_small_threshold;         /* minDimSmallThreshold                               */
    int32_t gpu_gemm_mode;                   /* F4J_MODE_* that AUTO uses above the small rules   */
    int32_t loaded;                          /* 1 when the dispatcher's file was read             */
} f4j_dispatch_config;

/* The CPU kernels the reference's dispatchers choose between
 * (ReDeMatMultDispatcher.getFunc, ReDeMatMultDispatcher.java:184-237;
 *  Cm128DeMatMultDispatcher.getFunc, Cm128DeMatMultDispatcher.java:184-226). */
enum {
    F4J_REF_STRD = 0, F4J_REF_REORD, F4J_REF_BLK, F4J_REF_BLK_REORD, F4J_REF_MT_STRD, F4J_REF_MT_REORD,
    F4J_REF_MT_BLK, F4J_REF_MT_BLK_REORD, F4J_REF_STRD_VEC_AS_MAT, F4J_REF_BLK_VEC_AS_MAT,
    F4J_REF_MT_STRD_VEC_AS_MAT, F4J_REF_MT_BLK_VEC_AS_MAT
};

/* Reads dir/ReDeMatMult.properties, dir/CmDeMatMult.properties and
 * dir/GeneralConfigs.properties (dir NULL: "./configs"); absent files keep the
 * defaults.  F4J_ERR_ARG (message with Java's NumberFormatException text) for
 * a value Integer.parseInt / Double.parseDouble would reject, or a bad
 * gpuGemmMode; the previous configuration then stays in force. */
int f4j_config_load(const char* dir);
/* Back to the built-in defaults (no files). */
int f4j_config_reset(void);
/* The configuration in force for real (cplx 0) or complex (cplx 1) products. */
int f4j_config_get(int cplx, f4j_dispatch_config* out);
/* GeneralConfigs.properties: blockSize and the resolved parallelism
 * (ThreadManager.setParallelismLevel: values <= 0 mean processors + value, at least 1). */
int f4j_config_general(int32_t* block_size, int32_t* parallelism);
/* The mode a product C (m x n) = A (m x k) B (k x n) runs in under `mode`
 * (F4J_MODE_AUTO resolved by the rules above), and the reference kernel
 * (F4J_REF_*) Flag4j's dispatcher would run for the same shapes. */
int f4j_dispatch(int cplx, int64_t m, int64_t n, int64_t k, int mode, int32_t* mode_out, int32_t* ref_kernel_out);
/* Name of an F4J_REF_* kernel as the dispatcher spells it ("MT_BLK_REORD"). */
const char* f4j_ref_kernel_name(int code);

/* ---- library / context --------------------------------------------------- */
int f4j_version(void); /* 10000*major + 100*minor + patch */
const char* f4j_last_error(void);
int f4j_create(int device, f4j_ctx** out);
int f4j_destroy(f4j_ctx* ctx);
int f4j_sync(f4j_ctx* ctx);
/* Diagnostic of the bounded device waits (no Flag4j counterpart): queues a
 * kernel whose wait on an mbarrier that nothing completes gives up after
 * limit_us (1 ms .. 2 s), as the GEMM kernels' waits do after about 2 s.  The
 * next f4j_sync then returns F4J_ERR_TIMEOUT (message with code
 * F4J_SELFTEST_WAIT_CODE), consumes the status, and the context stays usable. */
int f4j_selftest_wait(f4j_ctx* ctx, int64_t limit_us);
/* Run this context's work on an existing cudaStream_t (NULL = own stream). */
int f4j_set_stream(f4j_ctx* ctx, void* cuda_stream);
void* f4j_get_stream(f4j_ctx* ctx);
/* Kernels launched by this context so far. */
int64_t f4j_launch_count(f4j_ctx* ctx);
/* CUDA-event timing on the context stream: record into slot (0..15), then
 * read the elapsed ms between two recorded slots (synchronises the end slot). */
int f4j_timer_record(f4j_ctx* ctx, int slot);
int f4j_timer_elapsed(f4j_ctx* ctx, int slot_begin, int slot_end, float* ms);
/* Opt-in per-kernel timing: with profiling on, kernels are bracketed by CUDA
 * events tagged 0 (the product kernel: slice GEMM, DMMA GEMM, SpMV, SpMM, ...)
 * or 1 (preparation: exponent statistics, slicing, structure).  read returns
 * the summed ms and count for one tag (-1: all) since the last reset
 * (synchronises); set_profiling and reset clear the record. */
int f4j_set_profiling(f4j_ctx* ctx, int on);
int f4j_profile_read(f4j_ctx* ctx, int tag, double* total_ms, int64_t* count);
int f4j_profile_reset(f4j_ctx* ctx);

/* ---- device buffers ------------------------------------------------------ */
int f4j_buf_alloc(f4j_ctx* ctx, size_t bytes, f4j_buf* out);
int f4j_buf_free(f4j_ctx* ctx, f4j_buf buf);
size_t f4j_buf_size(f4j_buf buf);
void* f4j_buf_device_ptr(f4j_buf buf);
/* Copies are stream-ordered.  Synchronous variants wait for completion;
 * async variants return at once (host memory must stay valid, and should be
 * pinned, until the stream reaches the copy). */
int f4j_buf_upload(f4j_ctx* ctx, f4j_buf buf, const void* host, size_t bytes, size_t offset);
int f4j_buf_download(f4j_ctx* ctx, f4j_buf buf, void* host, size_t bytes, size_t offset);
int f4j_buf_upload_async(f4j_ctx* ctx, f4j_buf buf, const void* host, size_t bytes, size_t offset);
int f4j_buf_download_async(f4j_ctx* ctx, f4j_buf buf, void* host, size_t bytes, size_t offset);
int f4j_buf_zero(f4j_ctx* ctx, f4j_buf buf);
/* Pin / unpin caller-owned host memory (e.g. a Java MemorySegment). */
int f4j_host_register(void* host, size_t bytes);
int f4j_host_unregister(void* host);
/* Page-locked host memory from the CUDA allocator, for the host-buffer entry
 * points (f4j_dgemm_host) and async copies.  On GB300, copies from it run at
 * the host link's full rate (about 210 GB/s to the device); copies from
 * registered memory that is not 2 MiB aligned measured about 190 GB/s. */
int f4j_host_alloc(size_t bytes, void** out);
int f4j_host_free(void* host);
/* A buffer handle over memory the device can address, without copying it:
 * device memory from another allocator, host memory pinned with
 * f4j_host_register, or plain host memory where the device walks the host's
 * page tables.  Kernels then read and write that memory in place; for host
 * memory each access crosses the host link (on GB300 a split product writing
 * its 8192^2 C this way ran about 1 ms slower than writing device memory and
 * downloading it, so this is for callers that cannot spare the device copy).
 * ptr must be 16-byte aligned.  The handle does not own the
 * memory: f4j_buf_free releases the handle only.  F4J_ERR_ARG if the device
 * cannot address ptr.  No counterpart in Flag4j, whose matrices live in Java
 * heap arrays. */
int f4j_buf_wrap(f4j_ctx* ctx, void* ptr, size_t bytes, f4j_buf* out);

/* ---- dense products ------------------------------------------------------ */
/* C(m x n) = op(A) * op(B), op(A) m x k, op(B) k x n, real float64.
 * Replaces Matrix.mult -> ReDeMatMultDispatcher.dispatch
 *   (src/main/java/org/flag4j/arrays/dense/Matrix.java:638-640,
 *    src/main/java/org/flag4j/linalg/ops/dispatch/ReDeMatMultDispatcher.java:157-237)
 * and, with opB = F4J_OP_T, Matrix.multTranspose
 *   (Matrix.java:655-663, RealDenseMatrixMultiplyDispatcher.java:148-154).
 * A is stored m x k (opA N) or k x m (opA T); B k x n (N) or n x k (T). */
int f4j_dgemm(f4j_ctx* ctx, int64_t m, int64_t n, int64_t k, f4j_buf A, int opA, f4j_buf B,
              int opB, f4j_buf C, int mode, f4j_report* report);
/* f4j_dgemm from and to host memory: A, B, C are host pointers (row-major;
 * page-locked by f4j_host_alloc or f4j_host_register for full copy speed,
 * pageable works), and the call returns when C is in host memory.  A split
 * product with opA = N is pipelined: A's first rows are uploaded first, then B
 * in column parts, then the rest of A in row parts, back to back; each part is
 * sliced as it arrives and each product (B's column parts by A's first rows,
 * then A's later row parts by all of B) runs on its own stream, its block of C
 * downloaded behind it.  The slice count is taken from the first parts of A
 * and B; when all of A and B ask for another count (or an operand holds a
 * NaN / Inf) the product runs again through the f4j_dgemm path.  A
 * product that splits K (fewer than 152 output tiles and K <= 4096), fits one
 * 128 x 128 tile of C, or has opA != N uploads, multiplies and downloads in
 * turn.  The result is bitwise the f4j_dgemm result.  This is
 * the entry a JVM binding calls with its arrays' native copies for Flag4j's
 * Matrix.mult(Matrix) (src/main/java/org/flag4j/arrays/dense/Matrix.java:638-640),
 * same arguments and result. */
int f4j_dgemm_host(f4j_ctx* ctx, int64_t m, int64_t n, int64_t k, const double* A, int opA, const double* B,
                   int opB, double* C, int mode, f4j_report* report);
/* f4j_zgemm from and to host memory: A, B, C are interleaved (re, im) complex
 * host arrays (Flag4j's Complex128[] marshalled to double[2n]), opA, opB in
 * {N, T, C}; same contract as f4j_dgemm_host.  A split product with opA = N
 * is pipelined with B uploaded whole (its column parts would fall on both
 * halves of the [Re | Im] concatenation) and A in row parts; the result is
 * bitwise the f4j_zgemm result.  This is the entry a JVM binding calls with
 * the marshalled arrays for CMatrix.mult(CMatrix)
 * (src/main/java/org/flag4j/arrays/dense/CMatrix.java:463-465) and, with
 * opB = F4J_OP_T, CMatrix.multTranspose (this.mult(b.T()),
 * src/main/java/org/flag4j/arrays/backend/semiring_arrays/
 * AbstractDenseSemiringMatrix.java:330-334); non-square results are returned
 * correctly where the reference's kernels mis-size them
 * (Cm128DeMatMultKernels.java:46-77). */
int f4j_zgemm_host(f4j_ctx* ctx, int64_t m, int64_t n, int64_t k, const double* A, int opA, const double* B,
                   int opB, double* C, int mode, f4j_report* report);
/* Host pinning for the host-buffer products (f4j_dgemm_host, f4j_zgemm_host;
 * off by default, no counterpart in Flag4j).  On, each call page-locks A, B
 * and C for its duration (cudaHostRegister) and releases them before it
 * returns; arrays already page-locked, or whose pages cannot be registered,
 * are used as they are.  For callers whose arrays are pageable and live only
 * for the call: a JVM binding passing Java heap arrays through a critical
 * downcall (Linker.Option.critical(true)), where registering costs about 1-2
 * ms per 512 MiB operand against about 37 ms to copy it into native memory,
 * and the copies then run at the page-locked rate. */
int f4j_set_host_pinning(f4j_ctx* ctx, int on);

/* Complex128 C = op(A) * op(B), interleaved (re, im); op may be N, T or C.
 * Replaces CMatrix.mult -> Cm128DeMatMultDispatcher.dispatch
 *   (src/main/java/org/flag4j/arrays/dense/CMatrix.java:463-465,
 *    src/main/java/org/flag4j/linalg/ops/dispatch/Cm128DeMatMultDispatcher.java:155-226). */
int f4j_zgemm(f4j_ctx* ctx, int64_t m, int64_t n, int64_t k, f4j_buf A, int opA, f4j_buf B,
              int opB, f4j_buf C, int mode, f4j_report* report);

/* Reverse-mode adjoint of C = A * B (A m x k, B k x n, both op N):
 *   dA = dC * B^T (m x k),  dB = A^T * dC (k x n)   (real)
 *   dA = dC * B^H,          dB = A^H * dC           (complex: f4j_zgemm_adjoint)
 * run on the same GEMM kernels with transposed operand descriptors (no
 * transpose is materialised).  Either output may be NULL to skip it.
 * No Flag4j counterpart (Flag4j has no autodiff); its CPU oracle is
 * W.multTranspose(B) and A.T().mult(W). */
int f4j_dgemm_adjoint(f4j_ctx* ctx, int64_t m, int64_t n, int64_t k, f4j_buf A, f4j_buf B,
                      f4j_buf dC, f4j_buf dA, f4j_buf dB, int mode, f4j_report* report);
int f4j_zgemm_adjoint(f4j_ctx* ctx, int64_t m, int64_t n, int64_t k, f4j_buf A, f4j_buf B,
                      f4j_buf dC, f4j_buf dA, f4j_buf dB, int mode, f4j_report* report);

/* No-allocation variant of the split GEMM (no counterpart in the reference).
 * For callers that may not allocate device memory: engines that own a fixed
 * memory pool and forbid allocation after start-up, and JVM or other hosts
 * that only pass in buffers they already hold.  Same arithmetic as
 * f4j_dgemm(..., F4J_MODE_SPLIT, ...) on real float64, bitwise; A, B and C are
 * the caller's device pointers, `stream` a cudaStream_t (NULL = default
 * stream).  Scratch comes from a static 32 MiB device array inside the library
 * (held on every GPU that loads it until exit); a call is rejected with
 * F4J_ERR_ARG exactly when
 *   12 * (m + n) * roundup(k, 64) + 24 * (m + n) + 16384 > 32 MiB
 * (e.g. 1024 x 1024 x 1344 fits, 1024 x 1024 x 1408 does not).  The first call
 * on a device looks up the array's address (cudaGetSymbolAddress), so make
 * that call before any stream capture.  All calls share the array and it
 * keeps the last call's contents: calls whose GPU work overlaps race.  The
 * call queues its kernels on `stream`, then waits for them once and returns
 * F4J_OK with C written; F4J_ERR_ARG for a NaN/Inf operand and
 * F4J_ERR_UNSUPPORTED when no split plan fits (C not written; f4j_dgemm
 * handles both); F4J_ERR_TIMEOUT when a bounded device wait gave up (C
 * incomplete).  Calls no cudaMalloc/cudaFree or allocating library routine.
 * `slices_out` (may be NULL) receives the slice count used. */
int f4j_dgemm_split_noalloc(int64_t m, int64_t n, int64_t k, const double* A, int opA, const double* B,
                            int opB, double* C, void* stream, int32_t* slices_out);

/* Sampled accuracy check of a computed C = op(A) op(B): evaluates `samples`
 * seeded entries in double-double (compensated Dot2) on the GPU and returns
 * max |C - C_true| and max |C - C_true| / sum|a||b| over the samples. */
int f4j_gemm_check(f4j_ctx* ctx, int cplx, int64_t m, int64_t n, int64_t k, f4j_buf A, int opA,
                   f4j_buf B, int opB, f4j_buf C, int64_t samples, uint64_t seed,
                   double* max_abs_err, double* max_rel_err);

/* ---- CSR matrices ---------------------------------------------------------- */
/* Wrap device arrays as a CSR matrix (rowptr int32[rows+1], colidx int32[nnz],
 * vals float64[nnz]); the handle borrows the buffers.  validate != 0 runs
 * SparseValidation.validateCsr's checks on the GPU
 *   (src/main/java/org/flag4j/arrays/sparse/SparseValidation.java:151-206;
 *    constructor CsrMatrix.java:175-185). */
int f4j_csr_wrap(f4j_ctx* ctx, int64_t rows, int64_t cols, int64_t nnz, f4j_buf rowptr,
                 f4j_buf colidx, f4j_buf vals, int validate, f4j_csr* out);
/* Build CSR from COO triplets exactly as CooMatrix.toCsr does
 *   (src/main/java/org/flag4j/arrays/sparse/CooMatrix.java:457-470):
 * rowptr = inclusive scan of per-row counts; colidx and vals are copied
 * unchanged (so the COO must already be row-sorted).  The new handle owns
 * its three buffers. */
int f4j_csr_from_coo(f4j_ctx* ctx, int64_t rows, int64_t cols, int64_t nnz, f4j_buf rowidx,
                     f4j_buf colidx, f4j_buf vals, f4j_csr* out);
/* Stable lexicographic (row, col) sort of COO triplets in place, as
 * CooMatrix.sortIndices -> CooDataSorter.sparseSort
 *   (CooMatrix.java:476-479, src/main/java/org/flag4j/linalg/ops/sparse/coo/
 *    CooDataSorter.java:176-259). vals may be NULL. */
int f4j_coo_sort(f4j_ctx* ctx, int64_t nnz, f4j_buf rowidx, f4j_buf colidx, f4j_buf vals);
int f4j_csr_free(f4j_ctx* ctx, f4j_csr csr);
int f4j_csr_info(f4j_csr csr, int64_t* rows, int64_t* cols, int64_t* nnz);
int f4j_csr_buffers(f4j_csr csr, f4j_buf* rowptr, f4j_buf* colidx, f4j_buf* vals);
/* Materialised transpose, CsrMatrix.T() -> RealCsrOps.transpose
 *   (CsrMatrix.java:1431-1433, src/main/java/org/flag4j/linalg/ops/sparse/csr/real/
 *    RealCsrOps.java:195-225); bit-identical structure and order. */
int f4j_csr_transpose(f4j_ctx* ctx, f4j_csr S, f4j_csr* out);
/* Copy out the cached transpose permutation (int32[nnz]: for each position of
 * S^T in RealCsrOps.transpose order, the source nnz index of S). */
int f4j_csr_transpose_perm(f4j_ctx* ctx, f4j_csr S, f4j_buf perm_out);
/* CSR x CSR with a dense result, CsrMatrix.mult(CsrMatrix) ->
 *   RealCsrMatMult.standard (CsrMatrix.java:748-749,
 *   src/main/java/org/flag4j/linalg/ops/sparse/csr/real/RealCsrMatMult.java:53-75):
 *   C (A.rows x B.cols, row-major, overwritten) accumulates a * b over A's row
 *   nonzeros in storage order, each product and sum rounded; bit-identical.
 *   CsrMatrix.multTranspose(CsrMatrix) (CsrMatrix.java:809-810) is this with
 *   f4j_csr_transpose(B).  F4J_ERR_SHAPE when A.cols != B.rows. */
int f4j_csr_mult_dense(f4j_ctx* ctx, f4j_csr A, f4j_csr B, f4j_buf C, f4j_report* report);
/* CSR x CSR with a CSR result (owned by *out), CsrMatrix.mult2Csr(CsrMatrix) ->
 *   RealCsrMatMult.standardAsSparse (CsrMatrix.java:778-779,
 *   RealCsrMatMult.java:92-131): every column a row's products touch is
 *   stored, ascending, even where the products cancel; per entry the products
 *   are summed in the reference's loop order starting from the first
 *   (HashMap.merge).  Bit-identical.  F4J_ERR_UNSUPPORTED when the product
 *   count (sum over A's nonzeros of the length of B's row) exceeds 2^31 - 1. */
int f4j_csr_mult_csr(f4j_ctx* ctx, f4j_csr A, f4j_csr B, f4j_csr* out, f4j_report* report);
/* The same two products for complex operands: a_complex / b_complex say
 * whether A's / B's values are complex (interleaved, 16 * nnz bytes); the
 * result (C, or *out's values) is complex when either is.
 *   real x complex  CsrMatrix.mult(CsrCMatrix) / mult2Csr(CsrCMatrix) ->
 *     RealComplexCsrMatMult.standard / standardAsSparse
 *     (src/main/java/org/flag4j/linalg/ops/sparse/csr/real_complex/
 *      RealComplexCsrMatMult.java:58-83, :133-181): per part b * a
 *   complex x real  CsrCMatrix.mult(CsrMatrix) / mult2Csr(CsrMatrix)
 *     (same file :93-118, :190-238): per part a * b
 *   complex x complex  CsrCMatrix.mult(CsrCMatrix) / mult2Csr(CsrCMatrix) ->
 *     SemiringCsrMatMult.standard / standardToSparse
 *     (…/semiring_ops/SemiringCsrMatMult.java:58-87, :109-158) with
 *     Complex128.mult(b, a) (Complex128.java:336-341)
 * each product and sum rounded as there; bit-identical. */
int f4j_csr_mult_dense_ex(f4j_ctx* ctx, f4j_csr A, int a_complex, f4j_csr B, int b_complex, f4j_buf C,
                          f4j_report* report);
int f4j_csr_mult_csr_ex(f4j_ctx* ctx, f4j_csr A, int a_complex, f4j_csr B, int b_complex, f4j_csr* out,
                        f4j_report* report);

/* y = S x.  Replaces CsrMatrix.mult(Vector) -> RealCsrDenseMatMult.standardVector
 *   (CsrMatrix.java:1170-1171, src/main/java/org/flag4j/linalg/ops/dense_sparse/csr/
 *    real/RealCsrDenseMatMult.java:172-192).  Bit-identical: each y[i] is summed in
 * storage order with separately rounded products, like the reference. */
int f4j_spmv(f4j_ctx* ctx, f4j_csr S, f4j_buf x, f4j_buf y, f4j_report* report);
/* Y(rows x ncols) = S X, X cols x ncols row-major.  Replaces CsrMatrix.mult(Matrix)
 * -> RealCsrDenseMatMult.standard (CsrMatrix.java:1498-1499,
 * RealCsrDenseMatMult.java:55-82).  Bit-identical. */
int f4j_spmm(f4j_ctx* ctx, f4j_csr S, f4j_buf X, int64_t ncols, f4j_buf Y, f4j_report* report);
/* Rounding modes of the real CSR products: F4J_SPARSE_EXACT is the reference's
 * order (each product and each sum rounded; f4j_spmv / f4j_spmm); F4J_SPARSE_FMA
 * accumulates fma(v, x, acc) in the same storage order, one FP64 instruction
 * per term instead of two, within the componentwise bound
 * |y - y_ref| <= 2 k u |S||x| (k = the row length).  GB300's FP64 pipe bounds
 * the exact products; FMA halves that work.  No counterpart in Flag4j. */
enum { F4J_SPARSE_EXACT = 0, F4J_SPARSE_FMA = 1 };
int f4j_spmv_ex(f4j_ctx* ctx, f4j_csr S, f4j_buf x, f4j_buf y, int mode, f4j_report* report);
int f4j_spmm_ex(f4j_ctx* ctx, f4j_csr S, f4j_buf X, int64_t ncols, f4j_buf Y, int mode, f4j_report* report);
/* Y(rows x ncols) = S X for a complex CSR S and complex dense X, Y
 * (interleaved re/im): S is a CSR handle whose value buffer holds nnz complex
 * values (16 bytes each, as CsrCMatrix.data).  Bit-identical to
 * CsrCMatrix.mult(CMatrix) -> DenseCsrSemiringMatMult.standard
 * (src/main/java/org/flag4j/linalg/ops/dense_sparse/csr/semiring_ops/
 * DenseCsrSemiringMatMult.java:59-98), ncols = 1 for CsrCMatrix.mult(CVector).
 * A real CSR times a complex dense matrix (CsrMatrix.mult(CMatrix),
 * RealFieldDenseCsrMatMult.java:62-91) is f4j_spmm on X's interleaved storage
 * with 2 * ncols real columns. */
int f4j_zspmm(f4j_ctx* ctx, f4j_csr S, f4j_buf X, int64_t ncols, f4j_buf Y, f4j_report* report);
/* dX(cols x ncols) = S^T dC without forming S^T: gathers through a cached
 * transpose permutation (built on first use); atomic-free.  Bit-identical to
 * S.T().mult(dC) in the reference. */
int f4j_spmm_t(f4j_ctx* ctx, f4j_csr S, f4j_buf dC, int64_t ncols, f4j_buf dX,
               f4j_report* report);
/* SDDMM on S's pattern: out[q] = dot(A[row(q), :], B[col(q), :]) over ncols
 * (A rows x ncols, B cols x ncols) -- the gradient dS = (dC X^T) restricted to
 * pattern(S) for C = S X.  No Flag4j counterpart. */
int f4j_sddmm(f4j_ctx* ctx, f4j_csr S, f4j_buf A, f4j_buf B, int64_t ncols, f4j_buf out,
              f4j_report* report);

#ifdef __cplusplus
}
#endif
#endif /* FLAG4J_CUDA_H */
