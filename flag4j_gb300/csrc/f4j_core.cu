// f4j_core.cu -- contexts, device buffers, errors, timers and the dense
// front ends of libflag4j_cuda.so.
#include <mutex>

#include "f4j_internal.cuh"
#include "f4j_ptx.cuh"

// ------------------------------------------------------------------ errors
static thread_local std::string g_last_error;

int f4j_fail(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int f4j_cuda_fail(cudaError_t e, const char* what) {
    int code = (e == cudaErrorMemoryAllocation) ? F4J_ERR_OOM : F4J_ERR_CUDA;
    return f4j_fail(code, "CUDA error in %s: %s (%s)", what, cudaGetErrorName(e),
                    cudaGetErrorString(e));
}

int f4j_shape_error(int64_t r1, int64_t c1, int64_t r2, int64_t c2) {
    return f4j_fail(F4J_ERR_SHAPE, "Cannot multiply matrices/vector with shapes (%lld, %lld) and (%lld, %lld).",
                    (long long)r1, (long long)c1, (long long)r2, (long long)c2);
}

extern "C" const char* f4j_last_error(void) { return g_last_error.c_str(); }
extern "C" int f4j_version(void) { return 100; }

// ------------------------------------------------------------------ TMA encode
f4j_encode_tiled_fn f4j_encode_fn() {
    static std::once_flag once;
    static f4j_encode_tiled_fn fn = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<f4j_encode_tiled_fn>(p);
    });
    return fn;
}

// ------------------------------------------------------------------ contexts
extern "C" int f4j_create(int device, f4j_ctx** out) {
    if (!out) return f4j_fail(F4J_ERR_ARG, "null output pointer");
    *out = nullptr;
    int ndev = 0;
    F4J_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev)
        return f4j_fail(F4J_ERR_ARG, "device %d out of range (%d devices)", device, ndev);
    F4J_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    F4J_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major < 10)
        return f4j_fail(F4J_ERR_UNSUPPORTED, "device %d is sm_%d%d; this library is built for sm_103a",
                        device, prop.major, prop.minor);
    f4j_ctx* c = new f4j_ctx();
    c->device = device;
    c->sm_count = prop.multiProcessorCount;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return f4j_cuda_fail(e, "cudaStreamCreate");
    }
    c->own_stream = true;
    {   // keep freed pool memory for reuse by later calls (temporaries, CSR results)
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        cudaGetLastError();
    }
    e = cudaMalloc(&c->d_status, F4J_ST_WORDS * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(c->d_status, 0, F4J_ST_WORDS * sizeof(int));
    if (e != cudaSuccess) {
        cudaStreamDestroy(c->stream);
        delete c;
        return f4j_cuda_fail(e, "status allocation");
    }
    *out = c;
    return F4J_OK;
}

extern "C" int f4j_destroy(f4j_ctx* ctx) {
    F4J_CHECK_CTX(ctx);
    std::unique_lock<std::recursive_mutex> lock(ctx->mu);  // waits for a call in flight on another thread
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (int i = 0; i < 16; i++)
        if (ctx->ev_init[i]) cudaEventDestroy(ctx->ev[i]);
    if (ctx->prof_init)
        for (int i = 0; i < 1024; i++) cudaEventDestroy(ctx->prof_ev[i]);
    if (ctx->aux_stream) {
        cudaStreamSynchronize(ctx->aux_stream);
        cudaStreamDestroy(ctx->aux_stream);
        cudaEventDestroy(ctx->ev_fork);
        cudaEventDestroy(ctx->ev_join);
    }
    if (ctx->parts_init) {
        for (int i = 0; i < F4J_HOST_STREAMS; i++) {
            cudaStreamSynchronize(ctx->part_stream[i]);
            cudaStreamDestroy(ctx->part_stream[i]);
            cudaEventDestroy(ctx->part_ev[i]);
            cudaEventDestroy(ctx->part_prep_ev[i]);
            cudaEventDestroy(ctx->up_ev[i]);
        }
        cudaStreamSynchronize(ctx->up_stream);
        cudaStreamDestroy(ctx->up_stream);
        cudaEventDestroy(ctx->up_start);
    }
    for (int i = 0; i < 8; i++)
        if (ctx->ws[i]) cudaFree(ctx->ws[i]);
    for (int i = 0; i < 2; i++)
        if (ctx->plan_tab[i]) cudaFree(ctx->plan_tab[i]);
    if (ctx->d_status) cudaFree(ctx->d_status);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    lock.unlock();
    delete ctx;
    return F4J_OK;
}

extern "C" int f4j_sync(f4j_ctx* ctx) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    F4J_CUDA(cudaStreamSynchronize(ctx->stream));
    int t = 0;
    int rc = f4j_status_take(ctx, F4J_ST_TIMEOUT, &t);
    if (rc) return rc;
    if (t) return f4j_fail(F4J_ERR_TIMEOUT, "a device-side wait gave up (code %d)", t);
    return F4J_OK;
}

// Self-test of the bounded device waits: one thread waits on an mbarrier
// phase that nothing completes, with the wait primitive the GEMM kernels use,
// gives up after limit_ns, records `code` in the timeout status word and
// returns.
__global__ void k_wait_selftest(int* status, unsigned long long limit_ns, int code) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) mbar_wait_ns(&bar, 0, status, code, limit_ns);
    __syncthreads();
}

extern "C" int f4j_selftest_wait(f4j_ctx* ctx, int64_t limit_us) {
    F4J_LOCK(ctx);
    if (limit_us < 1000 || limit_us > 2000000) return f4j_fail(F4J_ERR_ARG, "limit must be 1 ms .. 2 s");
    F4J_CUDA(cudaSetDevice(ctx->device));
    k_wait_selftest<<<1, 32, 0, ctx->stream>>>(ctx->d_status + F4J_ST_TIMEOUT,
                                               (unsigned long long)limit_us * 1000ull, F4J_SELFTEST_WAIT_CODE);
    F4J_LAUNCHED(ctx);
    return F4J_OK;
}

extern "C" int f4j_set_stream(f4j_ctx* ctx, void* s) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    F4J_CUDA(cudaStreamSynchronize(ctx->stream));
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    if (s) {
        ctx->stream = (cudaStream_t)s;
        ctx->own_stream = false;
    } else {
        F4J_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        ctx->own_stream = true;
    }
    return F4J_OK;
}

extern "C" void* f4j_get_stream(f4j_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }
extern "C" int64_t f4j_launch_count(f4j_ctx* ctx) { return ctx ? ctx->launches : -1; }

extern "C" int f4j_timer_record(f4j_ctx* ctx, int slot) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (slot < 0 || slot >= 16) return f4j_fail(F4J_ERR_ARG, "timer slot %d out of range", slot);
    if (!ctx->ev_init[slot]) {
        F4J_CUDA(cudaEventCreate(&ctx->ev[slot]));
        ctx->ev_init[slot] = true;
    }
    F4J_CUDA(cudaEventRecord(ctx->ev[slot], ctx->stream));
    return F4J_OK;
}

extern "C" int f4j_timer_elapsed(f4j_ctx* ctx, int a, int b, float* ms) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (a < 0 || a >= 16 || b < 0 || b >= 16 || !ctx->ev_init[a] || !ctx->ev_init[b] || !ms)
        return f4j_fail(F4J_ERR_ARG, "timer slots not recorded");
    F4J_CUDA(cudaEventSynchronize(ctx->ev[b]));
    F4J_CUDA(cudaEventElapsedTime(ms, ctx->ev[a], ctx->ev[b]));
    return F4J_OK;
}

void f4j_prof_begin(f4j_ctx* ctx, int tag) {
    if (!ctx->prof || ctx->prof_n >= 512) return;
    ctx->prof_tag[ctx->prof_n] = tag;
    cudaEventRecord(ctx->prof_ev[2 * ctx->prof_n], ctx->stream);
}

void f4j_prof_end(f4j_ctx* ctx) {
    if (!ctx->prof || ctx->prof_n >= 512) return;
    cudaEventRecord(ctx->prof_ev[2 * ctx->prof_n + 1], ctx->stream);
    ctx->prof_n++;
}

extern "C" int f4j_set_profiling(f4j_ctx* ctx, int on) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (on && !ctx->prof_init) {
        for (int i = 0; i < 1024; i++) F4J_CUDA(cudaEventCreate(&ctx->prof_ev[i]));
        ctx->prof_init = true;
    }
    ctx->prof = on != 0;
    ctx->prof_n = 0;
    return F4J_OK;
}

extern "C" int f4j_profile_read(f4j_ctx* ctx, int tag, double* total_ms, int64_t* count) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (!total_ms || !count) return f4j_fail(F4J_ERR_ARG, "null output");
    double t = 0;
    int64_t c = 0;
    for (int i = 0; i < ctx->prof_n; i++) {
        if (tag >= 0 && ctx->prof_tag[i] != tag) continue;
        float ms = 0;
        F4J_CUDA(cudaEventSynchronize(ctx->prof_ev[2 * i + 1]));
        F4J_CUDA(cudaEventElapsedTime(&ms, ctx->prof_ev[2 * i], ctx->prof_ev[2 * i + 1]));
        t += ms;
        c++;
    }
    *total_ms = t;
    *count = c;
    return F4J_OK;
}

extern "C" int f4j_profile_reset(f4j_ctx* ctx) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    F4J_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->prof_n = 0;
    return F4J_OK;
}

int f4j_status_take(f4j_ctx* ctx, int idx, int* value) {
    int h[F4J_ST_WORDS];
    F4J_CUDA(cudaMemcpyAsync(h, ctx->d_status, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    F4J_CUDA(cudaStreamSynchronize(ctx->stream));
    *value = h[idx];
    if (h[idx]) F4J_CUDA(cudaMemsetAsync(ctx->d_status + idx, 0, sizeof(int), ctx->stream));
    return F4J_OK;
}

int f4j_workspace(f4j_ctx* ctx, int slot, size_t bytes, void** out) {
    if (slot < 0 || slot >= 8) return f4j_fail(F4J_ERR_ARG, "workspace slot %d", slot);
    if (bytes == 0) bytes = 256;
    if (bytes > ctx->ws_bytes[slot]) {
        F4J_CUDA(cudaStreamSynchronize(ctx->stream));
        if (ctx->ws[slot]) cudaFree(ctx->ws[slot]);
        ctx->ws[slot] = nullptr;
        ctx->ws_bytes[slot] = 0;
        size_t want = bytes + bytes / 8;
        cudaError_t e = cudaMalloc(&ctx->ws[slot], want);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return f4j_fail(F4J_ERR_OOM, "workspace of %zu bytes: %s", want, cudaGetErrorString(e));
        }
        ctx->ws_bytes[slot] = want;
    }
    *out = ctx->ws[slot];
    return F4J_OK;
}

int f4j_dev_alloc(f4j_ctx* ctx, size_t bytes, void** out) {
    cudaError_t e = cudaMallocAsync(out, bytes ? bytes : 16, ctx->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return f4j_fail(F4J_ERR_OOM, "device allocation of %zu bytes: %s", bytes, cudaGetErrorString(e));
    }
    return F4J_OK;
}

void f4j_dev_free(f4j_ctx* ctx, void* p) {
    if (p) cudaFreeAsync(p, ctx->stream);
}

// ------------------------------------------------------------------ buffers
extern "C" int f4j_buf_alloc(f4j_ctx* ctx, size_t bytes, f4j_buf* out) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (!out) return f4j_fail(F4J_ERR_ARG, "null output pointer");
    *out = nullptr;
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return f4j_fail(F4J_ERR_OOM, "device buffer of %zu bytes: %s", bytes, cudaGetErrorString(e));
    }
    *out = new f4j_buf_s{p, bytes, true, false};
    return F4J_OK;
}

extern "C" int f4j_buf_wrap(f4j_ctx* ctx, void* ptr, size_t bytes, f4j_buf* out) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (!out) return f4j_fail(F4J_ERR_ARG, "null output pointer");
    *out = nullptr;
    if (!ptr) return f4j_fail(F4J_ERR_ARG, "null memory to wrap");
    if (reinterpret_cast<uintptr_t>(ptr) & 15) return f4j_fail(F4J_ERR_ARG, "wrapped memory must be 16-byte aligned");
    cudaPointerAttributes a;
    cudaError_t e = cudaPointerGetAttributes(&a, ptr);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return f4j_fail(F4J_ERR_ARG, "cannot query the memory to wrap: %s", cudaGetErrorString(e));
    }
    void* dev = nullptr;
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) {
        if (a.type == cudaMemoryTypeDevice && a.device != ctx->device)
            return f4j_fail(F4J_ERR_ARG, "wrapped device memory belongs to device %d, context is on %d", a.device,
                            ctx->device);
        dev = ptr;
    } else if (a.type == cudaMemoryTypeHost) {
        dev = a.devicePointer;  // pinned / registered host memory, mapped into the device's address space
    } else {
        int pageable = 0;
        F4J_CUDA(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, ctx->device));
        if (!pageable)
            return f4j_fail(F4J_ERR_ARG, "the device cannot address unregistered host memory (register it first)");
        dev = ptr;
    }
    if (!dev) return f4j_fail(F4J_ERR_ARG, "the memory to wrap has no device address");
    *out = new f4j_buf_s{dev, bytes, false, false};
    return F4J_OK;
}

extern "C" int f4j_buf_free(f4j_ctx* ctx, f4j_buf b) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (!b) return F4J_OK;
    if (b->owned && b->pooled) {
        F4J_CUDA(cudaFreeAsync(b->ptr, ctx->stream));  // after the work queued on it
    } else {
        F4J_CUDA(cudaStreamSynchronize(ctx->stream));
        if (b->owned) cudaFree(b->ptr);
    }
    delete b;
    return F4J_OK;
}

int f4j_buf_alloc_pooled(f4j_ctx* ctx, size_t bytes, f4j_buf* out) {
    void* p = nullptr;
    int rc = f4j_dev_alloc(ctx, bytes, &p);
    if (rc) return rc;
    *out = new f4j_buf_s{p, bytes, true, true};
    return F4J_OK;
}

extern "C" size_t f4j_buf_size(f4j_buf b) { return b ? b->bytes : 0; }
extern "C" void* f4j_buf_device_ptr(f4j_buf b) { return b ? b->ptr : nullptr; }

static int copy_check(f4j_ctx* ctx, f4j_buf b, const void* host, size_t bytes, size_t off) {
    F4J_CHECK_CTX(ctx);
    if (!b) return f4j_fail(F4J_ERR_ARG, "null buffer");
    if (!host && bytes) return f4j_fail(F4J_ERR_ARG, "null host pointer");
    if (off > b->bytes || bytes > b->bytes - off)
        return f4j_fail(F4J_ERR_ARG, "copy of %zu bytes at offset %zu exceeds buffer of %zu bytes",
                        bytes, off, b->bytes);
    return F4J_OK;
}

extern "C" int f4j_buf_upload_async(f4j_ctx* ctx, f4j_buf b, const void* host, size_t bytes, size_t off) {
    F4J_LOCK(ctx);
    int rc = copy_check(ctx, b, host, bytes, off);
    if (rc) return rc;
    if (bytes)
        F4J_CUDA(cudaMemcpyAsync((char*)b->ptr + off, host, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return F4J_OK;
}

extern "C" int f4j_buf_download_async(f4j_ctx* ctx, f4j_buf b, void* host, size_t bytes, size_t off) {
    F4J_LOCK(ctx);
    int rc = copy_check(ctx, b, host, bytes, off);
    if (rc) return rc;
    if (bytes)
        F4J_CUDA(cudaMemcpyAsync(host, (char*)b->ptr + off, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return F4J_OK;
}

extern "C" int f4j_buf_upload(f4j_ctx* ctx, f4j_buf b, const void* host, size_t bytes, size_t off) {
    F4J_LOCK(ctx);
    int rc = f4j_buf_upload_async(ctx, b, host, bytes, off);
    if (rc) return rc;
    F4J_CUDA(cudaStreamSynchronize(ctx->stream));
    return F4J_OK;
}

extern "C" int f4j_buf_download(f4j_ctx* ctx, f4j_buf b, void* host, size_t bytes, size_t off) {
    F4J_LOCK(ctx);
    int rc = f4j_buf_download_async(ctx, b, host, bytes, off);
    if (rc) return rc;
    F4J_CUDA(cudaStreamSynchronize(ctx->stream));
    return F4J_OK;
}

extern "C" int f4j_buf_zero(f4j_ctx* ctx, f4j_buf b) {
    F4J_LOCK(ctx);
    F4J_CHECK_CTX(ctx);
    if (!b) return f4j_fail(F4J_ERR_ARG, "null buffer");
    F4J_CUDA(cudaMemsetAsync(b->ptr, 0, b->bytes, ctx->stream));
    return F4J_OK;
}

extern "C" int f4j_host_register(void* host, size_t bytes) {
    if (!host || !bytes) return f4j_fail(F4J_ERR_ARG, "null host range");
    F4J_CUDA(cudaHostRegister(host, bytes, cudaHostRegisterDefault));
    return F4J_OK;
}

extern "C" int f4j_host_unregister(void* host) {
    if (!host) return f4j_fail(F4J_ERR_ARG, "null host pointer");
    F4J_CUDA(cudaHostUnregister(host));
    return F4J_OK;
}

extern "C" int f4j_host_alloc(size_t bytes, void** out) {
    if (!out) return f4j_fail(F4J_ERR_ARG, "null output pointer");
    *out = nullptr;
    if (!bytes) return f4j_fail(F4J_ERR_ARG, "zero-byte host allocation");
    F4J_CUDA(cudaHostAlloc(out, bytes, cudaHostAllocPortable));
    return F4J_OK;
}

extern "C" int f4j_host_free(void* host) {
    if (!host) return F4J_OK;
    F4J_CUDA(cudaFreeHost(host));
    return F4J_OK;
}

// ------------------------------------------------------------------ dense front ends
static int check_gemm_args(f4j_ctx* ctx, bool cplx, int64_t m, int64_t n, int64_t k, f4j_buf A,
                           int opA, f4j_buf B, int opB, f4j_buf C, int mode) {
    F4J_CHECK_CTX(ctx);
    if (!A || !B || !C) return f4j_fail(F4J_ERR_ARG, "null matrix buffer");
    if (m < 0 || n < 0 || k < 0) return f4j_fail(F4J_ERR_ARG, "negative dimension");
    if (m > INT32_MAX || n > INT32_MAX || k > INT32_MAX)
        return f4j_fail(F4J_ERR_ARG, "dimension exceeds Flag4j's int range");
    int maxop = cplx ? F4J_OP_C : F4J_OP_C;
    if (opA < 0 || opA > maxop || opB < 0 || opB > maxop) return f4j_fail(F4J_ERR_ARG, "bad op");
    if (mode < F4J_MODE_PLAIN || mode > F4J_MODE_EXACT) return f4j_fail(F4J_ERR_ARG, "bad mode %d", mode);
    size_t es = cplx ? 16 : 8;
    if ((size_t)m * k * es > A->bytes) return f4j_fail(F4J_ERR_ARG, "A buffer too small for %lldx%lld", (long long)m, (long long)k);
    if ((size_t)k * n * es > B->bytes) return f4j_fail(F4J_ERR_ARG, "B buffer too small for %lldx%lld", (long long)k, (long long)n);
    if ((size_t)m * n * es > C->bytes) return f4j_fail(F4J_ERR_ARG, "C buffer too small for %lldx%lld", (long long)m, (long long)n);
    if (C->ptr == A->ptr || C->ptr == B->ptr) return f4j_fail(F4J_ERR_ARG, "C must not alias A or B");
    return F4J_OK;
}

int f4j_gemm_impl(f4j_ctx* ctx, bool cplx, int64_t m, int64_t n, int64_t k, const double* A,
                  int opA, const double* B, int opB, double* C, int mode, f4j_report* rep,
                  const int** gate_out) {
    if (gate_out) *gate_out = nullptr;
    int64_t l0 = ctx->launches;
    if (rep) {
        *rep = f4j_report{};
        rep->flops = (cplx ? 8.0 : 2.0) * (double)m * (double)n * (double)k;
        rep->max_abs_err = rep->max_rel_err = rep->plain_max_abs_err = rep->plain_max_rel_err = -1.0;
    }
    if (!cplx) {  // conjugation is the identity for real data
        if (opA == F4J_OP_C) opA = F4J_OP_T;
        if (opB == F4J_OP_C) opB = F4J_OP_T;
    }
    if (m == 0 || n == 0) return F4J_OK;
    // AUTO follows the dispatcher configuration: the reference's small-product
    // rule and products of a few microseconds of work run Flag4j's own order
    // (bit-identical); larger ones take the configured GPU path (f4j_config.cu).
    if (mode == F4J_MODE_AUTO) {
        mode = f4j_resolve_mode(cplx, m, n, k, mode);
        if (mode == F4J_MODE_AUTO) mode = F4J_MODE_SPLIT;
    }
    int rc = F4J_OK;
    int used = mode;
    if (k == 0) {
        F4J_CUDA(cudaMemsetAsync(C, 0, (size_t)m * n * (cplx ? 16 : 8), ctx->stream));
    } else if (mode == F4J_MODE_EXACT) {
        rc = f4j_gemm_exact(ctx, cplx, m, n, k, A, opA, B, opB, C);
    } else if (n == 1) {
        // a matrix-vector product: one FP64 FMA dot product per row reads A once,
        // where slicing A and a GEMM with one column would waste the tiles
        rc = f4j_gemv(ctx, cplx, m, k, A, opA, B, opB == F4J_OP_C, C);
        used = F4J_MODE_PLAIN;
    } else if (mode == F4J_MODE_PLAIN) {
        rc = f4j_gemm_dmma(ctx, cplx, m, n, k, A, opA, B, opB, C);
    } else {
        // NaN/Inf cannot be sliced: the split kernels stand down on the device
        // and the gated DMMA launch (a no-op otherwise) propagates them like
        // the reference.  Nothing here waits for the GPU.
        const int* gate = nullptr;
        rc = f4j_gemm_split(ctx, cplx, m, n, k, A, opA, B, opB, C, 0, rep, &gate);
        if (gate_out) *gate_out = gate;
        used = F4J_MODE_SPLIT;
        if (rc == F4J_OK) rc = f4j_gemm_dmma(ctx, cplx, m, n, k, A, opA, B, opB, C, gate);
        if (rc == F4J_OK && rep && rep->slices == 0) used = F4J_MODE_PLAIN;
    }
    if (rep) {
        rep->mode_used = used;
        rep->launches = (int32_t)(ctx->launches - l0);
    }
    return rc;
}

// The accuracy part of a dense product's report (f4j_report's check fields):
// the sampled double-double error of C, the plain FP64 bound on the same
// scale, and with F4J_CHECK_PLAIN the plain DMMA product's error on the same
// entries (that product goes to pool scratch and is freed again).

int f4j_report_accuracy(f4j_ctx* ctx, bool cplx, int64_t m, int64_t n, int64_t k, const double* A, int opA,
                        const double* B, int opB, const double* C, int samples, int flags, f4j_report* rep) {
    if (!rep) return F4J_OK;
    rep->check_samples = samples;
    rep->check_flags = flags;
    int32_t rk = 0;
    f4j_dispatch(cplx ? 1 : 0, m, n, k, F4J_MODE_AUTO, nullptr, &rk);
    rep->ref_kernel = rk;
    rep->plain_bound_rel = (cplx ? 2.0 : 1.0) * (double)k * 0x1p-53;
    rep->max_abs_err = rep->max_rel_err = -1.0;
    rep->plain_max_abs_err = rep->plain_max_rel_err = -1.0;
    if (samples <= 0 || m == 0 || n == 0) return F4J_OK;
    int rc = f4j_check_sampled(ctx, cplx, m, n, k, A, opA, B, opB, C, samples, F4J_CHECK_SEED, &rep->max_abs_err,
                               &rep->max_rel_err);
    if (rc || !(flags & F4J_CHECK_PLAIN)) return rc;
    void* C2 = nullptr;
    rc = f4j_dev_alloc(ctx, (size_t)m * n * (cplx ? 16 : 8), &C2);
    if (rc) return rc;
    rc = f4j_gemm_impl(ctx, cplx, m, n, k, A, opA, B, opB, (double*)C2, F4J_MODE_PLAIN, nullptr);
    if (rc == F4J_OK)
        rc = f4j_check_sampled(ctx, cplx, m, n, k, A, opA, B, opB, (const double*)C2, samples, F4J_CHECK_SEED,
                               &rep->plain_max_abs_err, &rep->plain_max_rel_err);
    f4j_dev_free(ctx, C2);
    return rc;
}

static int dense_entry(f4j_ctx* ctx, bool cplx, int64_t m, int64_t n, int64_t k, f4j_buf A, int opA, f4j_buf B,
                       int opB, f4j_buf C, int mode, f4j_report* rep) {
    int rc = check_gemm_args(ctx, cplx, m, n, k, A, opA, B, opB, C, mode);
    if (rc) return rc;
    if (rep && rep->check_samples < 0) return f4j_fail(F4J_ERR_ARG, "negative check_samples");
    const int samples = rep ? rep->check_samples : 0, flags = rep ? rep->check_flags : 0;
    F4J_CUDA(cudaSetDevice(ctx->device));
    rc = f4j_gemm_impl(ctx, cplx, m, n, k, (const double*)A->ptr, opA, (const double*)B->ptr, opB,
                       (double*)C->ptr, mode, rep);
    if (rc) return rc;
    return f4j_report_accuracy(ctx, cplx, m, n, k, (const double*)A->ptr, opA, (const double*)B->ptr, opB,
                               (const double*)C->ptr, samples, flags, rep);
}

extern "C" int f4j_dgemm(f4j_ctx* ctx, int64_t m, int64_t n, int64_t k, f4j_buf A, int opA,
                         f4j_buf B, int opB, f4j_buf C, int mode, f4j_report* rep) {
    F4J_LOCK(ctx);
    return dense_entry(ctx, false, m, n, k, A, opA, B, opB, C, mode, rep);
}

extern "C" int f4j_zgemm(f4j_ctx* ctx, int64_t m, int64_t n, int64_t k, f4j_buf A, int opA,
                         f4j_buf B, int opB, f4j_buf C, int mode, f4j_report* rep) {
    F4J_LOCK(ctx);
    return dense_entry(ctx, true, m, n, k, A, opA, B, opB, C, mode, rep);
}

static int adjoint(f4j_ctx* ctx, bool cplx, int64_t m, int64_t n, int64_t k, f4j_buf A, f4j_buf B,
                   f4j_buf dC, f4j_buf dA, f4j_buf dB, int mode, f4j_report* rep) {
    F4J_CHECK_CTX(ctx);
    if (!A || !B || !dC) return f4j_fail(F4J_ERR_ARG, "null operand buffer");
    if (!dA && !dB) return f4j_fail(F4J_ERR_ARG, "both gradient outputs are null");
    F4J_CUDA(cudaSetDevice(ctx->device));
    const int opH = cplx ? F4J_OP_C : F4J_OP_T;
    f4j_report r1{}, r2{};
    int64_t l0 = ctx->launches;
    if (dA && dB) {
        // Both products at once: dA on the context stream, dB on a second stream
        // with its own split workspace (slots 4-5).  Each product's persistent
        // kernel leaves a partly empty last wave; on two streams the other
        // product's CTAs fill those SMs.  No report is read until both are queued.
        int rc = check_gemm_args(ctx, cplx, m, k, n, dC, F4J_OP_N, B, opH, dA, mode);
        if (rc) return rc;
        rc = check_gemm_args(ctx, cplx, k, n, m, A, opH, dC, F4J_OP_N, dB, mode);
        if (rc) return rc;
        if (!ctx->aux_stream) {
            F4J_CUDA(cudaStreamCreateWithFlags(&ctx->aux_stream, cudaStreamNonBlocking));
            F4J_CUDA(cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
            F4J_CUDA(cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
        }
        F4J_CUDA(cudaEventRecord(ctx->ev_fork, ctx->stream));
        F4J_CUDA(cudaStreamWaitEvent(ctx->aux_stream, ctx->ev_fork, 0));
        const int* g1 = nullptr;
        const int* g2 = nullptr;
        rc = f4j_gemm_impl(ctx, cplx, m, k, n, (const double*)dC->ptr, F4J_OP_N, (const double*)B->ptr, opH,
                           (double*)dA->ptr, mode, nullptr, &g1);
        const cudaStream_t main_stream = ctx->stream;
        if (rc == F4J_OK) {
            ctx->stream = ctx->aux_stream;
            ctx->ws_base = 4;
            rc = f4j_gemm_impl(ctx, cplx, k, n, m, (const double*)A->ptr, opH, (const double*)dC->ptr, F4J_OP_N,
                               (double*)dB->ptr, mode, nullptr, &g2);
            ctx->stream = main_stream;
            ctx->ws_base = 0;
        }
        F4J_CUDA(cudaEventRecord(ctx->ev_join, ctx->aux_stream));
        F4J_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
        if (rc) return rc;
        if (rep) {
            *rep = f4j_report{};
            rep->flops = 2.0 * (cplx ? 8.0 : 2.0) * (double)m * (double)n * (double)k;
            rep->mode_used = f4j_resolve_mode(cplx, m, k, n, mode);  // dA's shape; dB's resolves alike
            rep->launches = (int32_t)(ctx->launches - l0);
            if (g1 || g2) {
                // the plans' headers: s, nrounds, ubits, nonfinite, spread (the gate is nonfinite)
                F4J_CUDA(cudaStreamSynchronize(ctx->stream));
                int h[2][5] = {};
                if (g1) F4J_CUDA(cudaMemcpy(h[0], g1 - 3, sizeof h[0], cudaMemcpyDeviceToHost));
                if (g2) F4J_CUDA(cudaMemcpy(h[1], g2 - 3, sizeof h[1], cudaMemcpyDeviceToHost));
                int s = 0, nonfinite = 0;
                float spread = 0.f;
                for (int u = 0; u < 2; u++) {
                    if (!(u ? g2 : g1)) continue;
                    float sp;
                    memcpy(&sp, &h[u][4], 4);
                    s = h[u][0] > s ? h[u][0] : s;
                    nonfinite |= h[u][3];
                    spread = sp > spread ? sp : spread;
                }
                rep->slices = nonfinite ? 0 : s;
                rep->frac_bits = s ? 4 + 5 * (s - 1) : 0;
                rep->exp_spread = spread;
                rep->mode_used = nonfinite ? F4J_MODE_PLAIN : F4J_MODE_SPLIT;
            }
        }
        return F4J_OK;
    }
    if (dA) {  // dA (m x k) = dC (m x n) * op(B) (n x k), B stored k x n
        int rc = check_gemm_args(ctx, cplx, m, k, n, dC, F4J_OP_N, B, opH, dA, mode);
        if (rc) return rc;
        rc = f4j_gemm_impl(ctx, cplx, m, k, n, (const double*)dC->ptr, F4J_OP_N,
                           (const double*)B->ptr, opH, (double*)dA->ptr, mode, &r1);
        if (rc) return rc;
    }
    if (dB) {  // dB (k x n) = op(A) (k x m) * dC (m x n), A stored m x k
        int rc = check_gemm_args(ctx, cplx, k, n, m, A, opH, dC, F4J_OP_N, dB, mode);
        if (rc) return rc;
        rc = f4j_gemm_impl(ctx, cplx, k, n, m, (const double*)A->ptr, opH, (const double*)dC->ptr,
                           F4J_OP_N, (double*)dB->ptr, mode, &r2);
        if (rc) return rc;
    }
    if (rep) {
        *rep = dA ? r1 : r2;
        rep->flops = r1.flops + r2.flops;
        rep->slices = r1.slices > r2.slices ? r1.slices : r2.slices;
        rep->launches = (int32_t)(ctx->launches - l0);
    }
    return F4J_OK;
}

extern "C" int f4j_dgemm_adjoint(f4j_ctx* ctx, int64_t m, int64_t n, int64_t k, f4j_buf A,
                                 f4j_buf B, f4j_buf dC, f4j_buf dA, f4j_buf dB, int mode,
                                 f4j_report* rep) {
    F4J_LOCK(ctx);
    return adjoint(ctx, false, m, n, k, A, B, dC, dA, dB, mode, rep);
}

extern "C" int f4j_zgemm_adjoint(f4j_ctx* ctx, int64_t m, int64_t n, int64_t k, f4j_buf A,
                                 f4j_buf B, f4j_buf dC, f4j_buf dA, f4j_buf dB, int mode,
                                 f4j_report* rep) {
    F4J_LOCK(ctx);
    return adjoint(ctx, true, m, n, k, A, B, dC, dA, dB, mode, rep);
}
