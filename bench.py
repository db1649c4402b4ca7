"""Benchmark of the GB300 engine for Flag4j's product path.

One step = one FP64-accurate GEMM C = A B at 8192^3 (real float64, entries
u 2^e, u ~ U[-1,1), integer e ~ U[-8, 8] per row of A / column of B) through
the split path: exponent statistics, FP8 slicing and the tcgen05 slice GEMM.
value = 2 m n k / step time (TFLOP/s, FP64-equivalent), inputs resident in
HBM (A, B: 512 MiB each, larger than L2, so no flush is needed).  The same JSON
line carries the plain DMMA path, errors against the double-double check for
phi in {0, 8, 32}, the Complex128 4096^3 product, CSR SpMV/SpMM GB/s at 2^20
rows (Poisson(16) row lengths), the dense adjoint step ratio, the roofline of
the slice GEMM kernel, the CPU baseline and an end-to-end number through the
host-buffer API (host<->device copies inside the timed region).  After all GPU
timing, the oracle's restatements of the reference's loops are timed on this
host beside the sparse, complex and adjoint rows (their cpu_baseline keys).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
  python bench.py --case small        # 2048^3 / 2^16-row variant (profiling)
Under torchrun each rank runs an independent replica on its own GPU
(replicas only: the path does not shard); rank 0 prints the max-over-ranks line.
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FP64-accurate GEMM TFLOP/s (split vs plain DMMA) at stated err; CSR SpMM GB/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--case", default="full", choices=["full", "small"])
    p.add_argument("--n", type=int, default=0, help="override the GEMM size n (profiling)")
    p.add_argument("--skip-extras", action="store_true", help="headline GEMM only (for profiling)")
    p.add_argument("--only-sparse", action="store_true", help="CSR products only (for profiling)")
    p.add_argument("--only-dmma", action="store_true", help="plain DMMA GEMM only (for profiling)")
    p.add_argument("--only-spmv", action="store_true",
                   help="SpMV alone at 2^20 rows, exact then FMA (for profiling; about 220 MB on the device)")
    p.add_argument("--only-sddmm", action="store_true",
                   help="SDDMM alone at 2^20 rows x 64 columns (for profiling; about 1.4 GB on the device)")
    return p.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier and max over ranks (torch.distributed when WORLD_SIZE > 1)."""

    def __init__(self, ws):
        self.ws = ws
        self.pg = None
        if ws > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, x):
        if self.ws == 1:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


class Clocks:
    """nvidia-smi samples during the timed region (median SM clock, reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- helpers
class Eng:
    def __init__(self, device):
        import flag4j_gb300 as f
        from flag4j_gb300 import _lib
        from flag4j_gb300.device import check
        self.f, self.L, self.check = f, _lib, check
        self.ctx = f.Context(device)
        self.lib = self.ctx.lib

    def dev(self, arr):
        return self.ctx.from_numpy(arr)

    def gemm(self, A, B, C, m, n, k, mode, cplx=False, opA=0, opB=0, report=False, check_samples=0):
        """One product; with report=True the call also fills (and waits for) the report, and with
        check_samples > 0 the report carries the sampled double-double error of this result."""
        rep = self.L.f4j_report() if report else None
        if report:
            rep.check_samples = check_samples
        fn = self.lib.f4j_zgemm if cplx else self.lib.f4j_dgemm
        self.check(fn(self.ctx.handle, m, n, k, A.handle, opA, B.handle, opB, C.handle, mode,
                      ctypes.byref(rep) if report else None))
        return rep

    def check_err(self, A, B, C, m, n, k, cplx=False, samples=4096, seed=1234):
        ea, er = ctypes.c_double(), ctypes.c_double()
        self.check(self.lib.f4j_gemm_check(self.ctx.handle, int(cplx), m, n, k, A.handle, 0, B.handle, 0,
                                           C.handle, samples, seed, ctypes.byref(ea), ctypes.byref(er)))
        return ea.value, er.value

    def kernel_ms(self, fn, steps, with_prep=False):
        """Average CUDA-event time per call of the main product kernel inside
        fn() (and of the preparation kernels when with_prep)."""
        self.check(self.lib.f4j_set_profiling(self.ctx.handle, 1))
        for _ in range(steps):
            fn()
        out = []
        for tag in (0, 1):
            tot, cnt = ctypes.c_double(), ctypes.c_int64()
            self.check(self.lib.f4j_profile_read(self.ctx.handle, tag, ctypes.byref(tot), ctypes.byref(cnt)))
            out.append(tot.value / steps)
        self.check(self.lib.f4j_set_profiling(self.ctx.handle, 0))
        return tuple(out) if with_prep else out[0]

    def timed(self, fn, steps, warmup):
        """Average ms per call with CUDA events on the context stream."""
        for _ in range(warmup):
            fn()
        self.ctx.sync()
        self.ctx.timer_record(0)
        for _ in range(steps):
            fn()
        self.ctx.timer_record(1)
        ms = self.ctx.timer_elapsed(0, 1) / steps
        self.ctx.sync()
        return ms


def fp8_peak_tflops():
    """Dense E4M3 peak measured with cuBLASLt (torch._scaled_mm), 8192^3, best of 10."""
    try:
        import torch
        n = 8192
        a = torch.randn(n, n, device="cuda").to(torch.float8_e4m3fn)
        b = torch.randn(n, n, device="cuda").to(torch.float8_e4m3fn).t()
        one = torch.tensor(1.0, device="cuda")
        for _ in range(3):
            torch._scaled_mm(a, b, scale_a=one, scale_b=one, out_dtype=torch.bfloat16)
        best = 1e9
        for _ in range(10):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            torch._scaled_mm(a, b, scale_a=one, scale_b=one, out_dtype=torch.bfloat16)
            e.record()
            torch.cuda.synchronize()
            best = min(best, s.elapsed_time(e))
        del a, b
        torch.cuda.empty_cache()
        return 2 * n ** 3 / (best * 1e-3) / 1e12, "cuBLASLt e4m3 8192^3 via torch._scaled_mm, best of 10, this run"
    except Exception as ex:  # noqa: BLE001
        v, src = fp8_peak_from_file()
        return v, "%s (fp8 measurement failed: %s)" % (src, type(ex).__name__)


def fp8_peak_from_file():
    """2 x the dense bf16 burst rate in MEASURED_PEAKS.json (FP8 runs at twice bf16 on the tensor pipe);
    the recipe's 1.9 PFLOP/s bf16 fallback when the file is absent."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return 2 * json.load(open(p))["bf16_tflops"], "2 x measured bf16 (MEASURED_PEAKS.json)"
    return 2 * 1900.0, "2 x fallback bf16 1.9 PFLOP/s"


# DRAM bytes of one k_split_gemm launch at 8192^3 by slice count, from one ncu
# capture each (dram__bytes_read.sum + dram__bytes_write.sum, 1 pass):
#   ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum --clock-control none
#       -k regex:k_split_gemm -s 2 -c 1 python bench.py --skip-extras --steps 2 --warmup 3
SPLIT_GEMM_DRAM_BYTES_8192 = {11: 15.077633e9 + 0.636095e9, 10: 12.27e9 + 0.65615e9}

# DRAM bytes of one 2^20-row, 32-column SpMM launch (k_spmm), exact and FMA
# modes, from the ncu capture in profiles/k_spmm_1M_rows_32cols.md
SPMM_DRAM_BYTES_1M = {"exact": 3.255e9 + 0.266e9, "fma": 3.257e9 + 0.265e9}
# FP64-pipe activity of the same launches (sm__pipe_fp64_cycles_active, of active cycles)
SPMM_FP64_PIPE_1M = {"exact": 0.839, "fma": 0.933}


def fp64_peak_tflops():
    """FP64 GEMM peak measured with cuBLAS DGEMM (torch.matmul float64), 8192^3, best of 3."""
    try:
        import torch
        n = 8192
        a = torch.randn(n, n, device="cuda", dtype=torch.float64)
        b = torch.randn(n, n, device="cuda", dtype=torch.float64)
        torch.matmul(a, b)
        best = 1e9
        for _ in range(3):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            torch.matmul(a, b)
            e.record()
            torch.cuda.synchronize()
            best = min(best, s.elapsed_time(e))
        del a, b
        torch.cuda.empty_cache()
        return 2 * n ** 3 / (best * 1e-3) / 1e12
    except Exception:  # noqa: BLE001
        return None


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "MEASURED_PEAKS.json hbm_gbs"
    return 6800.0, "fallback 6.8 TB/s"


# ---------------------------------------------------------------- CPU baseline
def cpu_baseline(n, k, seconds_target=15.0):
    """Flag4j's GEMM loop order (C restatement of RealDenseMatMult.concurrentBlockedReordered,
    bit-identical to the Java kernel) on all host cores, over a row sample of the
    same 8192^3 product (C rows 0..r-1 need A rows 0..r-1 and all of B)."""
    from oracle import oracle as O
    from flag4j_gb300 import synth
    threads = os.cpu_count() or 1
    B = synth.scaled(k, n, 8, 2, "col")
    rows = threads
    A = synth.scaled(rows, k, 8, 1, "row")
    t0 = time.perf_counter()
    O.dgemm(A, B, threads=threads)
    dt = time.perf_counter() - t0
    rows = max(threads, int(rows * seconds_target / max(dt, 1e-3)) // threads * threads)
    rows = min(rows, 4096, n)
    A = synth.scaled(rows, k, 8, 1, "row")
    t0 = time.perf_counter()
    O.dgemm(A, B, threads=threads)
    dt = time.perf_counter() - t0
    flops = 2.0 * rows * n * k
    return {"value": flops / dt / 1e12, "unit": "TFLOP/s", "cores": threads, "kind": "port",
            "sample": "%d of %d rows of C = A B (k = n = %d), C restatement of Flag4j's k-ascending no-FMA loop "
                      "(gcc -O3 -ffp-contract=off), %d pthreads, %.1f s" % (rows, n, n, threads, dt)}


def dense_cpu_baselines(nz, ma, ka, seconds=1.5):
    """Complex nz^3 (DenseSemiringMatMult over Complex128) and the C4 adjoint step
    (A B forward; W.multTranspose(B) and A.T().mult(W) backward) as the oracle's
    restatements of the reference's loops, on all host cores, each over a row
    sample of about `seconds` scaled to the full product by rows."""
    from oracle import oracle as O
    from flag4j_gb300 import synth
    O.build()
    threads = os.cpu_count() or 1

    def sampled(fn, full_rows):
        r = threads
        t = _wall(lambda: fn(r))
        r = min(full_rows, max(threads, int(r * seconds / max(t, 1e-4)) // threads * threads))
        t = _wall(lambda: fn(r))
        return t * full_rows / r, r

    Bz = synth.scaled(nz, nz, 8, 4, "col", cplx=True)
    tz, rz = sampled(lambda r: O.zgemm(synth.scaled(r, nz, 8, 3, "row", cplx=True), Bz, threads=threads), nz)
    del Bz
    A, B, W = synth.normal(ma, ka, 5), synth.normal(ka, ma, 6), synth.normal(ma, ma, 7)
    tf, rf = sampled(lambda r: O.dgemm(A[:r], B, threads=threads), ma)
    ta, ra = sampled(lambda r: O.dgemm_abt(W[:r], B, threads=threads), ma)
    At = np.ascontiguousarray(A.T)
    tb, rb = sampled(lambda r: O.dgemm(At[:r], W, threads=threads), ka)
    return {"complex": {"value": 8.0 * nz ** 3 / tz / 1e12, "unit": "TFLOP/s", "cores": threads, "kind": "port",
                        "sample": "%d of %d rows, scaled" % (rz, nz)},
            "adjoint": {"forward_ms": 1e3 * tf, "fwd_bwd_ms": 1e3 * (tf + ta + tb), "ratio": (tf + ta + tb) / tf,
                        "cores": threads, "kind": "port",
                        "sample": "row samples of A B (%d rows), W B^T (%d rows), A^T W (%d rows), scaled" % (rf, ra, rb)}}


def headline_config(n, ws):
    """The headline workload's config, the same dict on both arms."""
    return {"workload": "FP64-accurate GEMM %d^3 (split path), A u*2^e per row, B per column, "
                        "u~U[-1,1), e~U[-8,8]" % n,
            "l2": ("inputs larger than L2 (A, B %d MiB each), no flush" % (8 * n * n >> 20)
                   if 8 * n * n > (129 << 20) else
                   "A, B %d MiB each: L2-resident across steps" % (8 * n * n >> 20)),
            "parallelism": "replicas" if ws > 1 else "1 GPU"}


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    from flag4j_gb300 import synth
    O.build()
    n = 8192 if args.case == "full" else 2048
    threads = os.cpu_count() or 1
    B = synth.scaled(n, n, 8, 2, "col")
    # calibrate a row sample of about 2 s per step
    rows = threads
    A = synth.scaled(rows, n, 8, 1, "row")
    t0 = time.perf_counter()
    O.dgemm(A, B, threads=threads)
    dt = time.perf_counter() - t0
    rows = min(4096, max(threads, int(rows * 2.0 / max(dt, 1e-3)) // threads * threads))
    A = synth.scaled(rows, n, 8, 1, "row")
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        O.dgemm(A, B, threads=threads)
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    v = 2.0 * rows * n * n / t / 1e12
    cb = {"value": v, "unit": "TFLOP/s", "cores": threads, "kind": "port",
          "sample": "%d of %d rows of C = A B per step (k = n = %d), C restatement of Flag4j's k-ascending no-FMA "
                    "loop (gcc -O3 -ffp-contract=off), %d pthreads, median of %d steps" % (rows, n, n, threads,
                                                                                            len(times))}
    line = {"metric": METRIC, "value": v, "unit": "TFLOP/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded PCG64)",
            "impl": "reference",
            "config": headline_config(n, ws),
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "notes": "Flag4j is pure Java and neither machine has a JVM; the reference arm is the C "
                     "restatement of its GEMM loop (bit-identical to the Java kernel on the golden vectors) on "
                     "all host cores, timed on a row sample of the workload each step."}
    print(json.dumps(line))


# ---------------------------------------------------------------- sparse products
def _wall(fn):
    t0 = time.perf_counter()
    fn()
    return time.perf_counter() - t0


def sparse_cpu_baselines(rp, ci, v, g):
    """The oracle's restatements of the reference's sparse loops on this host,
    single-threaded as Flag4j runs them (RealCsrDenseMatMult, CooMatrix.toCsr,
    CooDataSorter, RealCsrOps.transpose + standard, RealCsrMatMult), each on a
    bounded sample of the bench's own workload and scaled to it as stated."""
    from oracle import oracle as O
    from flag4j_gb300 import synth
    O.build()
    rows, nnz = len(rp) - 1, len(v)
    out = {"kind": "port", "cores": 1}
    x = synth.normal(rows, 1, 5).ravel()
    t = _wall(lambda: O.spmv(rp, ci, v, x))
    out["spmv_ms"] = 1e3 * t
    # row samples: the first r rows, all of X (their columns span the whole range)
    r = max(1, rows // 16)
    rps, q = rp[:r + 1], int(rp[r])
    X = synth.normal(rows, 32, 6)
    t = _wall(lambda: O.spmm(rps, ci[:q], v[:q], X))
    out["spmm_ms"] = 1e3 * t * nnz / max(q, 1)
    del X
    X64 = synth.normal(rows, 64, 8)
    dC64 = synth.normal(rows, 64, 9)
    t = _wall(lambda: O.sddmm(rps, ci[:q], dC64, X64))
    out["sddmm64_ms"] = 1e3 * t * nnz / max(q, 1)
    # S^T dC as the reference does it: S.T() then standard(S^T, dC)
    t1 = _wall(lambda: O.csr_transpose(rows, rows, rp, ci, v))
    trp, tci, tv, _ = O.csr_transpose(rows, rows, rp, ci, v)
    qt = int(trp[r])
    t2 = _wall(lambda: O.spmm(trp[:r + 1], tci[:qt], tv[:qt], dC64))
    out["spmm_t64_ms"] = 1e3 * (t1 + t2 * nnz / max(qt, 1))
    del X64, dC64
    rs, cs, vs = synth.coo_shuffled(rp, ci, v, seed=7)
    m = min(nnz, 1 << 20)
    t = _wall(lambda: O.coo_sort(rs[:m], cs[:m], vs[:m]))
    out["coo_sort_ms"] = 1e3 * t * (nnz * math.log2(nnz)) / (m * math.log2(max(m, 2)))
    rsorted = np.repeat(np.arange(rows, dtype=np.int32), np.diff(rp))
    out["coo_to_csr_ms"] = 1e3 * _wall(lambda: O.coo_to_csr(rows, rsorted))
    grp, gci, gv = g
    gr = max(1, (len(grp) - 1) // 8)
    gq = int(grp[gr])
    t = _wall(lambda: O.spgemm_csr(grp[:gr + 1], gci[:gq], gv[:gq], grp, gci, gv, len(grp) - 1))
    products = int(np.diff(grp)[gci].sum())
    products_s = int(np.diff(grp)[gci[:gq]].sum())
    out["spgemm_csr_ms"] = 1e3 * t * products / max(products_s, 1)
    out["sample"] = ("SpMV and COO -> CSR on the whole matrix; SpMM, SDDMM, S^T dC and CSR x CSR on the first "
                     "1/16 (1/8 for CSR x CSR) of the rows, scaled by nonzeros (products); COO sort on 2^20 of the "
                     "shuffled triplets, scaled by n log n; S^T dC includes the full transpose")
    return out


def sparse_section(E, full, steps=20, cpu=False):
    """CSR SpMV / SpMM (32 and 64 columns), S^T dC and SDDMM (64 columns), COO sort and COO -> CSR,
    at 2^20 rows with Poisson(16) row lengths; CSR x CSR into CSR at rows / 4.  With cpu, the
    oracle's single-threaded restatements timed beside each (cpu_baseline)."""
    from flag4j_gb300 import synth
    rows = (1 << 20) if full else (1 << 16)
    rp, ci, v = synth.csr_poisson(rows, rows, seed=2024)
    nnz = len(v)
    S = E.f.CsrMatrix((rows, rows), v, rp, ci)
    hS = S.handle(E.ctx)
    x = E.dev(synth.normal(rows, 1, 5).ravel())
    y = E.ctx.alloc(8 * rows)
    X = E.dev(synth.normal(rows, 32, 6))
    Y = E.ctx.alloc(8 * rows * 32)
    t_spmv = E.timed(lambda: E.check(E.lib.f4j_spmv(E.ctx.handle, hS, x.handle, y.handle, None)), steps, 3)
    t_spmm = E.timed(lambda: E.check(E.lib.f4j_spmm(E.ctx.handle, hS, X.handle, 32, Y.handle, None)), steps, 3)
    FMA = E.L.SPARSE_FMA
    t_spmv_f = E.timed(lambda: E.check(E.lib.f4j_spmv_ex(E.ctx.handle, hS, x.handle, y.handle, FMA, None)),
                       steps, 3)
    t_spmm_f = E.timed(lambda: E.check(E.lib.f4j_spmm_ex(E.ctx.handle, hS, X.handle, 32, Y.handle, FMA, None)),
                       steps, 3)
    b_spmv = 12.0 * nnz + 4.0 * (rows + 1) + 16.0 * rows
    b_spmm = 12.0 * nnz + 4.0 * (rows + 1) + 2 * 8.0 * 32 * rows
    b_spmm_g = 12.0 * nnz + 8.0 * 32 * nnz + 8.0 * 32 * rows
    hbm, hbm_src = measured_peaks()
    # SpMM's binding resource is the FP64 pipe (2 lane-operations per clock per SM on GB300):
    # 2 * 32 * nnz lane-operations exact, 32 * nnz with FMA.  DRAM GB/s uses the bytes ncu
    # measured for the same launch (the X-row gathers miss L2 80 % of the time), not a byte
    # count: gather-inclusive bytes count L2 hits as well.
    dram = SPMM_DRAM_BYTES_1M if full else None

    def spmm_keys(t, mode):
        d = {"spmm_ms": t, "spmm_gbs_compulsory": b_spmm / t / 1e6, "spmm_frac_compulsory": b_spmm / t / 1e6 / hbm,
             "spmm_gbs_gather_inclusive": b_spmm_g / t / 1e6,
             "spmm_fp64_lane_ops_per_s": (2.0 if mode == "exact" else 1.0) * 32 * nnz / (t * 1e-3)}
        if dram:
            d.update({"spmm_dram_gbs_ncu_bytes": dram[mode] / t / 1e6, "spmm_dram_frac": dram[mode] / t / 1e6 / hbm,
                      "spmm_fp64_pipe_busy_ncu": SPMM_FP64_PIPE_1M[mode],
                      "spmm_bound": "FP64 pipe (%.1f %% busy in ncu)" % (100 * SPMM_FP64_PIPE_1M[mode])})
        return d

    res = {"rows": rows, "nnz": nnz, "spmv_ms": t_spmv,
           "spmv_gbs": b_spmv / t_spmv / 1e6, "spmv_frac": b_spmv / t_spmv / 1e6 / hbm,
           "hbm_peak_gbs": hbm, "hbm_peak_source": hbm_src, "bit_identical_to_reference_order": True,
           "spmm_bytes_note": "compulsory = 12 nnz + 4 (rows + 1) + 2 * 8 * 32 rows; gather-inclusive counts "
                              "a 256-byte X row per nonzero, L2 hits included; DRAM from ncu's bytes",
           "fma_mode": {"spmv_ms": t_spmv_f, "spmv_gbs": b_spmv / t_spmv_f / 1e6,
                        "spmv_frac": b_spmv / t_spmv_f / 1e6 / hbm,
                        "bound": "|y - y_ref| <= 2 k u |S||x| per row"}}
    res.update(spmm_keys(t_spmm, "exact"))
    res["fma_mode"].update(spmm_keys(t_spmm_f, "fma"))
    del x, y, X, Y

    # ---- structure: stable COO sort of shuffled triplets, then COO -> CSR
    # (CooMatrix.sortIndices, CooMatrix.toCsr); each timed around the call only
    r_s, c_s, v_s = synth.coo_shuffled(rp, ci, v, seed=7)
    r_s, c_s = r_s.astype(np.int32), c_s.astype(np.int32)
    dr, dc, dv = E.ctx.alloc(4 * nnz), E.ctx.alloc(4 * nnz), E.ctx.alloc(8 * nnz)
    sort_ms = []
    for i in range(3 + steps // 4):
        dr.upload(r_s), dc.upload(c_s), dv.upload(v_s)
        E.ctx.sync()
        E.ctx.timer_record(0)
        E.check(E.lib.f4j_coo_sort(E.ctx.handle, nnz, dr.handle, dc.handle, dv.handle))
        E.ctx.timer_record(1)
        if i >= 3:
            sort_ms.append(E.ctx.timer_elapsed(0, 1))
    conv_ms = []
    for i in range(3 + steps // 4):
        h = ctypes.c_void_p()
        E.ctx.sync()
        E.ctx.timer_record(0)
        E.check(E.lib.f4j_csr_from_coo(E.ctx.handle, rows, rows, nnz, dr.handle, dc.handle, dv.handle,
                                       ctypes.byref(h)))
        E.ctx.timer_record(1)
        if i >= 3:
            conv_ms.append(E.ctx.timer_elapsed(0, 1))
        E.lib.f4j_csr_free(E.ctx.handle, h)
    t_sort, t_conv = statistics.median(sort_ms), statistics.median(conv_ms)
    b_sort = 2 * 16.0 * nnz  # triplets read and written once (algorithmic; a radix pass moves them more)
    b_conv = 16.0 * nnz + 4.0 * nnz + 8.0 * nnz + 4.0 * (rows + 1)  # triplets in; cols, vals, rowptr out
    res.update({"coo_sort_ms": t_sort, "coo_sort_gbs": b_sort / t_sort / 1e6,
                "coo_to_csr_ms": t_conv, "coo_to_csr_gbs": b_conv / t_conv / 1e6,
                "coo_to_csr_note": "time includes the new handle's device allocations and the range checks"})
    del dr, dc, dv

    # ---- sparse adjoint at 64 columns (S^T dC through the cached permutation, SDDMM)
    X64 = E.dev(synth.normal(rows, 64, 8))
    dC64 = E.dev(synth.normal(rows, 64, 9))
    Y64 = E.ctx.alloc(8 * rows * 64)
    dS = E.ctx.alloc(8 * nnz)
    t_spmm64 = E.timed(lambda: E.check(E.lib.f4j_spmm(E.ctx.handle, hS, X64.handle, 64, Y64.handle, None)), steps, 3)
    t_spmmt = E.timed(lambda: E.check(E.lib.f4j_spmm_t(E.ctx.handle, hS, dC64.handle, 64, Y64.handle, None)),
                      steps, 3)
    t_sddmm = E.timed(lambda: E.check(E.lib.f4j_sddmm(E.ctx.handle, hS, dC64.handle, X64.handle, 64, dS.handle,
                                                      None)), steps, 3)
    b_spmm64 = 12.0 * nnz + 4.0 * (rows + 1) + 2 * 8.0 * 64 * rows
    b_spmmt = b_spmm64 + 4.0 * nnz
    b_sddmm = 4.0 * nnz + 4.0 * (rows + 1) + 2 * 8.0 * 64 * rows + 8.0 * nnz
    res.update({"spmm64_ms": t_spmm64, "spmm64_gbs_compulsory": b_spmm64 / t_spmm64 / 1e6,
                "spmm_t64_ms": t_spmmt, "spmm_t64_gbs_compulsory": b_spmmt / t_spmmt / 1e6,
                "sddmm64_ms": t_sddmm, "sddmm64_gbs_compulsory": b_sddmm / t_sddmm / 1e6,
                "sddmm64_gflops": 2.0 * 64 * nnz / t_sddmm / 1e6})
    del X64, dC64, Y64, dS, S

    # ---- CSR x CSR with a CSR result (CsrMatrix.mult2Csr): G G, G of rows/4 rows, Poisson(8)
    g_rows = rows // 4
    grp, gci, gv = synth.csr_poisson(g_rows, g_rows, lam=8.0, seed=77)
    G = E.f.CsrMatrix((g_rows, g_rows), gv, grp, gci)
    hG = G.handle(E.ctx)
    nnz_out = []

    def spgemm():
        h = ctypes.c_void_p()
        E.check(E.lib.f4j_csr_mult_csr(E.ctx.handle, hG, hG, ctypes.byref(h), None))
        if not nnz_out:
            nz = ctypes.c_int64()
            E.check(E.lib.f4j_csr_info(h, None, None, ctypes.byref(nz)))
            nnz_out.append(nz.value)
        E.lib.f4j_csr_free(E.ctx.handle, h)
    t_spgemm = E.timed(spgemm, max(3, steps // 4), 2)
    products = int(np.diff(grp)[gci].sum())
    res["spgemm_csr"] = {"rows": g_rows, "nnz_a": len(gv), "products": products, "nnz_c": nnz_out[0],
                         "ms": t_spgemm, "gproducts_per_s": products / t_spgemm / 1e6,
                         "note": "includes the result's device allocation and two host reads of sizes"}
    del G
    if cpu:
        attach_sparse_cpu(res, full)
    return res


def attach_sparse_cpu(res, full):
    """Adds the single-threaded CPU baselines beside the sparse section's GPU times
    (inputs regenerated from the same seeds)."""
    from flag4j_gb300 import synth
    rows = (1 << 20) if full else (1 << 16)
    rp, ci, v = synth.csr_poisson(rows, rows, seed=2024)
    g = synth.csr_poisson(rows // 4, rows // 4, lam=8.0, seed=77)
    cb = sparse_cpu_baselines(rp, ci, v, g)
    gpu_ms = {"spmv_ms": res["spmv_ms"], "spmm_ms": res["spmm_ms"], "sddmm64_ms": res["sddmm64_ms"],
              "spmm_t64_ms": res["spmm_t64_ms"], "coo_sort_ms": res["coo_sort_ms"],
              "coo_to_csr_ms": res["coo_to_csr_ms"], "spgemm_csr_ms": res["spgemm_csr"]["ms"]}
    cb["gpu_speedup"] = {k: cb[k] / gpu_ms[k] for k in gpu_ms}
    res["cpu_baseline"] = cb


def run_sparse_only(args):
    """Profiling helper: the CSR products alone (prints their numbers, not the contract line)."""
    from flag4j_gb300 import build
    build.build()
    E = Eng(dist_env()[2])
    print(json.dumps(sparse_section(E, args.case == "full", steps=args.steps, cpu=True)))


# ---------------------------------------------------------------- our arm
def run_ours(args):
    ws, rank, local = dist_env()
    dist = Dist(ws)
    from flag4j_gb300 import build, synth
    build.build()
    E = Eng(local)
    L = E.L
    full = args.case == "full"
    n = args.n if args.n > 0 else (8192 if full else 2048)
    out = {}

    # ---- headline: split GEMM n^3, phi = 8
    A_h = synth.scaled(n, n, 8, 1, "row")
    B_h = synth.scaled(n, n, 8, 2, "col")
    A, B = E.dev(A_h), E.dev(B_h)
    C = E.ctx.alloc(8 * n * n)
    rep = E.gemm(A, B, C, n, n, n, L.MODE_SPLIT, report=True)
    E.ctx.sync()
    clk = Clocks(local)
    dist.barrier()
    E.ctx.sync()
    l0 = E.ctx.launches()
    clk.start()
    for _ in range(args.warmup):
        E.gemm(A, B, C, n, n, n, L.MODE_SPLIT)
    E.ctx.sync()
    dist.barrier()
    E.ctx.sync()
    l0 = E.ctx.launches()
    E.ctx.timer_record(0)
    for _ in range(args.steps):
        E.gemm(A, B, C, n, n, n, L.MODE_SPLIT)
    E.ctx.timer_record(1)
    ms_local = E.ctx.timer_elapsed(0, 1) / args.steps
    E.ctx.sync()
    launches = E.ctx.launches() - l0
    dist.barrier()
    clocks = clk.stop()
    ms = dist.max(ms_local)
    flops = 2.0 * n ** 3
    value = ws * flops / (ms * 1e-3) / 1e12
    abs_err, rel_err = E.check_err(A, B, C, n, n, n)
    # the library's own per-result accuracy report on one more product (outside the timed region)
    arep = E.gemm(A, B, C, n, n, n, L.MODE_SPLIT, report=True, check_samples=4096)
    accuracy_report = {"check_samples": arep.check_samples, "max_abs_err": arep.max_abs_err,
                       "max_rel_err": arep.max_rel_err, "plain_bound_rel": arep.plain_bound_rel,
                       "ref_kernel": L.REF_KERNELS[arep.ref_kernel],
                       "note": "f4j_report accuracy fields: sampled Dot2 error of this result, k u bound of a plain "
                               "FP64 product on the same scale, the CPU kernel Flag4j's dispatcher would run"}

    # dominant kernel time: the tcgen05 slice GEMM alone (same inputs), for the roofline
    s = rep.slices
    prods = s * (s + 1) // 2
    kp = math.ceil(n / 128) * 128
    fp8_flops = prods * 2.0 * n * n * kp
    out["split"] = {"slices": s, "frac_bits": rep.frac_bits, "exp_spread_bits": round(rep.exp_spread, 3),
                    "launches_per_step": launches / args.steps, "max_abs_err": abs_err, "max_rel_err": rel_err,
                    "ms": ms_local, "fp8_products": prods, "accuracy_report": accuracy_report}

    if not args.skip_extras:
        # ---- plain DMMA path on the same inputs
        pms = E.timed(lambda: E.gemm(A, B, C, n, n, n, L.MODE_PLAIN), 1 if full else 3, 1)
        pa, pr = E.check_err(A, B, C, n, n, n)
        out["plain_dmma"] = {"tflops": flops / (pms * 1e-3) / 1e12, "ms": pms, "max_abs_err": pa, "max_rel_err": pr}
        out["split_vs_plain_speedup"] = pms / ms_local
        # ---- errors for phi in {0, 8, 32}: split vs plain (double-double sampled check)
        errs = {}
        for phi in (0, 8, 32):
            Ap, Bp = E.dev(synth.scaled(n, n, phi, 10 + phi, "row")), E.dev(synth.scaled(n, n, phi, 20 + phi, "col"))
            r = E.gemm(Ap, Bp, C, n, n, n, L.MODE_SPLIT, report=True)
            se = E.check_err(Ap, Bp, C, n, n, n)
            E.gemm(Ap, Bp, C, n, n, n, L.MODE_PLAIN)
            pe = E.check_err(Ap, Bp, C, n, n, n)
            errs[str(phi)] = {"slices": r.slices, "split_max_rel_err": se[1], "plain_max_rel_err": pe[1],
                              "split_max_abs_err": se[0], "plain_max_abs_err": pe[0]}
            del Ap, Bp
        out["errors_by_phi"] = errs
        del A, B
        # ---- C1: Matrix.mult at 1024^3, U[-1,1) entries, in AUTO (split), PLAIN and EXACT modes
        c1n = 1024
        A1, B1 = synth.uniform(c1n, c1n, 61), synth.uniform(c1n, c1n, 62)
        dA1, dB1, dC1 = E.dev(A1), E.dev(B1), E.ctx.alloc(8 * c1n * c1n)
        c1 = {"n": c1n}
        for name, md in (("auto", L.MODE_AUTO), ("plain", L.MODE_PLAIN), ("exact", L.MODE_EXACT)):
            r1 = E.gemm(dA1, dB1, dC1, c1n, c1n, c1n, md, report=True)
            t1 = E.timed(lambda: E.gemm(dA1, dB1, dC1, c1n, c1n, c1n, md), 10, 3)
            c1[name] = {"ms": t1, "tflops": 2.0 * c1n ** 3 / (t1 * 1e-3) / 1e12, "mode_used": r1.mode_used,
                        "slices": r1.slices}
        out["c1_gemm_1024"] = c1
        out["c1_gemm_1024"]["l2"] = "A, B 8 MiB each: L2-resident across steps (a 1024^3 product fits in L2)"
        del dA1, dB1, dC1
        # ---- matrix-vector product n x n (Matrix.mult(Vector) in AUTO mode: one FP64 FMA dot product per
        # row, A read once; A is 512 MiB at 8192, larger than L2)
        Av, xv, yv = E.dev(synth.normal(n, n, 51)), E.dev(synth.normal(n, 1, 52)), E.ctx.alloc(8 * n)
        mrep = E.gemm(Av, xv, yv, n, 1, n, L.MODE_AUTO, report=True)
        t_mv = E.timed(lambda: E.gemm(Av, xv, yv, n, 1, n, L.MODE_AUTO), 20, 3)
        hbm_peak, _ = measured_peaks()
        out["matvec"] = {"n": n, "ms": t_mv, "gbs": 8.0 * n * n / t_mv / 1e6,
                         "frac_hbm": 8.0 * n * n / t_mv / 1e6 / hbm_peak, "gflops": 2.0 * n * n / t_mv / 1e6,
                         "mode_used": mrep.mode_used, "basis": "A's 8 n^2 bytes read once per product"}
        del Av, xv, yv
        # ---- Complex128 n/2 ^3 (8mnk basis)
        nz = n // 2
        Az = synth.scaled(nz, nz, 8, 3, "row", cplx=True)
        Bz = synth.scaled(nz, nz, 8, 4, "col", cplx=True)
        dAz, dBz, dCz = E.dev(Az), E.dev(Bz), E.ctx.alloc(16 * nz * nz)
        zr = E.gemm(dAz, dBz, dCz, nz, nz, nz, L.MODE_SPLIT, cplx=True, report=True)
        zms = E.timed(lambda: E.gemm(dAz, dBz, dCz, nz, nz, nz, L.MODE_SPLIT, cplx=True), 3, 1)
        zs = E.check_err(dAz, dBz, dCz, nz, nz, nz, cplx=True)
        zpms = E.timed(lambda: E.gemm(dAz, dBz, dCz, nz, nz, nz, L.MODE_PLAIN, cplx=True), 1, 1)
        zp = E.check_err(dAz, dBz, dCz, nz, nz, nz, cplx=True)
        zf = 8.0 * nz ** 3
        out["complex"] = {"n": nz, "split_tflops": zf / (zms * 1e-3) / 1e12, "split_ms": zms, "slices": zr.slices,
                          "split_max_rel_err": zs[1], "plain_tflops": zf / (zpms * 1e-3) / 1e12,
                          "plain_max_rel_err": zp[1]}
        del dAz, dBz, dCz
        # the same product end to end from page-locked host memory (f4j_zgemm_host, CMatrix.mult's entry)
        from flag4j_gb300.device import pinned_empty
        Azh, Bzh, Czh = (pinned_empty((nz, nz), np.complex128), pinned_empty((nz, nz), np.complex128),
                         pinned_empty((nz, nz), np.complex128))
        Azh[...] = Az
        Bzh[...] = Bz
        zhe = E.timed(lambda: E.check(E.lib.f4j_zgemm_host(E.ctx.handle, nz, nz, nz, Azh.ctypes.data, 0,
                                                           Bzh.ctypes.data, 0, Czh.ctypes.data, L.MODE_SPLIT,
                                                           None)), 3, 1)
        out["complex"]["e2e"] = {"value": zf / (zhe * 1e-3) / 1e12, "unit": "TFLOP/s", "ms": zhe,
                                 "h2d_bytes_per_step": Azh.nbytes + Bzh.nbytes, "d2h_bytes_per_step": Czh.nbytes,
                                 "path": "f4j_zgemm_host on page-locked host A, B, C (interleaved complex): B up "
                                         "whole, then A in 4 row parts, each sliced and multiplied as it arrives "
                                         "and its rows of C downloaded behind its product"}
        del Azh, Bzh, Czh
        # ---- dense adjoint step: A (n/2 x n/4), B (n/4 x n/2), split
        ma, ka = n // 2, n // 4
        Aa, Ba, Wa = (E.dev(synth.normal(ma, ka, 5)), E.dev(synth.normal(ka, ma, 6)),
                      E.dev(synth.normal(ma, ma, 7)))
        Ca, dA, dB = E.ctx.alloc(8 * ma * ma), E.ctx.alloc(8 * ma * ka), E.ctx.alloc(8 * ka * ma)
        fwd = E.timed(lambda: E.gemm(Aa, Ba, Ca, ma, ma, ka, L.MODE_SPLIT), 3, 1)

        def step():
            E.gemm(Aa, Ba, Ca, ma, ma, ka, L.MODE_SPLIT)
            E.check(E.lib.f4j_dgemm_adjoint(E.ctx.handle, ma, ma, ka, Aa.handle, Ba.handle, Wa.handle, dA.handle,
                                            dB.handle, L.MODE_SPLIT, None))
        fb = E.timed(step, 3, 1)
        out["adjoint"] = {"shape": [ma, ka, ma], "forward_ms": fwd, "fwd_bwd_ms": fb, "ratio": fb / fwd}
        del Aa, Ba, Wa, Ca, dA, dB
        out["spmm"] = sparse_section(E, full)

    # ---- roofline of the dominant kernel (the tcgen05 slice GEMM), timed alone
    # with CUDA events around its launch on the context stream
    A, B = E.dev(A_h), E.dev(B_h)
    kms, prep_ms = E.kernel_ms(lambda: E.gemm(A, B, C, n, n, n, L.MODE_SPLIT), max(3, args.steps // 2), True)
    out["split"]["prep_kernels_ms"] = prep_ms
    out["split"]["gemm_kernel_ms"] = kms
    del A, B
    # peak: the measured dense bf16 burst rate of MEASURED_PEAKS.json, doubled for
    # E4M3 (the tcgen05 pipe runs kind::f8f6f4 at twice kind::f16); the FP8 rate
    # cuBLASLt reaches in this run is reported beside it
    fp8_peak, fp8_src = fp8_peak_from_file()
    fp8_run, fp8_run_src = fp8_peak_tflops() if not args.skip_extras else (None, None)
    achieved = fp8_flops / (kms * 1e-3) / 1e12
    traffic = SPLIT_GEMM_DRAM_BYTES_8192.get(s) if n == 8192 else None
    roofline = {"bound": "tensor", "achieved": achieved, "peak": fp8_peak, "unit": "TFLOP/s",
                "frac": achieved / fp8_peak, "traffic": traffic,
                "traffic_note": "DRAM bytes per launch from one ncu capture of the 8192^3 launch (read + write); "
                                "the kernel is tensor-bound, 0.76 GB/ms of DRAM" if traffic else None,
                "kernel": "k_split_gemm (tcgen05 kind::f8f6f4)",
                "kernel_ms": kms, "kernel_share_of_step": kms / ms_local,
                "basis": "FP8 MMA flops per launch: s(s+1)/2 slice products x 2 n n Kp",
                "peak_source": fp8_src + ", of measured",
                "cublaslt_fp8_this_run": fp8_run, "frac_of_cublaslt_fp8_this_run":
                    achieved / fp8_run if fp8_run else None, "cublaslt_fp8_source": fp8_run_src}
    fp64_peak = fp64_peak_tflops() if not args.skip_extras else None
    if fp64_peak:
        out["fp64_dgemm_peak_tflops"] = fp64_peak
        # plain DMMA against the same run's cuBLAS DGEMM: GB300 issues mma.sync f64 to its FP64
        # pipe, which ncu shows 93 % busy in k_gemm_dmma (profiles/k_gemm_dmma_2048cube.md)
        pt = out["plain_dmma"]["tflops"]
        out["plain_dmma"]["roofline"] = {"bound": "fp64 (DMMA on the FP64 pipe)", "achieved": pt, "peak": fp64_peak,
                                         "unit": "TFLOP/s", "frac": pt / fp64_peak, "kernel": "k_gemm_dmma",
                                         "peak_source": "cuBLAS DGEMM 8192^3 (torch.matmul float64) in this run, "
                                                        "best of 3; MEASURED_PEAKS.json has no FP64 figure",
                                         "basis": "2 n^3 flops per product"}

    # ---- end to end through the host-buffer API (page-locked host memory from f4j_host_alloc)
    from flag4j_gb300.device import pinned_empty
    Ah, Bh, Ch = pinned_empty((n, n)), pinned_empty((n, n)), pinned_empty((n, n))
    Ah[...] = A_h
    Bh[...] = B_h
    # the host-buffer entry point: A, B up, split product, C down, C's download
    # overlapping the later row parts' products (f4j_dgemm_host)
    def e2e():
        E.check(E.lib.f4j_dgemm_host(E.ctx.handle, n, n, n, Ah.ctypes.data, 0, Bh.ctypes.data, 0, Ch.ctypes.data,
                                     L.MODE_SPLIT, None))
    e2e_ms = E.timed(e2e, max(3, args.steps // 3), 2)
    e2e_ms = dist.max(e2e_ms)
    # the same call on pageable arrays page-locked per call (f4j_set_host_pinning): what a JVM binding
    # passing its heap arrays through a critical downcall gets
    Ahp, Bhp, Chp = np.array(A_h), np.array(B_h), np.empty((n, n))
    E.check(E.lib.f4j_set_host_pinning(E.ctx.handle, 1))

    def e2e_pageable():
        E.check(E.lib.f4j_dgemm_host(E.ctx.handle, n, n, n, Ahp.ctypes.data, 0, Bhp.ctypes.data, 0,
                                     Chp.ctypes.data, L.MODE_SPLIT, None))
    e2e_pg_ms = dist.max(E.timed(e2e_pageable, 3, 1))
    E.check(E.lib.f4j_set_host_pinning(E.ctx.handle, 0))
    del Ahp, Bhp, Chp

    cb = None
    if rank == 0 and ws == 1:
        from oracle import oracle as O
        O.build()
        cb = cpu_baseline(n, n, seconds_target=15.0 if full else 3.0)
        # CPU baselines of the other rows, after every GPU measurement
        if not args.skip_extras:
            attach_sparse_cpu(out["spmm"], full)
            dcb = dense_cpu_baselines(n // 2, n // 2, n // 4)
            out["complex"]["cpu_baseline"] = dcb["complex"]
            out["adjoint"]["cpu_baseline"] = dcb["adjoint"]
            # C1 on the CPU: the whole 1024^3 product, all cores, 3 warm-ups, median of 5
            A1, B1 = synth.uniform(1024, 1024, 61), synth.uniform(1024, 1024, 62)
            threads = os.cpu_count() or 1
            for _ in range(3):
                O.dgemm(A1, B1, threads=threads)
            t1 = statistics.median(_wall(lambda: O.dgemm(A1, B1, threads=threads)) for _ in range(5))
            out["c1_gemm_1024"]["cpu_baseline"] = {"value": 2.0 * 1024 ** 3 / t1 / 1e12, "unit": "TFLOP/s",
                                                   "ms": 1e3 * t1, "cores": threads, "kind": "port",
                                                   "sample": "the whole 1024^3 product, median of 5 after 3 warm-ups"}

    dist.close()
    if rank != 0:
        return
    line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 (FP8 E4M3 slices, exact FP32/int64 accumulation)",
            "data": "synthetic (seeded PCG64)",
            "config": headline_config(n, ws),
            "roofline": roofline, "cpu_baseline": cb,
            "e2e": {"value": ws * flops / (e2e_ms * 1e-3) / 1e12, "unit": "TFLOP/s", "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": Ah.nbytes + Bh.nbytes, "d2h_bytes_per_step": Ch.nbytes,
                    "path": "f4j_dgemm_host (split) on page-locked host A, B, C (f4j_host_alloc): uploads back "
                            "to back (A's first 1024 rows, B in 4 column parts, the rest of A in 3 row parts), "
                            "each part sliced as it arrives, B's column parts multiplied by A's first rows and "
                            "A's later parts by all of B, each block of C downloaded behind its product (the "
                            "slice count from the first parts, checked against all of A and B)"},
            "e2e_pageable_pinned_per_call": {"value": ws * flops / (e2e_pg_ms * 1e-3) / 1e12, "unit": "TFLOP/s",
                                             "ms_per_step": e2e_pg_ms,
                                             "path": "f4j_dgemm_host on pageable host A, B, C with "
                                                     "f4j_set_host_pinning on (each call page-locks and "
                                                     "releases them), as a JVM binding passing heap arrays "
                                                     "through a critical downcall"},
            "gpu_launches": launches, "clocks": clocks}
    line.update(out)
    print(json.dumps(line))


def run_dmma_only(args):
    """Profiling helper: the plain DMMA GEMM alone, n^3 (2048 with --case small), uniform[-1, 1) operands;
    prints its own numbers, not the contract line."""
    from flag4j_gb300 import build, synth
    build.build()
    E = Eng(dist_env()[2])
    n = args.n if args.n > 0 else (8192 if args.case == "full" else 2048)
    A, B, C = E.dev(synth.uniform(n, n, 1)), E.dev(synth.uniform(n, n, 2)), E.ctx.alloc(8 * n * n)
    ms = E.timed(lambda: E.gemm(A, B, C, n, n, n, E.L.MODE_PLAIN), args.steps, args.warmup)
    print(json.dumps({"kernel": "k_gemm_dmma", "n": n, "ms": ms, "tflops": 2.0 * n ** 3 / (ms * 1e-3) / 1e12,
                      "steps": args.steps, "warmup": args.warmup}))


def run_spmv_only(args):
    """Profiling helper: SpMV y = S x at 2^20 rows, Poisson(16) row lengths (S is 200 MB, larger than
    L2), `warmup` + `steps` exact launches, then as many FMA launches; prints its own numbers."""
    from flag4j_gb300 import build, synth
    build.build()
    E = Eng(dist_env()[2])
    rows = 1 << 20
    rp, ci, v = synth.csr_poisson(rows, rows, seed=2024)
    S = E.f.CsrMatrix((rows, rows), v, rp, ci)  # owns the handle's buffers: keep it alive
    hS = S.handle(E.ctx)
    x, y = E.dev(synth.normal(rows, 1, 5).ravel()), E.ctx.alloc(8 * rows)
    out = {"kernel": "k_spmv", "rows": rows, "nnz": len(v)}
    for name, mode in (("exact", E.L.SPARSE_EXACT), ("fma", E.L.SPARSE_FMA)):
        out[name + "_ms"] = E.timed(lambda: E.check(E.lib.f4j_spmv_ex(E.ctx.handle, hS, x.handle, y.handle, mode,
                                                                        None)), args.steps, args.warmup)
    print(json.dumps(out))
    del S


def run_sddmm_only(args):
    """Profiling helper: SDDMM on S's pattern at 2^20 rows x 64 columns, `warmup` + `steps` launches."""
    from flag4j_gb300 import build, synth
    build.build()
    E = Eng(dist_env()[2])
    rows = 1 << 20
    rp, ci, v = synth.csr_poisson(rows, rows, seed=2024)
    S = E.f.CsrMatrix((rows, rows), v, rp, ci)  # owns the handle's buffers: keep it alive
    hS = S.handle(E.ctx)
    A, B, o = E.dev(synth.normal(rows, 64, 9)), E.dev(synth.normal(rows, 64, 8)), E.ctx.alloc(8 * len(v))
    ms = E.timed(lambda: E.check(E.lib.f4j_sddmm(E.ctx.handle, hS, A.handle, B.handle, 64, o.handle, None)),
                 args.steps, args.warmup)
    print(json.dumps({"kernel": "k_sddmm64s", "rows": rows, "nnz": len(v), "ms": ms,
                      "fp64_lane_ops_per_s": 64.0 * len(v) / (ms * 1e-3)}))
    del S


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.only_sparse:
        run_sparse_only(args)
    elif args.only_dmma:
        run_dmma_only(args)
    elif args.only_spmv:
        run_spmv_only(args)
    elif args.only_sddmm:
        run_sddmm_only(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
