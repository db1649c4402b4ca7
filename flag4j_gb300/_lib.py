"""ctypes binding of libflag4j_cuda.so (the C ABI in include/flag4j_cuda.h).

The library is built in-tree by ``flag4j_gb300.build``.  Loading fails loudly
when it is missing: there is no CPU fallback for any product.
"""
import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libflag4j_cuda.so")

F4J_OK = 0
F4J_ERR_ARG = -1
F4J_ERR_SHAPE = -2
F4J_ERR_CSR = -3
F4J_ERR_OOM = -4
F4J_ERR_CUDA = -5
F4J_ERR_TIMEOUT = -6
F4J_ERR_UNSUPPORTED = -7

OP_N, OP_T, OP_C = 0, 1, 2
MODE_PLAIN, MODE_SPLIT, MODE_AUTO, MODE_EXACT = 0, 1, 2, 3
SPARSE_EXACT, SPARSE_FMA = 0, 1
SPARSE_MODES = {"exact": SPARSE_EXACT, "fma": SPARSE_FMA}
MODES = {"plain": MODE_PLAIN, "split": MODE_SPLIT, "auto": MODE_AUTO, "exact": MODE_EXACT}


CHECK_PLAIN = 1

REF_KERNELS = ["STRD", "REORD", "BLK", "BLK_REORD", "MT_STRD", "MT_REORD", "MT_BLK", "MT_BLK_REORD",
               "STRD_VEC_AS_MAT", "BLK_VEC_AS_MAT", "MT_STRD_VEC_AS_MAT", "MT_BLK_VEC_AS_MAT"]


class f4j_report(ctypes.Structure):
    _fields_ = [("mode_used", ctypes.c_int32), ("slices", ctypes.c_int32), ("launches", ctypes.c_int32),
                ("frac_bits", ctypes.c_int32), ("flops", ctypes.c_double), ("bytes", ctypes.c_double),
                ("exp_spread", ctypes.c_double), ("check_samples", ctypes.c_int32), ("check_flags", ctypes.c_int32),
                ("max_abs_err", ctypes.c_double), ("max_rel_err", ctypes.c_double),
                ("plain_bound_rel", ctypes.c_double), ("plain_max_abs_err", ctypes.c_double),
                ("plain_max_rel_err", ctypes.c_double), ("ref_kernel", ctypes.c_int32), ("reserved", ctypes.c_int32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


class f4j_dispatch_config(ctypes.Structure):
    _fields_ = [("cache_size", ctypes.c_double), ("aspect_threshold", ctypes.c_double),
                ("small_threshold", ctypes.c_int32), ("square_mt_standard_threshold", ctypes.c_int32),
                ("square_mt_reordered_threshold", ctypes.c_int32), ("wide_mt_reordered_threshold", ctypes.c_int32),
                ("square_sequential_vec_threshold", ctypes.c_int32), ("min_dim_small_threshold", ctypes.c_int32),
                ("gpu_gemm_mode", ctypes.c_int32), ("loaded", ctypes.c_int32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


# Every symbol declared in include/flag4j_cuda.h with its ctypes signature.
_v, _i, _i64, _u64, _sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_uint64, ctypes.c_size_t
_pv = ctypes.POINTER(ctypes.c_void_p)
_rep = ctypes.POINTER(f4j_report)
_pd = ctypes.POINTER(ctypes.c_double)
_pf = ctypes.POINTER(ctypes.c_float)
_pi64 = ctypes.POINTER(ctypes.c_int64)
SIGNATURES = {
    "f4j_version": (_i, []),
    "f4j_last_error": (ctypes.c_char_p, []),
    "f4j_create": (_i, [_i, _pv]),
    "f4j_destroy": (_i, [_v]),
    "f4j_sync": (_i, [_v]),
    "f4j_selftest_wait": (_i, [_v, _i64]),
    "f4j_set_stream": (_i, [_v, _v]),
    "f4j_get_stream": (_v, [_v]),
    "f4j_launch_count": (_i64, [_v]),
    "f4j_timer_record": (_i, [_v, _i]),
    "f4j_timer_elapsed": (_i, [_v, _i, _i, _pf]),
    "f4j_set_profiling": (_i, [_v, _i]),
    "f4j_profile_read": (_i, [_v, _i, _pd, _pi64]),
    "f4j_profile_reset": (_i, [_v]),
    "f4j_buf_alloc": (_i, [_v, _sz, _pv]),
    "f4j_buf_wrap": (_i, [_v, _v, _sz, _pv]),
    "f4j_buf_free": (_i, [_v, _v]),
    "f4j_buf_size": (_sz, [_v]),
    "f4j_buf_device_ptr": (_v, [_v]),
    "f4j_buf_upload": (_i, [_v, _v, _v, _sz, _sz]),
    "f4j_buf_download": (_i, [_v, _v, _v, _sz, _sz]),
    "f4j_buf_upload_async": (_i, [_v, _v, _v, _sz, _sz]),
    "f4j_buf_download_async": (_i, [_v, _v, _v, _sz, _sz]),
    "f4j_buf_zero": (_i, [_v, _v]),
    "f4j_host_register": (_i, [_v, _sz]),
    "f4j_host_alloc": (_i, [_sz, ctypes.POINTER(ctypes.c_void_p)]),
    "f4j_host_free": (_i, [_v]),
    "f4j_host_unregister": (_i, [_v]),
    "f4j_dgemm": (_i, [_v, _i64, _i64, _i64, _v, _i, _v, _i, _v, _i, _rep]),
    "f4j_dgemm_host": (_i, [_v, _i64, _i64, _i64, _v, _i, _v, _i, _v, _i, _rep]),
    "f4j_zgemm_host": (_i, [_v, _i64, _i64, _i64, _v, _i, _v, _i, _v, _i, _rep]),
    "f4j_set_host_pinning": (_i, [_v, _i]),
    "f4j_zgemm": (_i, [_v, _i64, _i64, _i64, _v, _i, _v, _i, _v, _i, _rep]),
    "f4j_dgemm_adjoint": (_i, [_v, _i64, _i64, _i64, _v, _v, _v, _v, _v, _i, _rep]),
    "f4j_zgemm_adjoint": (_i, [_v, _i64, _i64, _i64, _v, _v, _v, _v, _v, _i, _rep]),
    "f4j_gemm_check": (_i, [_v, _i, _i64, _i64, _i64, _v, _i, _v, _i, _v, _i64, _u64, _pd, _pd]),
    "f4j_dgemm_split_noalloc": (_i, [_i64, _i64, _i64, _v, _i, _v, _i, _v, _v, ctypes.POINTER(ctypes.c_int32)]),
    "f4j_config_load": (_i, [ctypes.c_char_p]),
    "f4j_config_reset": (_i, []),
    "f4j_config_get": (_i, [_i, ctypes.POINTER(f4j_dispatch_config)]),
    "f4j_config_general": (_i, [ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]),
    "f4j_dispatch": (_i, [_i, _i64, _i64, _i64, _i, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]),
    "f4j_ref_kernel_name": (ctypes.c_char_p, [_i]),
    "f4j_csr_wrap": (_i, [_v, _i64, _i64, _i64, _v, _v, _v, _i, _pv]),
    "f4j_csr_from_coo": (_i, [_v, _i64, _i64, _i64, _v, _v, _v, _pv]),
    "f4j_coo_sort": (_i, [_v, _i64, _v, _v, _v]),
    "f4j_csr_free": (_i, [_v, _v]),
    "f4j_csr_info": (_i, [_v, _pi64, _pi64, _pi64]),
    "f4j_csr_buffers": (_i, [_v, _pv, _pv, _pv]),
    "f4j_csr_transpose": (_i, [_v, _v, _pv]),
    "f4j_csr_mult_dense": (_i, [_v, _v, _v, _v, _rep]),
    "f4j_csr_mult_csr": (_i, [_v, _v, _v, _pv, _rep]),
    "f4j_csr_mult_dense_ex": (_i, [_v, _v, _i, _v, _i, _v, _rep]),
    "f4j_csr_mult_csr_ex": (_i, [_v, _v, _i, _v, _i, _pv, _rep]),
    "f4j_csr_transpose_perm": (_i, [_v, _v, _v]),
    "f4j_spmv": (_i, [_v, _v, _v, _v, _rep]),
    "f4j_spmv_ex": (_i, [_v, _v, _v, _v, _i, _rep]),
    "f4j_spmm": (_i, [_v, _v, _v, _i64, _v, _rep]),
    "f4j_zspmm": (_i, [_v, _v, _v, _i64, _v, _rep]),
    "f4j_spmm_ex": (_i, [_v, _v, _v, _i64, _v, _i, _rep]),
    "f4j_spmm_t": (_i, [_v, _v, _v, _i64, _v, _rep]),
    "f4j_sddmm": (_i, [_v, _v, _v, _v, _i64, _v, _rep]),
}

_lock = threading.Lock()
_lib = None


class Flag4jDeviceException(RuntimeError):
    """Device-side failure (CUDA error, allocation failure, bounded wait expiry)."""


def load():
    """Load libflag4j_cuda.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise Flag4jDeviceException(
                    "libflag4j_cuda.so is not built (run `python -m flag4j_gb300.build`); "
                    "there is no CPU fallback")
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def last_error():
    msg = load().f4j_last_error()
    return msg.decode() if msg else ""
