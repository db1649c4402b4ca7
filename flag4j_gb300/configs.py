"""The dense-product dispatcher's configuration files, through the C ABI.

Flag4j reads ./configs/ReDeMatMult.properties, ./configs/CmDeMatMult.properties
and ./configs/GeneralConfigs.properties at class initialisation
(src/main/java/org/flag4j/linalg/ops/dispatch/configs/ReDeMatMultDispatchConfigs.java:89-121,
Cm128DeMatMultDispatchConfigs.java:85-108,
src/main/java/org/flag4j/concurrency/Configurations.java:68-88).  The library
reads the same files (f4j_config_load; on the first AUTO product from
./configs when never loaded) and adds the key gpuGemmMode = auto | split |
plain | exact.  F4J_MODE_AUTO then runs EXACT (the reference's order) below
smallThreshold entries of A plus B and for products of at most 2^24 flops, and
the configured GPU path otherwise.
"""
import ctypes

from . import _lib
from .device import check

_MODE_NAMES = {v: k for k, v in _lib.MODES.items()}


def load(directory=None):
    """Read the three files from `directory` (None: ./configs of the working directory)."""
    lib = _lib.load()
    check(lib.f4j_config_load(None if directory is None else str(directory).encode()))


def reset():
    """Back to the built-in defaults."""
    check(_lib.load().f4j_config_reset())


def get(complex=False):
    """The configuration in force: ReDeMatMult (real) or CmDeMatMult (complex) values."""
    out = _lib.f4j_dispatch_config()
    check(_lib.load().f4j_config_get(1 if complex else 0, ctypes.byref(out)))
    d = out.as_dict()
    d["gpu_gemm_mode"] = _MODE_NAMES[d["gpu_gemm_mode"]]
    return d


def general():
    """(blockSize, parallelism) from GeneralConfigs.properties."""
    bs, par = ctypes.c_int32(), ctypes.c_int32()
    check(_lib.load().f4j_config_general(ctypes.byref(bs), ctypes.byref(par)))
    return bs.value, par.value


def dispatch(m, n, k, mode="auto", complex=False):
    """(mode that runs, reference kernel name) for C (m x n) = A (m x k) B (k x n)."""
    md, rk = ctypes.c_int32(), ctypes.c_int32()
    check(_lib.load().f4j_dispatch(1 if complex else 0, m, n, k, _lib.MODES[mode], ctypes.byref(md),
                                   ctypes.byref(rk)))
    return _MODE_NAMES[md.value], _lib.REF_KERNELS[rk.value]
