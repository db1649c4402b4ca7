"""Build libflag4j_cuda.so in-tree for sm_103a (nvcc, no cmake).

Each translation unit is compiled in parallel, then linked into
``flag4j_gb300/libflag4j_cuda.so``.  The library is rebuilt unless a stamp
beside it holds the SHA-256 of everything that goes into it (sources,
headers, flags, the nvcc version and the machine), so a library built
elsewhere or from other sources is never reused.
``python -m flag4j_gb300.build [--force] [--verbose]``.
"""
import concurrent.futures as cf
import hashlib
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libflag4j_cuda.so")
STAMP = LIB + ".sha256"
SOURCES = ["f4j_core.cu", "f4j_dense.cu", "f4j_split.cu", "f4j_sparse.cu", "f4j_config.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-I", os.path.join(ROOT, "include")]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _deps():
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    hdrs.append(os.path.join(ROOT, "include", "flag4j_cuda.h"))
    return hdrs


def _nvcc_version():
    r = subprocess.run([nvcc(), "--version"], capture_output=True, text=True)
    return r.stdout


def source_hash():
    """SHA-256 over the sources, headers, flags, nvcc version and machine."""
    h = hashlib.sha256()
    for path in [os.path.join(CSRC, s) for s in SOURCES] + sorted(_deps()):
        h.update(os.path.basename(path).encode())
        with open(path, "rb") as f:
            h.update(f.read())
    h.update(repr((ARCH, FLAGS, platform.machine())).encode())
    h.update(_nvcc_version().encode())
    return h.hexdigest()


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    digest = source_hash()
    if not force and os.path.exists(LIB) and os.path.exists(STAMP):
        with open(STAMP) as f:
            if f.read().strip() == digest:
                return LIB
    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc(), *ARCH, "-shared", "-Xlinker", "--no-undefined", "-o", tmp, *[o for o, _ in results]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    with open(STAMP + ".tmp%d" % os.getpid(), "w") as f:
        f.write(digest + "\n")
    os.replace(STAMP + ".tmp%d" % os.getpid(), STAMP)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv))
