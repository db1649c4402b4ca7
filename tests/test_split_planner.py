"""The split GEMM's device planner, walked on the host (no GPU needed).

tests/native/split_plan_check.cu includes the kernel source and calls its
__host__ __device__ plan_build for every slice count, band width and a range of
K, checking coverage, index ranges, stage sizes, the FP32 exactness budget and
group continuation (see the file's header)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not on PATH")
def test_split_planner_program_is_complete_and_in_range(tmp_path):
    exe = str(tmp_path / "split_plan_check")
    csrc = os.path.join(ROOT, "flag4j_gb300", "csrc")
    cmd = ["nvcc", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "--expt-relaxed-constexpr",
           "-I", os.path.join(ROOT, "include"), "-o", exe, os.path.join(HERE, "native", "split_plan_check.cu"),
           os.path.join(csrc, "f4j_core.cu"), os.path.join(csrc, "f4j_dense.cu"), os.path.join(csrc, "f4j_config.cu")]
    subprocess.run(cmd, check=True, capture_output=True, timeout=600)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout[-2000:] + out.stderr[-2000:]
    assert "plan check: ok" in out.stdout
