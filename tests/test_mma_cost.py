"""The tensor-core cost model the contractions are built on, measured on the
GPU (tests/mma_cost.cu): a cta_group::1 M = 128 tcgen05.mma costs nearly the
same below N = 128 as at N = 128, so one MMA of N = 256 does four N = 64
MMAs' work for well under twice the cycles. tc_gemm64.cu groups B's BF16
slices into MMAs of N up to 256 and tc_gemm.cu pairs B's TF32 high and low
parts in one MMA on this basis."""

import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.gpu
def test_wide_mmas_cost_little_more_than_narrow_ones(gpu):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "mma_cost")
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-o", exe,
                        os.path.join(HERE, "mma_cost.cu")], check=True, capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=120).stdout
    cycles = {}
    for line in out.splitlines():
        parts = line.split()
        name = " ".join(parts[:3])
        assert parts[-1] == "0", line  # no wait gave up
        cycles[name] = float(parts[parts.index("cycles") + 1])
    assert cycles["f16 N256 R1"] < 2.0 * cycles["f16 N64 R1"], cycles
    assert cycles["f16 N128 R1"] < 1.25 * cycles["f16 N64 R1"], cycles
    assert cycles["tf32 N256 R1"] < 2.0 * cycles["tf32 N128 R1"], cycles
