"""The double-float arithmetic of the complex<double> pipelined kernels
(heffte_gb300/csrc/gbfft_common.cuh), compiled for the host from the same
header and checked against long double arithmetic (no GPU): the scaled
double <-> float-pair conversions, sums, products, the fused twiddle dot
product, the complex product and the radix-2/4/8 butterflies (one
renormalisation per output), each within its normwise bound."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_double_float_arithmetic_on_the_host(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "check_df")
    subprocess.run([nvcc, "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "df_host", "check_df.cu")],
                   check=True, capture_output=True, cwd=str(tmp_path), timeout=300)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
    assert r.stdout.count(" ok") == 12
