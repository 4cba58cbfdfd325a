"""Host checks of device-side tables and arithmetic (no GPU): the
double-float arithmetic of the complex<double> pipelined kernels
(heffte_gb300/csrc/gbfft_common.cuh), compiled for the host from the same
header and checked against long double arithmetic (the scaled double <->
float-pair conversions, sums, products, the fused twiddle dot product, the
complex product and the radix-2/4/8 butterflies, each within its normwise
bound); the compile-time tables of the pipelined kernels; and the
compile-time radix plans of the runtime-radix kernels against the library's
plans."""
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


def test_pipelined_plans_and_swizzle_on_the_host(tmp_path):
    """The compile-time tables of the pipelined kernels (heffte_gb300/csrc/
    gbfft_pipe.cuh) evaluated on the host: radix plans multiply to their
    lengths (double-float plans with radices up to 8 and 8 values per
    thread), twiddle offsets in the Stockham layout, and the swizzle of the
    double-float line exchange a conflict-free permutation for every stage."""
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not found")
    root = os.path.dirname(HERE)
    exe = str(tmp_path / "check_plans")
    subprocess.run([nvcc, "-O1", "-std=c++17", "--expt-relaxed-constexpr", "-I" + os.path.join(root, "include"),
                    "-gencode", "arch=compute_103a,code=sm_103a", "-o", exe,
                    os.path.join(HERE, "df_host", "check_plans.cu")],
                   check=True, capture_output=True, cwd=str(tmp_path), timeout=600)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "plans and swizzle ok" in r.stdout, r.stdout


def test_compile_time_radix_plans_match_the_library(tmp_path, gb):
    """The constexpr radix plans of the runtime-radix pipelined kernels
    (ct_plan, heffte_gb300/csrc/gbfft_pipe_rt.cuh) against the plans the
    library builds, for every direct length up to 8192 that is not a power of
    two (linked against the built library; no GPU call)."""
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not found")
    from heffte_gb300 import build
    root = os.path.dirname(HERE)
    libdir = os.path.dirname(build.LIB)
    exe = str(tmp_path / "check_ct_plans")
    subprocess.run([nvcc, "-O1", "-std=c++17", "--expt-relaxed-constexpr", "-I" + os.path.join(root, "include"),
                    "-gencode", "arch=compute_103a,code=sm_103a", "-o", exe,
                    os.path.join(HERE, "df_host", "check_ct_plans.cu"), "-L" + libdir, "-lheffte_gb300",
                    "-Xlinker", "-rpath", "-Xlinker", libdir],
                   check=True, capture_output=True, cwd=str(tmp_path), timeout=600)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "compile-time plans ok" in r.stdout, r.stdout
