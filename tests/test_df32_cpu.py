"""Compensated FP32 ("float-float") arithmetic of the complex128 kernels, checked on the
host: the header is __host__ __device__, so the same code compiles with g++."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_df32_error_bounds(tmp_path):
    exe = str(tmp_path / "df32_check")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "qtnh_gb300", "csrc"),
                           "-o", exe, os.path.join(HERE, "cpp", "df32_check.cpp")])
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "ok" in out.stdout


def test_ozaki_slices_exact_and_accurate(tmp_path):
    exe = str(tmp_path / "ozaki_check")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "qtnh_gb300", "csrc"),
                           "-o", exe, os.path.join(HERE, "cpp", "ozaki_check.cpp")])
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "ok" in out.stdout


def test_ozaki_gemm_arithmetic(tmp_path):
    """The digit GEMM's chunked exact level sums, integer/FP32 accumulation and final
    scaling (ozaki.cuh, as gemm_oz.cu uses them) against long double."""
    exe = str(tmp_path / "ozaki_gemm_check")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "qtnh_gb300", "csrc"),
                           "-o", exe, os.path.join(HERE, "cpp", "ozaki_gemm_check.cpp")])
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "ok" in out.stdout


def test_ozaki_fixed_point_chain(tmp_path):
    """Consecutive fused gate pairs passing the state as 64-bit fixed point (ozaki.cuh, as
    gate_umma.cu's chain uses it) against long double."""
    exe = str(tmp_path / "ozaki_chain_check")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "qtnh_gb300", "csrc"),
                           "-o", exe, os.path.join(HERE, "cpp", "ozaki_chain_check.cpp")])
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "ok" in out.stdout
