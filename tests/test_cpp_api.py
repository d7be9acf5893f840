"""The C++ mirror of the crate's API (concrete-fft_gb300/cpp/concrete_fft.hpp):
it compiles against the C ABI here, and on a GPU its test program (the
reference's own tests, restated) passes."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "concrete-fft_gb300")


def build_cpp_test(cfft_lib, out):
    src = os.path.join(PKG, "cpp", "test_plan_api.cpp")
    libdir = os.path.join(PKG, "lib")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), src, "-o", out, "-L", libdir,
           "-lcfft_gb300", "-Wl,-rpath," + libdir]
    if os.uname().machine == "x86_64":
        cmd.append("-lquadmath")
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_cpp_api_compiles(cfft_lib, tmp_path):
    build_cpp_test(cfft_lib, str(tmp_path / "test_plan_api"))


@pytest.mark.gpu
def test_cpp_api_reference_tests_pass(cuda, tmp_path):
    import concrete_fft as cf
    exe = build_cpp_test(cf.load(), str(tmp_path / "test_plan_api"))
    r = subprocess.run([exe, os.path.join(ROOT, "tests", "golden")], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "ALL OK" in r.stdout, r.stdout[-4000:] + r.stderr[-2000:]
