"""The C++ drop-in header (include/fdcl_gb300.hpp): it compiles against the C
ABI (CPU) and its port of the reference's gtest checks passes on the GPU."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "test_dropin.cpp")


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.isdir(os.path.join(c, "include")):
            return c
    pytest.skip("CUDA headers not found")


def _compile(out, gblib):
    cuda = _cuda_home()
    cxx = shutil.which("g++") or pytest.skip("g++ not found")
    libdir = os.path.join(ROOT, "fftso3_gb300")
    cmd = [cxx, "-std=c++17", "-O2", "-fopenmp", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(cuda, "include"), SRC, "-o", out, "-L", libdir, "-lfftso3_gb300",
           "-L", os.path.join(cuda, "lib64"), "-lcudart", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_dropin_header_compiles(gblib, tmp_path):
    _compile(str(tmp_path / "test_dropin"), gblib)


@pytest.mark.gpu
def test_dropin_reference_checks_pass_on_gpu(gblib, tmp_path):
    exe = str(tmp_path / "test_dropin")
    _compile(exe, gblib)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PASSED" in r.stdout
