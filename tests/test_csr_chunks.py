"""The bottom solve's row chunks (csrc/ae_csr_chunks.h, host code): compiled with g++ and run on
random row lengths and chunk sizes (tests/cpp/csr_chunks_check.cpp)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_csr_chunks(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "csr_chunks_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "anisotropicfracture_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "csr_chunks_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
