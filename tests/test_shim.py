"""The C++ shim (include/alamo_elastic.H) compiles, agrees with the Python model constructors,
and drives a full solve through the C ABI like an Alamo integrator would."""
import os
import subprocess

import numpy as np
import pytest

from anisotropicfracture_gb300 import _lib, build, models

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OUT = os.path.join(ROOT, "anisotropicfracture_gb300", "_build")


def _compile(src, exe, link):
    os.makedirs(OUT, exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "shim", src),
           "-o", os.path.join(OUT, exe)]
    if link:
        cmd += ["-L", os.path.dirname(_lib.LIB_PATH), "-laefast", "-Wl,-rpath," + os.path.dirname(_lib.LIB_PATH)]
    subprocess.run(cmd, check=True)
    return os.path.join(OUT, exe)


def test_shim_cubic_define_matches_python():
    exe = _compile("cubic_define.cpp", "cubic_define", link=False)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    for line, ang in zip(out, [(0.3, 0.2, 0.1), (1.0, 2.0, 0.5), (0.0, np.pi / 2, 0.0)]):
        c = np.array([float(v) for v in line.split()])
        ref = models.cubic(1.68, 1.21, 0.75, models.euler_rotation(*ang))
        assert np.allclose(c, ref, rtol=0, atol=1e-14)


@pytest.mark.gpu
def test_shim_uniaxial_solve():
    build.build()
    exe = _compile("uniaxial_shim.cpp", "uniaxial_shim", link=True)
    r = subprocess.run([exe, "32"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert '"converged": 1' in r.stdout
