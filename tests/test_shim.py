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


@pytest.mark.gpu
def test_shim_neohookean_newton():
    """Newton<Elastic::NeoHookean> from C++ (the FiniteKinematics integrator's call): the uniaxial
    stretch lands on the exact homogeneous finite-strain solution."""
    build.build()
    exe = _compile("neohookean_shim.cpp", "neohookean_shim", link=True)
    r = subprocess.run([exe, "8"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_shim_writes_a_plotfile_without_a_gpu(tmp_path):
    """alamo::WritePlotFile (host fabs only) from C++: the reference's directory naming and .visit
    list, and the valid-box values of each level read back."""
    from anisotropicfracture_gb300 import plotfile
    build.build()
    exe = _compile("plotfile_shim.cpp", "plotfile_shim", link=True)
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == str(tmp_path / "00003node")
    with open(tmp_path / "nodeoutput.visit") as f:
        assert f.read() == "00000node/Header\n00003node/Header\n"
    p = plotfile.read_plotfile(str(tmp_path / "00003node"))
    assert p["time"] == 1.5 and p["names"] == ["disp001", "disp002", "disp003"]
    for lev, (lo, hi) in zip(p["levels"], [((0, 0, 0), (8, 8, 8)), ((4, 4, 4), (12, 12, 12))]):
        k, j, i = np.meshgrid(*[np.arange(lo[d], hi[d] + 1) for d in (2, 1, 0)], indexing="ij")
        want = np.stack([100.0 * q + i + 10.0 * j + 0.5 * k for q in range(3)])
        assert np.array_equal(lev["data"], want)


def test_shim_templates_instantiate():
    """Every member of Operator::Elastic<T> and Solver::Nonlocal::Newton<T> compiles for the
    isotropic, cubic and Laplacian models (explicit instantiation, compile only)."""
    src = os.path.join(ROOT, "tests", "shim", "instantiate_all.cpp")
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), src], check=True)
