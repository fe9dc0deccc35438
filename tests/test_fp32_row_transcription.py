"""The FP32 branch of div_mm (csrc/ae_device.cuh) spells the MajorMinor divergence out in
explicitly rounded operations (fx_sop / __fadd_rn), beside the FP64 branch that keeps the
expression of src/Set/Matrix4_MajorMinor.H:287-345.  Both branches must be the same sum of
products: this test reads the two branches from the source and compares them symbolically
(b[p][q][r] symmetric in q, r, as the stencil fills it)."""
import os
import re

import pytest

sp = pytest.importorskip("sympy")

SRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "anisotropicfracture_gb300", "csrc",
                   "ae_device.cuh")


def _branches():
    src = open(SRC).read()
    a = src.index("__device__ __forceinline__ void div_mm(")
    body = src[a:src.index("#undef B", a)]
    fp32 = body[body.index("if constexpr (sizeof(R) == 4)"):body.index("return;")]
    fp64 = body[body.index("return;"):]
    return fp32, fp64


def _rows(text):
    a = sp.symbols("a0:21")
    syms = {}

    def B(p, q, r):
        key = (p,) + tuple(sorted((q, r)))
        if key not in syms:
            syms[key] = sp.Symbol("b%d%d%d" % key)
        return syms[key]

    def fx_sop(*args):
        return sum(args[i] * args[i + 1] for i in range(0, len(args), 2))

    env = {"a": a, "B": B, "fx_sop": fx_sop, "S2": lambda x, y: x + y, "S3": lambda x, y, z: x + y + z,
           "S4": lambda x, y, z, w: x + y + z + w}
    flat = " ".join(text.split())
    rows = {int(i): sp.expand(eval(e, env)) for i, e in re.findall(r"f\[(\d)\] = (.*?);", flat)}
    assert sorted(rows) == [0, 1, 2]
    return rows


def test_fp32_divergence_is_the_fp64_expression():
    fp32, fp64 = _branches()
    r32, r64 = _rows(fp32), _rows(fp64)
    for i in range(3):
        assert sp.expand(r32[i] - r64[i]) == 0, i


def test_divergence_is_symmetric_in_the_row_and_the_displacement_component():
    """Major and minor symmetry of C: the coefficient of u_p,jl in row i equals that of u_i,jl in
    row p (the operator is self-adjoint up to the boundary rows)."""
    _, fp64 = _branches()
    rows = _rows(fp64)
    for i in range(3):
        for p in range(3):
            ci = {s: rows[i].coeff(s) for s in rows[i].free_symbols if s.name.startswith("b%d" % p)}
            cp = {s: rows[p].coeff(s) for s in rows[p].free_symbols if s.name.startswith("b%d" % i)}
            for s, v in ci.items():
                t = sp.Symbol("b%d%s" % (i, s.name[2:]))
                assert sp.expand(v - cp.get(t, 0)) == 0, (i, p, s)
