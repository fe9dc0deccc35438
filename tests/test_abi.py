"""The C-ABI library builds, loads and exports every symbol include/aefast.h declares.
No GPU calls: only host-side entry points are invoked."""
import ctypes as C
import os
import re
import subprocess

import pytest

from anisotropicfracture_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return set(re.findall(r"\b(ae_[a-z0-9_]+)\s*\(", src))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def test_header_symbols_exported(lib):
    declared = _declared("aefast.h")
    assert len(declared) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True, check=True)
    exported = set(re.findall(r"\sT\s(ae_[a-z0-9_]+)", out.stdout))
    assert declared <= exported, "declared but not exported: %s" % sorted(declared - exported)
    for name in declared:
        assert hasattr(lib, name)


def test_binding_covers_header(lib):
    assert set(_lib.SIGNATURES) == _declared("aefast.h")


def test_struct_layouts_match_header():
    # sizes of the ABI structs as a C compiler lays them out
    code = r"""
#include <stdio.h>
#include <stddef.h>
#include "aefast.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(ae_level_desc), sizeof(ae_fab), sizeof(ae_solver_opts),
         sizeof(ae_solve_stats), offsetof(ae_solver_opts, omega), sizeof(ae_cell_desc), sizeof(ae_cell_stats),
         offsetof(ae_cell_stats, mean_stress));
  return 0;
}
"""
    tmp = os.path.join(ROOT, "anisotropicfracture_gb300", "_build")
    os.makedirs(tmp, exist_ok=True)
    src = os.path.join(tmp, "abi_sizes.c")
    exe = os.path.join(tmp, "abi_sizes")
    open(src, "w").write(code)
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
    sizes = [int(v) for v in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert sizes == [C.sizeof(_lib.LevelDesc), C.sizeof(_lib.Fab), C.sizeof(_lib.SolverOpts),
                     C.sizeof(_lib.SolveStats), _lib.SolverOpts.omega.offset, C.sizeof(_lib.CellDesc),
                     C.sizeof(_lib.CellStats), _lib.CellStats.mean_stress.offset]


def test_host_only_entry_points(lib):
    o = _lib.default_opts()
    assert o.sweeps == 2 and abs(o.omega - 2.0 / 3.0) < 1e-15 and o.bottom_reltol == 1e-4
    assert o.nuf == 8 and o.max_iter == 200 and o.bottom_max_iter == 200
    assert lib.ae_version().decode().startswith("aefast")
    # argument errors are reported without touching a device
    h = C.c_void_p()
    assert lib.ae_op_create(None, 0, 0, C.byref(h)) == _lib.AE_ERR_ARG
    assert b"level" in lib.ae_last_error()
    assert lib.ae_op_num_amr_levels(None) == 0


def _levels(*descs):
    arr = (_lib.LevelDesc * len(descs))()
    for a, (cells, lo, hi, dx) in enumerate(descs):
        for d in range(3):
            arr[a].domain_cells[d], arr[a].lo[d], arr[a].hi[d], arr[a].dx[d] = cells, lo, hi, dx
    return arr


@pytest.mark.parametrize("descs,model,what", [
    ([(8, 0, 8, 0.125)], 4, b"model"),                                   # unknown stiffness kind
    ([(8, 0, 8, 0.0)], 0, b"dx"),                                        # non-positive spacing
    ([(8, 0, 9, 0.125)], 0, b"outside"),                                 # patch beyond the domain
    ([(8, 2, 8, 0.125)], 0, b"whole domain"),                            # level 0 must cover it
    ([(8, 0, 8, 0.125), (12, 4, 8, 0.0625)], 0, b"refine by 2"),         # refinement ratio
    ([(8, 0, 8, 0.125), (16, 3, 9, 0.0625)], 0, b"align"),               # odd fine patch corners
    ([(8, 0, 8, 0.125), (16, 2, 6, 0.0625), (16, 8, 12, 0.0625)], 0, b"separated"),  # patches' ghosts meet
    ([(8, 0, 8, 0.125), (16, 2, 6, 0.0625), (32, 20, 28, 0.03125)], 0, b"nest"),    # no parent patch
])
def test_level_descriptions_are_checked_on_the_host(lib, descs, model, what):
    """Operator::Elastic<T>::define's preconditions (src/Operator/Elastic.cpp:30-55) are checked
    before any device work, with the reference's Util::Abort turned into AE_ERR_ARG."""
    h = C.c_void_p()
    assert lib.ae_op_create(_levels(*descs), len(descs), model, C.byref(h)) == _lib.AE_ERR_ARG
    assert what in lib.ae_last_error()
    assert not h.value


def test_null_handles_are_argument_errors(lib):
    fab = _lib.Fab()
    assert lib.ae_op_set_model(None, 0, C.byref(fab)) == _lib.AE_ERR_ARG
    assert lib.ae_op_set_model_mixture(None, 0, C.byref(fab), 1, None, None, None) == _lib.AE_ERR_ARG
    assert lib.ae_op_set_model_degraded(None, 0, None, 0, 1.0, 1.0) == _lib.AE_ERR_ARG
    assert lib.ae_fapply(None, 0, 0, C.byref(fab), C.byref(fab)) == _lib.AE_ERR_ARG
    assert b"null" in lib.ae_last_error()
