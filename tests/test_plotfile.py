"""Nodal plotfiles (ae_write_plotfile, plotfile.WritePlotFile) on CPU: round trip through the
reader, the layout the reference's own reader (scripts/analyze.py) expects, the reference's
naming, and the error behaviour."""
import os
import re

import numpy as np
import pytest

from anisotropicfracture_gb300 import plotfile
from anisotropicfracture_gb300._lib import AeError
from anisotropicfracture_gb300.elastic import Field, level_desc
from oracle import pyoracle as po

pytestmark = pytest.mark.filterwarnings("ignore::UserWarning")


def two_levels():
    Ls = po.amr_levels(8, 2)
    descs = [level_desc(tuple(L.dom_hi), lo=tuple(L.lo), hi=tuple(L.hi), dx=tuple(L.dx)) for L in Ls]
    return Ls, descs


def fields(Ls, ncomp, seed):
    rng = np.random.default_rng(seed)
    return [Field(rng.standard_normal((ncomp,) + L.shape), tuple(L.lo[d] - L.ng for d in range(3))) for L in Ls]


def valid(L, a):
    g = L.ng
    return a if g == 0 else a[:, g:-g, g:-g, g:-g]


def test_round_trip(tmp_path):
    Ls, descs = two_levels()
    fl = fields(Ls, 4, 1)
    names = ["disp001", "disp002", "disp003", "energy"]
    out = str(tmp_path / "plt")
    plotfile.write_plotfile(out, descs, fl, names, time=0.25, steps=[7, 14])
    p = plotfile.read_plotfile(out)
    assert p["version"] == "HyperCLaw-V1.1" and p["names"] == names and p["dim"] == 3
    assert p["time"] == 0.25 and p["finest_level"] == 1 and p["ref_ratio"] == [2] and p["steps"] == [7, 14]
    assert p["prob_lo"] == [0.0] * 3 and p["prob_hi"] == [1.0] * 3
    assert p["domains"] == [(0, 0, 0, 7, 7, 7, 0, 0, 0), (0, 0, 0, 15, 15, 15, 0, 0, 0)]
    assert p["dx"] == [[0.125] * 3, [0.0625] * 3]
    for L, f, lev in zip(Ls, fl, p["levels"]):
        assert lev["lo"] == list(L.lo) and lev["hi"] == list(L.hi) and lev["type"] == 1
        want = valid(L, f.arr)
        assert np.array_equal(lev["data"], want)
        assert np.allclose(lev["min"], want.min(axis=(1, 2, 3)), rtol=1e-14, atol=0)
        assert np.allclose(lev["max"], want.max(axis=(1, 2, 3)), rtol=1e-14, atol=0)
        assert lev["extent"] == [[L.lo[d] * L.dx[d], L.hi[d] * L.dx[d]] for d in range(3)]
        assert lev["fab_header"].startswith("FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1)))((")


def test_layout_the_reference_reader_expects(tmp_path):
    """The parse of scripts/analyze.py, restated: header values separated by single spaces with a
    trailing space, one dx line per level, and the 3-D box regex over Level_<l>/Cell_H giving each
    level's covered volume."""
    Ls, descs = two_levels()
    out = str(tmp_path / "plt")
    plotfile.write_plotfile(out, descs, fields(Ls, 3, 2), ["u001", "u002", "u003"])
    with open(os.path.join(out, "Header")) as f:
        f.readline()
        nfields = int(f.readline())
        for _ in range(nfields):
            f.readline()
        dim = int(f.readline())
        f.readline()
        namrlevs = int(f.readline())
        lo = [float(d) for d in f.readline().replace(" \n", "").split(" ")]
        hi = [float(d) for d in f.readline().replace(" \n", "").split(" ")]
        for _ in range(3):
            f.readline()
        dx = [[float(d) for d in f.readline().replace(" \n", "").split(" ")] for _ in range(namrlevs + 1)]
    assert (nfields, dim, namrlevs, lo, hi) == (3, 3, 1, [0.0] * 3, [1.0] * 3)
    exp = re.compile(r"\(\(([0-9]*),([0-9]*),([0-9]*)\) \(([0-9]*),([0-9]*),([0-9]*)\) \(([0-9]*),([0-9]*),([0-9]*)\)\)")
    volumes = []
    for lev in range(namrlevs + 1):
        vol, patches = 0.0, 0
        with open(os.path.join(out, "Level_%d" % lev, "Cell_H")) as f:
            for line in f.readlines():
                res = exp.findall(line)
                if not res:
                    continue
                n = [int(res[0][3]) - int(res[0][0]), int(res[0][4]) - int(res[0][1]), int(res[0][5]) - int(res[0][2])]
                vol += n[0] * dx[lev][0] * n[1] * dx[lev][1] * n[2] * dx[lev][2]
                patches += 1
        assert patches == 1
        volumes.append(vol)
    assert volumes == [1.0, 0.125]


def test_write_plotfile_naming_and_visit_list(tmp_path):
    Ls, descs = two_levels()
    disp = fields(Ls, 3, 3)
    energy = fields(Ls, 1, 4)
    root = str(tmp_path / "out")
    os.makedirs(root)
    d0 = plotfile.WritePlotFile(root, 0, descs, [("disp", disp), ("energy", energy)])
    d1 = plotfile.WritePlotFile(root, 1, descs, [("disp", disp), ("energy", energy)], time=0.5)
    assert os.path.basename(d0) == "00000node" and os.path.basename(d1) == "00001node"
    with open(os.path.join(root, "nodeoutput.visit")) as f:
        assert f.read() == "00000node/Header\n00001node/Header\n"
    p = plotfile.read_plotfile(d1)
    assert p["names"] == ["disp001", "disp002", "disp003", "energy"] and p["time"] == 0.5
    assert np.array_equal(p["levels"][1]["data"][3], valid(Ls[1], energy[1].arr)[0])


def test_nan_field_is_reset_to_zero_and_inf_is_an_error(tmp_path):
    Ls, descs = two_levels()
    disp = fields(Ls, 3, 5)
    disp[1].arr[0, 4, 4, 4] = np.nan
    root = str(tmp_path / "out")
    os.makedirs(root)
    with pytest.warns(UserWarning):
        d = plotfile.WritePlotFile(root, 0, descs, [("disp", disp)], initial=True)
    assert os.path.basename(d) == "00000initnode"
    p = plotfile.read_plotfile(d)
    assert all(np.all(lev["data"] == 0.0) for lev in p["levels"])
    disp[1].arr[0, 4, 4, 4] = np.inf
    with pytest.raises(ValueError):
        plotfile.WritePlotFile(root, 1, descs, [("disp", disp)])


def test_writer_rejects_bad_arguments(tmp_path):
    Ls, descs = two_levels()
    fl = fields(Ls, 1, 6)
    with pytest.raises(AeError):  # whitespace in a component name
        plotfile.write_plotfile(str(tmp_path / "a"), descs, fl, ["bad name"])
    with pytest.raises(AeError):  # the fab does not cover the valid box
        short = [fl[0], Field(fl[1].arr[:, 3:, 3:, 3:], tuple(v + 3 for v in fl[1].lo))]
        plotfile.write_plotfile(str(tmp_path / "b"), descs, short, ["e"])
    bad = fields(Ls, 1, 7)
    bad[0].arr[0, 0, 0, 0] = np.nan
    with pytest.raises(AeError) as e:
        plotfile.write_plotfile(str(tmp_path / "c"), descs, bad, ["e"])
    assert e.value.code == -2
