"""Nodal AMReX plotfiles: the "node" half of Integrator::WritePlotFile
(src/Integrator/Integrator.cpp:582-681), written by libaefast's ae_write_plotfile, and a reader
for them.

A plotfile is a directory: `Header` (HyperCLaw-V1.1), then per level `Level_<l>/Cell_H` (the VisMF
header) and `Level_<l>/Cell_D_00000` (one FAB: a text line, then raw doubles).  VisIt and yt read
it; so does the reference's scripts/analyze.py."""
import ctypes as C
import os
import re
import warnings

import numpy as np

from ._lib import Fab, check, load
from .elastic import Field


def component_names(name, ncomp):
    """Names of a field's components as the reference writes them: the name itself for one
    component, else name001, name002, ... (amrex::Concatenate(name, j, 3),
    src/Integrator/Integrator.cpp:600-607)."""
    return [name] if ncomp == 1 else ["%s%03d" % (name, j) for j in range(1, ncomp + 1)]


def write_plotfile(path, levels, fields, names, time=0.0, steps=None):
    """Write one plotfile directory.  levels: one ae_level_desc per AMR level (elastic.level_desc);
    fields: one Field per level (host numpy FP64, ncomp components, box covering the level's valid
    box); names: ncomp component names."""
    n = len(levels)
    if len(fields) != n:
        raise ValueError("one field per level")
    descs = (type(levels[0]) * n)(*levels)
    keep = [np.ascontiguousarray(f.arr, dtype=np.float64) for f in fields]
    fabs = (Fab * n)()
    for l, (f, a) in enumerate(zip(fields, keep)):
        fabs[l] = Field(a, f.lo).fab()
    cnames = (C.c_char_p * len(names))(*[s.encode() for s in names])
    st = None if steps is None else (C.c_int * n)(*[int(s) for s in steps])
    check(load().ae_write_plotfile(os.fsencode(path), n, descs, fabs, len(names), cnames, float(time), st))


def WritePlotFile(plot_file, step, levels, node_fields, time=0.0, initial=False, steps=None):
    """Integrator::WritePlotFile for the node fields (src/Integrator/Integrator.cpp:582-681).
    node_fields: list of (name, [Field per level]).  Writes <plot_file>/<step:05d>[init]node and
    appends its Header to <plot_file>/nodeoutput.visit (created at step 0), as the reference does.
    A field holding NaN is reset to zero with a warning, as the reference does; an infinite value
    is an error.  Returns the plotfile directory."""
    nlev = len(levels)
    names, per_level = [], [[] for _ in range(nlev)]
    for name, flds in node_fields:
        arrs = [np.asarray(f.arr, dtype=np.float64) for f in flds]
        if any(np.isinf(a).any() for a in arrs):
            raise ValueError("%s contains inf" % name)
        if any(np.isnan(a).any() for a in arrs):
            warnings.warn("%s contains nan. Resetting to zero." % name)
            arrs = [np.zeros_like(a) for a in arrs]
        names += component_names(name, arrs[0].shape[0])
        for l in range(nlev):
            per_level[l].append((arrs[l], flds[l].lo))
    fields = []
    for l in range(nlev):
        lo0 = per_level[l][0][1]
        if any(lo != lo0 or a.shape[1:] != per_level[l][0][0].shape[1:] for a, lo in per_level[l]):
            raise ValueError("the node fields of a level must share one box")
        fields.append(Field(np.concatenate([a for a, _ in per_level[l]], axis=0), lo0))
    name = "%05d" % int(step) + ("init" if initial else "") + "node"
    out = os.path.join(plot_file, name)
    write_plotfile(out, levels, fields, names, time, steps)
    with open(os.path.join(plot_file, "nodeoutput.visit"), "w" if int(step) == 0 else "a") as f:
        f.write(name + "/Header\n")
    return out


_BOX = re.compile(r"\(\((-?\d+),(-?\d+),(-?\d+)\) \((-?\d+),(-?\d+),(-?\d+)\) \((\d+),(\d+),(\d+)\)\)")


def read_plotfile(path):
    """Read a plotfile written as above: returns a dict with the header fields ("names", "time",
    "finest_level", "prob_lo", "prob_hi", "ref_ratio", "domains", "steps", "dx") and "levels",
    one dict per level with "lo", "hi" (index box), "type" (0 cell, 1 node), "data"
    (ncomp, nz, ny, nx), "min", "max" (per component, from Cell_H) and "extent" (physical box)."""
    with open(os.path.join(path, "Header")) as f:
        lines = f.read().split("\n")
    it = iter(lines)
    out = {"version": next(it)}
    ncomp = int(next(it))
    out["names"] = [next(it) for _ in range(ncomp)]
    out["dim"] = int(next(it))
    out["time"] = float(next(it))
    out["finest_level"] = fl = int(next(it))
    out["prob_lo"] = [float(v) for v in next(it).split()]
    out["prob_hi"] = [float(v) for v in next(it).split()]
    out["ref_ratio"] = [int(v) for v in next(it).split()]
    out["domains"] = [tuple(int(v) for v in m) for m in _BOX.findall(next(it))]
    out["steps"] = [int(v) for v in next(it).split()]
    out["dx"] = [[float(v) for v in next(it).split()] for _ in range(fl + 1)]
    out["coord"] = int(next(it))
    out["bwidth"] = int(next(it))
    levels = []
    for _ in range(fl + 1):
        lev, nbox, t = next(it).split()
        step = int(next(it))
        extents = [[[float(v) for v in next(it).split()] for _ in range(out["dim"])] for _ in range(int(nbox))]
        prefix = next(it)
        levels.append(_read_level(path, prefix, int(lev), extents, step))
    out["levels"] = levels
    return out


def _read_level(path, prefix, lev, extents, step):
    ldir = os.path.join(path, os.path.dirname(prefix))
    with open(os.path.join(path, prefix + "_H")) as f:
        h = f.read().split("\n")
    ncomp = int(h[2])
    boxes = [m for m in _BOX.findall("\n".join(h))]
    fods = [ln.split() for ln in h if ln.startswith("FabOnDisk:")]
    mm = [ln for ln in h if re.match(r"^\d+,\d+$", ln)]
    vals = []
    for hdr in mm:
        i = h.index(hdr)
        vals.append([float(v) for v in h[i + 1].split(",") if v])
        h = h[i + 2:]
    b = [int(v) for v in boxes[0]]
    lo, hi, typ = b[0:3], b[3:6], b[6]
    _, fname, off = fods[0]
    with open(os.path.join(ldir, fname), "rb") as f:
        f.seek(int(off))
        line = f.readline().decode()
        fb = [int(v) for v in _BOX.findall(line)[0]]
        nc = int(line.rsplit(None, 1)[1])
        shape = (nc, fb[5] - fb[2] + 1, fb[4] - fb[1] + 1, fb[3] - fb[0] + 1)
        data = np.frombuffer(f.read(8 * int(np.prod(shape))), dtype="<f8").reshape(shape)
    return {"level": lev, "step": step, "lo": lo, "hi": hi, "type": typ, "ncomp": ncomp, "data": data,
            "min": vals[0], "max": vals[1], "extent": extents[0], "fab_header": line.rstrip("\n")}
