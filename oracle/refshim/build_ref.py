"""Recipe: compile the reference's own per-node operator code into oracle/_ref/libref.so.

TEST INFRASTRUCTURE ONLY.  It reads the reference tree (default /root/reference/src, or
$AE_REFERENCE_SRC), copies nothing into the repository, and writes only under oracle/_ref/
(git-ignored):

  oracle/_ref/extracted.inc  the member-function definitions listed in FUNCTIONS, cut verbatim out
                             of src/Operator/Elastic.cpp and src/Operator/Operator.cpp (with #line
                             directives pointing back at them)
  oracle/_ref/libref.so      oracle/refshim/ref_driver.cpp + extracted.inc + the reference's
                             headers, compiled against the stand-ins in oracle/refshim/include

The reference itself cannot be built here (it needs AMReX 20.05, Eigen and MPI, none of which is
in the image); this compiles the parts of it that the per-node operator path consists of.  Flags:
-O2 -ffp-contract=off, i.e. every multiply and add rounded separately, as the reference's x86-64
build without FMA instructions rounds them.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
LIB = os.path.join(OUT, "libref.so")
INC = os.path.join(OUT, "extracted.inc")

# (file under src/, signature prefix, occurrence) -> a function definition extracted verbatim
FUNCTIONS = [
    ("Operator/Elastic.cpp", "Elastic<T>::Fapply (", 0),
    ("Operator/Elastic.cpp", "Elastic<T>::Diagonal (", 0),
    ("Operator/Elastic.cpp", "Elastic<T>::Strain  (", 0),
    ("Operator/Elastic.cpp", "Elastic<T>::Stress (", 0),
    ("Operator/Elastic.cpp", "Elastic<T>::Energy (", 0),
    ("Operator/Elastic.cpp", "Elastic<T>::averageDownCoeffsSameAmrLevel (", 0),
    ("Operator/Operator.cpp", "void Operator<Grid::Node>::Fsmooth (", 0),
    ("Operator/Operator.cpp", "void Operator<Grid::Node>::restriction (", 0),
    ("Operator/Operator.cpp", "void Operator<Grid::Node>::interpolation (", 0),
]


def reference_src():
    return os.environ.get("AE_REFERENCE_SRC", "/root/reference/src")


def available():
    return os.path.isfile(os.path.join(reference_src(), "Operator", "Elastic.cpp"))


def _match_brace(text, start):
    """Index just past the brace that closes the one at `start`, skipping comments and literals."""
    depth, i, n = 0, start, len(text)
    while i < n:
        c = text[i]
        if text.startswith("//", i):
            i = text.find("\n", i)
            i = n if i < 0 else i
            continue
        if text.startswith("/*", i):
            i = text.find("*/", i + 2) + 2
            continue
        if c in "\"'":
            j = i + 1
            while j < n and text[j] != c:
                j += 2 if text[j] == "\\" else 1
            i = j + 1
            continue
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                return i + 1
        i += 1
    raise ValueError("unbalanced braces")


def extract(path, prefix, occurrence=0):
    """(first line number, text) of one function definition: from the `template<...>` line (or
    the signature line itself) through its closing brace."""
    text = open(path).read()
    pos, idx = -1, -1
    for _ in range(occurrence + 1):
        pos = text.find(prefix, pos + 1)
        if pos < 0:
            raise ValueError("%s: %r not found" % (path, prefix))
    line_start = text.rfind("\n", 0, pos) + 1
    # include a `template<class T>\nvoid\n` preamble when the definition has one
    pre = text[:line_start]
    m = re.search(r"template\s*<\s*class\s+T\s*>\s*\n(?:[^\n]*\n)?$", pre)
    begin = m.start() if m else line_start
    body = text.find("{", pos)
    end = _match_brace(text, body)
    first_line = text.count("\n", 0, begin) + 1
    return first_line, text[begin:end]


def generate(src=None):
    src = src or reference_src()
    os.makedirs(OUT, exist_ok=True)
    parts = ["// GENERATED by oracle/refshim/build_ref.py from the reference tree; not committed.\n"]
    for rel, prefix, occ in FUNCTIONS:
        path = os.path.join(src, rel)
        line, code = extract(path, prefix, occ)
        parts.append('#line %d "%s"\n%s\n' % (line, path, code))
    with open(INC, "w") as f:
        f.write("".join(parts))
    return INC


def build(force=False, verbose=False):
    """Build oracle/_ref/libref.so; returns its path, or None when the reference tree is absent."""
    if not available():
        return None
    deps = [os.path.join(HERE, "ref_driver.cpp"), os.path.abspath(__file__)]
    for root, _, files in os.walk(os.path.join(HERE, "include")):
        deps += [os.path.join(root, f) for f in files]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    generate()
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w",
           "-I", OUT, "-I", os.path.join(HERE, "include"), "-I", reference_src(),
           os.path.join(HERE, "ref_driver.cpp"), "-o", LIB + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("building the reference-code library failed:\n%s\n%s" % (r.stdout, r.stderr[-6000:]))
    os.replace(LIB + ".tmp", LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    p = build(force=True, verbose=True)
    if p is None:
        sys.exit("reference tree not found at %s" % reference_src())
