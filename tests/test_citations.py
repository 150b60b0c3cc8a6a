"""Every `File.F90:line` citation of the reference in this repository's code
and design notes points inside the cited file.

The line counts come from tests/golden/reference_line_counts.json (written by
tests/golden/make_reference_line_counts.py from the reference tree); where
the reference tree itself is present, the fixture is checked against it too.
"""
import json
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIXTURE = os.path.join(ROOT, "tests", "golden", "reference_line_counts.json")
REFERENCE_DIRS = ("/root/reference",)

# name.F90:12, name.F90:12-40, name.F90:12,40-44
CITE = re.compile(r"\b([A-Za-z0-9_]+\.(?:F90|f90|sbatch))((?::\d+(?:-\d+)?(?:,\s?\d+(?:-\d+)?)*))")
# a bare "_QR.F90:..." shorthand would escape the check above: forbid it
SHORTHAND = re.compile(r"(?<![A-Za-z0-9])_Q[TRZ]\.F90:")

SCANNED_DIRS = ("include", "taylor-couette-afid_gb300", "oracle", "tests")
SCANNED_FILES = ("bench.py", "__graft_entry__.py", "DESIGN.md", "INTEGRATION.md", "README.md",
                 "BASELINE.md")
SUFFIXES = (".h", ".c", ".cu", ".cuh", ".cpp", ".py", ".F90", ".md", ".txt")


def _files():
    out = []
    for d in SCANNED_DIRS:
        for dp, dn, fn in os.walk(os.path.join(ROOT, d)):
            dn[:] = [x for x in dn if x not in ("_build", "__pycache__", "_ref")]
            out += [os.path.join(dp, f) for f in fn if f.endswith(SUFFIXES)]
    out += [os.path.join(ROOT, f) for f in SCANNED_FILES if os.path.exists(os.path.join(ROOT, f))]
    prof = os.path.join(ROOT, "profiles")
    if os.path.isdir(prof):
        out += [os.path.join(prof, f) for f in os.listdir(prof)]
    me = os.path.abspath(__file__)
    return sorted(p for p in out if os.path.abspath(p) != me)


def _citations():
    for path in _files():
        with open(path, errors="replace") as f:
            for ln, line in enumerate(f, 1):
                for m in CITE.finditer(line):
                    for part in m.group(2)[1:].split(","):
                        a = part.strip().split("-")
                        yield path, ln, m.group(1), int(a[0]), int(a[-1])


def _counts():
    with open(FIXTURE) as f:
        return json.load(f)


def test_fixture_matches_reference_tree():
    ref = next((d for d in REFERENCE_DIRS if os.path.isdir(d)), None)
    if ref is None:
        pytest.skip("reference tree not present on this machine")
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "mk", os.path.join(ROOT, "tests", "golden", "make_reference_line_counts.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    assert mk.line_counts(ref) == _counts()


def test_every_citation_is_inside_its_file():
    counts = _counts()
    bad, n = [], 0
    for path, ln, name, lo, hi in _citations():
        n += 1
        rel = os.path.relpath(path, ROOT)
        if name not in counts:
            bad.append(f"{rel}:{ln}: unknown reference file {name}")
        elif not (1 <= lo <= hi <= counts[name]):
            bad.append(f"{rel}:{ln}: {name}:{lo}-{hi} but the file has {counts[name]} lines")
    assert n > 100, "citation scan found too little: the pattern is broken"
    assert not bad, "\n".join(bad)


def test_no_citation_split_over_lines():
    """A `File.F90:` whose line numbers continue on the next line escapes
    the range check above."""
    bad = []
    for path in _files():
        with open(path, errors="replace") as f:
            for ln, line in enumerate(f, 1):
                if re.search(r"\.(?:F90|f90):\s*$", line):
                    bad.append(f"{os.path.relpath(path, ROOT)}:{ln}")
    assert not bad, "keep each citation on one line: " + ", ".join(bad)


def test_no_bare_line_citations():
    """"(:123)" inherits a file named somewhere above it: name the file."""
    bare = re.compile(r"[(\s,]:\d{2,4}(?:-\d+)?[),]")
    bad = []
    for path in _files():
        if not path.endswith((".h", ".c", ".cu", ".cuh", ".cpp", ".F90")) and not path.endswith("tc_np.py"):
            continue
        with open(path, errors="replace") as f:
            for ln, line in enumerate(f, 1):
                if bare.search(line):
                    bad.append(f"{os.path.relpath(path, ROOT)}:{ln}")
    assert not bad, "name the reference file of: " + ", ".join(bad)


def test_no_shorthand_citations():
    bad = []
    for path in _files():
        with open(path, errors="replace") as f:
            for ln, line in enumerate(f, 1):
                if SHORTHAND.search(line):
                    bad.append(f"{os.path.relpath(path, ROOT)}:{ln}")
    assert not bad, "cite SolveImpEqnUpdate_Q*.F90 by its full name: " + ", ".join(bad)
