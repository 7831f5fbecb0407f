"""Every reference citation in the sources points at lines that exist.

The code cites the reference as ``<path>.jl:<line>[-<line>][,...]`` (also .m,
.txt, .toml, .sh files).  This test resolves each cited path against the
reference checkout (the directory in PTD_REFERENCE_DIR, by default the
reference's checkout next to this build) and checks every cited line number
against the length of that file.  It is skipped where no reference checkout
is present (the GPU machines carry none).
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("PTD_REFERENCE_DIR", "/root/reference")
SCANNED = ["oracle", "include", "pseudotransientdiffusion.jl_gb300", "tests", "bench.py", "__graft_entry__.py",
           "INTEGRATION.md", "DESIGN.md", "README.md"]
EXTS = (".c", ".h", ".cu", ".cuh", ".py", ".jl", ".md", "Makefile")
CITE = re.compile(r"([A-Za-z0-9_./-]+\.(?:jl|m|txt|toml|sh)):((?:\d+(?:-\d+)?)(?:,\s?\d+(?:-\d+)?)*)")


def _reference_files():
    out = {}
    for dp, _, fn in os.walk(REF):
        for f in fn:
            full = os.path.join(dp, f)
            out[os.path.relpath(full, REF)] = full
    return out


def _sources():
    for r in SCANNED:
        p = os.path.join(ROOT, r)
        if os.path.isfile(p):
            yield p
            continue
        for dp, _, fn in os.walk(p):
            if "_build" in dp or "__pycache__" in dp:
                continue
            for f in fn:
                if f.endswith(EXTS):
                    yield os.path.join(dp, f)


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "scripts")), reason="no reference checkout here")
def test_every_cited_line_exists():
    files = _reference_files()
    lengths = {}
    checked, bad = 0, []
    for src in _sources():
        with open(src, errors="replace") as fh:
            for ln, line in enumerate(fh, 1):
                for m in CITE.finditer(line):
                    name, ranges = m.group(1), m.group(2)
                    cands = sorted(f for f in files if f == name or f.endswith("/" + name))
                    if not cands:
                        continue   # not a reference file (e.g. a file of this repository)
                    path = cands[0]
                    if path not in lengths:
                        with open(files[path], errors="replace") as rf:
                            lengths[path] = sum(1 for _ in rf)
                    n = lengths[path]
                    for part in ranges.split(","):
                        lo, _, hi = part.strip().partition("-")
                        lo, hi = int(lo), int(hi or lo)
                        checked += 1
                        if not (1 <= lo <= hi <= n):
                            bad.append(f"{os.path.relpath(src, ROOT)}:{ln}: {name}:{part} ({path} has {n} lines)")
    assert checked > 100, checked
    assert not bad, "\n".join(bad)
