"""Every reference citation in the sources resolves: `path:line[-line][, line[-line]]` names one file
of the reference project and lines inside it.

A citation may name a file by its base name when that name is unique in the reference; where several
files share it (the library's primitives/*.cpp and vren_test's test files of the same name) enough of
the path must be given to pick one, e.g. ``vren/primitives/reduce.cpp`` or
``vren_test/primitives/reduce.cpp``.  The reference tree is located by ``VREN_REFERENCE_DIR``
(default: the reference checkout beside the build container); the test skips where it is absent.
"""
from __future__ import annotations

import collections
import os
import re
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
REFERENCE = Path(os.environ.get("VREN_REFERENCE_DIR", "/root/reference"))

# files and folders of this repository whose comments and docstrings cite the reference
CITING = ["include", "oracle", "vren_gb300", "tests", "DESIGN.md", "INTEGRATION.md", "bench.py",
          "__graft_entry__.py", "README.md"]
SKIP_SUFFIXES = (".so", ".o", ".pyc", ".a")
EXTENSIONS = "cpp|hpp|comp|glsl|h|cmake|txt|json|rst|md|frag|vert|mesh|task"
CITATION = re.compile(r"((?:[\w.\-]+/)*[\w\-]+\.(?:" + EXTENSIONS + r")):(\d+(?:-\d+)?(?:,\s?\d+(?:-\d+)?)*)")


def _reference_index() -> dict[str, list[str]]:
    index: dict[str, list[str]] = collections.defaultdict(list)
    for root, dirs, files in os.walk(REFERENCE):
        dirs[:] = [d for d in dirs if d != ".git"]
        for f in files:
            index[f].append(os.path.relpath(os.path.join(root, f), REFERENCE).replace(os.sep, "/"))
    return index


def _citing_files() -> list[Path]:
    out = []
    for entry in CITING:
        p = REPO / entry
        if p.is_file():
            out.append(p)
        elif p.is_dir():
            for q in sorted(p.rglob("*")):
                if q.is_file() and not q.name.endswith(SKIP_SUFFIXES) and "__pycache__" not in q.parts \
                        and "_build" not in q.parts and "_ref" not in q.parts:
                    out.append(q)
    return out


def _line_count(path: Path, cache: dict) -> int:
    if path not in cache:
        cache[path] = len(path.read_text(encoding="utf-8", errors="replace").splitlines())
    return cache[path]


@pytest.mark.skipif(not REFERENCE.is_dir(), reason="reference tree not present")
def test_every_reference_citation_resolves():
    index = _reference_index()
    counts: dict = {}
    problems = []
    checked = 0
    for src in _citing_files():
        text = src.read_text(encoding="utf-8", errors="replace")
        for lineno, line in enumerate(text.splitlines(), 1):
            for m in CITATION.finditer(line):
                name, ranges = m.group(1), m.group(2)
                base = name.rsplit("/", 1)[-1]
                cands = [c for c in index.get(base, []) if c == name or c.endswith("/" + name)]
                if not cands:
                    continue  # not a file of the reference (this repository's own files)
                where = f"{src.relative_to(REPO)}:{lineno}: {name}:{ranges}"
                if len(cands) > 1:
                    problems.append(f"{where}: ambiguous, matches {cands}")
                    continue
                n = _line_count(REFERENCE / cands[0], counts)
                checked += 1
                for part in ranges.replace(" ", "").split(","):
                    a, _, b = part.partition("-")
                    lo, hi = int(a), int(b) if b else int(a)
                    if not 1 <= lo <= hi <= n:
                        problems.append(f"{where}: lines {lo}-{hi} outside {cands[0]} ({n} lines)")
    assert checked > 200, f"only {checked} citations found"
    assert not problems, "\n".join(problems)
