"""Every `path:line` citation of the reference in this repository points inside
the cited file, and names that file unambiguously.

Sources, headers, tests, the oracle and the design notes cite the reference
(fionser/YELL) as `include/yell/details/ntt.hpp:106-166` and the like.  This
test finds each such citation, resolves the path against the reference
checkout (a suffix must match exactly one file there) and checks that the line
range lies within that file.  It needs the reference checkout and is skipped
where it is absent.
"""
from __future__ import annotations

import os
import re

import pytest

REF = os.environ.get("YELL_REFERENCE_DIR", "/root/reference")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# Files written for this repository (the survey, the review and the baseline
# notes are inputs to it and are not checked).
SKIP_TOP = {"SURVEY.md", "VERDICT.md", "ADVICE.md", "BASELINE.md"}
SKIP_DIRS = ("_work", ".git", "gpurun_out", "oracle/_ref", "baseline", ".pytest_cache")
EXTS = (".py", ".c", ".cpp", ".cu", ".cuh", ".h", ".hpp", ".md", ".inc", ".txt", "Makefile")
CITE = re.compile(
    r"(?<![A-Za-z0-9_./-])((?:[A-Za-z0-9_.-]+/)*[A-Za-z0-9_.-]+\.(?:hpp|cpp|h|cc|txt|md|s)):(\d+)(?:-(\d+))?")


def _ref_files():
    out = []
    for d, _, fs in os.walk(REF):
        if "/.git" in d:
            continue
        out += [os.path.relpath(os.path.join(d, f), REF) for f in fs]
    return out


def _line_count(path):
    with open(path, "rb") as fh:
        data = fh.read()
    return data.count(b"\n") + (0 if data.endswith(b"\n") or not data else 1)


def _repo_files():
    for d, dirs, fs in os.walk(ROOT):
        rel = os.path.relpath(d, ROOT)
        if rel.startswith(SKIP_DIRS) or "_build" in rel or "__pycache__" in rel:
            dirs[:] = []
            continue
        for f in fs:
            if rel == "." and f in SKIP_TOP:
                continue
            if f.endswith(EXTS):
                yield os.path.join(d, f)


def _citations():
    ref_files = _ref_files()
    lengths = {}
    for path in _repo_files():
        with open(path, errors="replace") as fh:
            for ln, line in enumerate(fh, 1):
                for m in CITE.finditer(line):
                    cited = m.group(1)
                    cands = [r for r in ref_files if r == cited or r.endswith("/" + cited)]
                    if not cands:
                        continue  # not a reference path (a file of this repository)
                    a = int(m.group(2))
                    b = int(m.group(3) or a)
                    for c in cands:
                        if c not in lengths:
                            lengths[c] = _line_count(os.path.join(REF, c))
                    yield os.path.relpath(path, ROOT), ln, cited, a, b, cands, [lengths[c] for c in cands]


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "include", "yell")), reason="reference checkout absent")
def test_reference_citations_resolve():
    bad = []
    n = 0
    for where, ln, cited, a, b, cands, lens in _citations():
        n += 1
        if len(cands) > 1:
            bad.append(f"{where}:{ln}: {cited}:{a}-{b} is ambiguous ({', '.join(cands)})")
        elif not (1 <= a <= b <= lens[0]):
            bad.append(f"{where}:{ln}: {cited}:{a}-{b} outside {cands[0]} ({lens[0]} lines)")
    assert n > 100, f"only {n} citations found: the scan is broken"
    assert not bad, "\n".join(bad)
