"""Every reference citation `path/to/file.cc:12-34` in the sources and the
integration documents names lines that exist in the reference checkout (CPU).

A citation names a reference file by its path inside the reference project,
or by its bare file name; it counts as valid when some reference file with
that path (or name) has at least as many lines as the highest cited line.
Names that are not reference files (this repository's own files) are not
checked.  Skipped where the reference checkout is absent."""
import os
import re
import runpy

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SCAN = ["include", "mpas-o-flecsi-2.0_gb300", "oracle", "tests", "bench.py", "__graft_entry__.py",
        "DESIGN.md", "INTEGRATION.md", "README.md"]
EXT = (".py", ".c", ".cc", ".cu", ".cuh", ".h", ".hh", ".md")
CITE = re.compile(r"((?:[A-Za-z0-9_.\-]+/)*[A-Za-z0-9_\-]+\.(?:cc|hh|h|txt|cmake|py|yml))\s*:\s*(\d+)"
                  r"(?:\s*[-–]\s*(\d+))?((?:\s*,\s*\d+(?:\s*[-–]\s*\d+)?)*)")


def _reference_dir():
    ref = runpy.run_path(os.path.join(ROOT, "oracle", "build.py"), run_name="oracle_build_paths")["REF"]
    return ref if os.path.isdir(os.path.join(ref, "apps")) else None


def _sources():
    for d in SCAN:
        p = os.path.join(ROOT, d)
        if os.path.isfile(p):
            yield p
            continue
        for dp, dn, fn in os.walk(p):
            dn[:] = [x for x in dn if x not in ("_build", "_ref", "__pycache__", "lib")]
            for f in fn:
                if f.endswith(EXT):
                    yield os.path.join(dp, f)


def test_reference_citations_exist():
    ref = _reference_dir()
    if ref is None:
        pytest.skip("reference checkout absent")
    by_name = {}
    for dp, dn, fn in os.walk(ref):
        dn[:] = [x for x in dn if x != ".git"]
        for f in fn:
            by_name.setdefault(f, []).append(os.path.join(dp, f))
    lines = {}

    def n_lines(p):
        if p not in lines:
            with open(p, errors="replace") as fh:
                lines[p] = sum(1 for _ in fh)
        return lines[p]

    bad, checked = [], 0
    for src in _sources():
        with open(src, errors="replace") as fh:
            for ln, text in enumerate(fh, 1):
                for m in CITE.finditer(text):
                    path = m.group(1)
                    cands = [c for c in by_name.get(os.path.basename(path), [])
                             if "/" not in path or c.endswith("/" + path)]
                    if not cands:
                        continue
                    hi = max([int(m.group(3) or m.group(2))] +
                             [int(b or a) for a, b in re.findall(r"(\d+)(?:\s*[-–]\s*(\d+))?", m.group(4) or "")])
                    checked += 1
                    if not any(n_lines(c) >= hi for c in cands):
                        bad.append(f"{os.path.relpath(src, ROOT)}:{ln}: {m.group(0)}")
    assert checked > 100, f"only {checked} citations found: the scan is broken"
    assert not bad, "citations past the end of the reference file:\n" + "\n".join(bad)
