"""Every reference citation `file:line` or `file:first-last` in the C ABI
header, the oracle and the package names lines that exist in the reference
sources. Skipped where the reference sources are absent."""
from __future__ import annotations

import os
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
REF = Path(os.environ.get("TEALEAF_REF",
                         Path(__file__).resolve().parents[2] / "reference" / "TeaLeaf"))
CITATION = re.compile(
    r"((?:[\w.-]+/)*[\w.-]+\.(?:c|h|cpp|hpp|in|problems|out|cl)):(\d+)(?:-(\d+))?")
SCANNED = [ROOT / "include", ROOT / "oracle", ROOT / "exploringsycl_gb300", ROOT / "bench.py",
           ROOT / "__graft_entry__.py"]
SOURCE_SUFFIXES = {".c", ".h", ".cpp", ".cu", ".cuh", ".py", ".hpp"}


def _reference_files() -> dict[str, list[Path]]:
    out: dict[str, list[Path]] = {}
    for p in REF.parent.rglob("*"):
        if p.is_file() and p.suffix in {".c", ".h", ".cpp", ".hpp", ".in", ".problems", ".out",
                                         ".cl"} | {""} and "_ref" not in p.parts:
            out.setdefault(p.name, []).append(p)
    return out


def _sources():
    for s in SCANNED:
        if s.is_file():
            yield s
        elif s.is_dir():
            for q in sorted(s.rglob("*")):
                if q.is_file() and q.suffix in SOURCE_SUFFIXES and "_build" not in q.parts:
                    yield q


@pytest.mark.skipif(not REF.is_dir(), reason="reference sources not present")
def test_every_reference_citation_names_existing_lines():
    files = _reference_files()
    checked, bad = 0, []
    for src in _sources():
        for ln, line in enumerate(src.read_text(errors="replace").splitlines(), 1):
            for m in CITATION.finditer(line):
                path, first = m.group(1), int(m.group(2))
                last = int(m.group(3)) if m.group(3) else first
                cands = files.get(os.path.basename(path), [])
                exact = [c for c in cands if str(c).endswith(path)]
                cands = exact or cands
                where = f"{src.relative_to(ROOT)}:{ln}: {m.group(0)}"
                if not cands:
                    bad.append(f"{where} (no such reference file)")
                    continue
                n = max(len(c.read_text(errors="replace").splitlines()) for c in cands)
                if not 1 <= first <= last <= n:
                    bad.append(f"{where} (the file has {n} lines)")
                checked += 1
    assert checked > 100, f"only {checked} citations found"
    assert not bad, "\n".join(bad)
