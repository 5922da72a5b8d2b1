"""Every reference citation (``file.py:a-b``, ``file.cl:a``, with ``, c-d``
continuations) in the C header, the integration notes and the sources must
point inside the cited reference file, and where a citation follows the name
it documents (``depose_scalar (grid_methods_cl.py:44-69``), that name must
occur in the cited lines.

Needs the reference tree (the directory ``reference`` beside the repository,
or ``CHIMERACL_REFERENCE``); skipped where it is absent.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("CHIMERACL_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")

CITE = re.compile(r"(?:(\w+)\s+\(\s*)?((?:[\w./]+/)?(\w+\.(?:py|cl))):(\d+)(?:-(\d+))?"
                  r"((?:,\s*:?\d+(?:-\d+)?)*)")
MORE = re.compile(r":?(\d+)(?:-(\d+))?")
SCANNED_EXT = (".py", ".h", ".cu", ".cuh", ".c", ".cpp", ".hpp", ".md")
# repository files whose names could collide with a reference file
OWN_PREFIXES = ("tests/", "chimeracl_gb300/", "methods/particles_methods_cu", "oracle/",
                "csrc/", "bench")


def _ref_files():
    out = {}
    for dp, _, fs in os.walk(REF):
        for f in fs:
            if f.endswith((".py", ".cl")) and f != "__init__.py":
                out.setdefault(f, []).append(os.path.join(dp, f))
    return out


def _scanned():
    files = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    files += [os.path.join(ROOT, f) for f in ("INTEGRATION.md", "DESIGN.md", "README.md", "bench.py",
                                                "__graft_entry__.py")]
    for top in ("chimeracl_gb300", "oracle", "tests"):
        for dp, _, fs in os.walk(os.path.join(ROOT, top)):
            if "_build" in dp or "__pycache__" in dp or "_ref" in dp:
                continue
            files += [os.path.join(dp, f) for f in fs if f.endswith(SCANNED_EXT)]
    return [f for f in files if os.path.isfile(f) and not f.endswith("test_citations.py")]


def _citations():
    refs = _ref_files()
    for path in _scanned():
        text = open(path, encoding="utf-8", errors="replace").read()
        for mt in CITE.finditer(text):
            name, cited, base, a, b, more = mt.groups()
            if cited.startswith(OWN_PREFIXES) or base not in refs:
                continue
            cands = [p for p in refs[base] if p.replace(os.sep, "/").endswith(cited)]
            if len(cands) != 1:
                continue
            ranges = [(int(a), int(b or a))]
            ranges += [(int(x), int(y or x)) for x, y in MORE.findall(more or "")]
            line = text.count("\n", 0, mt.start()) + 1
            yield os.path.relpath(path, ROOT), line, name, cands[0], ranges


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "chimeraCL")),
                    reason="reference tree not present")
def test_reference_citations_point_inside_their_files():
    bad, checked, named = [], 0, 0
    for where, line, name, ref, ranges in _citations():
        lines = open(ref, encoding="utf-8", errors="replace").read().splitlines()
        for a, b in ranges:
            checked += 1
            if not 1 <= a <= b <= len(lines):
                bad.append(f"{where}:{line}: {os.path.basename(ref)}:{a}-{b} outside 1..{len(lines)}")
        whole = "\n".join(lines)
        # the name check applies where the name is a function or kernel that
        # the cited file defines
        if name and re.search(r"(def|void)\s+%s\s*\(" % re.escape(name), whole):
            named += 1
            body = "\n".join("\n".join(lines[a - 1:b]) for a, b in ranges)
            if not re.search(r"\b%s\b" % re.escape(name), body):
                bad.append(f"{where}:{line}: '{name}' not in {os.path.basename(ref)}:{ranges}")
    assert checked > 100 and named > 10, (checked, named)
    assert not bad, "\n".join(bad)
