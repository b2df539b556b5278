"""Every reference citation (``file.ml:N-M`` and the like) in the product, the
oracle and the tests names a file of the reference and lines inside it.

Runs only where the reference sources are present (skipped elsewhere).
"""
import collections
import os
import re

import pytest

REF = os.environ.get("PPLACER_REFERENCE", "/root/reference")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CITE = re.compile(r"\b([A-Za-z_0-9]+\.(?:ml|mli|mly|c|h)):(\d+(?:-\d+)?(?:,\d+(?:-\d+)?)*)")
SCANNED = ("oracle", "include", "pplacer_gb300", "tests")
TOP = ("bench.py", "__graft_entry__.py")
OWN = {"pplacer_gb300.h"}  # this project's own header, cited by name


def _sources():
    for d in SCANNED:
        for root, dirs, files in os.walk(os.path.join(ROOT, d)):
            dirs[:] = [x for x in dirs if not x.startswith(("_", "."))]
            for f in files:
                if f.endswith((".py", ".cu", ".cuh", ".cpp", ".c", ".h")):
                    yield os.path.join(root, f)
    for f in TOP:
        yield os.path.join(ROOT, f)


def _reference_lengths():
    lengths = collections.defaultdict(list)
    for root, _, files in os.walk(REF):
        for f in files:
            if f.endswith((".ml", ".mli", ".mly", ".c", ".h")):
                with open(os.path.join(root, f), errors="replace") as fh:
                    lengths[f].append(sum(1 for _ in fh))
    return lengths


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "pplacer_src")),
                    reason="reference sources absent")
def test_citations_point_inside_reference_files():
    lengths = _reference_lengths()
    bad = []
    n = 0
    for path in _sources():
        with open(path, errors="replace") as fh:
            for ln, line in enumerate(fh, 1):
                for m in CITE.finditer(line):
                    name, ranges = m.group(1), m.group(2)
                    if name in OWN:
                        continue
                    n += 1
                    where = f"{os.path.relpath(path, ROOT)}:{ln} {m.group(0)}"
                    if name not in lengths:
                        bad.append(f"{where}: no such reference file")
                        continue
                    last = max(int(x) for x in re.findall(r"\d+", ranges))
                    for part in ranges.split(","):
                        a, _, b = part.partition("-")
                        if b and int(b) < int(a):
                            bad.append(f"{where}: reversed range")
                    if all(last > L for L in lengths[name]):
                        bad.append(f"{where}: line {last} past the end ({lengths[name]})")
    assert n > 100, n
    assert not bad, "\n".join(bad)
