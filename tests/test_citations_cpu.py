"""Every ``file:line`` citation of the reference in this repository exists.

The index (tests/golden/reference_index.json, made by
tests/golden/make_reference_index.py from the reference sources) holds each
reference file's line count and the line span of each Fortran subroutine and
function.  A citation fails when a cited line lies past the end of its file,
when a range runs backwards, or when the citation directly follows the name
of a routine of that file (``compute_wall_model (wallmodel.f90:23-46)``) and
the cited lines lie outside that routine.
"""
import json
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
INDEX = os.path.join(HERE, "golden", "reference_index.json")

# product sources and their documents (the review and survey files are not
# this repository's own text)
SCAN_EXT = (".py", ".cu", ".cuh", ".h", ".c", ".cpp", ".f90", ".md")
SKIP_FILES = {"VERDICT.md", "ADVICE.md", "SURVEY.md", "test_citations_cpu.py"}   # (this file plants mistakes)
SKIP_DIRS = {".git", "_work", "gpurun_out", "_build", "baseline", "__pycache__", ".pytest_cache"}

CITE = re.compile(r"(?<![\w/.])((?:[\w./]*/)?([A-Za-z_][\w]*\.(?:f90|cpp|m|sh)|input_parameters_\d+|Makefile|README))"
                  r":(\d+(?:-\d+)?(?:,\s?\d+(?:-\d+)?)*)")
WORD = re.compile(r"([A-Za-z_]\w*)[\s`'\"(]*$")


def _index():
    with open(INDEX) as f:
        idx = json.load(f)
    by_name = {}
    for path, ent in idx.items():
        by_name.setdefault(os.path.basename(path), []).append(ent)
    return by_name


def _sources():
    for dp, dns, fns in os.walk(ROOT):
        dns[:] = [d for d in dns if d not in SKIP_DIRS]
        for fn in fns:
            if fn.endswith(SCAN_EXT) and fn not in SKIP_FILES and not fn.startswith(("BENCH_", "GPUTEST_")):
                yield os.path.join(dp, fn)


def _ranges(spec):
    for part in spec.replace(" ", "").split(","):
        a, _, b = part.partition("-")
        yield int(a), int(b) if b else int(a)


def check_text(text, label, by_name):
    """(list of bad citations, number of reference citations) in one text."""
    bad, seen = [], 0
    for m in CITE.finditer(text):
        ents = by_name.get(m.group(2))
        if not ents:
            continue                          # not a reference file (e.g. this repo's own sources)
        ent = max(ents, key=lambda e: e["lines"])
        seen += 1
        line = text.count("\n", 0, m.start()) + 1
        where = f"{label}:{line}: {m.group(0)}"
        spans = list(_ranges(m.group(3)))
        for a, b in spans:
            if b < a or b > ent["lines"] or a < 1:
                bad.append(f"{where} (file has {ent['lines']} lines)")
        w = WORD.search(text[max(0, m.start() - 80):m.start()])
        if w and w.group(1).lower() in ent["routines"]:
            lo, hi = ent["routines"][w.group(1).lower()]
            if not any(a <= hi and b >= lo for a, b in spans):
                bad.append(f"{where} (outside {w.group(1)}, lines {lo}-{hi})")
    return bad, seen


def find_bad_citations():
    by_name = _index()
    bad, seen = [], 0
    for path in _sources():
        with open(path, errors="replace") as f:
            b, s = check_text(f.read(), os.path.relpath(path, ROOT), by_name)
        bad += b
        seen += s
    return bad, seen


def test_checker_catches_planted_mistakes():
    by_name = _index()
    ok = "compute_wall_model (wallmodel.f90:23-46); the shift (time_integration.f90:89-94)"
    assert check_text(ok, "t", by_name) == ([], 2)
    past_end, _ = check_text("the shift (mass_flow.f90:360-413)", "t", by_name)
    wrong_routine, _ = check_text("compute_dPx_for_constant_mass_flow (mass_flow.f90:24-61)", "t", by_name)
    backwards, _ = check_text("`subgrid.f90:537-379`", "t", by_name)
    assert len(past_end) == 1 and len(wrong_routine) == 1 and len(backwards) == 1


def test_reference_citations_exist():
    bad, seen = find_bad_citations()
    assert seen > 100, seen                   # the scan found the citations at all
    assert not bad, "\n".join(bad)
