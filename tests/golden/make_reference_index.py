"""Regenerate tests/golden/reference_index.json from the reference sources.

For every file of the reference's ``code/`` and ``scripts/`` trees the index
holds its line count and, for the Fortran files, the first and last line of
each subroutine and function (``Subroutine name`` .. ``End Subroutine name``).
tests/test_citations_cpu.py checks every ``file:line`` citation of this
repository against it, so the check runs wherever the tests run, without the
reference sources.

    python tests/golden/make_reference_index.py [reference root]
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "reference_index.json")
START = re.compile(r"^\s*(?:(?:pure|elemental|recursive|module)\s+)*(subroutine|function)\s+([A-Za-z_]\w*)", re.I)
END = re.compile(r"^\s*end\s*(subroutine|function)\s+([A-Za-z_]\w*)", re.I)


def index_file(path):
    with open(path, errors="replace") as f:
        lines = f.read().split("\n")
    if lines and lines[-1] == "":
        lines.pop()
    spans, open_ = {}, {}
    if path.endswith(".f90"):
        for n, ln in enumerate(lines, 1):
            if ln.lstrip().startswith("!"):
                continue
            m = END.match(ln)
            if m:
                name = m.group(2).lower()
                if name in open_:
                    spans[name] = [open_.pop(name), n]
                continue
            m = START.match(ln)
            if m:
                open_[m.group(2).lower()] = n
    return {"lines": len(lines), "routines": spans}


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    idx = {}
    for sub in ("code", "scripts"):
        for dp, _, fs in os.walk(os.path.join(root, sub)):
            for fn in sorted(fs):
                if fn.endswith((".f90", ".cpp", ".m", ".sh")) or fn == "Makefile" or fn.startswith("input_parameters"):
                    rel = os.path.relpath(os.path.join(dp, fn), root)
                    idx[rel] = index_file(os.path.join(dp, fn))
    for fn in ("README",):
        p = os.path.join(root, fn)
        if os.path.exists(p):
            idx[fn] = index_file(p)
    with open(OUT, "w") as f:
        json.dump(idx, f, indent=1, sort_keys=True)
    print(f"{len(idx)} files -> {OUT}")


if __name__ == "__main__":
    main()
