"""Confirm that every known-answer value in reference_kats.json is literally
present in the reference test lines it cites.

Run where a casa-rs checkout is available, giving its root as the argument
or in the CASA_RS_ROOT environment variable:
    python tests/golden/check_reference_citations.py <casa-rs root>
It prints one line per KAT and exits non-zero if a literal is missing.  The
unit tests only load the JSON and need no checkout.
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(root: str) -> int:
    with open(os.path.join(HERE, "reference_kats.json")) as fh:
        kats = json.load(fh)["kats"]
    bad = 0
    for kat in kats:
        path, lines = kat["cite"].rsplit(":", 1)
        first, last = (int(x) for x in lines.split("-"))
        with open(os.path.join(root, path)) as fh:
            text = "".join(fh.readlines()[first - 1:last])
        missing = [lit for lit in kat.get("literals", []) if lit not in text]
        status = "ok" if not missing else f"MISSING {missing}"
        bad += bool(missing)
        print(f"{kat['name']:40s} {kat['cite']:55s} {status}")
    return 1 if bad else 0


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CASA_RS_ROOT")
    if not root:
        sys.exit("usage: check_reference_citations.py <casa-rs root> (or set CASA_RS_ROOT)")
    sys.exit(main(root))
