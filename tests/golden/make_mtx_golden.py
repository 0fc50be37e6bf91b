"""Generate tests/golden/mtx2egr.json: .mtx inputs and the sha256 of the .egr
bytes that the reference's own converter (tools/efficient_converter.py,
imported from the reference tree) writes for each.  Run where the reference
tree is present; the tests read only the JSON.

Usage: python tests/golden/make_mtx_golden.py <reference_root>  (or set MISFIT_REF_ROOT)
"""
import hashlib
import importlib.util
import io
import json
import os
import sys
import tempfile
from contextlib import redirect_stdout

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def cases():
    rng = np.random.default_rng(2024)
    out = {}
    # an ER-like edge list in random order, both directions, with repeats,
    # comments, a weight column and the edge count on the size line
    n = 60
    a = rng.integers(1, n + 1, 300)
    b = rng.integers(1, n + 1, 300)
    keep = a != b
    a, b = a[keep], b[keep]
    lines = ["%%MatrixMarket matrix coordinate pattern general", "% a comment", "%d %d %d" % (n, n, 2 * a.size)]
    for x, y in zip(a, b):
        lines.append("%d %d" % (x, y))
        lines.append("%d\t%d 1.0" % (y, x))
    out["er60_both_directions"] = "\n".join(lines) + "\n"
    # no edge count on the size line, a non-square size line, blank and
    # one-field lines, entries whose source is beyond the vertex count
    lines = ["% size line without an edge count", "40 55"]
    for _ in range(120):
        x, y = int(rng.integers(1, 60)), int(rng.integers(1, 56))
        lines.append("%d %d" % (x, y))
        if rng.random() < 0.05:
            lines.append("")
        if rng.random() < 0.05:
            lines.append("7")
    out["nonsquare_no_count"] = "\n".join(lines) + "\n"
    # CRLF line ends, extra spaces, vertices with no entries, no final newline
    lines = ["%comment", "  10   10  6 ", "1 2", "2 1", " 3  9", "9 3", "10 1", "1 10"]
    out["crlf_spacing"] = "\r\n".join(lines)
    return out


def main(root):
    spec = importlib.util.spec_from_file_location("efficient_converter",
                                                  os.path.join(root, "tools", "efficient_converter.py"))
    conv = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(conv)
    golden = {}
    with tempfile.TemporaryDirectory() as d:
        for name, text in cases().items():
            src, dst = os.path.join(d, name + ".mtx"), os.path.join(d, name + ".egr")
            with open(src, "w", newline="") as f:
                f.write(text)
            with redirect_stdout(io.StringIO()):
                conv.convert_mtx_to_egr(src, dst)
            data = open(dst, "rb").read()
            golden[name] = {"mtx": text, "sha256": hashlib.sha256(data).hexdigest(), "size": len(data)}
    with open(os.path.join(HERE, "mtx2egr.json"), "w") as f:
        json.dump(golden, f, indent=1, sort_keys=True)
    print("wrote", len(golden), "cases")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MISFIT_REF_ROOT")
    if not root:
        raise SystemExit("usage: make_mtx_golden.py <reference_root>  (or set MISFIT_REF_ROOT)")
    main(root)
