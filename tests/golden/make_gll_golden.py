"""Generate tests/golden/gll_05.json from the reference's GLL table src/gll_xwh/gll_05.tab.

The table is the only data the reference ships for the hot path (GetGLL.jl:17-28 reads it:
row 1 = nodes x, row 2 = weights w, rows 3-7 = H with H[i,j] = h'_i(x_j)).  It pins the
oracle's and the product's GLL computation.  Run with the root of a checkout of the reference:
    python tests/golden/make_gll_golden.py <reference checkout>
"""
import json
import os
import sys

if len(sys.argv) != 2:
    sys.exit(__doc__)
path = os.path.join(sys.argv[1], "src", "gll_xwh", "gll_05.tab")
rows = []
with open(path) as f:
    for line in f:
        if line.strip():
            rows.append([float(t) for t in line.split()])
out = {"source": "src/gll_xwh/gll_05.tab", "x": rows[0], "w": rows[1], "H": rows[2:7]}
dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "gll_05.json")
with open(dst, "w") as f:
    json.dump(out, f, indent=1)
print(dst, file=sys.stderr)
