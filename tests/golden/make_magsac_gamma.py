"""Extracts a subset of the reference's MAGSAC++ weight table as a golden fixture.

Reads stored_gamma_values from the reference checkout
(src/pygcransac/include/gamma_values.cpp:2012) as text and writes every 100th
entry to magsac_gamma_subset.json next to this script. Run from the repository
root with the reference checkout's path:
python tests/golden/make_magsac_gamma.py <path to the graph-cut-ransac checkout>
"""
import json
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: make_magsac_gamma.py <path to the graph-cut-ransac checkout>")
ref = sys.argv[1]
path = os.path.join(ref, "src/pygcransac/include/gamma_values.cpp")
text = open(path).read()
start = text.index("stored_gamma_values[]")
body = text[text.index("{", start) + 1:text.index("}", start)]
vals = [float(v) for v in re.split(r"[,\s]+", body.strip()) if v]
subset = {str(i): vals[i] for i in range(0, len(vals), 100)}
subset[str(len(vals) - 1)] = vals[-1]
out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "magsac_gamma_subset.json")
json.dump({"source": "src/pygcransac/include/gamma_values.cpp:2012 stored_gamma_values",
           "length": len(vals), "entries": subset}, open(out, "w"), indent=0)
print(out, len(vals))
