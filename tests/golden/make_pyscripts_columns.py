"""Writes pyscripts_columns.json: the column names the reference's plotting
scripts select from swm_tests' text outputs.

The reference's readers (pyscripts/imodel_data.py, imodel_data_evol.py) load
a file with pandas.read_csv(delim_whitespace=True) and pick the columns
named in their option files (pyscripts/options_*.csv: the InLoop, MidLoop,
OutLoop, xVar and yVar rows).  Run from the repository root with the
reference checked out at the path given (default /root/reference); the JSON
is committed so that the tests do not need the reference.
"""
import csv
import json
import os
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "pyscripts_columns.json")
KEYS = ("InLoop", "MidLoop", "OutLoop", "xVar", "yVar")


def columns(path):
    cols = []
    with open(path) as f:
        rows = csv.reader(f)
        next(rows)  # comment line
        for row in rows:
            if row and row[0] in KEYS:
                cols.extend(c for c in row[1:] if c)
    return cols


out = {}
for name in ("options_swm_conv.csv", "options_template.csv", "options_template_evol.csv"):
    out[name] = columns(os.path.join(REF, "pyscripts", name))
with open(OUT, "w") as f:
    json.dump(out, f, indent=1)
print(json.dumps(out))
