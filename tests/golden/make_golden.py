"""Regenerates the fixtures in this folder from the reference tree.

dlaruv_mm.json : the 128 x 4 multiplier table MM of SRC/dlaruv.f (the
                 DATA statements), against which the oracle's generator
                 (powers of the base multiplier) is checked.
test_inputs.json : the dimension / block-size / right-hand-side lists of the
                 reference test inputs TESTING/dtest.in (GE lines) and
                 TESTING/dstest.in, which the parity tests sweep.

Usage: python tests/golden/make_golden.py [reference_root]
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def dlaruv_table(ref):
    src = open(os.path.join(ref, "SRC", "dlaruv.f")).read()
    rows = {}
    pat = re.compile(r"DATA\s+\(\s*MM\(\s*(\d+),\s*J\s*\),\s*J\s*=\s*1,\s*4\s*\)\s*/\s*([\d\s,$]+?)/")
    for m in pat.finditer(src):
        rows[int(m.group(1))] = [int(v) for v in re.findall(r"\d+", m.group(2))]
    assert sorted(rows) == list(range(1, 129)), "unexpected DLARUV table"
    return [rows[i] for i in range(1, 129)]


def _ints(line):
    return [int(v) for v in line.split()[:50] if re.fullmatch(r"-?\d+", v)]


def test_inputs(ref):
    d = open(os.path.join(ref, "TESTING", "dtest.in")).read().splitlines()
    # dtest.in: line 1 title; 2 NM; 3 M values; 4 NN; 5 N values; 6 NNS; 7 NRHS values; 8 NNB; 9 NB values;
    # 10 NX values; 11 NRANK; 12 ranks; 13 THRESH
    out = {
        "dtest": {"m": _ints(d[2]), "n": _ints(d[4]), "nrhs": _ints(d[6]), "nb": _ints(d[8]),
                  "thresh": float(d[12].split()[0])},
    }
    s = open(os.path.join(ref, "TESTING", "dstest.in")).read().splitlines()
    # dstest.in: line 1 title; 2 NM; 3 M values; 4 NNS; 5 NRHS values; 6 THRESH
    out["dstest"] = {"n": _ints(s[2]), "nrhs": _ints(s[4]), "thresh": float(s[5].split()[0])}
    return out


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LAPACK_REFERENCE_DIR", "")
    if not ref:
        sys.exit("usage: make_golden.py <reference tree>  (or set LAPACK_REFERENCE_DIR)")
    with open(os.path.join(HERE, "dlaruv_mm.json"), "w") as f:
        json.dump({"source": "SRC/dlaruv.f DATA MM(128,4)", "mm": dlaruv_table(ref)}, f)
    with open(os.path.join(HERE, "test_inputs.json"), "w") as f:
        json.dump(test_inputs(ref), f, indent=1)


if __name__ == "__main__":
    main()
