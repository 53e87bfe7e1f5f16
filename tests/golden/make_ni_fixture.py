"""Generate tests/golden/check_values_lj_Ni.json from the reference's golden deck data.

Source: contribs/microStamp/samples/benchmark_lj_snap/check_values_lj_Ni.dat of the
exaNBody tree (100 sampled atoms after 100 steps of input_lj_Ni.msp; each row is
[id, rx, ry, rz, ax, ay, az, vx, vy, vz] in hex floats, units angstrom / ps).
Run once where the reference tree is mounted:
    python tests/golden/make_ni_fixture.py /path/to/exaNBody
"""
import json
import os
import sys

if len(sys.argv) != 2:
    sys.exit("usage: python %s <root of the exaNBody source tree>" % sys.argv[0])
src_root = sys.argv[1]
src = os.path.join(src_root, "contribs/microStamp/samples/benchmark_lj_snap/check_values_lj_Ni.dat")
rows = []
with open(src) as f:
    for line in f:
        if line.startswith("- ["):
            toks = [t.strip() for t in line.strip()[3:-1].split(",")]
            rows.append({"id": int(toks[0]), "hex": toks[1:]})
out = {
    "source": "contribs/microStamp/samples/benchmark_lj_snap/check_values_lj_Ni.dat",
    "deck": "contribs/microStamp/samples/benchmark_lj_snap/input_lj_Ni.msp",
    "fields": ["rx", "ry", "rz", "ax", "ay", "az", "vx", "vy", "vz"],
    "thresholds": {"pos": 1e-5, "vel": 1e-5, "acc": 1e-5},
    "rows": rows,
}
dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "check_values_lj_Ni.json")
with open(dst, "w") as f:
    json.dump(out, f, indent=0)
print("wrote", dst, len(rows), "rows")
# the same rows in the check_values file layout (values: - [id, 9 hex floats]),
# read by the deck runner's check_values operator
dat = os.path.join(os.path.dirname(os.path.abspath(__file__)), "check_values_lj_Ni.dat")
with open(dat, "w") as f:
    f.write("length_unit: 1.0 ang\nvalues:\n")
    for r in rows:
        f.write("- [%d, %s]\n" % (r["id"], ", ".join(r["hex"])))
print("wrote", dat)
