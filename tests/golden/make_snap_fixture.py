"""Copy the reference's SNAP golden data into tests/golden/snap/.

Sources in the exaNBody tree (benchmark_lj_snap: 100 NVE steps of FCC Ni / BCC Mo
with snap_force_generic, 100 sampled atoms [id, rx, ry, rz, ax, ay, az, vx, vy, vz]
in hex floats):
    contribs/microStamp/samples/benchmark_lj_snap/check_values_snap_{Ni,Mo}.dat
    contribs/microStamp/samples/benchmark_lj_snap/input_snap_{Ni,Mo}.msp (the decks)
and the LAMMPS potential files those decks read:
    contribs/microStamp/potentials/{Ni,Mo}_Zuo_JPCA2020.snap{param,coeff}
Run once where the reference tree is mounted:
    python tests/golden/make_snap_fixture.py /path/to/exaNBody
"""
import os
import shutil
import sys

if len(sys.argv) != 2:
    sys.exit("usage: python %s <root of the exaNBody source tree>" % sys.argv[0])
src_root = sys.argv[1]
dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "snap")
os.makedirs(dst, exist_ok=True)
bench = os.path.join(src_root, "contribs/microStamp/samples/benchmark_lj_snap")
pots = os.path.join(src_root, "contribs/microStamp/potentials")
for el in ("Ni", "Mo"):
    with open(os.path.join(bench, "check_values_snap_%s.dat" % el)) as f:
        rows = [l for l in f if l.startswith("- [")]
    with open(os.path.join(dst, "check_values_snap_%s.dat" % el), "w") as f:
        f.write("length_unit: 1.0 ang\nvalues:\n")
        f.writelines(rows)
    for ext in ("snapparam", "snapcoeff"):
        name = "%s_Zuo_JPCA2020.%s" % (el, ext)
        shutil.copyfile(os.path.join(pots, name), os.path.join(dst, name))
    print(el, len(rows), "rows")
