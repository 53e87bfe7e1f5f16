"""The SNAP restatement of the oracle (oracle/xnb_snap_oracle.h) pinned against
the reference's own golden data (contribs/microStamp/samples/benchmark_lj_snap:
check_values_snap_{Ni,Mo}.dat after 100 NVE steps of input_snap_{Ni,Mo}.msp), and
its adjoint forces checked against finite differences of its energy."""
import os

import numpy as np
import pytest

from exanbody_gb300 import snap, workloads
from oracle.oracle import OracleSystem

G = os.path.join(os.path.dirname(__file__), "golden", "snap")
DECKS = {
    # box, cell, rcut_max, mass, structure, lattice constant, noise sigma (input_snap_*.msp)
    "Ni": (55.68, 13.92, 4.1, 58.693, "FCC", 3.48, 0.05),
    "Mo": (50.4, 12.6, 4.6, 95.96, "BCC", 3.15, 0.1),
}


def potential(el):
    return snap.read_lammps(os.path.join(G, "%s_Zuo_JPCA2020.snapparam" % el),
                            os.path.join(G, "%s_Zuo_JPCA2020.snapcoeff" % el))


def golden(el):
    ref = {}
    with open(os.path.join(G, "check_values_snap_%s.dat" % el)) as f:
        for line in f:
            if line.startswith("- ["):
                t = [x.strip() for x in line.strip()[3:-1].split(",")]
                ref[int(t[0])] = np.array([float.fromhex(h) for h in t[1:]])
    return ref


def golden_errors(P, ref, L):
    idx = {int(i): k for k, i in enumerate(P["id"])}
    er = ea = ev = 0.0
    for pid, v in ref.items():
        k = idx[pid]
        d = np.array([P["rx"][k], P["ry"][k], P["rz"][k]]) - v[0:3]
        d -= L * np.round(d / L)
        er += float((d ** 2).sum())
        ea += float(((np.array([P["fx"][k], P["fy"][k], P["fz"][k]]) - v[3:6]) ** 2).sum())
        ev += float(((np.array([P["vx"][k], P["vy"][k], P["vz"][k]]) - v[6:9]) ** 2).sum())
    return er ** 0.5, ea ** 0.5, ev ** 0.5


def test_parameter_files_and_coefficient_order():
    ni, mo = potential("Ni"), potential("Mo")
    assert ni["twojmax"] == 8 and ni["rcutfac"] == 4.1 and ni["bzeroflag"] == 0 and ni["switchflag"] == 1
    assert ni["ncoeffall"] == 56 and len(ni["elements"]) == 1 and ni["elements"][0]["radelem"] == 0.5
    assert mo["twojmax"] == 6 and mo["ncoeffall"] == 31
    # coefficient count = number of (j1 >= j2, j >= j1) triples + 1 (sna.cpp:236-259)
    for cfg in (ni, mo):
        J = cfg["twojmax"]
        n = sum(1 for j1 in range(J + 1) for j2 in range(j1 + 1)
                for j in range(j1 - j2, min(J, j1 + j2) + 1, 2) if j >= j1)
        assert n + 1 == cfg["ncoeffall"]


@pytest.mark.parametrize("el", ["Ni", "Mo"])
def test_adjoint_forces_match_energy_derivative(el):
    """dE/dx by central differences of the full-matrix energy equals the adjoint
    force (the beta multiplicities, the unique-half weights and dU/dr)."""
    cfg = potential(el)
    a = 3.52 if el == "Ni" else 3.15
    structure = "FCC" if el == "Ni" else "BCC"
    n = 4
    L = n * a
    basis = {"FCC": workloads.FCC_BASIS, "BCC": np.array([[0, 0, 0], [0.5, 0.5, 0.5]])}[structure]
    cells = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"), -1).reshape(-1, 3)
    r = ((cells[:, None, :] + basis[None]).reshape(-1, 3) * a)
    r = (r + np.random.default_rng(3).normal(0, 0.1, r.shape)) % L
    ids = np.arange(1, len(r) + 1, dtype=np.uint64)

    def evaluate(rr):
        o = OracleSystem((0, 0, 0), (L, L, L), (2, 2, 2), L / 2, cfg["rcutfac"], 0.3, 1.0, 1.0, 0.001, kind="omp")
        o.set_snap(cfg, snap.energy_unit(), with_energy=True)
        o.load_flat(rr, np.zeros_like(rr), ids)
        o.init()
        return o.particles()

    p0 = evaluate(r)
    order = np.argsort(p0["id"])
    F = np.stack([p0["fx"], p0["fy"], p0["fz"]], 1)[order]
    h = 1e-5
    for atom in (0, 37):
        for k in range(3):
            rp, rm = r.copy(), r.copy()
            rp[atom, k] += h
            rm[atom, k] -= h
            fd = -(evaluate(rp)["pe"].sum() - evaluate(rm)["pe"].sum()) / (2 * h)
            assert abs(fd - F[atom, k]) <= 2e-8 * np.abs(F).max(), (atom, k, fd, F[atom, k])


@pytest.mark.parametrize("el", ["Mo", "Ni"])
def test_golden_check_values(el):
    """check_values (debug/check_values.cpp:243-401) after 100 steps: L2 errors of
    the 100 sampled atoms far below the deck's 1e-5 thresholds."""
    L, cs, rc, mass, structure, a, sigma = DECKS[el]
    s = OracleSystem((0, 0, 0), (L, L, L), (4, 4, 4), cs, rc, 2.0, 1.0, 1.0, 2e-3, mass=mass,
                     divide_by_mass=True, kind="omp")
    s.set_snap(potential(el), snap.energy_unit())
    s.load_lattice_noise(structure, a, sigma)
    s.init()
    assert s.n == (16384 if el == "Ni" else 8192)
    for _ in range(100):
        s.step()
    er, ea, ev = golden_errors(s.particles(), golden(el), L)
    assert er < 1e-9 and ea < 1e-6 and ev < 1e-8, (er, ea, ev)
