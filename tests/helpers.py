"""Shared helpers of the GPU parity tests (CUDA library vs CPU oracle)."""
import os

import numpy as np

from exanbody_gb300 import units, workloads, xnb
from oracle.oracle import OracleSystem

FIELDS = ("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz")


def oracle_threads():
    return max(1, os.cpu_count() or 1)


def new_batch(systems_atoms, systems_cells, list_per_atom=170.0, max_systems=None):
    P = int(sum(systems_atoms)) + 64
    Cc = int(sum(systems_cells)) + 64
    L = int(list_per_atom * P) + 4096
    return xnb.Batch(P, Cc, L, max_systems=max_systems or max(1, len(systems_atoms)))


def ncells(geom):
    d = geom["dims"]
    return int(d[0]) * int(d[1]) * int(d[2])


def oracle_from(w, kind="omp"):
    g = w["geom"]
    s = OracleSystem(g["origin"], g["extent"], g["dims"], g["cell_size"], 2.5, 0.3, 1.0, 1.0, 0.005, kind=kind)
    s.set_threads(oracle_threads())
    s.load_flat(w["r"], w["v"], w["id"])
    return s


def force_error(f_test, f_ref):
    """max and RMS of |dF_i| / max(|F_i|, F_rms) (relative error robust to near-zero forces)."""
    d = np.linalg.norm(f_test - f_ref, axis=1)
    mag = np.linalg.norm(f_ref, axis=1)
    frms = float(np.sqrt((mag ** 2).mean()))
    rel = d / np.maximum(mag, frms)
    return float(rel.max()), float(np.sqrt((rel ** 2).mean()))


def forces(P):
    return np.stack([P["fx"], P["fy"], P["fz"]], axis=1)


def assert_bitwise_equal(G, O, fields=FIELDS):
    assert np.array_equal(G["id"], O["id"]), "particle order differs"
    for k in fields:
        a, b = G[k], O[k]
        if not np.array_equal(a.view(np.uint64), b.view(np.uint64)):
            bad = np.nonzero(a.view(np.uint64) != b.view(np.uint64))[0]
            raise AssertionError("%s differs at %d entries, first %d: %r vs %r" % (k, len(bad), bad[0], a[bad[0]], b[bad[0]]))


def ni_deck_oracle():
    s = OracleSystem((0, 0, 0), (55.68, 55.68, 55.68), (4, 4, 4), 13.92, 4.1, 2.0, units.ev_to_internal(0.3729),
                     2.2808, 2e-3, mass=58.693, divide_by_mass=True, amr=True, kind="omp")
    s.set_threads(oracle_threads())
    s.load_lattice_noise_fcc(3.48, 0.05)
    return s


def ni_deck_params():
    geom = {"origin": (0.0, 0.0, 0.0), "extent": (55.68, 55.68, 55.68), "dims": (4, 4, 4), "cell_size": 13.92}
    return xnb.lj_params(geom, epsilon=units.ev_to_internal(0.3729), sigma=2.2808, rcut=4.1, rcut_inc=2.0, dt=2e-3,
                         mass=58.693, divide_by_mass=True, amr=True)


def translated(w, origin):
    """The same workload with its domain and every position moved by `origin`
    (domain [origin, origin + extent))."""
    o = np.asarray(origin, np.float64)
    g = dict(w["geom"])
    g["origin"] = tuple(float(x) for x in o)
    g["extent"] = tuple(float(o[a] + w["geom"]["extent"][a]) for a in range(3))
    out = dict(w)
    out["geom"] = g
    out["r"] = w["r"] + o
    return out


def compare_pairs_sliced(b, s, o, G=None, slice_particles=400_000):
    """Pair lists of the library (system s of batch b) and of the oracle o, as
    particle ids in list order, compared slice by slice over interior cells so
    that host memory stays bounded at any system size. The particle order must
    already be equal (G: a download of the system; its ids are checked here).
    Returns the number of entries compared."""
    counts = o.cell_counts()
    if G is not None:
        O_ids = o.particles()["id"]
        assert np.array_equal(G["id"], O_ids), "particle order differs"
    first = np.concatenate([[0], np.cumsum(counts)])
    nc = len(counts)
    total = 0
    c0 = 0
    while c0 < nc:
        # the largest cell range starting at c0 holding at most slice_particles (at least one cell)
        c1 = int(np.searchsorted(first, first[c0] + slice_particles, side="right")) - 1
        c1 = max(c0 + 1, min(nc, c1))
        p0, p1 = int(first[c0]), int(first[c1])
        ob, ocnt = o.pairs_of_cells(c0, c1, p1 - p0)
        try:
            gb, gcnt = b.pairs_range(s, p0, p1 - p0, len(ob) + 1)
        except xnb.XnbError as e:
            raise AssertionError("cells [%d, %d): the library lists more entries than the oracle (%s)" % (c0, c1, e))
        if not np.array_equal(gcnt, ocnt):
            bad = np.nonzero(gcnt != ocnt)[0]
            raise AssertionError("cells [%d, %d): %d per-particle counts differ, first particle %d: %d vs %d"
                                 % (c0, c1, len(bad), p0 + bad[0], gcnt[bad[0]], ocnt[bad[0]]))
        if not np.array_equal(gb, ob):
            bad = np.nonzero(gb != ob)[0]
            raise AssertionError("cells [%d, %d): %d list entries differ, first at %d" % (c0, c1, len(bad), bad[0]))
        total += len(ob)
        c0 = c1
    return total
