"""Ragged batches: systems of 0, 1 and 2 atoms beside a 32,000-atom cube.

The reference runs a domain whose grid holds no particle, or a lone particle,
like any other (cell loops over empty cells, lists of length zero). Here:
- an empty system keeps zero particles, zero list entries and zero energy;
- a single atom moves ballistically across cells and through the periodic
  boundary (rebuilds of its own, no neighbours);
- two atoms interact only through the periodic z boundary;
and the cube beside them keeps its own result. FP64_EXACT is compared with
the oracle bit for bit (positions, velocities, forces, per-particle energy,
rebuild steps); MIXED through the CUDA-graph path equals each system run alone.
"""
import numpy as np
import pytest

from exanbody_gb300 import workloads, xnb
from helpers import assert_bitwise_equal, ncells, new_batch, oracle_from

pytestmark = pytest.mark.gpu

ALL = ("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz", "pe")


def tiny_system(geom, n):
    """n = 0, 1 or 2 atoms in the cube's box; the pair sits across the z boundary."""
    o, L = geom["origin"], geom["extent"]
    r = np.array([[o[0] + 1.3, o[1] + 2.1, o[2] + L[2] - 0.05],
                  [o[0] + 2.5, o[1] + 2.1, o[2] + 0.4]])[:n].reshape(n, 3)
    v = np.array([[0.7, -0.4, 1.9], [-0.3, 0.2, -1.1]])[:n].reshape(n, 3)
    ids = np.arange(n, dtype=np.uint64) + 7
    return {"r": r, "v": v, "id": ids, "geom": geom, "n_atoms": n}


def ragged_workloads():
    cube = workloads.lj_fcc_system(20, 0.8442, 1.44, 12345)
    return [tiny_system(cube["geom"], 0), tiny_system(cube["geom"], 1), tiny_system(cube["geom"], 2), cube]


def add_all(b, ws):
    return [b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"]) for w in ws]


def test_empty_and_few_atom_systems_exact_against_oracle():
    ws = ragged_workloads()
    b = new_batch([w["n_atoms"] for w in ws], [ncells(w["geom"]) for w in ws], max_systems=len(ws) + 1)
    ss = add_all(b, ws)
    b.init_particles(-1, xnb.PREC_FP64_EXACT)
    os_ = [oracle_from(w) for w in ws]
    for o in os_:
        o.init()
    rebuilds = [0] * len(ws)
    for step in range(60):
        r0 = [b.info(s).rebuilds for s in ss]
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC | xnb.STEP_ENERGY)
        for k, (s, o) in enumerate(zip(ss, os_)):
            rebuilt = o.step()
            assert b.info(s).rebuilds - r0[k] == rebuilt, "rebuild decision differs (system %d, step %d)" % (k, step)
            rebuilds[k] += rebuilt
    assert rebuilds[0] == 0 and rebuilds[1] >= 2 and rebuilds[3] >= 1, rebuilds
    for s, o in zip(ss, os_):
        assert_bitwise_equal(b.download(s), o.particles(), fields=ALL)
        assert tuple(b.energy(s)) == tuple(o.energy())
    empty = b.info(ss[0])
    assert empty.n_particles == 0 and empty.list_used == 0 and empty.error_bits == 0
    assert b.energy(ss[0]) == (0.0, 0.0)
    lone = b.download(ss[1])
    assert lone["fx"][0] == 0.0 and lone["pe"][0] == 0.0
    pair = b.download(ss[2])
    assert pair["pe"][0] < 0.0 and pair["fx"][0] != 0.0  # the pair sees each other only through z
    b.check_errors()

    # the empty slot taken back and reused by another two-atom system
    b.remove_system(ss[0])
    w2 = tiny_system(ws[3]["geom"], 2)
    s2 = b.add_system(xnb.lj_params(w2["geom"]), w2["r"], w2["v"], w2["id"])
    b.init_particles(s2, xnb.PREC_FP64_EXACT)
    o2 = oracle_from(w2)
    o2.init()
    for _ in range(10):
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC | xnb.STEP_ENERGY)
        o2.step()
    assert_bitwise_equal(b.download(s2), o2.particles(), fields=ALL)
    b.check_errors()
    b.close()


def test_ragged_batch_mixed_graph_equals_each_alone():
    ws = ragged_workloads()
    big = new_batch([w["n_atoms"] for w in ws], [ncells(w["geom"]) for w in ws], max_systems=len(ws))
    ss = add_all(big, ws)
    big.init_particles(-1, xnb.PREC_MIXED)
    big.step(80, xnb.PREC_MIXED, 0)
    big.check_errors()
    for w, s in zip(ws, ss):
        b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
        so = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
        b.init_particles(so, xnb.PREC_MIXED)
        b.step(80, xnb.PREC_MIXED, 0)
        assert_bitwise_equal(big.download(s), b.download(so))
        assert big.info(s).rebuilds == b.info(so).rebuilds
        b.close()
    big.close()
