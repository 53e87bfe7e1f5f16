"""Parity at the benchmark size: the 4,000,000-atom FCC 100^3 system
(rho* = 0.8442, T* = 1.44, rc 2.5, skin 0.3, dt 0.005) against the CPU oracle.

FP64_EXACT through the C ABI with the host-synchronised schedule beside the
oracle's OpenMP build: the same rebuild steps; neighbour lists (ids in the
reference's stream order, compared slice by slice) equal at init and after every
rebuild; positions, velocities, forces and energies bitwise after 100 steps.
On that final state the FP64 traversal (full and Newton lists) stays within
1e-12 relative force error and 1e-12 relative potential energy of the oracle,
and the mixed path within 1e-5.

The same comparison over the full 1000 steps of the configuration is
tests/parity_lj4m.py (writes results/parity_lj4m_1000_steps.json).
"""
import numpy as np
import pytest

from exanbody_gb300 import workloads, xnb
from helpers import (assert_bitwise_equal, compare_pairs_sliced, force_error, forces, ncells, new_batch,
                     oracle_from)

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-5
STEPS = 100
ALL = ("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz", "pe")


def test_lj4m_fp64_exact_matches_oracle_over_100_steps():
    w = workloads.lj_fcc_system(100, 0.8442, 1.44, 12345)
    assert w["n_atoms"] == 4_000_000
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    G = b.download(s)
    assert_bitwise_equal(G, o.particles(), fields=ALL)
    entries = compare_pairs_sliced(b, s, o, G)
    assert 77 * w["n_atoms"] < entries < 79 * w["n_atoms"]

    rebuilds = 0
    for step in range(STEPS):
        r0 = b.info(s).rebuilds
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC | xnb.STEP_ENERGY)
        rebuilt = o.step()
        assert (b.info(s).rebuilds - r0) == rebuilt, "rebuild decision differs at step %d" % step
        if rebuilt:
            rebuilds += 1
            compare_pairs_sliced(b, s, o, b.download(s))
    assert rebuilds >= 5
    G, O = b.download(s), o.particles()
    assert_bitwise_equal(G, O, fields=ALL)
    ke_g, pe_g = b.energy(s)
    ke_o, pe_o = o.energy()
    assert ke_g == ke_o and pe_g == pe_o

    ref = forces(O)
    for prec, tol in ((xnb.PREC_FP64, FP64_TOL), (xnb.PREC_FP64 | xnb.PREC_NEWTON, FP64_TOL),
                      (xnb.PREC_MIXED, MIXED_TOL)):
        b.lennard_jones_force(s, prec, True)
        e, _ = force_error(forces(b.download(s)), ref)
        assert e <= tol, (prec, e)
        _, pe = b.energy(s)
        assert abs(pe - pe_o) <= tol * abs(pe_o), (prec, pe, pe_o)
    b.close()
