"""A box longer than 1024 sigma in one batch with an ordinary one.

The mixed traversal packs each particle's FP32 position residuals into the
mirror's fourth word as 10-bit multiples of ulp(X) / 1024 (X bounds
|x - origin|). Their absolute error grows with X, so a system with X above
1024 sigma reads the residual mirror instead (SysDesc::packed_lo = 0, a
uniform branch per system). Here an elongated FCC system (8.4 x 8.4 x 1030
sigma, 61k atoms) shares a batch with the 32,000-atom cube. Both systems'
mixed forces (full and Newton lists) stay within 1e-5 of their FP64 forces, and
the FP64_EXACT trajectory of the long system equals the oracle's bit for bit
over 30 steps.
"""
import numpy as np
import pytest

from exanbody_gb300 import workloads, xnb
from helpers import assert_bitwise_equal, force_error, forces, ncells, new_batch, oracle_from

pytestmark = pytest.mark.gpu

RHO = 0.8442


def long_system(seed=21):
    r, a = workloads.fcc_lattice(5, RHO, nz=613)
    L = 5 * a
    geom = workloads.geometry((L, L, 613 * a))
    v = workloads.maxwell_boltzmann(len(r), 1.2, seed)
    ids = np.arange(len(r), dtype=np.uint64)
    return {"r": r, "v": v, "id": ids, "geom": geom, "a": a, "n_atoms": len(r), "rho": RHO, "T": 1.2}


def test_long_box_and_cube_mixed_forces_within_tolerance():
    wl = long_system()
    wc = workloads.lj_fcc_system(20, RHO, 1.44, 12345)
    assert max(wl["geom"]["extent"]) > 1024.0
    b = new_batch([wl["n_atoms"], wc["n_atoms"]], [ncells(wl["geom"]), ncells(wc["geom"])], max_systems=2)
    sl = b.add_system(xnb.lj_params(wl["geom"]), wl["r"], wl["v"], wl["id"])
    sc = b.add_system(xnb.lj_params(wc["geom"]), wc["r"], wc["v"], wc["id"])
    for s in (sl, sc):
        b.init_particles(s, xnb.PREC_MIXED)
    b.step(40, xnb.PREC_MIXED, xnb.STEP_HOST_SYNC)  # off the lattice
    for s in (sl, sc):
        b.lennard_jones_force(s, xnb.PREC_FP64, False)
        ref = forces(b.download(s))
        for prec in (xnb.PREC_MIXED, xnb.PREC_MIXED | xnb.PREC_NEWTON):
            b.lennard_jones_force(s, prec, False)
            e, _ = force_error(forces(b.download(s)), ref)
            assert e <= 1e-5, (s, prec, e)
    b.check_errors()
    b.close()


def test_long_box_exact_trajectory_equals_oracle():
    w = long_system(5)
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    for _ in range(30):
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC | xnb.STEP_ENERGY)
        o.step()
    assert_bitwise_equal(b.download(s), o.particles())
    b.close()
