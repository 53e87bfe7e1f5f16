"""A domain far from the coordinate origin, in every precision.

The 32,000-atom configuration translated to origin (-500, 1000, 7500) sigma:
positions there carry ~12 fewer fraction bits than in a domain at 0, the FP32
mirrors are taken relative to the domain origin, and the mixed path's FP64
displacement sum (sum pd r_b - r_a sum pd) runs on large coordinates.

FP64_EXACT stays bit-identical to the oracle for 100 steps (same rebuild steps,
same lists at every rebuild); on the final state the FP64 traversal is within
1e-12 and the mixed path within 1e-5 relative force error of the oracle's
forces (full and Newton lists); a dump of the far domain, restored through
read_dump's placement, continues bit for bit.
"""
import numpy as np
import pytest

from exanbody_gb300 import dump, workloads, xnb
from helpers import (assert_bitwise_equal, compare_pairs_sliced, force_error, forces, ncells, new_batch,
                     oracle_from, translated)

pytestmark = pytest.mark.gpu

FAR = (-500.0, 1000.0, 7500.0)
FP64_TOL = 1e-12
MIXED_TOL = 1e-5
ALL = ("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz", "pe")


def far_system():
    return translated(workloads.lj_fcc_system(20, 0.8442, 1.44, 12345), FAR)


def test_far_origin_exact_trajectory_and_all_precisions():
    w = far_system()
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    assert_bitwise_equal(b.download(s), o.particles(), fields=ALL)
    compare_pairs_sliced(b, s, o, b.download(s))
    rebuilds = 0
    for step in range(100):
        r0 = b.info(s).rebuilds
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC | xnb.STEP_ENERGY)
        rebuilt = o.step()
        assert (b.info(s).rebuilds - r0) == rebuilt, "rebuild decision differs at step %d" % step
        if rebuilt:
            rebuilds += 1
            compare_pairs_sliced(b, s, o, b.download(s))
    assert rebuilds >= 1
    O = o.particles()
    assert_bitwise_equal(b.download(s), O, fields=ALL)
    assert float(np.min(O["rz"])) > 7400.0  # the state really is far out
    ref = forces(O)
    _, pe_o = o.energy()
    errs = {}
    for prec, tol in ((xnb.PREC_FP64, FP64_TOL), (xnb.PREC_FP64 | xnb.PREC_NEWTON, FP64_TOL),
                      (xnb.PREC_MIXED, MIXED_TOL), (xnb.PREC_MIXED | xnb.PREC_NEWTON, MIXED_TOL)):
        b.lennard_jones_force(s, prec, True)
        e, _ = force_error(forces(b.download(s)), ref)
        errs[prec] = e
        assert e <= tol, (prec, e)
        _, pe = b.energy(s)
        assert abs(pe - pe_o) <= tol * abs(pe_o), (prec, pe, pe_o)
    b.close()


def test_far_origin_mixed_and_fp64_steps_track_the_exact_path():
    """100 steps in each precision from the same state: the rebuild steps equal
    the exact path's, and the trajectories stay within a few 1e-9 (FP64) and
    1e-5 (mixed) of it in position after 100 steps of a chaotic dynamics."""
    w = far_system()
    runs = {}
    for prec in (xnb.PREC_FP64_EXACT, xnb.PREC_FP64, xnb.PREC_MIXED):
        b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
        s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
        b.init_particles(s, prec)
        steps = []
        for step in range(100):
            r0 = b.info(s).rebuilds
            b.step(1, prec, xnb.STEP_HOST_SYNC)
            if b.info(s).rebuilds != r0:
                steps.append(step)
        P = b.download(s)
        order = np.argsort(P["id"])
        runs[prec] = (steps, np.stack([P[k][order] for k in ("rx", "ry", "rz")], 1))
        b.check_errors()
        b.close()
    steps_x, r_x = runs[xnb.PREC_FP64_EXACT]
    L = np.array(w["geom"]["extent"]) - np.array(w["geom"]["origin"])
    for prec, tol in ((xnb.PREC_FP64, 1e-8), (xnb.PREC_MIXED, 1e-4)):
        steps_p, r_p = runs[prec]
        assert steps_p == steps_x, (prec, steps_p, steps_x)
        d = r_p - r_x
        d -= L * np.round(d / L)  # a particle wrapped on one side only
        assert float(np.abs(d).max()) <= tol, (prec, float(np.abs(d).max()))


def test_far_origin_dump_restart_continues_bit_for_bit(tmp_path):
    w = far_system()
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    r0 = b.info(s).rebuilds
    steps = 0
    while b.info(s).rebuilds == r0:
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC)
        steps += 1
        assert steps < 200
    path = tmp_path / "far.dump"
    dump.write_system(b, s, path, timestep=steps, physical_time=steps * 0.005)
    info = dump.read_info(path)
    assert tuple(info["domain"]["origin"]) == tuple(w["geom"]["origin"])
    assert tuple(info["domain"]["extent"]) == tuple(w["geom"]["extent"])
    b2 = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s2, _ = dump.restore_system(b2, path)
    b2.init_particles(s2, xnb.PREC_FP64_EXACT)
    keys = ("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz")
    assert_bitwise_equal(b.download(s), b2.download(s2), fields=keys)
    for _ in range(3):
        b.step(10, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC)
        b2.step(10, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC)
        assert_bitwise_equal(b.download(s), b2.download(s2), fields=keys)
    b.close()
    b2.close()
