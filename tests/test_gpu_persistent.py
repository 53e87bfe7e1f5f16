"""The persistent step loop (xnb_step_persistent): one cooperative launch
advances every system step after step, with grid barriers between the phases,
until a step's displacement trigger fires; that step's rebuild path and forces
run as separate launches and the loop resumes.

FP64_EXACT through the loop stays bitwise equal to the oracle for 100 steps of
the 32,000-atom configuration (same rebuild count); FP64 and mixed runs equal
xnb_step bit for bit, alone and for a batch of systems of different sizes. The
barrier's time limit is exercised without a hang: XNB_STEP_BARRIER_CHECK makes
the first barrier wait for a block that does not exist, every wait runs out
after 20 ms, the call reports XNB_ERR_DEVICE, no state changes, and the batch
steps normally afterwards.
"""
import numpy as np
import pytest

from exanbody_gb300 import workloads, xnb
from helpers import assert_bitwise_equal, ncells, new_batch, oracle_from

pytestmark = pytest.mark.gpu

ALL = ("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz", "pe")
MOTION = ("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz")


def batch_of(ws):
    b = new_batch([w["n_atoms"] for w in ws], [ncells(w["geom"]) for w in ws], max_systems=len(ws))
    ss = [b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"]) for w in ws]
    return b, ss


def test_exact_loop_equals_oracle_100_steps():
    w = workloads.lj_fcc_system(20, 0.8442, 1.44, 12345)
    b, (s,) = batch_of([w])
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    rebuilt = 0
    for _ in range(100):
        rebuilt += int(o.step())
    b.step_persistent(100, xnb.PREC_FP64_EXACT, xnb.STEP_ENERGY)
    assert b.info(s).rebuilds == rebuilt >= 10
    assert_bitwise_equal(b.download(s), o.particles(), fields=ALL)
    b.check_errors()
    b.close()


@pytest.mark.parametrize("prec", [xnb.PREC_FP64, xnb.PREC_MIXED])
def test_loop_equals_fused_steps(prec):
    ws = [workloads.lj_fcc_system(n, rho, T, seed) for n, rho, T, seed in
          ((14, 0.8442, 1.44, 1), (9, 0.95, 0.9, 2), (17, 0.75, 1.3, 3))]
    out = []
    for persistent in (False, True):
        b, ss = batch_of(ws)
        for s in ss:
            b.init_particles(s, prec)
        if persistent:
            b.step_persistent(150, prec, xnb.STEP_ENERGY)
        else:
            b.step(150, prec, xnb.STEP_HOST_SYNC | xnb.STEP_ENERGY)
        b.check_errors()
        out.append([(b.download(s), b.info(s).rebuilds) for s in ss])
        b.close()
    for (g, rg), (p, rp) in zip(out[0], out[1]):
        assert rg == rp >= 5
        assert_bitwise_equal(p, g, fields=ALL)


def test_barrier_wait_runs_out_without_changing_state():
    w = workloads.lj_fcc_system(12, 0.8442, 1.44, 8)
    b, (s,) = batch_of([w])
    b.init_particles(s, xnb.PREC_MIXED)
    b.step_persistent(20, xnb.PREC_MIXED)
    before = b.download(s)
    with pytest.raises(xnb.XnbError) as e:
        b.step_persistent(5, xnb.PREC_MIXED, xnb.STEP_BARRIER_CHECK)
    assert e.value.code == -5
    assert_bitwise_equal(b.download(s), before, fields=MOTION)
    # the context and the batch stay usable: the loop resumes where it was
    b.step_persistent(30, xnb.PREC_MIXED)
    b.check_errors()
    ref, (r,) = batch_of([w])
    ref.init_particles(r, xnb.PREC_MIXED)
    ref.step(50, xnb.PREC_MIXED, xnb.STEP_HOST_SYNC)
    assert_bitwise_equal(b.download(s), ref.download(r), fields=MOTION)
    b.close()
    ref.close()


def test_newton_lists_are_refused():
    w = workloads.lj_fcc_system(6, 0.8442, 1.44, 3)
    b, (s,) = batch_of([w])
    b.init_particles(s, xnb.PREC_MIXED)
    with pytest.raises(xnb.XnbError) as e:
        b.step_persistent(2, xnb.PREC_MIXED | xnb.PREC_NEWTON)
    assert e.value.code == -1
    b.close()
