"""The staged mixed force traversal (xnb_batch_set_force_form(XNB_FORCE_STAGED)).

Blocks stage the neighbourhood of a segment of cells in shared memory and walk
the lists in their compact (cell group, index in cell) form; entry order, the
FP32 prefilter and the pair body are those of the one-thread traversal, so
forces, energies and velocities must be bitwise equal to it: on a liquid state,
on small domains whose neighbourhoods repeat cells through periodic images, on
a batch of several systems, on dense cells that overflow the stage (the
segment then runs from global memory), after switching the form on with lists
already built, and over a graph-captured run with rebuilds."""
import ctypes

import numpy as np
import pytest

from exanbody_gb300 import workloads, xnb
from helpers import assert_bitwise_equal, ncells, new_batch

pytestmark = pytest.mark.gpu

F = ("fx", "fy", "fz", "pe")


def forces_both(b, s, energy=True):
    b.set_force_form(xnb.FORCE_THREAD)
    b.lennard_jones_force(s, xnb.PREC_MIXED, energy)
    one = b.download(s)
    b.set_force_form(xnb.FORCE_STAGED)
    b.lennard_jones_force(s, xnb.PREC_MIXED, energy)
    staged = b.download(s)
    b.set_force_form(xnb.FORCE_THREAD)
    return one, staged


@pytest.mark.parametrize("n,rho,T,seed,steps", [
    (20, 0.8442, 1.44, 12345, 30),  # 32,000 atoms, 11^3 cells: segments of 8 and 3 cells
    (6, 0.8442, 1.44, 2, 10),       # 3^3 cells: rows shorter than a segment, images in every row
    (4, 1.0, 1.0, 3, 10),           # 2^3 cells: each neighbour cell staged twice through images
    (5, 1.0, 1.2, 8, 10),           # 62 atoms per cell: the neighbourhood overflows the stage
])
def test_staged_forces_bitwise_equal_thread_forces(n, rho, T, seed, steps):
    w = workloads.lj_fcc_system(n, rho, T, seed)
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
    b.init_particles(s, xnb.PREC_MIXED)
    b.step(steps, xnb.PREC_MIXED, xnb.STEP_HOST_SYNC)
    for energy in (True, False):
        one, staged = forces_both(b, s, energy)
        assert_bitwise_equal(staged, one, fields=F if energy else F[:3])
    b.check_errors()
    b.close()


def test_staged_batch_of_systems_and_form_switch():
    ws = [workloads.lj_fcc_system(n, rho, 1.2, 10 + n) for n, rho in ((7, 0.8), (10, 0.9), (5, 0.75))]
    b = new_batch([w["n_atoms"] for w in ws], [ncells(w["geom"]) for w in ws], max_systems=3)
    ids = [b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"]) for w in ws]
    b.init_particles(-1, xnb.PREC_MIXED)
    b.step(20, xnb.PREC_MIXED, xnb.STEP_HOST_SYNC)
    for s in ids:
        one, staged = forces_both(b, s)
        assert_bitwise_equal(staged, one, fields=F)
    b.close()


def test_staged_captured_run_equals_thread_run():
    """200 mixed steps as replays of a 50-step graph (rebuilds inside, lists
    compacted on the device after each build): bitwise the same trajectory."""
    import torch

    w = workloads.lj_fcc_system(12, 0.8442, 1.44, 8)
    out = {}
    for form in (xnb.FORCE_THREAD, xnb.FORCE_STAGED):
        stream = torch.cuda.Stream()
        b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
        b.stream = ctypes.c_void_p(stream.cuda_stream)
        s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
        b.set_force_form(form)
        b.init_particles(s, xnb.PREC_MIXED)
        g = b.graph(50, xnb.PREC_MIXED, xnb.STEP_ENERGY)
        for _ in range(4):
            g.launch()
        stream.synchronize()
        b.check_errors()
        out[form] = (b.download(s), b.info(s).rebuilds)
        g.close()
        b.close()
    assert out[xnb.FORCE_STAGED][1] == out[xnb.FORCE_THREAD][1] > 0
    assert_bitwise_equal(out[xnb.FORCE_STAGED][0], out[xnb.FORCE_THREAD][0],
                         fields=("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz", "pe"))
