"""Threads per particle of the force traversal (xnb_batch_set_force_lanes), and
graphs that no longer cover a grown batch.

With 2 or 4 threads per particle the FP64 and mixed full-list traversals split
each list in 8-entry blocks and combine the partial sums in a fixed order:
forces agree with one thread per particle within the precision's tolerance
(1e-12 FP64, 1e-5 mixed, |dF_i| / max(|F_i|, F_rms)), repeated calls give the
same bits, and a graph-captured mixed run stays within tolerance of the
one-thread run. FP64_EXACT ignores the setting (bit-exact with the oracle)."""
import ctypes

import numpy as np
import pytest

from exanbody_gb300 import workloads, xnb
from helpers import assert_bitwise_equal, force_error, forces, ncells, new_batch, oracle_from

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("lanes", [2, 4])
def test_lanes_agree_with_one_thread_and_repeat_bitwise(lanes):
    w = workloads.lj_fcc_system(16, 0.8442, 1.44, 21)
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    b.step(25, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC)
    for prec, tol in ((xnb.PREC_FP64, 1e-12), (xnb.PREC_MIXED, 1e-5)):
        b.set_force_lanes(1)
        b.lennard_jones_force(s, prec, True)
        one = b.download(s)
        b.set_force_lanes(lanes)
        b.lennard_jones_force(s, prec, True)
        many = b.download(s)
        b.lennard_jones_force(s, prec, True)
        again = b.download(s)
        e, _ = force_error(forces(many), forces(one))
        assert e <= tol, (prec, lanes, e)
        assert abs(many["pe"].sum() - one["pe"].sum()) <= tol * abs(one["pe"].sum())
        assert_bitwise_equal(many, again, fields=("fx", "fy", "fz", "pe"))
    b.close()


def test_exact_path_ignores_lanes():
    w = workloads.lj_fcc_system(10, 0.8442, 1.44, 4)
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
    b.set_force_lanes(4)
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    for _ in range(20):
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC | xnb.STEP_ENERGY)
        o.step()
    assert_bitwise_equal(b.download(s), o.particles())
    b.close()


def test_lanes_in_a_captured_mixed_run():
    """A 200-step graph-captured mixed run with 4 threads per particle stays
    within tolerance of the one-thread run (same rebuild count)."""
    import torch

    w = workloads.lj_fcc_system(12, 0.8442, 1.44, 8)
    res = {}
    for lanes in (1, 4):
        stream = torch.cuda.Stream()
        b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
        b.stream = ctypes.c_void_p(stream.cuda_stream)
        s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
        b.set_force_lanes(lanes)
        b.init_particles(s, xnb.PREC_MIXED)
        g = b.graph(50, xnb.PREC_MIXED, 0)
        for _ in range(4):
            g.launch()
        stream.synchronize()
        b.check_errors()
        P = b.download(s)
        order = np.argsort(P["id"])
        res[lanes] = (np.stack([P[k][order] for k in ("rx", "ry", "rz")], 1), b.info(s).rebuilds)
        g.close()
        b.close()
    L = np.array(w["geom"]["extent"]) - np.array(w["geom"]["origin"])
    d = res[4][0] - res[1][0]
    d -= L * np.round(d / L)
    assert float(np.abs(d).max()) <= 1e-4
    assert res[4][1] == res[1][1]


def test_graph_refuses_a_grown_batch():
    """A graph captured before a system joined beyond the captured extent is not
    current and refuses to launch (it would not step the new system)."""
    import torch

    ws = [workloads.lj_fcc_system(6, 0.8442, 1.44, k) for k in (1, 2)]
    stream = torch.cuda.Stream()
    b = new_batch([w["n_atoms"] for w in ws], [ncells(w["geom"]) for w in ws], max_systems=2)
    b.stream = ctypes.c_void_p(stream.cuda_stream)
    s0 = b.add_system(xnb.lj_params(ws[0]["geom"]), ws[0]["r"], ws[0]["v"], ws[0]["id"])
    b.init_particles(s0, xnb.PREC_MIXED)
    g = b.graph(5, xnb.PREC_MIXED, 0)
    assert g.current()
    g.launch()
    s1 = b.add_system(xnb.lj_params(ws[1]["geom"]), ws[1]["r"], ws[1]["v"], ws[1]["id"])
    b.init_particles(s1, xnb.PREC_MIXED)
    assert not g.current()
    with pytest.raises(xnb.XnbError):
        g.launch()
    g.close()
    g2 = b.graph(5, xnb.PREC_MIXED, 0)
    g2.launch()
    stream.synchronize()
    b.check_errors()
    g2.close()
    b.close()
