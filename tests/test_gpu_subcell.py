"""Sub-cell pair pruning of the neighbour build (xnb_batch_set_subcell_pruning).

Cells with an AMR sub-grid (side 2 or 3) search only the sub-cells of their 27
neighbour cells that lie within reach of each of their own sub-cells
(max_distance_sub_cell_pairs, amr/lib/amr_grid_algorithm.cpp:102-218). The
systems are the 32,000-atom FCC configuration gridded with larger cells
(5.6, 6.72 and 8.4 sigma: 148, 256 and 500 atoms per cell, sub-grid sides 2, 3
and 4; a neighbourhood with side 4 goes to the unpruned build) and a slab whose
cells range from empty to dense. The lists equal the oracle's at init and at
every rebuild, the trajectories stay bit-identical, and the reference-format
streams with both offset tables (lower-half lengths included) equal the
unpruned build's word for word.
"""
import numpy as np
import pytest

from exanbody_gb300 import workloads, xnb
from helpers import assert_bitwise_equal, ncells, new_batch, oracle_from

pytestmark = pytest.mark.gpu

ALL = ("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz", "pe")


def compare_pairs(b, s, o):
    ga, gb, gc = b.pairs(s)
    oa, ob, oc = o.pairs()
    assert np.array_equal(gc, oc), "per-particle neighbour counts differ"
    assert np.array_equal(ga, oa) and np.array_equal(gb, ob), "neighbour lists differ"
    return len(ga)


def system(w, prune=True, stage_cap=0):
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    if stage_cap:
        b.set_tuning(stage_cap, 128)
    b.set_subcell_pruning(prune)
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
    return b, s


@pytest.mark.parametrize("factor,side", [(1.9, 2), (2.0, 3), (2.5, 4)])
def test_dense_cells_lists_and_trajectory_bit_exact(factor, side):
    w = workloads.lj_fcc_system(20, 0.8442, 1.44, 12345, cell_factor=factor)
    per_cell = w["n_atoms"] / ncells(w["geom"])
    assert int(np.floor(np.cbrt(per_cell / 6.5))) == side
    b, s = system(w)
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    assert_bitwise_equal(b.download(s), o.particles(), fields=ALL)
    npairs = compare_pairs(b, s, o)
    assert 75 * w["n_atoms"] < npairs < 80 * w["n_atoms"]
    rebuilds = 0
    for step in range(40):
        r0 = b.info(s).rebuilds
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC | xnb.STEP_ENERGY)
        rebuilt = o.step()
        assert (b.info(s).rebuilds - r0) == rebuilt, "rebuild decision differs at step %d" % step
        if rebuilt:
            rebuilds += 1
            compare_pairs(b, s, o)
    assert rebuilds >= 2
    assert_bitwise_equal(b.download(s), o.particles(), fields=ALL)
    b.check_errors()
    b.close()


def test_slab_of_empty_half_and_dense_cells_bit_exact():
    """Cells of 6.72 sigma across a liquid-vacuum slab: empty cells (side 1), half
    filled cells at the interfaces and full ones (sides 2 and 3) side by side."""
    w = workloads.lj_slab_system(12, 0.8442, 0.8, 7, cell_factor=2.0)
    b, s = system(w)
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    counts = o.cell_counts()
    sides = np.where(counts / 6.5 >= 8.0, np.floor(np.cbrt(counts / 6.5)), 1)
    assert (counts == 0).any() and (sides == 2).any() and (sides == 3).any()
    compare_pairs(b, s, o)
    for _ in range(40):
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC | xnb.STEP_ENERGY)
        if o.step():
            compare_pairs(b, s, o)
    assert_bitwise_equal(b.download(s), o.particles(), fields=ALL)
    b.close()


@pytest.mark.parametrize("stage_cap", [0, 128])
def test_pruned_streams_equal_unpruned_streams(stage_cap):
    """The reference-format streams with the per-particle offsets and lower-half
    lengths (offset_tables = 2), after init, after a rebuild and after a build
    without a rebin once positions have moved (the sub-cell keys are then stale
    and whole cells are searched): the pruned build gives the unpruned build's
    words. A 128-candidate stage takes each sub-cell's candidates in many rounds."""
    import torch

    w = workloads.lj_fcc_system(20, 0.8442, 1.44, 4242, cell_factor=2.0)
    runs = []
    for prune in (True, False):
        b, s = system(w, prune, stage_cap)
        b.init_particles(s, xnb.PREC_MIXED)
        first = [t.cpu().numpy().copy() for t in b.chunk_neighbors_stream(s, offset_tables=2)]
        b.step(30, xnb.PREC_MIXED, xnb.STEP_HOST_SYNC)
        b.update_particles_full(s)
        second = [t.cpu().numpy().copy() for t in b.chunk_neighbors_stream(s, offset_tables=2)]
        b.step(5, xnb.PREC_MIXED, xnb.STEP_HOST_SYNC)
        b.push_f_v_r(1.0, s)  # positions move without a rebin
        b.chunk_neighbors(s)
        third = [t.cpu().numpy().copy() for t in b.chunk_neighbors_stream(s, offset_tables=2)]
        b.check_errors()
        b.close()
        runs.append((first, second, third))
    torch.cuda.synchronize()
    for k in range(3):
        for x, y in zip(runs[0][k], runs[1][k]):
            assert np.array_equal(x, y)


def test_captured_steps_prune_like_host_synchronised_steps():
    """A CUDA graph of mixed steps (rebuilds inside the graph) equals the same
    steps run one by one with host synchronisation, positions bit for bit."""
    import ctypes

    import torch

    w = workloads.lj_fcc_system(16, 0.8442, 1.44, 5, cell_factor=2.0)
    out = []
    for graph in (False, True):
        b, s = system(w)
        stream = torch.cuda.Stream()
        b.stream = ctypes.c_void_p(stream.cuda_stream)
        b.init_particles(s, xnb.PREC_MIXED)
        if graph:
            g = b.graph(40, xnb.PREC_MIXED, 0)
            g.launch()
            stream.synchronize()
            g.close()
        else:
            b.step(40, xnb.PREC_MIXED, xnb.STEP_HOST_SYNC)
        b.check_errors()
        out.append((b.download(s), b.info(s).rebuilds))
        b.close()
    assert out[0][1] == out[1][1] >= 2
    assert_bitwise_equal(out[0][0], out[1][0], fields=("rx", "ry", "rz", "vx", "vy", "vz"))
