"""Every neighbour-build kernel gives the reference's lists.

XNB_BUILD_ROWS (lane per particle, rows of three cells bulk-copied into shared
memory; two particles per lane for cells of 33-64), XNB_BUILD_WARP (lane per
candidate, the 27-cell block staged per warp) and XNB_BUILD_HALF (each pair of
cells once, per-cell pair masks, lists written from the masks) against the
oracle: neighbour lists as ids in stream order at init and after every
rebuild, the same rebuild steps, and bitwise state after the run (FP64_EXACT);
on the final state the Newton traversal over the lower halves agrees with the
full lists to 1e-12. The systems cover a uniform liquid, cells of 33-64
particles, cells above 64 particles or with rows over the stage (the
block-per-cell build; the half-shell form passes the system to the warp build)
and the 2-cell periodic wrap (a neighbour cell seen through two images)."""
import numpy as np
import pytest

from exanbody_gb300 import workloads, xnb
from helpers import (assert_bitwise_equal, compare_pairs_sliced, force_error, forces, ncells, new_batch,
                     oracle_from)

pytestmark = pytest.mark.gpu

CASES = [
    (20, 0.8442, 1.44, 12345, 30),  # 32,000 atoms, 24 per cell
    (10, 1.05, 1.44, 5, 40),        # 32 per cell on the lattice: cells of 33+ after a few steps
    (6, 1.5, 1.0, 7, 5),            # 108 per cell: every cell block-per-cell
    (5, 1.0, 1.2, 8, 20),           # 62 per cell, 2 cells per axis: rows over the stage
]


@pytest.mark.parametrize("form", [xnb.BUILD_ROWS, xnb.BUILD_WARP, xnb.BUILD_HALF])
@pytest.mark.parametrize("n,rho,T,seed,steps", CASES)
def test_build_form_lists_equal_the_oracle(form, n, rho, T, seed, steps):
    w = workloads.lj_fcc_system(n, rho, T, seed)
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])], list_per_atom=max(170.0, 220.0 * rho))
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
    b.set_build_form(form)
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    compare_pairs_sliced(b, s, o, b.download(s))
    occupancy = {int(b.info(s).max_cell)}
    for step in range(steps):
        r0 = b.info(s).rebuilds
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC)
        rebuilt = o.step()
        assert (b.info(s).rebuilds - r0) == rebuilt, "rebuild decision differs at step %d" % step
        if rebuilt:
            compare_pairs_sliced(b, s, o, b.download(s))
            occupancy.add(int(b.info(s).max_cell))
    assert_bitwise_equal(b.download(s), o.particles())
    if n == 10:
        # the two-particles-per-lane path ran: some cell held 33..64 particles
        assert any(32 < m <= 64 for m in occupancy), occupancy
    b.lennard_jones_force(s, xnb.PREC_FP64, False)
    full = forces(b.download(s))
    b.lennard_jones_force(s, xnb.PREC_FP64 | xnb.PREC_NEWTON, False)
    e, _ = force_error(forces(b.download(s)), full)
    assert e <= 1e-12, e
    b.check_errors()
    b.close()


@pytest.mark.parametrize("form,factor", [(xnb.BUILD_WARP, 1.0), (xnb.BUILD_ROWS, 1.0), (xnb.BUILD_HALF, 1.0),
                                         (xnb.BUILD_WARP, 2.0)])
def test_sizing_build_of_a_new_system_leaves_resident_lists_alone(form, factor):
    """A system added to a batch is first built without list slots (the build
    that sizes them): its hits must go nowhere. The resident system's lists,
    which may start at the same offset of the list pool, stay as they were
    (warp, rows and half-shell forms; sub-cell pruned cells with factor 2)."""
    wa = workloads.lj_fcc_system(10, 0.8442, 1.44, 31, cell_factor=factor)
    wb = workloads.lj_fcc_system(8, 0.9, 1.2, 32, cell_factor=factor)
    b = new_batch([wa["n_atoms"], wb["n_atoms"]], [ncells(wa["geom"]), ncells(wb["geom"])], max_systems=2)
    b.set_build_form(form)
    sa = b.add_system(xnb.lj_params(wa["geom"]), wa["r"], wa["v"], wa["id"])
    b.init_particles(sa, xnb.PREC_MIXED)
    before = b.pairs(sa)
    sb = b.add_system(xnb.lj_params(wb["geom"]), wb["r"], wb["v"], wb["id"])
    b.init_particles(sb, xnb.PREC_MIXED)
    after = b.pairs(sa)
    for x, y in zip(before, after):
        assert np.array_equal(x, y)
    o = oracle_from(wb)
    o.init()
    compare_pairs_sliced(b, sb, o, b.download(sb))
    b.check_errors()
    b.close()
