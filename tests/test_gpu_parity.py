"""Parity of the sm_103a library (through its C ABI) with the CPU oracle.

FP64_EXACT must be bit-identical to the oracle: neighbour pair lists (as
particle ids, in the reference's stream order), positions, velocities and
forces after every step. FP64 must agree within 1e-12 relative force error and
MIXED within 1e-5 (|dF_i| / max(|F_i|, F_rms), max over particles).
"""
import json
import os

import numpy as np
import pytest

from exanbody_gb300 import workloads, xnb
from helpers import (assert_bitwise_equal, force_error, forces, ncells, new_batch, ni_deck_oracle,
                     ni_deck_params, oracle_from)

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-5


def gpu_system(w, batch=None, list_factor=1.3):
    b = batch or new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"], list_factor=list_factor)
    return b, s


def compare_pairs(b, s, o):
    ga, gb, gc = b.pairs(s)
    oa, ob, oc = o.pairs()
    assert np.array_equal(gc, oc), "per-particle neighbour counts differ"
    assert np.array_equal(ga, oa) and np.array_equal(gb, ob), "neighbour lists differ"
    return len(ga)


def test_init_bit_exact_config0():
    w = workloads.lj_fcc_system(20, 0.8442, 1.44, 12345)  # 32,000 atoms
    b, s = gpu_system(w)
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    G, O = b.download(s), o.particles()
    assert_bitwise_equal(G, O, fields=("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz", "pe"))
    npairs = compare_pairs(b, s, o)
    assert 75 * w["n_atoms"] < npairs < 80 * w["n_atoms"]


def test_trajectory_bit_exact_config0_100_steps():
    """Same rebuild steps, same pair lists at every rebuild, same bits after 100 steps."""
    w = workloads.lj_fcc_system(20, 0.8442, 1.44, 12345)
    b, s = gpu_system(w)
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    rebuild_steps = 0
    for step in range(100):
        r0 = b.info(s).rebuilds
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC | xnb.STEP_ENERGY)
        rebuilt = o.step()
        assert (b.info(s).rebuilds - r0) == rebuilt, "rebuild decision differs at step %d" % step
        if rebuilt:
            rebuild_steps += 1
            compare_pairs(b, s, o)
    assert rebuild_steps >= 1
    assert_bitwise_equal(b.download(s), o.particles(), fields=("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz", "pe"))
    ke_g, pe_g = b.energy(s)
    ke_o, pe_o = o.energy()
    assert ke_g == ke_o and pe_g == pe_o


def test_fp64_and_mixed_forces_on_same_state():
    w = workloads.lj_fcc_system(20, 0.8442, 1.44, 12345)
    b, s = gpu_system(w)
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    b.step(30, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC)  # a liquid-like state with rebuilds behind it
    ref = forces(b.download(s))
    b.lennard_jones_force(s, xnb.PREC_FP64, True)
    f64 = forces(b.download(s))
    b.lennard_jones_force(s, xnb.PREC_MIXED, True)
    fmx = forces(b.download(s))
    e64, _ = force_error(f64, ref)
    emx, rms = force_error(fmx, ref)
    assert e64 <= FP64_TOL, e64
    assert emx <= MIXED_TOL, emx
    assert rms < emx or rms == emx


def test_graph_equals_host_sync_exact():
    w = workloads.lj_fcc_system(12, 0.8442, 1.44, 99)
    b1, s1 = gpu_system(w)
    b1.init_particles(s1, xnb.PREC_FP64_EXACT)
    b1.step(60, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC)
    import torch
    stream = torch.cuda.Stream()
    b2 = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    b2.stream = __import__("ctypes").c_void_p(stream.cuda_stream)
    s2 = b2.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
    b2.init_particles(s2, xnb.PREC_FP64_EXACT)
    g = b2.graph(20, xnb.PREC_FP64_EXACT, 0)
    for _ in range(3):
        g.launch()
    stream.synchronize()
    b2.check_errors()
    assert_bitwise_equal(b2.download(s2), b1.download(s1))
    assert b1.info(s1).rebuilds == b2.info(s2).rebuilds


@pytest.mark.parametrize("n,rho,T", [(5, 1.0, 1.2), (4, 1.0, 0.9), (7, 0.7, 1.5)])
def test_small_and_dense_systems_bit_exact(n, rho, T):
    """D = 2 cells per axis, cells dense enough for AMR sub-grids (62 atoms/cell)."""
    w = workloads.lj_fcc_system(n, rho, T, 3 + n)
    b, s = gpu_system(w)
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    compare_pairs(b, s, o)
    for _ in range(50):
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC)
        if o.step():
            compare_pairs(b, s, o)
    assert_bitwise_equal(b.download(s), o.particles())


@pytest.mark.parametrize("cap", [32, 512, 544])
def test_stage_cap_splits_cells_between_builds(cap):
    """Cells whose candidates exceed the stage cap are built block-per-cell, the
    others warp-per-cell; a cap near the mean candidate count (~515 here) splits
    one system between both builds. Lists match the oracle's, and the lower-half
    lengths give Newton-list forces equal to the full-list ones."""
    w = workloads.lj_fcc_system(12, 0.8442, 1.44, 99)
    b, s = gpu_system(w)
    b.set_tuning(cap, 128)
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    compare_pairs(b, s, o)
    # off the lattice first: there the net forces are rounding-sized
    for _ in range(30):
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC)
        if o.step():
            compare_pairs(b, s, o)
    assert_bitwise_equal(b.download(s), o.particles())
    b.lennard_jones_force(s, xnb.PREC_FP64, True)
    full = forces(b.download(s))
    b.lennard_jones_force(s, xnb.PREC_FP64 | xnb.PREC_NEWTON, True)
    e, _ = force_error(forces(b.download(s)), full)
    assert e <= FP64_TOL, e


@pytest.mark.parametrize("list_factor", [8.0, 12.0])
def test_large_slots_take_the_block_build(list_factor):
    """Slots above 512 entries leave every cell to the block-per-cell build: its
    shared-memory list buffer up to 1024 entries (factor 8: ~760), direct global
    writes above (factor 12: ~1130). Lists and trajectories stay the oracle's."""
    w = workloads.lj_fcc_system(8, 0.8442, 1.44, 31)
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])], list_per_atom=1300.0)
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"], list_factor=list_factor)
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    compare_pairs(b, s, o)
    for _ in range(20):
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC)
        if o.step():
            compare_pairs(b, s, o)
    assert_bitwise_equal(b.download(s), o.particles())


def test_warp_build_cells_above_32_particles():
    """Cells of more than 32 particles whose candidates still fit the warp's
    stage: the warp build loads those particles' mirrors per pass instead of
    shuffling them across lanes. 3^3 cells of 3 sigma with ~25 uniformly random
    particles each (Poisson counts up to ~40), stage 1024: the oracle's lists."""
    rng = np.random.default_rng(7)
    geom = workloads.geometry((9.0, 9.0, 9.0))
    assert tuple(geom["dims"]) == (3, 3, 3)
    n = 675
    w = {"r": rng.uniform(0.0, 9.0, (n, 3)), "v": rng.normal(0.0, 0.1, (n, 3)),
         "id": np.arange(n, dtype=np.uint64), "geom": geom, "n_atoms": n}
    b, s = gpu_system(w)
    b.set_tuning(1024, 128)
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    assert o.cell_counts().max() > 32
    compare_pairs(b, s, o)
    assert_bitwise_equal(b.download(s), o.particles())


@pytest.mark.parametrize("cap", [640, 1024])
def test_ghost_filter_and_cutoff_boundaries_bit_exact(cap):
    """Periodic images placed on the ghost-filter bound (outer_lo = -nbh) and
    pairs placed on nbh itself, ulps apart: the FP32 tests are undecided there,
    so both builds take the reference's FP64 decisions (block build at stage
    640 < 691 candidates, warp build at 1024). The lists stay the oracle's."""
    rng = np.random.default_rng(11)
    geom = workloads.geometry((9.0, 9.0, 9.0))
    r = [rng.uniform(0.0, 9.0, (675, 3))]
    yz = rng.uniform(0.5, 8.5, (8, 2))
    xb = 9.0 - 2.8
    for k in range(8):
        # b's image through the -x wall sits ulps from -2.8; a at x = 0 faces it at ~2.8
        x = xb
        for _ in range(k - 4 if k >= 4 else 4 - k):
            x = np.nextafter(x, np.inf if k >= 4 else -np.inf)
        r.append(np.array([[0.0, yz[k, 0], yz[k, 1]], [x, yz[k, 0], yz[k, 1]]]))
    r = np.concatenate(r)
    n = len(r)
    w = {"r": r, "v": np.zeros((n, 3)), "id": np.arange(n, dtype=np.uint64), "geom": geom, "n_atoms": n}
    b, s = gpu_system(w)
    b.set_tuning(cap, 128)
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    compare_pairs(b, s, o)
    assert_bitwise_equal(b.download(s), o.particles())


def test_mixed_pair_set_at_the_cutoff():
    """Isolated pairs at rc shifted by 0..4 ulps either way: each particle's force
    is its one pair force or zero, so the mixed path's FP32 cutoff test (FP64
    inside its error band) must select exactly the FP64 pairs; the FP64-exact
    forces stay the oracle's bits."""
    geom = workloads.geometry((12.0, 12.0, 12.0))
    pts = []
    for k in range(8):
        a = np.array([1.0 + (k % 2) * 6.0, 1.0 + ((k // 2) % 2) * 6.0, 1.0 + (k // 4) * 6.0])
        x = a[0] + 2.5
        for _ in range(abs(k - 4)):
            x = np.nextafter(x, np.inf if k >= 4 else -np.inf)
        pts += [a, np.array([x, a[1], a[2]])]
    r = np.array(pts)
    n = len(r)
    w = {"r": r, "v": np.zeros((n, 3)), "id": np.arange(n, dtype=np.uint64), "geom": geom, "n_atoms": n}
    b, s = gpu_system(w)
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    assert_bitwise_equal(b.download(s), o.particles())
    b.lennard_jones_force(s, xnb.PREC_FP64, False)
    f64 = forces(b.download(s))
    b.lennard_jones_force(s, xnb.PREC_MIXED, False)
    fmx = forces(b.download(s))
    in64 = np.linalg.norm(f64, axis=1) > 0
    inmx = np.linalg.norm(fmx, axis=1) > 0
    assert np.array_equal(in64, inmx)
    assert 0 < in64.sum() < n  # pairs on both sides of rc
    e, _ = force_error(fmx, f64)
    assert e <= MIXED_TOL, e


def test_slab_with_empty_cells_bit_exact():
    w = workloads.lj_slab_system(8, 0.8442, 0.8, 5)
    b, s = gpu_system(w)
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    assert (o.cell_counts() == 0).sum() > 0
    compare_pairs(b, s, o)
    for _ in range(50):
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC)
        if o.step():
            compare_pairs(b, s, o)
    assert_bitwise_equal(b.download(s), o.particles())


def test_ni_golden_deck_on_gpu():
    """input_lj_Ni.msp through the library: cells as the lattice generator leaves
    them, 100 steps, check_values golden data within 1e-5 and bitwise = oracle."""
    o = ni_deck_oracle()
    P0 = o.particles()
    counts = o.cell_counts()
    r = np.stack([P0["rx"], P0["ry"], P0["rz"]], 1)
    v = np.stack([P0["vx"], P0["vy"], P0["vz"]], 1)
    b = new_batch([len(r)], [64], list_per_atom=260.0)
    s = b.add_system(ni_deck_params(), r, v, P0["id"], cell_counts=counts)
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o.init()
    for _ in range(100):
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC)
        o.step()
    G = b.download(s)
    assert_bitwise_equal(G, o.particles())
    here = os.path.dirname(__file__)
    with open(os.path.join(here, "golden", "check_values_lj_Ni.json")) as f:
        gold = json.load(f)
    idx = {int(i): k for k, i in enumerate(G["id"])}
    er = ea = ev = 0.0
    for row in gold["rows"]:
        ref = np.array([float.fromhex(h) for h in row["hex"]])
        k = idx[row["id"]]
        d = np.array([G["rx"][k], G["ry"][k], G["rz"][k]]) - ref[0:3]
        d -= 55.68 * np.round(d / 55.68)
        er += float((d ** 2).sum())
        ea += float(((np.array([G["fx"][k], G["fy"][k], G["fz"][k]]) - ref[3:6]) ** 2).sum())
        ev += float(((np.array([G["vx"][k], G["vy"][k], G["vz"][k]]) - ref[6:9]) ** 2).sum())
    assert er ** 0.5 <= 1e-5 and ea ** 0.5 <= 1e-5 and ev ** 0.5 <= 1e-5


def test_operator_sequence_equals_fused_step():
    """The unfused reference operators called one by one give the fused step's bits."""
    w = workloads.lj_fcc_system(10, 0.8442, 1.44, 21)
    b1, s1 = gpu_system(w)
    b1.init_particles(s1, xnb.PREC_FP64_EXACT)
    b2, s2 = gpu_system(w)
    b2.init_particles(s2, xnb.PREC_FP64_EXACT)
    for _ in range(40):
        b1.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC)
        b2.push_f_v_r(1.0, s2)
        b2.push_f_v(0.5, s2)
        if b2.particle_displ_over(s2) > 0:
            b2.update_particles_full(s2)
        b2.lennard_jones_force(s2, xnb.PREC_FP64_EXACT, False)
        b2.push_f_v(0.5, s2)
    assert_bitwise_equal(b1.download(s1), b2.download(s2))


def test_batched_systems_equal_alone():
    """Uneven systems advanced together in one batch give each system's solo result."""
    specs = workloads.ensemble_specs(5, seed=77, nmin=4, nmax=9)
    ws = [workloads.lj_fcc_system(sp["n"], sp["rho"], sp["T"], sp["seed"]) for sp in specs]
    big = new_batch([w["n_atoms"] for w in ws], [ncells(w["geom"]) for w in ws])
    ids = [big.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"]) for w in ws]
    big.init_particles(-1, xnb.PREC_MIXED)
    big.step(80, xnb.PREC_MIXED, 0)
    big.check_errors()
    for w, s in zip(ws, ids):
        b, so = gpu_system(w)
        b.init_particles(so, xnb.PREC_MIXED)
        b.step(80, xnb.PREC_MIXED, 0)
        assert_bitwise_equal(big.download(s), b.download(so))
        assert big.info(s).rebuilds == b.info(so).rebuilds


def test_list_overflow_is_reported_and_recovered():
    """A too-small list segment in graph mode is flagged, not written past."""
    w = workloads.lj_fcc_system(8, 0.8442, 1.44, 4)
    b, s = gpu_system(w, list_factor=1.0)
    b.init_particles(s, xnb.PREC_MIXED)
    # host-sync steps regrow the segment when a rebuild needs more room
    b.step(200, xnb.PREC_MIXED, xnb.STEP_HOST_SYNC)
    b.check_errors()
    assert b.info(s).rebuilds >= 1


def test_newton_half_list_forces_and_energy():
    """Each pair once (lower half of the sorted list) with FP64 reductions for the
    reaction: FP64 <= 1e-12 and MIXED <= 1e-5 against the full-list FP64 forces,
    potential energy to 1e-12 relative."""
    w = workloads.lj_fcc_system(20, 0.8442, 1.44, 12345)
    b, s = gpu_system(w)
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    b.step(30, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC)
    b.lennard_jones_force(s, xnb.PREC_FP64, True)
    ref = b.download(s)
    _, pe_ref = b.energy(s)
    b.lennard_jones_force(s, xnb.PREC_FP64 | xnb.PREC_NEWTON, True)
    g64 = b.download(s)
    _, pe64 = b.energy(s)
    b.lennard_jones_force(s, xnb.PREC_MIXED | xnb.PREC_NEWTON, True)
    gmx = b.download(s)
    e64, _ = force_error(forces(g64), forces(ref))
    emx, _ = force_error(forces(gmx), forces(ref))
    assert e64 <= FP64_TOL, e64
    assert emx <= MIXED_TOL, emx
    assert abs(pe64 - pe_ref) <= 1e-12 * abs(pe_ref)
    # momentum: the pair forces cancel exactly in pairs up to FP64 rounding
    assert np.abs(forces(g64).sum(axis=0)).max() < 1e-9


def test_newton_batched_systems_match_alone_within_tolerance():
    specs = workloads.ensemble_specs(4, seed=78, nmin=4, nmax=8)
    ws = [workloads.lj_fcc_system(sp["n"], sp["rho"], sp["T"], sp["seed"]) for sp in specs]
    prec = xnb.PREC_MIXED | xnb.PREC_NEWTON
    big = new_batch([w["n_atoms"] for w in ws], [ncells(w["geom"]) for w in ws])
    ids = [big.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"]) for w in ws]
    big.init_particles(-1, prec)
    big.step(40, prec, 0)
    big.check_errors()
    for w, s in zip(ws, ids):
        b, so = gpu_system(w)
        b.init_particles(so, prec)
        b.step(40, prec, 0)
        G, A = big.download(s), b.download(so)
        assert np.array_equal(G["id"], A["id"])
        for k in ("rx", "ry", "rz"):
            assert np.max(np.abs(G[k] - A[k])) < 1e-9
        e, _ = force_error(forces(G), forces(A))
        assert e <= MIXED_TOL
