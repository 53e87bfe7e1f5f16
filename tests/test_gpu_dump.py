"""write_dump / read_dump through resident systems (xnb_system_write_dump,
exanbody_gb300.dump.restore_system).

A dump written right after a neighbour-list rebuild holds every particle in its
cell in storage order; read back, placement puts the particles into the same
cells in the same order (read_dump appends in file order), so the restored
system computes the same forces and continues the trajectory bit for bit in
FP64_EXACT and in the mixed path. Types travel with their particles."""
import numpy as np
import pytest

from exanbody_gb300 import dump, workloads, xnb
from helpers import ncells, new_batch

pytestmark = pytest.mark.gpu

KEYS = ("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz", "id", "cell")


def same_state(a, b):
    return all(np.array_equal(a[k], b[k]) for k in KEYS)


@pytest.mark.parametrize("prec", [xnb.PREC_FP64_EXACT, xnb.PREC_MIXED])
def test_restart_at_a_rebuild_continues_bit_for_bit(tmp_path, prec):
    w = workloads.lj_fcc_system(12, 0.8442, 1.44, 77)  # 6912 atoms
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
    types = (w["id"] % 3).astype(np.uint8)
    assert b.set_types(s, w["id"], types) == w["n_atoms"]
    b.init_particles(s, prec)
    r0 = b.info(s).rebuilds
    steps = 0
    while b.info(s).rebuilds == r0:
        b.step(1, prec, xnb.STEP_HOST_SYNC)
        steps += 1
        assert steps < 200
    path = tmp_path / "restart.dump"
    dump.write_system(b, s, path, timestep=steps, physical_time=steps * 0.005)
    info = dump.read_info(path)
    assert info["n_particles"] == w["n_atoms"] and info["timestep"] == steps
    assert info["domain"]["dims"] == tuple(w["geom"]["dims"])

    b2 = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s2, _ = dump.restore_system(b2, path)
    b2.init_particles(s2, prec)
    assert same_state(b.download(s), b2.download(s2))
    assert np.array_equal(dump.system_types(b, s), dump.system_types(b2, s2))
    base1, base2 = b.info(s).rebuilds, b2.info(s2).rebuilds
    for _ in range(3):
        b.step(10, prec, xnb.STEP_HOST_SYNC)
        b2.step(10, prec, xnb.STEP_HOST_SYNC)
        assert same_state(b.download(s), b2.download(s2))
    assert b.info(s).rebuilds - base1 == b2.info(s2).rebuilds - base2 > 0


def test_dump_of_a_moving_system_reads_back_exactly(tmp_path):
    """Between rebuilds particles may sit outside their cells; the file keeps
    storage order and the exact coordinates, and a restore wraps and re-bins
    them as read_dump does."""
    w = workloads.lj_fcc_system(10, 0.8442, 1.44, 5)
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
    b.init_particles(s, xnb.PREC_MIXED)
    b.step(37, xnb.PREC_MIXED, xnb.STEP_HOST_SYNC)
    st = b.download(s)
    path = tmp_path / "m.dump"
    dump.write_system(b, s, path, compression_level=1, max_part_size=100000)
    d = dump.read(path)
    assert np.array_equal(d["r"][:, 0], st["rx"]) and np.array_equal(d["v"][:, 2], st["vz"])
    assert np.array_equal(d["id"], st["id"])
    b2 = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s2, _ = dump.restore_system(b2, path)
    b2.init_particles(s2, xnb.PREC_MIXED)
    st2 = b2.download(s2)
    order = np.argsort(st["id"])
    order2 = np.argsort(st2["id"])
    L = np.array(w["geom"]["extent"]) - np.array(w["geom"]["origin"])
    for a, k in enumerate(("rx", "ry", "rz")):
        d_ = st2[k][order2] - st[k][order]
        assert np.all(np.abs(d_ - L[a] * np.round(d_ / L[a])) <= 1e-12 * L[a])
    # forces agree to rounding (the pair order may differ where particles changed cells)
    f1 = np.stack([st[k][order] for k in ("fx", "fy", "fz")], 1)
    f2 = np.stack([st2[k][order2] for k in ("fx", "fy", "fz")], 1)
    assert np.max(np.abs(f1 - f2)) <= 1e-9 * np.max(np.abs(f1))
