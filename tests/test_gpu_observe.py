"""On-device observables: simulation_stats reductions and id sampling
(xnb_simulation_stats, xnb_sample_particles) against the downloaded state."""
import numpy as np
import pytest

from exanbody_gb300 import workloads, xnb
from helpers import ncells, new_batch

pytestmark = pytest.mark.gpu


def system(seed=11):
    w = workloads.lj_fcc_system(12, 0.8442, 1.44, seed)
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
    b.init_particles(s, xnb.PREC_MIXED)
    b.step(25, xnb.PREC_MIXED, xnb.STEP_HOST_SYNC | xnb.STEP_ENERGY)
    return w, b, s


def test_simulation_stats_match_host_reduction():
    w, b, s = system()
    st = b.simulation_stats(s)
    P = b.download(s)
    v2 = (P["vx"] * P["vx"] + P["vy"] * P["vy"]) + P["vz"] * P["vz"]
    f2 = (P["fx"] * P["fx"] + P["fy"] * P["fy"]) + P["fz"] * P["fz"]
    assert st["particle_count"] == w["n_atoms"]
    assert abs(st["kinetic_sum"] - v2.sum()) <= 1e-12 * v2.sum()
    assert abs(st["potential_energy"] - P["pe"].sum()) <= 1e-12 * abs(P["pe"]).sum()
    for key, ref in (("min_vel", np.sqrt(v2).min()), ("max_vel", np.sqrt(v2).max()),
                     ("min_acc", np.sqrt(f2).min()), ("max_acc", np.sqrt(f2).max())):
        assert abs(st[key] - ref) <= 1e-14 * max(1.0, abs(ref)), key
    # the reduction order is fixed: the same state gives the same bits
    assert b.simulation_stats(s) == st


def test_sample_particles_by_id():
    w, b, s = system(12)
    P = b.download(s)
    rng = np.random.default_rng(3)
    pick = rng.choice(w["n_atoms"], 200, replace=False)
    ids = np.concatenate([P["id"][pick], np.array([10 ** 12, 10 ** 12 + 7], np.uint64)])
    vals, found = b.sample_particles(s, ids)
    assert found[:200].all() and not found[200:].any()
    want = np.stack([P[k][pick] for k in ("rx", "ry", "rz", "fx", "fy", "fz", "vx", "vy", "vz")], 1)
    assert np.array_equal(vals[:200], want)
    with pytest.raises(xnb.XnbError):
        b.sample_particles(s, np.array([5, 5], np.uint64))
