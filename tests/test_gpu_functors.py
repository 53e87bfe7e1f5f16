"""A second pair functor through the same neighbour lists: gravitational_force
(contribs/pi/gravitational_force.cu) with per-type masses, against the oracle's
restatement over its own chunk streams. FP64_EXACT is bit-identical, including
after rebins (types follow their particles); FP64 within 1e-12."""
import numpy as np
import pytest

from exanbody_gb300 import workloads, xnb
from helpers import assert_bitwise_equal, force_error, forces, ncells, new_batch, oracle_from

pytestmark = pytest.mark.gpu

G = 0.8
MASSES = [1.0, 2.5, 0.7]


def setup(n=20, seed=12345):
    w = workloads.lj_fcc_system(n, 0.8442, 1.44, seed)
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    types = (w["id"] % 3).astype(np.uint8)
    assert b.set_types(s, w["id"], types) == w["n_atoms"]
    o.set_types(w["id"], types)
    return w, b, s, o


def test_gravity_bit_exact_at_init_and_after_rebins():
    w, b, s, o = setup()
    for rcut in (2.5, 2.0):
        b.gravitational_force(s, G, MASSES, rcut, xnb.PREC_FP64_EXACT, energy=True)
        o.gravitational_force(G, MASSES, rcut)
        assert_bitwise_equal(b.download(s), o.particles(), fields=("fx", "fy", "fz", "pe"))
    rebuilds = 0
    for _ in range(30):
        r0 = b.info(s).rebuilds
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC)
        o.step()
        rebuilds += b.info(s).rebuilds != r0
    assert rebuilds >= 2
    b.gravitational_force(s, G, MASSES, 2.5, xnb.PREC_FP64_EXACT, energy=True)
    o.gravitational_force(G, MASSES, 2.5)
    assert_bitwise_equal(b.download(s), o.particles(), fields=("fx", "fy", "fz", "pe"))


def test_gravity_fp64_and_accumulate():
    w, b, s, o = setup(12, 5)
    b.gravitational_force(s, G, MASSES, 2.5, xnb.PREC_FP64_EXACT)
    exact = forces(b.download(s))
    b.gravitational_force(s, G, MASSES, 2.5, xnb.PREC_FP64)
    emax, _ = force_error(forces(b.download(s)), exact)
    assert emax <= 1e-12, emax
    # LJ then gravity added onto it: the sum of the two force fields
    b.lennard_jones_force(s, xnb.PREC_FP64_EXACT, False)
    lj = forces(b.download(s))
    b.gravitational_force(s, G, MASSES, 2.5, xnb.PREC_FP64_EXACT, accumulate=True)
    emax, _ = force_error(forces(b.download(s)), lj + exact)
    assert emax <= 1e-12, emax


def test_gravity_needs_a_mass_per_type():
    w, b, s, o = setup(8, 3)
    with pytest.raises(xnb.XnbError):
        b.gravitational_force(s, G, MASSES[:2], 2.5, xnb.PREC_FP64_EXACT)
    with pytest.raises(xnb.XnbError):
        b.gravitational_force(s, G, MASSES, 3.5, xnb.PREC_FP64_EXACT)  # beyond the lists' reach
