"""A third pair potential through the pair-functor API (include/xnb_pair.cuh):
a Morse functor written against the public headers alone
(tests/functors/morse_pair.cu, built here into its own library) runs over a
resident system's lists through xnb_system_pair_view and matches the oracle's
restatement of the same potential over the reference-format streams: forces
within 1e-12 relative (|dF_i| / max(|F_i|, F_rms)) and energies within 1e-12,
as a buffer-less functor, as a compute-buffer functor (bitwise equal to the
buffer-less one: same pairs, same order) and as a symmetric (Newton, lower
half lists + atomic reactions) functor. The library's own Lennard-Jones and
gravitational functors run through the same traversal (tests/test_gpu_parity.py,
tests/test_gpu_functors.py)."""
import ctypes as C

import numpy as np
import pytest

from exanbody_gb300 import workloads, xnb
from helpers import force_error, forces, ncells, new_batch, oracle_from
from test_pair_api import build_user_functor

pytestmark = pytest.mark.gpu

TOL = 1e-12
MORSE = dict(D=0.5, alpha=1.6, r0=1.12, rcut=2.7)


@pytest.fixture(scope="module")
def morse_lib(tmp_path_factory):
    lib = C.CDLL(build_user_functor(tmp_path_factory.mktemp("morse")))
    lib.morse_force.argtypes = [C.POINTER(xnb.PairView), C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                C.c_void_p]
    lib.morse_force.restype = C.c_int
    return lib


def run_morse(lib, b, s, mode):
    v = b.pair_view(s)
    rc = lib.morse_force(C.byref(v), MORSE["D"], MORSE["alpha"], MORSE["r0"], MORSE["rcut"], mode, b.stream)
    assert rc == 0, rc
    P = b.download(s)
    return forces(P), P["pe"].copy()


@pytest.mark.parametrize("n,steps", [(12, 30), (5, 10)])
def test_user_morse_functor_matches_oracle(morse_lib, n, steps):
    """FCC 12^3 after 30 steps (rebuilds behind it), and a dense 2^3-cell system."""
    w = workloads.lj_fcc_system(n, 0.8442 if n > 5 else 1.0, 1.44, 31 + n)
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    for _ in range(steps):
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC)
        o.step()
    # both sides walk the lists of the last rebuild (equal: the FP64_EXACT path is bit-exact)
    o.morse_force(MORSE["D"], MORSE["alpha"], MORSE["r0"], MORSE["rcut"])
    O = o.particles()
    G = b.download(s)
    assert np.array_equal(G["id"], O["id"])
    ref_f, ref_pe = forces(O), O["pe"]

    f0, pe0 = run_morse(morse_lib, b, s, 0)
    e, _ = force_error(f0, ref_f)
    assert e <= TOL, e
    assert np.max(np.abs(pe0 - ref_pe)) <= TOL * np.max(np.abs(ref_pe))
    assert abs(pe0.sum() - ref_pe.sum()) <= TOL * abs(ref_pe.sum())

    f1, pe1 = run_morse(morse_lib, b, s, 1)
    assert np.array_equal(f1, f0) and np.array_equal(pe1, pe0)

    f2, pe2 = run_morse(morse_lib, b, s, 2)
    e, _ = force_error(f2, ref_f)
    assert e <= TOL, e
    assert abs(pe2.sum() - ref_pe.sum()) <= TOL * abs(ref_pe.sum())
    b.close()


def test_user_functor_rejects_a_cutoff_beyond_the_lists(morse_lib):
    w = workloads.lj_fcc_system(6, 0.8442, 1.44, 2)
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    v = b.pair_view(s)
    assert abs(v.nbh_dist - 2.8) < 1e-12 and v.n_particles == w["n_atoms"]
    assert morse_lib.morse_force(C.byref(v), 0.5, 1.6, 1.12, 2.9, 0, b.stream) == -1
    b.close()
