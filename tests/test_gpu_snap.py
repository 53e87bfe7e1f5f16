"""snap_force_generic on the GPU (xnb_snap_create / xnb_snap_force) against the
oracle's SNAP restatement, and the reference's SNAP golden decks through the
operator runner."""
import os
import subprocess

import numpy as np
import pytest

from exanbody_gb300 import build, snap, workloads, xnb
from helpers import ncells, new_batch
from oracle.oracle import OracleSystem
from test_snap_oracle import potential

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def block(el, n, a, seed, sigma=0.1):
    basis = workloads.FCC_BASIS if el == "Ni" else np.array([[0, 0, 0], [0.5, 0.5, 0.5]])
    cells = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"), -1).reshape(-1, 3)
    L = n * a
    r = ((cells[:, None, :] + basis[None]).reshape(-1, 3) * a)
    r = (r + np.random.default_rng(seed).normal(0, sigma, r.shape)) % L
    return r, L


@pytest.mark.parametrize("el,n,a,dims", [("Ni", 6, 3.52, 3), ("Mo", 7, 3.15, 4)])
def test_forces_and_energies_match_the_oracle(el, n, a, dims):
    cfg = potential(el)
    r, L = block(el, n, a, 5)
    rng = np.random.default_rng(1)
    v = rng.normal(0, 1, r.shape)
    ids = np.arange(1, len(r) + 1, dtype=np.uint64)
    rc, skin = cfg["rcutfac"], 0.5
    geom = {"origin": (0.0, 0.0, 0.0), "extent": (L, L, L), "dims": (dims,) * 3, "cell_size": L / dims}
    o = OracleSystem((0, 0, 0), (L, L, L), (dims,) * 3, L / dims, rc, skin, 1.0, 1.0, 1e-3, kind="omp")
    o.set_snap(cfg, snap.energy_unit(), with_energy=True)
    o.load_flat(r, v, ids)
    o.init()
    P = o.particles()
    b = new_batch([len(r)], [ncells(geom)])
    s = b.add_system(xnb.lj_params(geom, rcut=rc, rcut_inc=skin), r, v, ids)
    b.init_particles(s, xnb.PREC_FP64)
    pot = snap.Potential(cfg)
    pot.force(b, s, energy=True)
    D = b.download(s)
    o1, o2 = np.argsort(P["id"]), np.argsort(D["id"])
    F1 = np.stack([P[k][o1] for k in ("fx", "fy", "fz")], 1)
    F2 = np.stack([D[k][o2] for k in ("fx", "fy", "fz")], 1)
    assert np.max(np.abs(F1 - F2)) <= 1e-10 * np.max(np.abs(F1))
    assert np.allclose(P["pe"][o1], D["pe"][o2], rtol=1e-12, atol=1e-9 * np.max(np.abs(P["pe"])))
    # accumulate adds onto the current forces
    pot.force(b, s, accumulate=True)
    F3 = np.stack([b.download(s)[k][o2] for k in ("fx", "fy", "fz")], 1)
    assert np.max(np.abs(F3 - 2 * F2)) <= 1e-10 * np.max(np.abs(F2))


def test_errors_are_reported():
    cfg = potential("Ni")
    r, L = block("Ni", 6, 3.52, 2)
    ids = np.arange(1, len(r) + 1, dtype=np.uint64)
    geom = {"origin": (0.0, 0.0, 0.0), "extent": (L, L, L), "dims": (3, 3, 3), "cell_size": L / 3}
    b = new_batch([len(r)], [ncells(geom)])
    s = b.add_system(xnb.lj_params(geom, rcut=3.0, rcut_inc=0.5), r, np.zeros_like(r), ids)
    b.init_particles(s, xnb.PREC_FP64)
    pot = snap.Potential(cfg)
    with pytest.raises(xnb.XnbError):  # SNAP cutoff 4.1 above the lists' 3.5
        pot.force(b, s)
    b2 = new_batch([len(r)], [ncells(geom)])
    s2 = b2.add_system(xnb.lj_params(geom, rcut=4.1, rcut_inc=0.5), r, np.zeros_like(r), ids)
    b2.init_particles(s2, xnb.PREC_FP64)
    b2.set_types(s2, ids[:5], np.full(5, 3, np.uint8))
    with pytest.raises(xnb.XnbError):  # type 3 has no coefficients
        pot.force(b2, s2)


@pytest.mark.parametrize("el", ["Ni", "Mo"])
def test_golden_decks_through_the_operator_runner(tmp_path, el):
    """The reference's SNAP decks (100 NVE steps, snap_force_generic, divide by
    mass) reproduce their golden check_values."""
    exe = build.build_host()
    deck = os.path.join(HERE, "decks", "snap_%s_golden.msp" % el)
    r = subprocess.run([exe, deck], capture_output=True, text=True, timeout=600, cwd=tmp_path)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr
    vals = {}
    for line in r.stdout.splitlines():
        if line.startswith("** "):
            vals[line.split()[1]] = float(line.split("=")[1].split("/")[0])
    assert vals["Position"] < 1e-9 and vals["Acceleration"] < 1e-6 and vals["Velocity"] < 1e-8, vals
