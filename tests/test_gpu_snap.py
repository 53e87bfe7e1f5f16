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


@pytest.mark.parametrize("el,n,a,dims", [("Ni", 8, 3.52, 4), ("Mo", 8, 3.15, 4)])
def test_mixed_forces_within_1e5_of_fp64(el, n, a, dims):
    """XNB_FORCE_MIXED (FP32 U, Z, Y, adjoint; FP64 geometry and sums): force
    error |dF_i| / max(|F_i|, F_rms) <= 1e-5 (measured ~1e-6), energies to 1e-5."""
    cfg = potential(el)
    r, L = block(el, n, a, 9, sigma=0.15)
    ids = np.arange(1, len(r) + 1, dtype=np.uint64)
    geom = {"origin": (0.0, 0.0, 0.0), "extent": (L, L, L), "dims": (dims,) * 3, "cell_size": L / dims}
    b = new_batch([len(r)], [ncells(geom)])
    s = b.add_system(xnb.lj_params(geom, rcut=cfg["rcutfac"], rcut_inc=1.0), r, np.zeros_like(r), ids)
    b.init_particles(s, xnb.PREC_FP64)
    pot = snap.Potential(cfg)
    pot.force(b, s, energy=True)
    P64 = b.download(s)
    pot.force(b, s, energy=True, mixed=True)
    P32 = b.download(s)
    F64 = np.stack([P64[k] for k in ("fx", "fy", "fz")], 1)
    F32 = np.stack([P32[k] for k in ("fx", "fy", "fz")], 1)
    mag = np.linalg.norm(F64, axis=1)
    frms = np.sqrt((mag ** 2).mean())
    rel = np.linalg.norm(F32 - F64, axis=1) / np.maximum(mag, frms)
    assert rel.max() <= 1e-5, rel.max()
    assert np.max(np.abs(P32["pe"] - P64["pe"])) <= 1e-5 * np.max(np.abs(P64["pe"]))


def test_mixed_nve_drift_matches_fp64():
    """200 NVE steps of the Mo deck's system from a thermal start: the total
    energy of the mixed path drifts no more than the FP64 path's (plus 1e-7)."""
    from exanbody_gb300 import units

    cfg = potential("Mo")
    r = snap.lattice("BCC", 10, 3.15, 0.05, 3)
    L = 31.5
    geom = {"origin": (0.0, 0.0, 0.0), "extent": (L, L, L), "dims": (4, 4, 4), "cell_size": L / 4}
    mass = 95.96
    # 300 K Maxwell-Boltzmann velocities (k_B in Da A^2 / ps^2 / K)
    kb = units.ev_to_internal(8.617333262e-5)
    v = np.random.default_rng(4).normal(0.0, np.sqrt(kb * 300.0 / mass), r.shape)
    v -= v.mean(axis=0)
    ids = np.arange(1, len(r) + 1, dtype=np.uint64)
    drift = {}
    for mixed in (False, True):
        b = new_batch([len(r)], [ncells(geom)])
        s = b.add_system(xnb.lj_params(geom, rcut=cfg["rcutfac"], rcut_inc=1.0, dt=1e-3, mass=mass,
                                       divide_by_mass=True), r, v, ids)
        b.init_particles(s, xnb.PREC_FP64)
        pot = snap.Potential(cfg)
        pot.force(b, s, energy=True, mixed=mixed)
        e = []
        for _ in range(20):
            snap.md_steps(b, s, pot, 10, energy=True, mixed=mixed)
            P = b.download(s)
            ke = 0.5 * mass * float((P["vx"] ** 2 + P["vy"] ** 2 + P["vz"] ** 2).sum())
            e.append(ke + float(P["pe"].sum()))
        e = np.array(e)
        drift[mixed] = float(np.max(np.abs(e - e[0])) / abs(e[0]))
    assert drift[True] <= 2.0 * drift[False] + 1e-7, drift
