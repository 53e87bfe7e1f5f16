"""SNAP potentials: LAMMPS parameter/coefficient files and the GPU force operator.

read_lammps follows the reference's reader (contribs/md/snap/lib/snap_read_lammps.cpp:
30-132): `key value` lines of the .snapparam file (lines starting with '#'
skipped) over the defaults of SnapConfig (snap_config.h:62-77: rfac0 0.99363,
rmin0 0, twojmax 6, bzeroflag on, switchflag on, the other flags off); in the
.snapcoeff file, leading comment or empty lines, then `n_materials
coefs_per_material`, then per material a `name radelem weight` line and one
coefficient per line (constant term first). Coefficients stay in the file's
energy unit (eV); forces and energies are converted by `energy_unit`.
"""
import ctypes as C
import os

import numpy as np

from . import units, xnb

DEFAULTS = {"rfac0": 0.99363, "rmin0": 0.0, "rcutfac": 0.0, "twojmax": 6, "nelements": 1, "bzeroflag": 1,
            "switchflag": 1, "chemflag": 0, "bnormflag": 0, "wselfallflag": 0, "switchinnerflag": 0,
            "quadraticflag": 0}


def read_lammps(param_path, coef_path):
    cfg = dict(DEFAULTS)
    with open(param_path) as f:
        for line in f:
            if not line.strip() or line.startswith("#"):
                continue
            toks = line.split()
            if toks[0] in cfg and len(toks) > 1:
                cfg[toks[0]] = float(toks[1])
    for k in ("twojmax", "nelements", "bzeroflag", "switchflag", "chemflag", "bnormflag", "wselfallflag",
              "switchinnerflag", "quadraticflag"):
        cfg[k] = int(cfg[k])
    with open(coef_path) as f:
        lines = f.read().split("\n")
    k = 0
    while k < len(lines) and (not lines[k].strip() or lines[k].startswith("#")):
        k += 1
    nmat, ncoeff = (int(x) for x in lines[k].split()[:2])
    k += 1
    elements = []
    for _ in range(nmat):
        name, rad, w = lines[k].split()[:3]
        k += 1
        coeffs = [float(lines[k + c].split()[0]) for c in range(ncoeff)]
        k += ncoeff
        elements.append({"name": name, "radelem": float(rad), "weight": float(w), "coeffs": coeffs})
    cfg["elements"] = elements
    cfg["ncoeffall"] = ncoeff
    return cfg


def energy_unit():
    """1 eV in the internal energy unit (Da angstrom^2 / ps^2)."""
    return units.ev_to_internal(1.0)


class Potential:
    """A SNAP potential resident on one GPU (xnb_snap_create), applied to the
    systems of a batch with force(); cfg is a read_lammps() configuration."""

    def __init__(self, cfg, device=0, unit=None):
        self.lib = xnb.load()
        els = cfg["elements"]
        if len(els) > 16:
            raise ValueError("at most 16 element types")
        p = xnb.SnapParams()
        p.twojmax = int(cfg["twojmax"])
        p.rcutfac, p.rfac0, p.rmin0 = float(cfg["rcutfac"]), float(cfg["rfac0"]), float(cfg["rmin0"])
        p.switchflag, p.bzeroflag = int(cfg["switchflag"]), int(cfg["bzeroflag"])
        p.chemflag, p.bnormflag = int(cfg["chemflag"]), int(cfg["bnormflag"])
        p.quadraticflag, p.switchinnerflag = int(cfg["quadraticflag"]), int(cfg["switchinnerflag"])
        p.ntypes = len(els)
        for k, e in enumerate(els):
            p.radelem[k] = e["radelem"]
            p.wj[k] = e["weight"]
        p.ncoeffall = int(cfg["ncoeffall"])
        self._coeff = np.ascontiguousarray([c for e in els for c in e["coeffs"]], np.float64)
        p.coeff = self._coeff.ctypes.data_as(C.POINTER(C.c_double))
        p.energy_unit = energy_unit() if unit is None else float(unit)
        h = C.c_void_p()
        xnb._ck(self.lib.xnb_snap_create(C.byref(p), int(device), C.byref(h)))
        self.h = h
        self.cfg = cfg

    def close(self):
        if getattr(self, "h", None):
            self.lib.xnb_snap_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def force(self, batch, s=-1, energy=False, accumulate=False, mixed=False):
        """mixed: FP32 arithmetic for U, Z, Y and the adjoint; FP64 geometry and sums."""
        flags = ((xnb.FORCE_ENERGY if energy else 0) | (xnb.FORCE_ACCUMULATE if accumulate else 0)
                 | (xnb.FORCE_MIXED if mixed else 0))
        xnb._ck(self.lib.xnb_snap_force(batch.h, int(s), self.h, flags, batch.stream))

    @property
    def cutoff(self):
        return 2.0 * max(e["radelem"] for e in self.cfg["elements"]) * float(self.cfg["rcutfac"])


def md_steps(batch, s, pot, nsteps, energy=False, mixed=False):
    """Velocity-Verlet steps of system s with snap_force_generic as the force
    chain (numerical-scheme.msp:13-25 with update-particles.msp): push_f_v_r,
    push_f_v, particle_displ_over and, when triggered, move_particles +
    chunk_neighbors, then the SNAP forces and push_f_v."""
    for _ in range(nsteps):
        batch.push_f_v_r(1.0, s)
        batch.push_f_v(0.5, s)
        if batch.particle_displ_over(s) > 0:
            batch.update_particles_full(s)
        pot.force(batch, s, energy=energy, mixed=mixed)
        batch.push_f_v(0.5, s)


def lattice(structure, n, a, sigma, seed):
    """Sites of an n^3 block of unit cells (SC, BCC or FCC basis of the
    reference's lattice generator, lattice_generator.h:140-170) with Gaussian
    noise of sigma (seeded), wrapped into the [0, n a) box."""
    basis = {"SC": np.array([[0.5, 0.5, 0.5]]), "BCC": np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.5]]),
             "FCC": np.array([[0.0, 0.0, 0.0], [0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0]])}[structure]
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    cells = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float64)
    r = (cells[:, None, :] + basis[None]).reshape(-1, 3) * a
    r += np.random.default_rng(seed).normal(0.0, sigma, r.shape)
    return r % (n * a)
