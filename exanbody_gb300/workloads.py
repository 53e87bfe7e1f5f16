"""Seeded synthetic LJ workloads (reduced units, eps = sigma = m = 1).

The benchmark systems are FCC lattices at a reduced density with
Maxwell-Boltzmann velocities. The reference has no density-driven FCC builder
and no velocity initialiser, so both are defined here:
  * lattice constant a = (4/rho)^(1/3), FCC basis of grid_cell_particles/include/
    exanb/grid_cell_particles/lattice_generator.h:162-170, sites in (k, j, i, basis)
    order, ids 0..N-1 in that order;
  * domain: L = n*a per axis, D = floor(L / (rcut + skin)) cells of size L/D,
    origin 0, extent D*cell (one ghost layer, as nbh_dist.cpp gives for this skin);
  * velocities: numpy PCG64(seed) standard normals per component in id order,
    mean removed, rescaled to T with 3N-3 degrees of freedom.
"""
import math

import numpy as np

FCC_BASIS = np.array([[0.0, 0.0, 0.0], [0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0]])


def geometry(lengths, rcut=2.5, skin=0.3, cell_factor=1.0):
    """Periodic box of the given lengths cut into cubic cells of at least
    cell_factor * (rcut + skin) (cell_factor >= 1: denser cells, AMR sub-grids)."""
    nbh = (rcut + skin) * cell_factor
    lengths = [float(x) for x in lengths]
    dmin = [int(math.floor(L / nbh)) for L in lengths]
    # one cubic cell size for all axes: the smallest L/D over axes
    cs = max(L / d for L, d in zip(lengths, dmin))
    dims = [max(2, int(round(L / cs))) for L in lengths]
    extent = [d * cs for d in dims]
    return {"origin": (0.0, 0.0, 0.0), "extent": tuple(extent), "dims": tuple(dims), "cell_size": cs}


def fcc_lattice(n, rho, nz=None):
    """Sites of an n x n x nz FCC block, (k, j, i, basis) order."""
    nz = n if nz is None else nz
    a = (4.0 / rho) ** (1.0 / 3.0)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(n), np.arange(n), indexing="ij")
    cells = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float64)
    r = (cells[:, None, :] + FCC_BASIS[None, :, :]).reshape(-1, 3) * a
    return r, a


def maxwell_boltzmann(nparticles, temperature, seed, mass=1.0):
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((nparticles, 3))
    v -= v.mean(axis=0)
    ke = 0.5 * mass * float((v * v).sum())
    t_now = 2.0 * ke / (3.0 * nparticles - 3.0)
    v *= math.sqrt(temperature / t_now)
    return v


def lj_fcc_system(n, rho=0.8442, temperature=1.44, seed=12345, rcut=2.5, skin=0.3, cell_factor=1.0):
    """Periodic FCC n^3 system: positions, velocities, ids, geometry."""
    r, a = fcc_lattice(n, rho)
    L = n * a
    geom = geometry((L, L, L), rcut, skin, cell_factor)
    v = maxwell_boltzmann(len(r), temperature, seed)
    ids = np.arange(len(r), dtype=np.uint64)
    return {"r": r, "v": v, "id": ids, "geom": geom, "a": a, "n_atoms": len(r), "rho": rho, "T": temperature}


def lj_slab_system(n, rho=0.8442, temperature=0.8, seed=12345, rcut=2.5, skin=0.3, cell_factor=1.0):
    """Liquid-vacuum slab: FCC n^3 filling the middle half of a (L, L, 2L) box."""
    r, a = fcc_lattice(n, rho)
    L = n * a
    geom = geometry((L, L, 2.0 * L), rcut, skin, cell_factor)
    r = r.copy()
    r[:, 2] += 0.5 * geom["extent"][2] * 0.5
    v = maxwell_boltzmann(len(r), temperature, seed)
    ids = np.arange(len(r), dtype=np.uint64)
    return {"r": r, "v": v, "id": ids, "geom": geom, "a": a, "n_atoms": len(r), "rho": rho, "T": temperature}


def ensemble_specs(count=1024, seed=2024, nmin=4, nmax=25, rho=(0.70, 1.00), temp=(0.7, 1.5)):
    """Per-system (n, rho, T, seed) of the batched ensemble workload."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(nmin, nmax + 1, size=count)
    rhos = rng.uniform(rho[0], rho[1], size=count)
    temps = rng.uniform(temp[0], temp[1], size=count)
    seeds = rng.integers(0, 2**31 - 1, size=count)
    return [dict(n=int(a), rho=float(b), T=float(c), seed=int(d)) for a, b, c, d in zip(ns, rhos, temps, seeds)]


def serving_stream(count=10000, seed=4242, nmin=5, nmax=40, steps=(200, 2000), rate=1.0):
    """Seeded Poisson arrivals of LJ MD requests (arrival time in seconds)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=count)
    t = np.cumsum(gaps)
    ns = rng.integers(nmin, nmax + 1, size=count)
    rhos = rng.uniform(0.70, 1.00, size=count)
    temps = rng.uniform(0.7, 1.5, size=count)
    nsteps = rng.integers(steps[0], steps[1] + 1, size=count)
    seeds = rng.integers(0, 2**31 - 1, size=count)
    return [dict(arrival=float(a), n=int(b), rho=float(c), T=float(d), steps=int(e), seed=int(f))
            for a, b, c, d, e, f in zip(t, ns, rhos, temps, nsteps, seeds)]
