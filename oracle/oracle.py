"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, bench.py's CPU-baseline leg and __graft_entry__.smoke() import this
module, and only to check or time against it; the product library never calls it.
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

_LIBS = {}


class Params(C.Structure):
    _fields_ = [
        ("origin", C.c_double * 3),
        ("extent", C.c_double * 3),
        ("dims", C.c_int32 * 3),
        ("cell_size", C.c_double),
        ("rcut", C.c_double),
        ("rcut_inc", C.c_double),
        ("epsilon", C.c_double),
        ("sigma", C.c_double),
        ("dt", C.c_double),
        ("mass", C.c_double),
        ("divide_by_mass", C.c_int32),
        ("amr_enabled", C.c_int32),
        ("sub_grid_density", C.c_double),
    ]


def _lib(kind="parity"):
    if kind in _LIBS:
        return _LIBS[kind]
    out = build_oracle.build()
    lib = C.CDLL(os.path.join(out, "liboracle_%s.so" % kind))
    P = C.POINTER
    d, i64, u64, i32, u16 = C.c_double, C.c_int64, C.c_uint64, C.c_int32, C.c_uint16
    lib.xo_create.restype = C.c_void_p
    lib.xo_create.argtypes = [P(Params)]
    lib.xo_destroy.argtypes = [C.c_void_p]
    lib.xo_set_threads.argtypes = [C.c_int]
    lib.xo_load_flat.argtypes = [C.c_void_p, i64] + [P(d)] * 6 + [P(u64)]
    lib.xo_load_cells.argtypes = [C.c_void_p, P(i64)] + [P(d)] * 6 + [P(u64)]
    lib.xo_load_lattice_noise_fcc.argtypes = [C.c_void_p, d, d]
    lib.xo_load_lattice_noise.argtypes = [C.c_void_p, i32, d, d]
    lib.xo_set_snap.argtypes = [C.c_void_p, i32, d, d, d, i32, i32, i32, P(d), P(d), i32, P(d), d, i32]
    lib.xo_init.argtypes = [C.c_void_p]
    lib.xo_step.argtypes = [C.c_void_p]
    lib.xo_compute_forces.argtypes = [C.c_void_p]
    lib.xo_chunk_neighbors.argtypes = [C.c_void_p]
    for f in ("xo_num_particles", "xo_rebuild_count", "xo_num_cells", "xo_pair_count", "xo_displ_over_count"):
        getattr(lib, f).restype = i64
        getattr(lib, f).argtypes = [C.c_void_p]
    lib.xo_get_particles.argtypes = [C.c_void_p] + [P(d)] * 9 + [P(u64), P(i32), P(d)]
    lib.xo_set_types.argtypes = [C.c_void_p, P(u64), P(C.c_uint8), i64]
    lib.xo_gravitational_force.argtypes = [C.c_void_p, d, P(d), C.c_int32, d]
    lib.xo_morse_force.argtypes = [C.c_void_p, d, d, d, d]
    lib.xo_get_cell_counts.argtypes = [C.c_void_p, P(i64)]
    lib.xo_get_pairs.argtypes = [C.c_void_p, P(u64), P(u64), P(i32)]
    lib.xo_pair_count_cells.restype = i64
    lib.xo_pair_count_cells.argtypes = [C.c_void_p, i64, i64]
    lib.xo_get_pairs_cells.argtypes = [C.c_void_p, i64, i64, P(u64), P(i32)]
    lib.xo_cell_stream_size.restype = i64
    lib.xo_cell_stream_size.argtypes = [C.c_void_p, i64]
    lib.xo_get_cell_stream.argtypes = [C.c_void_p, i64, P(u16)]
    lib.xo_energy.argtypes = [C.c_void_p, P(d), P(d)]
    _LIBS[kind] = lib
    return lib


def _ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class OracleSystem:
    """One periodic LJ system advanced by the CPU restatement of the reference."""

    def __init__(self, origin, extent, dims, cell_size, rcut, rcut_inc, epsilon, sigma, dt,
                 mass=1.0, divide_by_mass=False, amr=True, sub_grid_density=6.5, kind="parity"):
        self.lib = _lib(kind)
        p = Params()
        for a in range(3):
            p.origin[a] = origin[a]
            p.extent[a] = extent[a]
            p.dims[a] = int(dims[a])
        p.cell_size = cell_size
        p.rcut, p.rcut_inc = rcut, rcut_inc
        p.epsilon, p.sigma, p.dt = epsilon, sigma, dt
        p.mass, p.divide_by_mass = mass, int(bool(divide_by_mass))
        p.amr_enabled, p.sub_grid_density = int(bool(amr)), sub_grid_density
        self.params = p
        self.h = self.lib.xo_create(C.byref(p))
        if not self.h:
            raise ValueError("oracle rejected the domain (needs one ghost layer and >=2 cells per axis)")
        self.dims = tuple(int(x) for x in dims)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.xo_destroy(h)
            self.h = None

    def set_threads(self, n):
        return self.lib.xo_set_threads(int(n))

    def load_flat(self, r, v, ids):
        r = np.ascontiguousarray(r, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        ids = np.ascontiguousarray(ids, dtype=np.uint64)
        cols = [np.ascontiguousarray(r[:, a]) for a in range(3)] + [np.ascontiguousarray(v[:, a]) for a in range(3)]
        rc = self.lib.xo_load_flat(self.h, len(ids), *[_ptr(c, C.c_double) for c in cols], _ptr(ids, C.c_uint64))
        assert rc == 0

    def load_lattice_noise_fcc(self, a, sigma):
        assert self.lib.xo_load_lattice_noise_fcc(self.h, a, sigma) == 0

    def load_lattice_noise(self, structure, a, sigma):
        """structure: "SC", "BCC" or "FCC" (the reference's lattice generator basis)."""
        code = {"SC": 0, "BCC": 1, "FCC": 2}[structure]
        assert self.lib.xo_load_lattice_noise(self.h, code, a, sigma) == 0

    def set_snap(self, cfg, energy_unit, with_energy=False):
        """Force chain = snap_force_generic with a read_lammps() configuration."""
        els = cfg["elements"]
        rad = np.ascontiguousarray([e["radelem"] for e in els], np.float64)
        wj = np.ascontiguousarray([e["weight"] for e in els], np.float64)
        coeff = np.ascontiguousarray([c for e in els for c in e["coeffs"]], np.float64)
        rc = self.lib.xo_set_snap(self.h, int(cfg["twojmax"]), float(cfg["rcutfac"]), float(cfg["rfac0"]),
                                  float(cfg["rmin0"]), int(cfg["switchflag"]), int(cfg["bzeroflag"]), len(els),
                                  _ptr(rad, C.c_double), _ptr(wj, C.c_double), int(cfg["ncoeffall"]),
                                  _ptr(coeff, C.c_double), float(energy_unit), int(bool(with_energy)))
        if rc != 0:
            raise RuntimeError("oracle set_snap failed: %d" % rc)

    def init(self):
        rc = self.lib.xo_init(self.h)
        if rc != 0:
            raise RuntimeError("oracle init failed: %d" % rc)

    def step(self):
        rc = self.lib.xo_step(self.h)
        if rc < 0:
            raise RuntimeError("oracle step failed: %d" % rc)
        return rc

    def compute_forces(self):
        """The force pass alone on the current state (CPU-baseline timing)."""
        if self.lib.xo_compute_forces(self.h) != 0:
            raise RuntimeError("oracle force pass failed")

    def chunk_neighbors(self):
        """The neighbour build alone on the current state (CPU-baseline timing)."""
        if self.lib.xo_chunk_neighbors(self.h) != 0:
            raise RuntimeError("oracle neighbour build failed")

    @property
    def n(self):
        return int(self.lib.xo_num_particles(self.h))

    @property
    def rebuilds(self):
        return int(self.lib.xo_rebuild_count(self.h))

    def displ_over_count(self):
        return int(self.lib.xo_displ_over_count(self.h))

    def particles(self):
        n = self.n
        arrs = {k: np.empty(n, np.float64) for k in ("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz", "pe")}
        ids = np.empty(n, np.uint64)
        cell = np.empty(n, np.int32)
        self.lib.xo_get_particles(self.h, *[_ptr(arrs[k], C.c_double) for k in ("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz")],
                                  _ptr(ids, C.c_uint64), _ptr(cell, C.c_int32), _ptr(arrs["pe"], C.c_double))
        arrs["id"] = ids
        arrs["cell"] = cell
        return arrs

    def cell_counts(self):
        nc = int(self.lib.xo_num_cells(self.h))
        out = np.empty(nc, np.int64)
        self.lib.xo_get_cell_counts(self.h, _ptr(out, C.c_int64))
        return out

    def pairs(self):
        m = int(self.lib.xo_pair_count(self.h))
        a = np.empty(m, np.uint64)
        b = np.empty(m, np.uint64)
        cnt = np.empty(self.n, np.int32)
        self.lib.xo_get_pairs(self.h, _ptr(a, C.c_uint64), _ptr(b, C.c_uint64), _ptr(cnt, C.c_int32))
        return a, b, cnt

    def pairs_of_cells(self, ci0, ci1, n_particles):
        """Partner ids (list order) and per-particle lengths of the n_particles
        particles of interior cells [ci0, ci1)."""
        m = int(self.lib.xo_pair_count_cells(self.h, int(ci0), int(ci1)))
        b = np.empty(m, np.uint64)
        cnt = np.empty(int(n_particles), np.int32)
        self.lib.xo_get_pairs_cells(self.h, int(ci0), int(ci1), _ptr(b, C.c_uint64), _ptr(cnt, C.c_int32))
        return b, cnt

    def cell_stream(self, interior_cell):
        m = int(self.lib.xo_cell_stream_size(self.h, interior_cell))
        out = np.empty(m, np.uint16)
        if m:
            self.lib.xo_get_cell_stream(self.h, interior_cell, _ptr(out, C.c_uint16))
        return out

    def set_types(self, ids, types):
        ids = np.ascontiguousarray(ids, np.uint64)
        types = np.ascontiguousarray(types, np.uint8)
        rc = self.lib.xo_set_types(self.h, _ptr(ids, C.c_uint64), _ptr(types, C.c_uint8), len(ids))
        if rc != 0:
            raise RuntimeError("oracle set_types matched nothing")

    def gravitational_force(self, G, masses, rcut):
        masses = np.ascontiguousarray(masses, np.float64)
        rc = self.lib.xo_gravitational_force(self.h, float(G), _ptr(masses, C.c_double), len(masses), float(rcut))
        if rc != 0:
            raise RuntimeError("oracle gravitational_force failed: %d" % rc)

    def morse_force(self, D, alpha, r0, rcut):
        rc = self.lib.xo_morse_force(self.h, float(D), float(alpha), float(r0), float(rcut))
        if rc != 0:
            raise RuntimeError("oracle morse_force failed: %d" % rc)

    def energy(self):
        ke, pe = C.c_double(), C.c_double()
        self.lib.xo_energy(self.h, C.byref(ke), C.byref(pe))
        return ke.value, pe.value
