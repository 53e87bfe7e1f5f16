"""ctypes binding of libxnb_gpu.so (include/xnb_gpu.h).

This is the Python face of the C ABI: no computation happens here. Every call
goes to the sm_103a library; if the library or a GPU is missing the calls fail
loudly (there is no CPU fallback).
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

PREC_FP64_EXACT = 0
PREC_FP64 = 1
PREC_MIXED = 2
PREC_NEWTON = 0x10
PRECISIONS = {"fp64_exact": PREC_FP64_EXACT, "fp64": PREC_FP64, "mixed": PREC_MIXED,
              "fp64_newton": PREC_FP64 | PREC_NEWTON, "mixed_newton": PREC_MIXED | PREC_NEWTON}

BUILD_ROWS = 0
BUILD_WARP = 1
BUILD_HALF = 2
FORCE_THREAD = 0
FORCE_STAGED = 1

STEP_HOST_SYNC = 1
STEP_ENERGY = 2
STEP_BARRIER_CHECK = 0x100

ERR_ARG = -1
ERR_CUDA = -2
ERR_NOMEM = -3
ERR_CAPACITY = -4
ERR_DEVICE = -5

ERRBIT_LIST_OVERFLOW = 1
ERRBIT_FAR_MOVER = 2
ERRBIT_CELL_INDEX = 4

EXPORTED = [
    "xnb_last_error_string", "xnb_version", "xnb_batch_create", "xnb_batch_destroy", "xnb_system_bytes",
    "xnb_system_add", "xnb_system_remove", "xnb_system_info_get", "xnb_system_download", "xnb_system_pairs",
    "xnb_system_energy", "xnb_init_particles", "xnb_push_f_v_r", "xnb_push_f_v", "xnb_particle_displ_over",
    "xnb_update_particles_full", "xnb_chunk_neighbors", "xnb_backup_r", "xnb_lennard_jones_force",
    "xnb_ghost_update_r", "xnb_step", "xnb_step_graph_create", "xnb_graph_launch", "xnb_graph_destroy",
    "xnb_check_errors", "xnb_stats_kernel_launches", "xnb_chunk_neighbors_noalloc", "xnb_chunk_neighbors_stream",
    "xnb_verify_chunk_neighbors", "xnb_simulation_stats", "xnb_sample_particles", "xnb_system_set_types",
    "xnb_gravitational_force", "xnb_batch_set_tuning", "xnb_autotune", "xnb_snap_create", "xnb_snap_destroy",
    "xnb_snap_force", "xnb_system_pairs_range", "xnb_system_pair_view", "xnb_batch_set_build_form",
    "xnb_graph_is_current", "xnb_batch_set_force_lanes", "xnb_batch_set_force_form",
    "xnb_batch_set_subcell_pruning", "xnb_step_persistent",
]

FORCE_ENERGY = 1
FORCE_ACCUMULATE = 2
FORCE_MIXED = 4

STREAM_CHECKS = ("format", "order", "self", "range", "far", "missing")


class LJParams(C.Structure):
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


class SimStats(C.Structure):
    _fields_ = [
        ("particle_count", C.c_int64),
        ("kinetic_sum", C.c_double),
        ("potential_energy", C.c_double),
        ("min_vel", C.c_double),
        ("max_vel", C.c_double),
        ("min_acc", C.c_double),
        ("max_acc", C.c_double),
    ]


class Tuning(C.Structure):
    _fields_ = [
        ("stage_cap", C.c_int32),
        ("force_block", C.c_int32),
        ("newton", C.c_int32),
        ("trials", C.c_int32),
        ("atom_steps_per_s", C.c_double),
        ("build_form", C.c_int32),
        ("force_lanes", C.c_int32),
        ("force_form", C.c_int32),
        ("reserved", C.c_int32),
    ]


class BatchConfig(C.Structure):
    _fields_ = [
        ("device", C.c_int32),
        ("max_systems", C.c_int32),
        ("particle_capacity", C.c_int64),
        ("cell_capacity", C.c_int64),
        ("list_capacity", C.c_int64),
        ("stage_cap", C.c_int32),
        ("force_block", C.c_int32),
    ]


class SystemInfo(C.Structure):
    _fields_ = [
        ("n_particles", C.c_int64),
        ("n_cells", C.c_int64),
        ("list_used", C.c_int64),
        ("list_cap", C.c_int64),
        ("rebuilds", C.c_int64),
        ("error_bits", C.c_uint32),
        ("max_cell", C.c_uint32),
        ("active", C.c_int32),
        ("max_nbr", C.c_uint32),
    ]


class PairView(C.Structure):
    """xnb_pair_view: device pointers of one system for pair functors (include/xnb_pair.cuh)."""
    _fields_ = [("n_particles", C.c_int64)] + [(k, C.c_void_p) for k in (
        "rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz", "pe", "id", "type", "mirror", "mirror_lo", "nbr",
        "nbr_start", "nbr_count", "nbr_half")] + [
        ("origin", C.c_double * 3), ("period", C.c_double * 3), ("nbh_dist", C.c_double),
        ("max_period", C.c_double), ("mass", C.c_double), ("divide_by_mass", C.c_int32), ("sys", C.c_int32)]


class SnapParams(C.Structure):
    _fields_ = [("twojmax", C.c_int32), ("rcutfac", C.c_double), ("rfac0", C.c_double), ("rmin0", C.c_double),
                ("switchflag", C.c_int32), ("bzeroflag", C.c_int32), ("chemflag", C.c_int32),
                ("bnormflag", C.c_int32), ("quadraticflag", C.c_int32), ("switchinnerflag", C.c_int32),
                ("ntypes", C.c_int32), ("radelem", C.c_double * 16), ("wj", C.c_double * 16),
                ("ncoeffall", C.c_int32), ("coeff", C.POINTER(C.c_double)), ("energy_unit", C.c_double)]


class XnbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("xnb error %d: %s" % (code, msg))
        self.code = code


_LIB = None


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libxnb_gpu.so (building it when missing) and declare the ABI."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError("libxnb_gpu.so not built: run exanbody_gb300/build.py")
        _build.build()
    lib = C.CDLL(path)
    P = C.POINTER
    d, i32, i64, u64, vp = C.c_double, C.c_int32, C.c_int64, C.c_uint64, C.c_void_p
    lib.xnb_last_error_string.restype = C.c_char_p
    lib.xnb_batch_create.argtypes = [P(BatchConfig), P(vp)]
    lib.xnb_batch_destroy.argtypes = [vp]
    lib.xnb_system_bytes.restype = i64
    lib.xnb_system_bytes.argtypes = [i64, i64, d]
    lib.xnb_system_add.argtypes = [vp, P(LJParams), i64] + [P(d)] * 6 + [P(u64), P(i64), d, vp, P(i32)]
    lib.xnb_system_remove.argtypes = [vp, i32, vp]
    lib.xnb_system_info_get.argtypes = [vp, i32, P(SystemInfo), vp]
    lib.xnb_system_download.argtypes = [vp, i32] + [P(d)] * 9 + [P(u64), P(i32), P(d), vp]
    lib.xnb_system_pairs.argtypes = [vp, i32, P(u64), P(u64), P(i32), i64, P(i64), vp]
    lib.xnb_system_pairs_range.argtypes = [vp, i32, i64, i64, P(u64), P(i32), i64, P(i64), vp]
    lib.xnb_system_pair_view.argtypes = [vp, i32, P(PairView)]
    lib.xnb_batch_set_build_form.argtypes = [vp, i32]
    lib.xnb_graph_is_current.argtypes = [vp]
    lib.xnb_batch_set_force_lanes.argtypes = [vp, i32]
    lib.xnb_batch_set_force_form.argtypes = [vp, i32]
    lib.xnb_batch_set_subcell_pruning.argtypes = [vp, i32]
    lib.xnb_step_persistent.argtypes = [vp, i32, i32, i32, vp]
    lib.xnb_system_energy.argtypes = [vp, i32, P(d), P(d), vp]
    lib.xnb_init_particles.argtypes = [vp, i32, i32, vp]
    lib.xnb_push_f_v_r.argtypes = [vp, i32, d, vp]
    lib.xnb_push_f_v.argtypes = [vp, i32, d, vp]
    lib.xnb_particle_displ_over.argtypes = [vp, i32, P(i64), vp]
    lib.xnb_update_particles_full.argtypes = [vp, i32, vp]
    lib.xnb_chunk_neighbors.argtypes = [vp, i32, vp]
    lib.xnb_backup_r.argtypes = [vp, i32, vp]
    lib.xnb_lennard_jones_force.argtypes = [vp, i32, i32, i32, vp]
    lib.xnb_ghost_update_r.argtypes = [vp, i32, vp]
    lib.xnb_step.argtypes = [vp, i32, i32, i32, vp]
    lib.xnb_step_graph_create.argtypes = [vp, i32, i32, i32, vp, P(vp)]
    lib.xnb_graph_launch.argtypes = [vp, vp]
    lib.xnb_graph_destroy.argtypes = [vp]
    lib.xnb_check_errors.argtypes = [vp, vp]
    lib.xnb_stats_kernel_launches.restype = i64
    lib.xnb_stats_kernel_launches.argtypes = [vp]
    u32p = P(C.c_uint32)
    lib.xnb_chunk_neighbors_noalloc.argtypes = [P(LJParams), i64, vp, vp, vp, vp, vp, vp, i64, vp, vp, P(i64), vp]
    lib.xnb_chunk_neighbors_stream.argtypes = [vp, i32, i32, vp, i64, vp, P(i64), vp]
    lib.xnb_verify_chunk_neighbors.argtypes = [vp, i32, i32, vp, i64, vp, P(i64), vp]
    lib.xnb_simulation_stats.argtypes = [vp, i32, P(SimStats), vp]
    lib.xnb_sample_particles.argtypes = [vp, i32, P(u64), i64, P(d), P(i32), vp]
    lib.xnb_system_set_types.argtypes = [vp, i32, P(u64), P(C.c_uint8), i64, P(i64), vp]
    lib.xnb_gravitational_force.argtypes = [vp, i32, d, P(d), i32, d, i32, i32, vp]
    lib.xnb_batch_set_tuning.argtypes = [vp, i32, i32]
    lib.xnb_autotune.argtypes = [vp, i32, i32, vp, P(Tuning)]
    lib.xnb_snap_create.argtypes = [P(SnapParams), i32, P(vp)]
    lib.xnb_snap_destroy.argtypes = [vp]
    lib.xnb_snap_force.argtypes = [vp, i32, vp, i32, vp]
    _LIB = lib
    return lib


def _ck(rc):
    if rc != 0:
        raise XnbError(rc, _LIB.xnb_last_error_string().decode())
    return rc


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def lj_params(geom, epsilon=1.0, sigma=1.0, rcut=2.5, rcut_inc=0.3, dt=0.005, mass=1.0, divide_by_mass=False,
              amr=True, sub_grid_density=6.5):
    """LJParams from a geometry dict (origin, extent, dims, cell_size)."""
    p = LJParams()
    for a in range(3):
        p.origin[a] = geom["origin"][a]
        p.extent[a] = geom["extent"][a]
        p.dims[a] = int(geom["dims"][a])
    p.cell_size = geom["cell_size"]
    p.rcut, p.rcut_inc = rcut, rcut_inc
    p.epsilon, p.sigma, p.dt = epsilon, sigma, dt
    p.mass, p.divide_by_mass = mass, int(bool(divide_by_mass))
    p.amr_enabled, p.sub_grid_density = int(bool(amr)), sub_grid_density
    return p


class Batch:
    """Device pools holding any number of resident systems (xnb_batch)."""

    def __init__(self, particle_capacity, cell_capacity, list_capacity, max_systems=1, device=0, stage_cap=0,
                 stream=None, force_block=0):
        self.lib = load()
        cfg = BatchConfig(int(device), int(max_systems), int(particle_capacity), int(cell_capacity),
                          int(list_capacity), int(stage_cap), int(force_block))
        h = C.c_void_p()
        _ck(self.lib.xnb_batch_create(C.byref(cfg), C.byref(h)))
        self.h = h
        self.stream = C.c_void_p(stream) if stream else None

    def close(self):
        if getattr(self, "h", None):
            self.lib.xnb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- systems ----
    def add_system(self, params, r, v, ids, cell_counts=None, list_factor=1.3):
        r = np.ascontiguousarray(r, np.float64)
        v = np.ascontiguousarray(v, np.float64)
        ids = np.ascontiguousarray(ids, np.uint64)
        cols = [np.ascontiguousarray(r[:, a]) for a in range(3)] + [np.ascontiguousarray(v[:, a]) for a in range(3)]
        cc = None
        if cell_counts is not None:
            cell_counts = np.ascontiguousarray(cell_counts, np.int64)
            cc = cell_counts.ctypes.data_as(C.POINTER(C.c_int64))
        sid = C.c_int32()
        _ck(self.lib.xnb_system_add(self.h, C.byref(params), len(ids), *[_dp(c) for c in cols],
                                    ids.ctypes.data_as(C.POINTER(C.c_uint64)), cc, float(list_factor),
                                    self.stream, C.byref(sid)))
        return sid.value

    def add_system_soa(self, params, cols, ids, list_factor=1.3):
        """add_system from contiguous float64 columns cols["rx" .. "vz"] and uint64 ids,
        passed to the library as they are (no copy: pinned buffers stay pinned)."""
        keys = ("rx", "ry", "rz", "vx", "vy", "vz")
        for k in keys:
            c = cols[k]
            if c.dtype != np.float64 or not c.flags["C_CONTIGUOUS"] or len(c) != len(ids):
                raise ValueError("column %s must be contiguous float64 of len(ids)" % k)
        if ids.dtype != np.uint64 or not ids.flags["C_CONTIGUOUS"]:
            raise ValueError("ids must be contiguous uint64")
        sid = C.c_int32()
        _ck(self.lib.xnb_system_add(self.h, C.byref(params), len(ids), *[_dp(cols[k]) for k in keys],
                                    ids.ctypes.data_as(C.POINTER(C.c_uint64)), None, float(list_factor),
                                    self.stream, C.byref(sid)))
        return sid.value

    def remove_system(self, s):
        _ck(self.lib.xnb_system_remove(self.h, s, self.stream))

    def info(self, s):
        inf = SystemInfo()
        _ck(self.lib.xnb_system_info_get(self.h, s, C.byref(inf), self.stream))
        return inf

    def download(self, s, out=None):
        """Particles in storage order; `out` may supply the arrays (e.g. pinned buffers)."""
        n = self.info(s).n_particles
        if out is None:
            out = {k: np.empty(n, np.float64) for k in ("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz", "pe")}
            out["id"] = np.empty(n, np.uint64)
            out["cell"] = np.empty(n, np.int32)
        ids, cell = out["id"], out["cell"]
        _ck(self.lib.xnb_system_download(self.h, s, *[_dp(out[k]) for k in ("rx", "ry", "rz", "vx", "vy", "vz",
                                                                            "fx", "fy", "fz")],
                                         ids.ctypes.data_as(C.POINTER(C.c_uint64)),
                                         cell.ctypes.data_as(C.POINTER(C.c_int32)), _dp(out["pe"]), self.stream))
        out["id"] = ids
        out["cell"] = cell
        return out

    def pairs(self, s):
        inf = self.info(s)
        m = inf.list_used
        a = np.empty(m, np.uint64)
        b = np.empty(m, np.uint64)
        cnt = np.empty(inf.n_particles, np.int32)
        nout = C.c_int64()
        _ck(self.lib.xnb_system_pairs(self.h, s, a.ctypes.data_as(C.POINTER(C.c_uint64)),
                                      b.ctypes.data_as(C.POINTER(C.c_uint64)),
                                      cnt.ctypes.data_as(C.POINTER(C.c_int32)), m, C.byref(nout), self.stream))
        return a[: nout.value], b[: nout.value], cnt

    def pairs_range(self, s, first, count, entries):
        """Partner ids (list order) and per-particle lengths of particles
        [first, first + count); `entries` bounds the id array (the range's list total)."""
        b = np.empty(int(entries), np.uint64)
        cnt = np.empty(int(count), np.int32)
        nout = C.c_int64()
        _ck(self.lib.xnb_system_pairs_range(self.h, s, int(first), int(count),
                                            b.ctypes.data_as(C.POINTER(C.c_uint64)),
                                            cnt.ctypes.data_as(C.POINTER(C.c_int32)), int(entries), C.byref(nout),
                                            self.stream))
        if nout.value > len(b):
            raise XnbError(-4, "pairs_range: %d entries, %d requested" % (nout.value, len(b)))
        return b[: nout.value], cnt

    def pair_view(self, s):
        """The system's xnb_pair_view (for functors compiled against include/xnb_pair.cuh)."""
        v = PairView()
        _ck(self.lib.xnb_system_pair_view(self.h, s, C.byref(v)))
        return v

    def energy(self, s):
        ke, pe = C.c_double(), C.c_double()
        _ck(self.lib.xnb_system_energy(self.h, s, C.byref(ke), C.byref(pe), self.stream))
        return ke.value, pe.value

    # ---- operators ----
    def init_particles(self, s=-1, precision=PREC_FP64_EXACT):
        _ck(self.lib.xnb_init_particles(self.h, s, precision, self.stream))

    def push_f_v_r(self, dt_scale=1.0, s=-1):
        _ck(self.lib.xnb_push_f_v_r(self.h, s, dt_scale, self.stream))

    def push_f_v(self, dt_scale=0.5, s=-1):
        _ck(self.lib.xnb_push_f_v(self.h, s, dt_scale, self.stream))

    def particle_displ_over(self, s):
        out = np.zeros(max(1, 1 if s >= 0 else 4096), np.int64)
        _ck(self.lib.xnb_particle_displ_over(self.h, s, out.ctypes.data_as(C.POINTER(C.c_int64)), self.stream))
        return int(out[0]) if s >= 0 else out

    def update_particles_full(self, s=-1):
        _ck(self.lib.xnb_update_particles_full(self.h, s, self.stream))

    def chunk_neighbors(self, s=-1):
        _ck(self.lib.xnb_chunk_neighbors(self.h, s, self.stream))

    def backup_r(self, s=-1):
        _ck(self.lib.xnb_backup_r(self.h, s, self.stream))

    def lennard_jones_force(self, s=-1, precision=PREC_FP64_EXACT, energy=True):
        _ck(self.lib.xnb_lennard_jones_force(self.h, s, precision, int(bool(energy)), self.stream))

    def step(self, nsteps=1, precision=PREC_FP64_EXACT, flags=STEP_HOST_SYNC):
        _ck(self.lib.xnb_step(self.h, int(nsteps), int(precision), int(flags), self.stream))

    def step_persistent(self, nsteps=1, precision=PREC_FP64_EXACT, flags=0):
        """xnb_step_persistent: the same steps as one cooperative launch per run
        of steps between rebuilds (bitwise the states of step())."""
        _ck(self.lib.xnb_step_persistent(self.h, int(nsteps), int(precision), int(flags), self.stream))

    def graph(self, nsteps, precision=PREC_MIXED, flags=0):
        g = C.c_void_p()
        _ck(self.lib.xnb_step_graph_create(self.h, int(nsteps), int(precision), int(flags), self.stream,
                                           C.byref(g)))
        return Graph(self, g)

    def chunk_neighbors_stream(self, s, offset_tables=1, device="cuda"):
        """Reference-format u16 streams of system s as device tensors
        (stream[total] as int16 bit patterns, cell_offsets[n_cells + 1] as int64)."""
        import torch

        ncells = self.info(s).n_cells
        off = torch.empty(ncells + 1, dtype=torch.int64, device=device)
        total = C.c_int64()
        _ck(self.lib.xnb_chunk_neighbors_stream(self.h, s, int(offset_tables), None, 0, C.c_void_p(off.data_ptr()),
                                                C.byref(total), self.stream))
        buf = torch.empty(max(1, total.value), dtype=torch.int16, device=device)
        _ck(self.lib.xnb_chunk_neighbors_stream(self.h, s, int(offset_tables), C.c_void_p(buf.data_ptr()),
                                                total.value, C.c_void_p(off.data_ptr()), C.byref(total), self.stream))
        return buf[: total.value], off

    def verify_chunk_neighbors(self, s, stream, cell_offsets, offset_tables=1):
        """verify_chunk_neighbors counts (dict over STREAM_CHECKS) for device tensors."""
        out = (C.c_int64 * 6)()
        _ck(self.lib.xnb_verify_chunk_neighbors(self.h, s, int(offset_tables), C.c_void_p(stream.data_ptr()),
                                                int(stream.numel()), C.c_void_p(cell_offsets.data_ptr()), out,
                                                self.stream))
        return dict(zip(STREAM_CHECKS, [int(x) for x in out]))

    def simulation_stats(self, s):
        """simulation_stats reduced on the GPU (dict of the xnb_sim_stats fields)."""
        st = SimStats()
        _ck(self.lib.xnb_simulation_stats(self.h, s, C.byref(st), self.stream))
        return {k: getattr(st, k) for k, _ in SimStats._fields_}

    def sample_particles(self, s, ids):
        """(values[n, 9] = r, f, v; found[n]) for the given particle ids, gathered on the GPU."""
        ids = np.ascontiguousarray(ids, np.uint64)
        vals = np.zeros((len(ids), 9))
        found = np.zeros(len(ids), np.int32)
        _ck(self.lib.xnb_sample_particles(self.h, s, ids.ctypes.data_as(C.POINTER(C.c_uint64)), len(ids),
                                          vals.ctypes.data_as(C.POINTER(C.c_double)),
                                          found.ctypes.data_as(C.POINTER(C.c_int32)), self.stream))
        return vals, found

    def set_types(self, s, ids, types):
        """field::type of the listed ids; returns how many particles of s were found."""
        ids = np.ascontiguousarray(ids, np.uint64)
        types = np.ascontiguousarray(types, np.uint8)
        matched = C.c_int64()
        _ck(self.lib.xnb_system_set_types(self.h, s, ids.ctypes.data_as(C.POINTER(C.c_uint64)),
                                          types.ctypes.data_as(C.POINTER(C.c_uint8)), len(ids), C.byref(matched),
                                          self.stream))
        return matched.value

    def gravitational_force(self, s, G, masses, rcut, precision=PREC_FP64_EXACT, energy=False, accumulate=False):
        masses = np.ascontiguousarray(masses, np.float64)
        flags = (FORCE_ENERGY if energy else 0) | (FORCE_ACCUMULATE if accumulate else 0)
        _ck(self.lib.xnb_gravitational_force(self.h, s, float(G), masses.ctypes.data_as(C.POINTER(C.c_double)),
                                             len(masses), float(rcut), int(precision), flags, self.stream))

    def set_tuning(self, stage_cap, force_block):
        _ck(self.lib.xnb_batch_set_tuning(self.h, int(stage_cap), int(force_block)))

    def set_force_lanes(self, lanes):
        """Threads per particle (1, 2 or 4) of the FP64 / mixed full-list force traversal."""
        _ck(self.lib.xnb_batch_set_force_lanes(self.h, int(lanes)))

    def set_force_form(self, form):
        """FORCE_THREAD (one thread per particle, default) or FORCE_STAGED (cell
        segments staged in shared memory) for the mixed full-list traversal."""
        _ck(self.lib.xnb_batch_set_force_form(self.h, int(form)))

    def set_build_form(self, form):
        """BUILD_ROWS (lane per particle, bulk-copied rows) or BUILD_WARP (lane per candidate)."""
        _ck(self.lib.xnb_batch_set_build_form(self.h, int(form)))

    def set_subcell_pruning(self, on):
        """Sub-cell pair pruning of the neighbour build (default on): while the
        positions are those of the last rebin, dense cells (AMR sub-grid side 2
        or 3) search only the neighbour sub-cells within reach of each sub-cell;
        the lists are the same."""
        _ck(self.lib.xnb_batch_set_subcell_pruning(self.h, 1 if on else 0))

    def autotune(self, trial_steps=20, precision=PREC_MIXED):
        """Online autotuner (xnb_autotune): the batch advances while it is timed and is
        left on the fastest configuration; returns it as a dict."""
        t = Tuning()
        _ck(self.lib.xnb_autotune(self.h, int(trial_steps), int(precision), self.stream, C.byref(t)))
        return {k: getattr(t, k) for k, _ in Tuning._fields_}

    def check_errors(self):
        _ck(self.lib.xnb_check_errors(self.h, self.stream))

    def kernel_launches(self):
        return int(self.lib.xnb_stats_kernel_launches(self.h))


def chunk_neighbors_noalloc(params, n, rx, ry, rz, cell_start, cell_count, nbr, nbr_capacity, nbr_start, nbr_count,
                            stream=None):
    """xnb_chunk_neighbors_noalloc on caller-owned device buffers (device pointers as ints).
    Returns the number of entries written; an XnbError carries `.total`, the
    entries needed, which the library sets with XNB_ERR_CAPACITY."""
    lib = load()
    total = C.c_int64(-1)
    rc = lib.xnb_chunk_neighbors_noalloc(C.byref(params), int(n), rx, ry, rz, cell_start, cell_count, nbr,
                                         int(nbr_capacity), nbr_start, nbr_count, C.byref(total),
                                         C.c_void_p(stream) if stream else None)
    if rc != 0:
        err = XnbError(rc, lib.xnb_last_error_string().decode())
        err.total = total.value  # entries needed (set with XNB_ERR_CAPACITY)
        raise err
    return total.value


class Graph:
    def __init__(self, batch, g):
        self.batch, self.g = batch, g

    def launch(self):
        _ck(self.batch.lib.xnb_graph_launch(self.g, self.batch.stream))

    def current(self):
        """False once systems were added beyond the captured extent (capture again)."""
        return bool(self.batch.lib.xnb_graph_is_current(self.g))

    def close(self):
        if self.g:
            self.batch.lib.xnb_graph_destroy(self.g)
            self.g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
