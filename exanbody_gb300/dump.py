"""Dump/restart files in the reference's .dump format (include/xnb_dump.h).

write_dump / read_dump of exaNBody (src/io/write_dump.cpp, src/io/read_dump.cpp)
exchange positions, velocities, ids and types with a header carrying the
domain, time step and physical time. Here:

    write(filename, r, v, ids, types, dom, ...)   host arrays -> file
    read(filename)                                file -> arrays in file order
    write_system(batch, s, filename, ...)         a resident system -> file
    restore_system(batch, filename, **lj)         file -> a new resident system

A restored system is placed as read_dump places particles: each into the cell
of its periodic location, cells filled in file order (the batch's placement of
flat input, domain_periodic_location + append, sim_dump_reader.h:293-352).
"""
import ctypes as C

import numpy as np

from . import xnb

DUMP_VERSION = 1003

PERIODIC_X, PERIODIC_Y, PERIODIC_Z = 1 << 0, 1 << 1, 1 << 2
MIRROR_X_MIN, MIRROR_X_MAX, MIRROR_Y_MIN, MIRROR_Y_MAX, MIRROR_Z_MIN, MIRROR_Z_MAX = (1 << k for k in range(3, 9))
EXPANDABLE = 1 << 16
XFORM_IDENTITY = 1 << 17

FIELDS = ("rx", "ry", "rz", "vx", "vy", "vz", "id", "type")

EXPORTED = [
    "xnb_dump_zlib_available", "xnb_dump_domain_init", "xnb_dump_write", "xnb_dump_read_info", "xnb_dump_read",
    "xnb_system_write_dump", "xnb_system_download_types",
]


class DumpDomain(C.Structure):
    _fields_ = [("bmin", C.c_double * 3), ("bmax", C.c_double * 3), ("grid_dims", C.c_int64 * 3),
                ("cell_size", C.c_double), ("xform", C.c_double * 9), ("inv_xform", C.c_double * 9),
                ("xform_min_scale", C.c_double), ("xform_max_scale", C.c_double), ("flags", C.c_uint32)]

    def as_dict(self):
        return {"origin": tuple(self.bmin), "extent": tuple(self.bmax), "dims": tuple(self.grid_dims),
                "cell_size": self.cell_size, "xform": tuple(self.xform), "inv_xform": tuple(self.inv_xform),
                "xform_min_scale": self.xform_min_scale, "xform_max_scale": self.xform_max_scale,
                "flags": self.flags,
                "periodic": tuple(bool(self.flags & (PERIODIC_X << a)) for a in range(3)),
                "expandable": bool(self.flags & EXPANDABLE)}


class DumpInfo(C.Structure):
    _fields_ = [("version", C.c_uint64), ("n_particles", C.c_uint64), ("timestep", C.c_uint64),
                ("physical_time", C.c_double), ("tuple_size", C.c_uint64), ("chunk_count", C.c_uint64),
                ("data_chunks", C.c_uint64), ("file_bytes", C.c_uint64), ("part_size", C.c_uint64),
                ("n_fields", C.c_int32), ("field_mask", C.c_uint32), ("domain", DumpDomain)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "domain"}
        d["fields"] = tuple(f for k, f in enumerate(FIELDS) if self.field_mask & (1 << k))
        d["domain"] = self.domain.as_dict()
        return d


_DECLARED = False


def _lib():
    global _DECLARED
    lib = xnb.load()
    if not _DECLARED:
        P = C.POINTER
        d, i32, i64, u64, u32, vp = C.c_double, C.c_int32, C.c_int64, C.c_uint64, C.c_uint32, C.c_void_p
        lib.xnb_dump_zlib_available.argtypes = []
        lib.xnb_dump_domain_init.argtypes = [P(DumpDomain), P(d), P(d), P(i64), d, u32]
        lib.xnb_dump_domain_init.restype = None
        lib.xnb_dump_write.argtypes = [C.c_char_p, P(DumpDomain), u64, d, i64] + [vp] * 8 + [vp, i64, i32, i64,
                                                                                              i64, i32]
        lib.xnb_dump_read_info.argtypes = [C.c_char_p, P(DumpInfo)]
        lib.xnb_dump_read.argtypes = [C.c_char_p, i64] + [vp] * 8 + [P(i64), P(DumpInfo)]
        lib.xnb_system_write_dump.argtypes = [vp, i32, C.c_char_p, u64, d, i32, i64, u32, vp]
        lib.xnb_system_download_types.argtypes = [vp, i32, vp, vp]
        _DECLARED = True
    return lib


def _ck(rc):
    if rc != 0:
        raise xnb.XnbError(rc, _lib().xnb_last_error_string().decode())


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def zlib_available():
    return bool(_lib().xnb_dump_zlib_available())


def domain(geom, periodic=(True, True, True), expandable=True):
    """DumpDomain of a geometry dict (origin, extent, dims, cell_size): identity
    transform; Domain() starts expandable (domain.h:104)."""
    flags = sum(PERIODIC_X << a for a in range(3) if periodic[a]) | (EXPANDABLE if expandable else 0)
    dom = DumpDomain()
    lo = (C.c_double * 3)(*[float(x) for x in geom["origin"]])
    hi = (C.c_double * 3)(*[float(x) for x in geom["extent"]])
    dims = (C.c_int64 * 3)(*[int(x) for x in geom["dims"]])
    _lib().xnb_dump_domain_init(C.byref(dom), lo, hi, dims, float(geom["cell_size"]), flags)
    return dom


def write(filename, r, v=None, ids=None, types=None, dom=None, timestep=0, physical_time=0.0, cell_counts=None,
          compression_level=6, max_part_size=-1, chunk_particles=0, threads=0):
    """Writes particles in the order given (see xnb_dump_write)."""
    r = np.asarray(r, np.float64)
    n = len(r)
    cols = [np.ascontiguousarray(r[:, a]) for a in range(3)]
    cols += [None] * 3 if v is None else [np.ascontiguousarray(np.asarray(v, np.float64)[:, a]) for a in range(3)]
    idc = None if ids is None else np.ascontiguousarray(ids, np.uint64)
    tyc = None if types is None else np.ascontiguousarray(types, np.uint8)
    for c in cols + [idc, tyc]:
        if c is not None and len(c) != n:
            raise ValueError("all particle arrays need %d entries" % n)
    cc = None if cell_counts is None else np.ascontiguousarray(cell_counts, np.int64)
    _ck(_lib().xnb_dump_write(str(filename).encode(), C.byref(dom), int(timestep), float(physical_time), n,
                              *[_ptr(c) for c in cols], _ptr(idc), _ptr(tyc), _ptr(cc),
                              0 if cc is None else len(cc), int(compression_level), int(max_part_size),
                              int(chunk_particles), int(threads)))


def read_info(filename):
    info = DumpInfo()
    _ck(_lib().xnb_dump_read_info(str(filename).encode(), C.byref(info)))
    return info.as_dict()


def read(filename):
    """Particles in file order: {"r", "v", "id", "type", "info"}."""
    info = read_info(filename)
    n = int(info["n_particles"])
    cols = [np.empty(n, np.float64) for _ in range(6)]
    ids = np.empty(n, np.uint64)
    types = np.empty(n, np.uint8)
    nout = C.c_int64()
    inf = DumpInfo()
    _ck(_lib().xnb_dump_read(str(filename).encode(), n, *[_ptr(c) for c in cols], _ptr(ids), _ptr(types),
                             C.byref(nout), C.byref(inf)))
    return {"r": np.stack(cols[:3], axis=1), "v": np.stack(cols[3:], axis=1), "id": ids, "type": types,
            "info": inf.as_dict()}


def system_types(batch, s):
    n = batch.info(s).n_particles
    t = np.empty(n, np.uint8)
    _ck(_lib().xnb_system_download_types(batch.h, s, _ptr(t), batch.stream))
    return t


def write_system(batch, s, filename, timestep=0, physical_time=0.0, compression_level=6, max_part_size=-1,
                 expandable=True):
    """write_dump of one resident system (storage order, chunks at cell boundaries)."""
    _ck(_lib().xnb_system_write_dump(batch.h, s, str(filename).encode(), int(timestep), float(physical_time),
                                     int(compression_level), int(max_part_size), 0 if expandable else EXPANDABLE,
                                     batch.stream))


def geometry(info):
    """Geometry dict (origin, extent, dims, cell_size) of a file's domain; only
    fully periodic domains with the identity transform are simulated here."""
    dom = info["domain"]
    if not all(dom["periodic"]):
        raise ValueError("the domain of this file is not periodic in x, y and z")
    if not dom["flags"] & XFORM_IDENTITY:
        raise ValueError("the domain of this file has a non-identity transform")
    return {"origin": dom["origin"], "extent": dom["extent"], "dims": dom["dims"], "cell_size": dom["cell_size"]}


def restore_system(batch, filename, list_factor=1.3, **lj):
    """read_dump into a new resident system of `batch`; lj: xnb.lj_params keyword
    arguments (rcut, rcut_inc, epsilon, sigma, dt, mass, ...). Returns (sys, info)."""
    d = read(filename)
    params = xnb.lj_params(geometry(d["info"]), **lj)
    s = batch.add_system(params, d["r"], d["v"], d["id"], list_factor=list_factor)
    if np.any(d["type"] != 0):
        step = 1 << 24  # xnb_system_set_types takes at most 2^24 ids per call
        for k in range(0, len(d["id"]), step):
            batch.set_types(s, d["id"][k:k + step], d["type"][k:k + step])
    return s, d["info"]
