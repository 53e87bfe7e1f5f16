""".dump files (include/xnb_dump.h, exanbody_gb300/dump.py) on the host.

An independent parser and writer below restate the reference's layout from its
declarations -- SimDumpHeader (src/io/include/exanb/io/sim_dump_io.h:105-128),
Domain (core/include/exanb/core/domain.h:96-105) and Domain_legacy_v1_2
(io/include/exanb/io/domain_legacy_v1.2.h:36-49) with natural member alignment,
DataChunkItem (sim_dump_io.h:42-49), zlib chunks (lib/mpi_file_io.cpp:397-440) and
file parts (mpi_file_io.cpp:110-176) -- with struct and zlib only. The library's
files must parse under it, its legacy and unpadded files must read back in the
library, and malformed files must raise, never crash."""
import os
import struct
import zlib

import numpy as np
import pytest

from exanbody_gb300 import dump, workloads, xnb

FIELDS = [("rx", 8, "<f8"), ("ry", 8, "<f8"), ("rz", 8, "<f8"), ("vx", 8, "<f8"), ("vy", 8, "<f8"),
          ("vz", 8, "<f8"), ("id", 8, "<u8"), ("type", 1, "u1")]


def _align(x, a=8):
    return (x + a - 1) // a * a


def header_layout():
    """Byte offsets of SimDumpHeader members under natural alignment (LP64)."""
    members = [("version", 8, 8), ("nb_fields", 4, 4), ("data_flags", 4, 1), ("tuple_size", 8, 8),
               ("field_size", 8 * 128, 8), ("fields", 32 * 128, 1), ("nb_particles", 8, 8), ("time_step", 8, 8),
               ("time", 8, 8), ("domain", 248, 8), ("optional_offset", 8, 8), ("table_offset", 8, 8),
               ("data_offset", 8, 8), ("optional_header_size", 8, 8), ("chunk_count", 8, 8)]
    off, lay = 0, {}
    for name, size, al in members:
        off = _align(off, al)
        lay[name] = off
        off += size
    lay["size"] = _align(off, 8)
    return lay


def domain_layout():
    """Domain: AABB(2 Vec3d), IJK(3 ssize_t), cell size, 2 Mat3d, 2 scales, then
    u32 flags + u32 padding (1.3) or 5 bools (1.2), padded to 8 bytes."""
    return {"bmin": 0, "bmax": 24, "dims": 48, "cell": 72, "xform": 80, "inv": 152, "min_scale": 224,
            "max_scale": 232, "flags": 240, "size": 248}


def read_logical(path):
    """Concatenation of the file's parts (the split size is the first part's size)."""
    data = open(path, "rb").read()
    k = 1
    while os.path.exists("%s.%d" % (path, k)):
        data += open("%s.%d" % (path, k), "rb").read()
        k += 1
    return data


def parse(path):
    """Independent reader of a version 1.3 file with the write_dump field set."""
    buf = read_logical(path)
    H, D = header_layout(), domain_layout()
    assert H["size"] == 5456 and H["domain"] == 5168
    version, = struct.unpack_from("<Q", buf, H["version"])
    nf, = struct.unpack_from("<I", buf, H["nb_fields"])
    sizes = struct.unpack_from("<%dQ" % nf, buf, H["field_size"])
    names = [buf[H["fields"] + 32 * k: H["fields"] + 32 * (k + 1)].split(b"\0")[0].decode() for k in range(nf)]
    out = {"version": version, "names": names, "sizes": list(sizes)}
    for key in ("tuple_size", "nb_particles", "time_step", "optional_offset", "table_offset", "data_offset",
                "optional_header_size", "chunk_count"):
        out[key], = struct.unpack_from("<Q", buf, H[key])
    out["time"], = struct.unpack_from("<d", buf, H["time"])
    dbase = H["domain"]
    out["bmin"] = struct.unpack_from("<3d", buf, dbase + D["bmin"])
    out["bmax"] = struct.unpack_from("<3d", buf, dbase + D["bmax"])
    out["dims"] = struct.unpack_from("<3q", buf, dbase + D["dims"])
    out["cell_size"], = struct.unpack_from("<d", buf, dbase + D["cell"])
    out["xform"] = struct.unpack_from("<9d", buf, dbase + D["xform"])
    out["flags"], out["pad"] = struct.unpack_from("<II", buf, dbase + D["flags"])
    table = [struct.unpack_from("<QIi", buf, out["table_offset"] + 16 * i) for i in range(out["chunk_count"])]
    out["table"] = table
    cols = {name: [] for name, _, _ in FIELDS}
    for i, (off, size, n) in enumerate(table):
        if size == 0 and n == 0:
            continue
        assert n > 0
        raw_len = sum(_align(n * s) for _, s, _ in FIELDS)
        blob = buf[off: off + size]
        raw = blob if size == raw_len else zlib.decompress(blob)
        assert len(raw) == raw_len
        at = 0
        for name, s, dt in FIELDS:
            at = _align(at)
            cols[name].append(np.frombuffer(raw[at: at + n * s], dtype=dt))
            at += n * s
    out["arrays"] = {k: (np.concatenate(v) if v else np.empty(0)) for k, v in cols.items()}
    out["file_size"] = len(buf)
    return out


def write_independent(path, r, v, ids, types, geom, version=1003, legacy_periodic=(1, 1, 1), legacy_expandable=1,
                      chunk=1000, level=6, pad_last=True, part=None):
    """Writer restated from the same declarations (for reader tests)."""
    H, D = header_layout(), domain_layout()
    n = len(r)
    spans = [(f, min(chunk, n - f)) for f in range(0, n, chunk)]
    chunk_count = 1 + n // chunk + 1
    data_offset = H["size"] + 16 * chunk_count
    blobs, table, at = [], [], data_offset
    for f, m in spans:
        arrays = [r[f:f + m, 0], r[f:f + m, 1], r[f:f + m, 2], v[f:f + m, 0], v[f:f + m, 1], v[f:f + m, 2],
                  ids[f:f + m], types[f:f + m]]
        raw = b""
        for (name, s, dt), a in zip(FIELDS, arrays):
            raw += b"\0" * (_align(len(raw)) - len(raw))
            raw += np.ascontiguousarray(a, dtype=dt).tobytes()
        if pad_last:
            raw += b"\0" * (_align(len(raw)) - len(raw))
        blob = zlib.compress(raw, level) if level else raw
        if len(blob) >= len(raw):
            blob = raw
        blobs.append(blob)
        table.append((at, len(blob), m))
        at += len(blob)
    table += [(at, 0, 0)] * (chunk_count - len(table))
    h = bytearray(H["size"])
    struct.pack_into("<Q", h, H["version"], version)
    struct.pack_into("<I", h, H["nb_fields"], len(FIELDS))
    struct.pack_into("<Q", h, H["tuple_size"], 64)
    for k, (name, s, _) in enumerate(FIELDS):
        struct.pack_into("<Q", h, H["field_size"] + 8 * k, s)
        h[H["fields"] + 32 * k: H["fields"] + 32 * k + len(name)] = name.encode()
    struct.pack_into("<QQd", h, H["nb_particles"], n, 7, 0.035)
    d0 = H["domain"]
    struct.pack_into("<3d", h, d0 + D["bmin"], *geom["origin"])
    struct.pack_into("<3d", h, d0 + D["bmax"], *geom["extent"])
    struct.pack_into("<3q", h, d0 + D["dims"], *geom["dims"])
    struct.pack_into("<d", h, d0 + D["cell"], geom["cell_size"])
    ident = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0)
    struct.pack_into("<9d", h, d0 + D["xform"], *ident)
    struct.pack_into("<9d", h, d0 + D["inv"], *ident)
    struct.pack_into("<2d", h, d0 + D["min_scale"], 1.0, 1.0)
    if version >= 1003:
        struct.pack_into("<I", h, d0 + D["flags"], 0x7 | (1 << 16) | (1 << 17))
    else:
        struct.pack_into("<5B", h, d0 + D["flags"], 1, *legacy_periodic, legacy_expandable)
    struct.pack_into("<5Q", h, H["optional_offset"], H["size"], H["size"], data_offset, 0, chunk_count)
    body = bytes(h) + b"".join(struct.pack("<QIi", *t) for t in table) + b"".join(blobs)
    if part is None:
        open(path, "wb").write(body)
    else:
        for k in range(0, (len(body) + part - 1) // part):
            open(path if k == 0 else "%s.%d" % (path, k), "wb").write(body[k * part:(k + 1) * part])


@pytest.fixture(scope="module")
def system():
    w = workloads.lj_fcc_system(9, 0.8442, 1.44, 21)  # 2916 atoms
    w["type"] = (np.arange(w["n_atoms"]) * 7 % 5).astype(np.uint8)
    return w


def test_round_trip_levels_chunks_and_parts(system, tmp_path):
    w = system
    dom = dump.domain(w["geom"])
    for level, part, chunk in ((6, -1, 0), (0, -1, 500), (1, 40000, 700), (-1, 9000, 333), (9, -1, 1)):
        fn = tmp_path / ("a_%d.dump" % level)
        dump.write(fn, w["r"], w["v"], w["id"], w["type"], dom, timestep=40, physical_time=0.2,
                   compression_level=level, max_part_size=part, chunk_particles=chunk, threads=3)
        d = dump.read(fn)
        assert np.array_equal(d["r"], w["r"]) and np.array_equal(d["v"], w["v"])
        assert np.array_equal(d["id"], w["id"]) and np.array_equal(d["type"], w["type"])
        inf = d["info"]
        assert inf["version"] == 1003 and inf["n_particles"] == w["n_atoms"]
        assert inf["timestep"] == 40 and inf["physical_time"] == 0.2
        per = chunk if chunk > 0 else 65536
        assert inf["chunk_count"] == 3 + w["n_atoms"] // per + 1
        assert inf["data_chunks"] == -(-w["n_atoms"] // per)
        assert inf["fields"] == dump.FIELDS and inf["tuple_size"] == 64
        dd = inf["domain"]
        assert dd["periodic"] == (True, True, True) and dd["expandable"]
        assert dd["dims"] == tuple(w["geom"]["dims"]) and dd["cell_size"] == w["geom"]["cell_size"]
        if part > 0:
            assert inf["part_size"] == part and os.path.exists(str(fn) + ".1")


def test_independent_parser_reads_library_files(system, tmp_path):
    w = system
    dom = dump.domain(w["geom"], expandable=False)
    fn = tmp_path / "b.dump"
    dump.write(fn, w["r"], w["v"], w["id"], w["type"], dom, timestep=123, physical_time=0.615,
               compression_level=6, max_part_size=20000, chunk_particles=800)
    p = parse(str(fn))
    assert p["version"] == 1003
    assert p["names"] == [f[0] for f in FIELDS] and p["sizes"] == [f[1] for f in FIELDS]
    assert p["tuple_size"] == 64 and p["nb_particles"] == w["n_atoms"]
    assert p["time_step"] == 123 and p["time"] == 0.615
    assert p["optional_offset"] == 5456 and p["table_offset"] == 5456 and p["optional_header_size"] == 0
    assert p["data_offset"] == 5456 + 16 * p["chunk_count"]
    assert p["bmin"] == tuple(w["geom"]["origin"]) and p["bmax"] == tuple(w["geom"]["extent"])
    assert p["dims"] == tuple(w["geom"]["dims"]) and p["cell_size"] == w["geom"]["cell_size"]
    assert p["xform"] == (1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0)
    assert p["flags"] == 0x7 | (1 << 17) and p["pad"] == 0  # periodic xyz, identity, not expandable
    offs = [t[0] for t in p["table"]]
    assert offs == sorted(offs) and offs[0] == p["data_offset"]
    ends = [t for t in p["table"] if t[1] == 0]
    assert ends and all(t == (p["file_size"], 0, 0) for t in ends)
    a = p["arrays"]
    assert np.array_equal(a["rx"], w["r"][:, 0]) and np.array_equal(a["vz"], w["v"][:, 2])
    assert np.array_equal(a["id"], w["id"]) and np.array_equal(a["type"], w["type"])


def test_chunks_close_at_cell_boundaries(system, tmp_path):
    w = system
    rng = np.random.default_rng(3)
    counts, total = [], 0
    while total < w["n_atoms"]:
        c = min(int(rng.integers(0, 40)), w["n_atoms"] - total)
        counts.append(c)
        total += c
    counts = np.array(counts)
    fn = tmp_path / "c.dump"
    dump.write(fn, w["r"], w["v"], w["id"], w["type"], dump.domain(w["geom"]), cell_counts=counts,
               chunk_particles=300, compression_level=1)
    p = parse(str(fn))
    bounds = set(np.cumsum(counts).tolist())
    sizes = [t[2] for t in p["table"] if t[2] > 0]
    cum = np.cumsum(sizes)
    assert cum[-1] == w["n_atoms"] and all(int(c) in bounds for c in cum)
    assert all(s >= 300 for s in sizes[:-1])
    assert np.array_equal(dump.read(fn)["r"], w["r"])


@pytest.mark.parametrize("version,periodic,expandable,want_exp", [(1002, (1, 0, 1), 0, False), (1001, (1, 1, 1), 0, True),
                                                                  (1002, (0, 1, 0), 1, True)])
def test_legacy_domain_versions(system, tmp_path, version, periodic, expandable, want_exp):
    w = system
    fn = tmp_path / "legacy.dump"
    write_independent(str(fn), w["r"], w["v"], w["id"], w["type"], w["geom"], version=version,
                      legacy_periodic=periodic, legacy_expandable=expandable)
    d = dump.read(fn)
    dd = d["info"]["domain"]
    assert d["info"]["version"] == version
    assert dd["periodic"] == tuple(bool(x) for x in periodic)
    assert dd["expandable"] == want_exp  # 1.1 files are made expandable (post_process)
    assert dd["flags"] & dump.XFORM_IDENTITY and dd["xform_min_scale"] == 1.0
    assert np.array_equal(d["r"], w["r"]) and np.array_equal(d["type"], w["type"])


@pytest.mark.parametrize("level,pad", [(0, False), (0, True), (6, False)])
def test_unpadded_and_raw_chunks_from_another_writer(system, tmp_path, level, pad):
    w = system
    fn = tmp_path / "other.dump"
    write_independent(str(fn), w["r"], w["v"], w["id"], w["type"], w["geom"], chunk=777, level=level, pad_last=pad,
                      part=50000)
    d = dump.read(fn)
    assert np.array_equal(d["r"], w["r"]) and np.array_equal(d["v"], w["v"])
    assert np.array_equal(d["id"], w["id"]) and np.array_equal(d["type"], w["type"])
    assert d["info"]["timestep"] == 7 and d["info"]["physical_time"] == 0.035


def test_stale_parts_are_removed(system, tmp_path):
    w = system
    fn = tmp_path / "s.dump"
    dom = dump.domain(w["geom"])
    dump.write(fn, w["r"], w["v"], w["id"], w["type"], dom, compression_level=0, max_part_size=30000)
    assert os.path.exists(str(fn) + ".3")
    dump.write(fn, w["r"], w["v"], w["id"], w["type"], dom, compression_level=0)
    assert not os.path.exists(str(fn) + ".1") and not os.path.exists(str(fn) + ".3")
    assert np.array_equal(dump.read(fn)["r"], w["r"])


def _expect_error(path):
    with pytest.raises(xnb.XnbError):
        dump.read(path)


def test_malformed_files_raise(system, tmp_path):
    w = system
    good = tmp_path / "g.dump"
    dump.write(good, w["r"], w["v"], w["id"], w["type"], dump.domain(w["geom"]), chunk_particles=500)
    blob = bytearray(open(good, "rb").read())
    H = header_layout()
    p = parse(str(good))

    def variant(name, mutate):
        b = bytearray(blob)
        mutate(b)
        path = tmp_path / name
        open(path, "wb").write(bytes(b))
        return path

    _expect_error(tmp_path / "missing.dump")
    _expect_error(variant("short.dump", lambda b: b.__delitem__(slice(4000, None))))
    _expect_error(variant("trunc.dump", lambda b: b.__delitem__(slice(len(b) - 100, None))))
    _expect_error(variant("ver.dump", lambda b: struct.pack_into("<Q", b, 0, 1004)))
    _expect_error(variant("nf.dump", lambda b: struct.pack_into("<I", b, H["nb_fields"], 500)))
    _expect_error(variant("norx.dump", lambda b: b.__setitem__(slice(H["fields"], H["fields"] + 2), b"qq")))
    _expect_error(variant("size.dump", lambda b: struct.pack_into("<Q", b, H["field_size"], 4)))
    _expect_error(variant("count.dump", lambda b: struct.pack_into("<Q", b, H["nb_particles"], w["n_atoms"] + 1)))
    t0 = p["table_offset"]
    _expect_error(variant("order.dump", lambda b: struct.pack_into("<Q", b, t0 + 16, 0)))
    _expect_error(variant("half.dump", lambda b: struct.pack_into("<I", b, t0 + 8, 0)))
    first = p["table"][0][0]
    _expect_error(variant("zdata.dump", lambda b: b.__setitem__(slice(first, first + 64), b"\xff" * 64)))
    with pytest.raises(xnb.XnbError):
        out = np.empty((10, 3))
        dump.write(tmp_path / "x.dump", out, dom=dump.domain(w["geom"]), compression_level=11)


def test_random_corruption_never_crashes(system, tmp_path):
    """Single-byte changes anywhere in the header, table or data: each read
    either succeeds or raises (the process must survive every one)."""
    w = system
    good = tmp_path / "f.dump"
    dump.write(good, w["r"][:600], w["v"][:600], w["id"][:600], w["type"][:600], dump.domain(w["geom"]),
               chunk_particles=200)
    blob = open(good, "rb").read()
    rng = np.random.default_rng(11)
    hot = [0, 8, 12, 16, 24, 1048, 5144, 5152, 5168 + 48, 5168 + 240, 5416, 5424, 5432, 5440, 5448]
    positions = [h + int(rng.integers(0, 8)) for h in hot for _ in range(4)]
    positions += [int(x) for x in rng.integers(5456, len(blob), size=120)]
    ok = 0
    for k, at in enumerate(positions):
        b = bytearray(blob)
        b[at] ^= int(rng.integers(1, 256))
        path = tmp_path / ("fz%d.dump" % k)
        open(path, "wb").write(bytes(b))
        try:
            dump.read(path)
            ok += 1
        except xnb.XnbError:
            pass
        os.remove(path)
    assert ok < len(positions)
