// .dump files (include/xnb_dump.h): the reference's SimDumpHeader, chunk table
// and zlib chunks (src/io/include/exanb/io/sim_dump_io.h:90-163, sim_dump_writer.h,
// sim_dump_reader.h, src/io/lib/mpi_file_io.cpp), written and read by one
// process. Host code only; zlib is bound at run time.
#include <dlfcn.h>
#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <exception>
#include <string>
#include <thread>
#include <vector>

#include "../../include/xnb_dump.h"

namespace xnb {
int set_error(int code, const std::string& msg);
}

namespace {

using xnb::set_error;

// ---------------------------------------------------------------------------
// SimDumpHeader byte layout (natural alignment of its members on LP64):
//   m_version u64 @0, m_nb_fields u32 @8, m_data_flags u8[4] @12,
//   m_tuple_size u64 @16, m_field_size u64[128] @24, m_fields char[128][32] @1048,
//   m_nb_particles u64 @5144, m_time_step u64 @5152, m_time f64 @5160,
//   m_domain Domain @5168 (248 bytes), m_optional_offset @5416, m_table_offset
//   @5424, m_data_offset @5432, m_optional_header_size @5440, m_chunk_count @5448.
constexpr uint64_t kVersion = XNB_DUMP_VERSION;
constexpr uint32_t kMaxFields = 128;
constexpr uint32_t kStrMaxLen = 32;
constexpr size_t kHVersion = 0, kHNbFields = 8, kHDataFlags = 12, kHTupleSize = 16, kHFieldSize = 24,
                 kHFields = kHFieldSize + 8 * kMaxFields, kHNbParticles = kHFields + kMaxFields * kStrMaxLen,
                 kHTimeStep = kHNbParticles + 8, kHTime = kHTimeStep + 8, kHDomain = kHTime + 8,
                 kDomainBytes = 248, kHOptOffset = kHDomain + kDomainBytes, kHTableOffset = kHOptOffset + 8,
                 kHDataOffset = kHTableOffset + 8, kHOptSize = kHDataOffset + 8, kHChunkCount = kHOptSize + 8,
                 kHeaderBytes = kHChunkCount + 8;
static_assert(kHFields == 1048 && kHDomain == 5168 && kHeaderBytes == 5456, "SimDumpHeader layout");

// Domain (core/include/exanb/core/domain.h:96-105): AABB (2 x Vec3d) @0,
// IJK (3 x ssize_t) @48, cell size @72, xform (Mat3d) @80, inverse @152, min and
// max scale @224/@232, then version 1.3: u32 flags @240 + u32 padding;
// version <= 1.2 (domain_legacy_v1.2.h:36-49): bool xform_is_identity @240,
// bool periodic[3] @241, bool expandable @244.
constexpr size_t kDBmin = 0, kDBmax = 24, kDDims = 48, kDCell = 72, kDXform = 80, kDInv = 152, kDMinScale = 224,
                 kDMaxScale = 232, kDFlags = 240;

constexpr size_t kChunkItemBytes = 16;  // DataChunkItem {u64 offset, u32 bytes, i32 particles}
constexpr int64_t kWriteBufferSize = 65536;
constexpr uint64_t kDefaultMaxFileSize = 128ull * 1024ull * 1024ull * 1024ull;
constexpr size_t kAlign = 8;  // FieldArrays<8, 1, ...>: each field array starts on 8 bytes

template <class T>
void put(std::vector<uint8_t>& b, size_t off, const T& v) {
  std::memcpy(b.data() + off, &v, sizeof(T));
}
template <class T>
T get(const uint8_t* b, size_t off) {
  T v;
  std::memcpy(&v, b + off, sizeof(T));
  return v;
}

size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// ---------------------------------------------------------------------------
// zlib (compress2 / uncompress, as MpiIO::compress_buffer / uncompress_buffer)
struct Zlib {
  using compress2_t = int (*)(unsigned char*, unsigned long*, const unsigned char*, unsigned long, int);
  using uncompress_t = int (*)(unsigned char*, unsigned long*, const unsigned char*, unsigned long);
  using bound_t = unsigned long (*)(unsigned long);
  compress2_t compress2 = nullptr;
  uncompress_t uncompress = nullptr;
  bound_t bound = nullptr;
  bool ok = false;
};

const Zlib& zlib() {
  static const Zlib z = [] {
    Zlib r;
    void* h = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!h) h = dlopen("libz.so", RTLD_NOW | RTLD_LOCAL);
    if (h) {
      r.compress2 = reinterpret_cast<Zlib::compress2_t>(dlsym(h, "compress2"));
      r.uncompress = reinterpret_cast<Zlib::uncompress_t>(dlsym(h, "uncompress"));
      r.bound = reinterpret_cast<Zlib::bound_t>(dlsym(h, "compressBound"));
      r.ok = r.compress2 && r.uncompress && r.bound;
    }
    return r;
  }();
  return z;
}

// ---------------------------------------------------------------------------
// The logical file over its parts: part k > 0 is named "<file>.<k>" and holds
// bytes [k * part, (k + 1) * part) (MpiIO::read_bytes / write_bytes).
class PartFile {
 public:
  ~PartFile() { close(); }
  bool open_write(const std::string& base, uint64_t part) {
    base_ = base;
    part_ = part;
    write_ = true;
    return file(0) != nullptr;
  }
  bool open_read(const std::string& base) {
    base_ = base;
    write_ = false;
    struct stat sb;
    if (stat(base.c_str(), &sb) != 0) return false;
    part_ = static_cast<uint64_t>(sb.st_size);
    total_ = part_;
    for (size_t k = 1; stat(part_name(k).c_str(), &sb) == 0; ++k) total_ += static_cast<uint64_t>(sb.st_size);
    return part_ > 0 && file(0) != nullptr;
  }
  uint64_t part_size() const { return part_; }
  uint64_t total_size() const { return total_; }  // bytes over the parts present (read mode)
  size_t parts_used() const { return files_.size(); }
  bool write(uint64_t off, const void* src, size_t n) { return io(off, const_cast<void*>(src), n); }
  bool read(uint64_t off, void* dst, size_t n) { return io(off, dst, n); }
  bool close() {
    bool ok = true;
    for (FILE*& f : files_)
      if (f) {
        ok = (std::fclose(f) == 0) && ok;
        f = nullptr;
      }
    return ok;
  }
  std::string part_name(size_t k) const { return k == 0 ? base_ : base_ + "." + std::to_string(k); }

 private:
  FILE* file(size_t k) {
    if (k >= files_.size()) files_.resize(k + 1, nullptr);
    if (!files_[k]) files_[k] = std::fopen(part_name(k).c_str(), write_ ? "w+b" : "rb");
    return files_[k];
  }
  bool io(uint64_t off, void* buf, size_t n) {
    uint8_t* p = static_cast<uint8_t*>(buf);
    while (n > 0) {
      const uint64_t k = off / part_, o = off % part_;
      const size_t m = static_cast<size_t>(std::min<uint64_t>(n, part_ - o));
      FILE* f = file(static_cast<size_t>(k));
      if (!f || fseeko(f, static_cast<off_t>(o), SEEK_SET) != 0) return false;
      const size_t done = write_ ? std::fwrite(p, 1, m, f) : std::fread(p, 1, m, f);
      if (done != m) return false;
      p += m;
      off += m;
      n -= m;
    }
    return true;
  }
  std::string base_;
  uint64_t part_ = kDefaultMaxFileSize;
  uint64_t total_ = 0;
  bool write_ = false;
  std::vector<FILE*> files_;
};

// ---------------------------------------------------------------------------
struct Field {
  const char* name;
  uint32_t size;
};
// write_dump / read_dump field set, in FieldSet order (write_dump.cpp:37, read_dump.cpp:38;
// FieldSetIntersection keeps the order of the dump field list, field_set_utils.h:229-244)
constexpr Field kDumpFields[8] = {{"rx", 8}, {"ry", 8}, {"rz", 8}, {"vx", 8},
                                  {"vy", 8}, {"vz", 8}, {"id", 8}, {"type", 1}};
// sizeof(FieldTuple<rx, ry, rz, vx, vy, vz, id, type>): 57 bytes of members, 8-aligned
constexpr uint64_t kDumpTupleSize = 64;

// Array offsets of one chunk of n particles (each field array starts on kAlign bytes).
struct ChunkLayout {
  std::vector<size_t> offset;
  size_t unpadded = 0, padded = 0;
};
ChunkLayout chunk_layout(const std::vector<uint32_t>& sizes, size_t n) {
  ChunkLayout L;
  size_t at = 0;
  for (uint32_t s : sizes) {
    at = align_up(at);
    L.offset.push_back(at);
    at += n * s;
  }
  L.unpadded = at;
  L.padded = align_up(at);
  return L;
}

void encode_domain(std::vector<uint8_t>& h, const xnb_dump_domain& d) {
  const size_t b = kHDomain;
  for (int a = 0; a < 3; ++a) {
    put(h, b + kDBmin + 8 * a, d.bmin[a]);
    put(h, b + kDBmax + 8 * a, d.bmax[a]);
    put(h, b + kDDims + 8 * a, d.grid_dims[a]);
  }
  put(h, b + kDCell, d.cell_size);
  for (int k = 0; k < 9; ++k) {
    put(h, b + kDXform + 8 * k, d.xform[k]);
    put(h, b + kDInv + 8 * k, d.inv_xform[k]);
  }
  put(h, b + kDMinScale, d.xform_min_scale);
  put(h, b + kDMaxScale, d.xform_max_scale);
  put(h, b + kDFlags, d.flags);
  put(h, b + kDFlags + 4, static_cast<uint32_t>(0));
}

bool is_identity(const double* m) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      if (m[3 * r + c] != (r == c ? 1.0 : 0.0)) return false;
  return true;
}

// Domain of a header; version < 1.3 holds Domain_legacy_v1_2 and is converted
// as SimDumpHeader::post_process does (sim_dump_io.h:131-160): mirrors off,
// periodic and expandable from the legacy bools, the identity bit and the
// scales from set_xform (domain.cpp:27-44; scales 1 for the identity).
void decode_domain(const uint8_t* h, uint64_t version, xnb_dump_domain& d) {
  const size_t b = kHDomain;
  for (int a = 0; a < 3; ++a) {
    d.bmin[a] = get<double>(h, b + kDBmin + 8 * a);
    d.bmax[a] = get<double>(h, b + kDBmax + 8 * a);
    d.grid_dims[a] = get<int64_t>(h, b + kDDims + 8 * a);
  }
  d.cell_size = get<double>(h, b + kDCell);
  for (int k = 0; k < 9; ++k) {
    d.xform[k] = get<double>(h, b + kDXform + 8 * k);
    d.inv_xform[k] = get<double>(h, b + kDInv + 8 * k);
  }
  d.xform_min_scale = get<double>(h, b + kDMinScale);
  d.xform_max_scale = get<double>(h, b + kDMaxScale);
  if (version >= 1003) {
    d.flags = get<uint32_t>(h, b + kDFlags);
    return;
  }
  uint32_t f = 0;
  for (int a = 0; a < 3; ++a)
    if (h[b + kDFlags + 1 + a]) f |= XNB_DOMAIN_PERIODIC_X << a;
  bool expandable = h[b + kDFlags + 4] != 0;
  if (version < 1002) expandable = true;  // 1.1 -> 1.2: forced true for backward compatibility
  if (expandable) f |= XNB_DOMAIN_EXPANDABLE;
  if (is_identity(d.xform)) {
    f |= XNB_DOMAIN_XFORM_IDENTITY;
    std::memcpy(d.inv_xform, d.xform, sizeof(d.xform));
    d.xform_min_scale = d.xform_max_scale = 1.0;
  }
  d.flags = f;
}

struct Chunk {
  int64_t first = 0, n = 0;
  std::vector<uint8_t> data;  // what goes into the file
  uint64_t raw = 0;
};

int compress_chunk(Chunk& c, const std::vector<const void*>& src, int level) {
  std::vector<uint32_t> sizes;
  for (const Field& f : kDumpFields) sizes.push_back(f.size);
  const ChunkLayout L = chunk_layout(sizes, static_cast<size_t>(c.n));
  std::vector<uint8_t> raw(L.padded, 0);
  for (size_t k = 0; k < sizes.size(); ++k) {
    uint8_t* dst = raw.data() + L.offset[k];
    const size_t bytes = static_cast<size_t>(c.n) * sizes[k];
    if (src[k]) {
      std::memcpy(dst, static_cast<const uint8_t*>(src[k]) + static_cast<size_t>(c.first) * sizes[k], bytes);
    } else if (k == 6) {  // id absent: the particle's index in the file
      for (int64_t q = 0; q < c.n; ++q) {
        const uint64_t v = static_cast<uint64_t>(c.first + q);
        std::memcpy(dst + 8 * q, &v, 8);
      }
    }
  }
  c.raw = raw.size();
  if (level == 0 || raw.empty()) {
    c.data.swap(raw);
    return 0;
  }
  const Zlib& z = zlib();
  unsigned long cs = z.bound(static_cast<unsigned long>(raw.size()));
  c.data.resize(cs);
  if (z.compress2(c.data.data(), &cs, raw.data(), static_cast<unsigned long>(raw.size()), level) != 0) return -1;
  if (cs >= raw.size()) {
    c.data.swap(raw);  // failed to shrink: raw data (MpiIO::compress_buffer)
  } else {
    c.data.resize(cs);
  }
  return 0;
}

}  // namespace

extern "C" {

int xnb_dump_zlib_available(void) { return zlib().ok ? 1 : 0; }

void xnb_dump_domain_init(xnb_dump_domain* d, const double bmin[3], const double bmax[3], const int64_t dims[3],
                          double cell_size, uint32_t flags) {
  std::memset(d, 0, sizeof(*d));
  for (int a = 0; a < 3; ++a) {
    d->bmin[a] = bmin[a];
    d->bmax[a] = bmax[a];
    d->grid_dims[a] = dims[a];
  }
  d->cell_size = cell_size;
  for (int k = 0; k < 9; ++k) d->xform[k] = d->inv_xform[k] = (k % 4 == 0) ? 1.0 : 0.0;
  d->xform_min_scale = d->xform_max_scale = 1.0;
  d->flags = flags | XNB_DOMAIN_XFORM_IDENTITY;
}

namespace {
int dump_write(const char* filename, const xnb_dump_domain* domain, uint64_t timestep, double physical_time,
               int64_t n, const double* rx, const double* ry, const double* rz, const double* vx, const double* vy,
               const double* vz, const uint64_t* id, const uint8_t* type, const int64_t* cell_counts,
               int64_t n_cells, int32_t compression_level, int64_t max_part_size, int64_t chunk_particles,
               int32_t threads) {
  if (!filename || !domain || n < 0 || (n > 0 && (!rx || !ry || !rz)))
    return set_error(XNB_ERR_ARG, "xnb_dump_write: filename, domain and positions are required");
  if (compression_level < -1 || compression_level > 9)
    return set_error(XNB_ERR_ARG, "xnb_dump_write: compression_level must be in [-1, 9]");
  if (compression_level != 0 && !zlib().ok)
    return set_error(XNB_ERR_IO, "xnb_dump_write: zlib (libz.so.1) not found; use compression_level 0");
  const int64_t per_chunk = chunk_particles > 0 ? chunk_particles : kWriteBufferSize;
  const uint64_t part = max_part_size > 0 ? static_cast<uint64_t>(max_part_size) : kDefaultMaxFileSize;
  int nt = threads > 0 ? threads : static_cast<int>(std::thread::hardware_concurrency());
  nt = std::max(1, std::min(nt, 64));

  // chunk boundaries: whole cells up to at least per_chunk particles, or fixed runs
  std::vector<std::pair<int64_t, int64_t>> spans;  // (first, count)
  if (cell_counts && n_cells > 0) {
    int64_t total = 0;
    for (int64_t c = 0; c < n_cells; ++c) {
      if (cell_counts[c] < 0) return set_error(XNB_ERR_ARG, "xnb_dump_write: negative cell count");
      total += cell_counts[c];
    }
    if (total != n) return set_error(XNB_ERR_ARG, "xnb_dump_write: cell counts do not sum to n");
    int64_t first = 0, acc = 0;
    for (int64_t c = 0; c < n_cells; ++c) {
      acc += cell_counts[c];
      if (acc >= per_chunk) {
        spans.emplace_back(first, acc);
        first += acc;
        acc = 0;
      }
    }
    if (acc > 0) spans.emplace_back(first, acc);
  } else {
    for (int64_t f = 0; f < n; f += per_chunk) spans.emplace_back(f, std::min(per_chunk, n - f));
  }
  for (const auto& s : spans)
    if (s.second > INT32_MAX) return set_error(XNB_ERR_ARG, "xnb_dump_write: a chunk exceeds 2^31 particles");

  // header (sim_dump_writer.h:114-127, 203-233): chunk table sized for the writer
  // threads plus one chunk per WRITE_BUFFER_SIZE particles plus the end marker
  const uint64_t chunk_count = static_cast<uint64_t>(nt) + static_cast<uint64_t>(n / per_chunk) + 1;
  std::vector<uint8_t> h(kHeaderBytes, 0);
  put(h, kHVersion, kVersion);
  put(h, kHNbFields, static_cast<uint32_t>(8));
  put(h, kHTupleSize, kDumpTupleSize);
  for (uint32_t k = 0; k < 8; ++k) {
    put(h, kHFieldSize + 8 * k, static_cast<uint64_t>(kDumpFields[k].size));
    std::strncpy(reinterpret_cast<char*>(h.data() + kHFields + kStrMaxLen * k), kDumpFields[k].name, kStrMaxLen - 1);
  }
  put(h, kHNbParticles, static_cast<uint64_t>(n));
  put(h, kHTimeStep, timestep);
  put(h, kHTime, physical_time);
  encode_domain(h, *domain);
  const uint64_t opt_offset = kHeaderBytes;
  const uint64_t table_offset = opt_offset;  // empty optional header
  const uint64_t data_offset = table_offset + chunk_count * kChunkItemBytes;
  put(h, kHOptOffset, opt_offset);
  put(h, kHTableOffset, table_offset);
  put(h, kHDataOffset, data_offset);
  put(h, kHOptSize, static_cast<uint64_t>(0));
  put(h, kHChunkCount, chunk_count);

  PartFile file;
  if (!file.open_write(filename, part))
    return set_error(XNB_ERR_IO, std::string("xnb_dump_write: cannot create ") + filename + ": " + std::strerror(errno));
  if (!file.write(0, h.data(), h.size())) return set_error(XNB_ERR_IO, "xnb_dump_write: write failed (header)");

  const std::vector<const void*> src = {rx, ry, rz, vx, vy, vz, id, type};
  std::vector<uint8_t> table(chunk_count * kChunkItemBytes, 0);
  uint64_t at = data_offset;
  size_t next = 0;
  // chunks compressed nt at a time in parallel, written in order
  for (size_t s0 = 0; s0 < spans.size(); s0 += static_cast<size_t>(nt)) {
    const size_t s1 = std::min(spans.size(), s0 + static_cast<size_t>(nt));
    std::vector<Chunk> chunks(s1 - s0);
    std::vector<int> rc(s1 - s0, 0);
    for (size_t s = s0; s < s1; ++s) {
      chunks[s - s0].first = spans[s].first;
      chunks[s - s0].n = spans[s].second;
    }
    std::vector<std::thread> pool;
    for (size_t t = 0; t < chunks.size(); ++t)
      pool.emplace_back([&, t] { rc[t] = compress_chunk(chunks[t], src, compression_level); });
    for (auto& th : pool) th.join();
    for (size_t t = 0; t < chunks.size(); ++t) {
      if (rc[t]) return set_error(XNB_ERR_IO, "xnb_dump_write: compression failed");
      const Chunk& c = chunks[t];
      if (!file.write(at, c.data.data(), c.data.size()))
        return set_error(XNB_ERR_IO, "xnb_dump_write: write failed (chunk data)");
      put(table, next * kChunkItemBytes, at);
      put(table, next * kChunkItemBytes + 8, static_cast<uint32_t>(c.data.size()));
      put(table, next * kChunkItemBytes + 12, static_cast<int32_t>(c.n));
      ++next;
      at += c.data.size();
    }
  }
  for (; next < chunk_count; ++next) {  // end markers {file size, 0, 0}
    put(table, next * kChunkItemBytes, at);
    put(table, next * kChunkItemBytes + 8, static_cast<uint32_t>(0));
    put(table, next * kChunkItemBytes + 12, static_cast<int32_t>(0));
  }
  if (!table.empty() && !file.write(table_offset, table.data(), table.size()))
    return set_error(XNB_ERR_IO, "xnb_dump_write: write failed (chunk table)");
  const size_t used = std::max<size_t>(1, static_cast<size_t>((at + part - 1) / part));
  if (!file.close()) return set_error(XNB_ERR_IO, "xnb_dump_write: close failed");
  // parts beyond the written ones, left by an earlier larger file of the same
  // name, are removed as MpiIO::close removes its unused pre-opened parts
  for (size_t k = used; k < used + 4; ++k) std::remove(file.part_name(k).c_str());
  return XNB_OK;
}
}  // namespace

int xnb_dump_write(const char* filename, const xnb_dump_domain* domain, uint64_t timestep, double physical_time,
                   int64_t n, const double* rx, const double* ry, const double* rz, const double* vx,
                   const double* vy, const double* vz, const uint64_t* id, const uint8_t* type,
                   const int64_t* cell_counts, int64_t n_cells, int32_t compression_level, int64_t max_part_size,
                   int64_t chunk_particles, int32_t threads) {
  try {
    return dump_write(filename, domain, timestep, physical_time, n, rx, ry, rz, vx, vy, vz, id, type, cell_counts,
                      n_cells, compression_level, max_part_size, chunk_particles, threads);
  } catch (const std::exception& e) {
    return set_error(XNB_ERR_IO, std::string("xnb_dump_write: ") + e.what());
  }
}

namespace {

struct Reader {
  PartFile file;
  xnb_dump_info info{};
  std::vector<std::string> names;
  std::vector<uint32_t> sizes;
  std::vector<uint8_t> table;

  int open(const char* filename) {
    if (!filename) return set_error(XNB_ERR_ARG, "xnb_dump_read: filename required");
    if (!file.open_read(filename)) return set_error(XNB_ERR_IO, std::string("xnb_dump_read: cannot open ") + filename);
    if (file.part_size() < kHeaderBytes) return set_error(XNB_ERR_IO, "xnb_dump_read: file shorter than its header");
    std::vector<uint8_t> h(kHeaderBytes);
    if (!file.read(0, h.data(), h.size())) return set_error(XNB_ERR_IO, "xnb_dump_read: cannot read the header");
    info.version = get<uint64_t>(h.data(), kHVersion);
    if (info.version > kVersion || info.version < 1000)
      return set_error(XNB_ERR_IO, "xnb_dump_read: bad version number " + std::to_string(info.version));
    const uint32_t nf = get<uint32_t>(h.data(), kHNbFields);
    if (nf == 0 || nf > kMaxFields) return set_error(XNB_ERR_IO, "xnb_dump_read: bad field count");
    info.n_fields = static_cast<int32_t>(nf);
    info.tuple_size = get<uint64_t>(h.data(), kHTupleSize);
    for (uint32_t k = 0; k < nf; ++k) {
      const char* s = reinterpret_cast<const char*>(h.data() + kHFields + kStrMaxLen * k);
      const size_t len = strnlen(s, kStrMaxLen);
      if (len == kStrMaxLen) return set_error(XNB_ERR_IO, "xnb_dump_read: unterminated field name");
      names.emplace_back(s, len);
      const uint64_t sz = get<uint64_t>(h.data(), kHFieldSize + 8 * k);
      if (sz == 0 || sz > 4096) return set_error(XNB_ERR_IO, "xnb_dump_read: bad size of field " + names.back());
      sizes.push_back(static_cast<uint32_t>(sz));
      for (uint32_t j = 0; j < k; ++j)
        if (names[j] == names.back()) return set_error(XNB_ERR_IO, "xnb_dump_read: field listed twice");
      for (int f = 0; f < 8; ++f)
        if (names.back() == kDumpFields[f].name) {
          if (sz != kDumpFields[f].size)
            return set_error(XNB_ERR_IO, "xnb_dump_read: field " + names.back() + " has an unexpected size");
          info.field_mask |= 1u << f;
        }
    }
    const uint32_t need = XNB_DUMP_F_RX | XNB_DUMP_F_RY | XNB_DUMP_F_RZ;
    if ((info.field_mask & need) != need) return set_error(XNB_ERR_IO, "xnb_dump_read: no rx/ry/rz fields");
    info.n_particles = get<uint64_t>(h.data(), kHNbParticles);
    info.timestep = get<uint64_t>(h.data(), kHTimeStep);
    info.physical_time = get<double>(h.data(), kHTime);
    decode_domain(h.data(), info.version, info.domain);
    const uint64_t opt_off = get<uint64_t>(h.data(), kHOptOffset);
    const uint64_t table_off = get<uint64_t>(h.data(), kHTableOffset);
    const uint64_t data_off = get<uint64_t>(h.data(), kHDataOffset);
    info.chunk_count = get<uint64_t>(h.data(), kHChunkCount);
    if (opt_off != kHeaderBytes || table_off < opt_off || info.chunk_count > file.total_size() / kChunkItemBytes ||
        data_off != table_off + info.chunk_count * kChunkItemBytes || data_off > file.total_size())
      return set_error(XNB_ERR_IO, "xnb_dump_read: inconsistent header offsets");
    info.part_size = file.part_size();
    table.resize(info.chunk_count * kChunkItemBytes);
    if (!table.empty() && !file.read(table_off, table.data(), table.size()))
      return set_error(XNB_ERR_IO, "xnb_dump_read: cannot read the chunk table");
    // the reader's consistency checks (sim_dump_reader.h:160-190)
    uint64_t last = data_off, total = 0;
    bool ended = false;
    info.file_bytes = data_off;
    for (uint64_t i = 0; i < info.chunk_count; ++i) {
      const uint64_t off = get<uint64_t>(table.data(), i * kChunkItemBytes);
      const uint32_t bytes = get<uint32_t>(table.data(), i * kChunkItemBytes + 8);
      const int32_t np = get<int32_t>(table.data(), i * kChunkItemBytes + 12);
      const bool empty = bytes == 0 && np == 0;
      if ((!empty && (bytes == 0 || np == 0)) || off < last || (ended && !empty) ||
          (!empty && np > 0 && off + bytes > file.total_size()))
        return set_error(XNB_ERR_IO, "xnb_dump_read: file corrupted, inconsistent chunk #" + std::to_string(i));
      last = off;
      if (empty) {
        ended = true;
        info.file_bytes = std::max(info.file_bytes, off);
        continue;
      }
      ++info.data_chunks;
      total += static_cast<uint64_t>(np < 0 ? -static_cast<int64_t>(np) : np);
      info.file_bytes = std::max(info.file_bytes, off + (np > 0 ? bytes : 0));
    }
    if (total != info.n_particles)
      return set_error(XNB_ERR_IO, "xnb_dump_read: chunk particle counts do not add up to the header's");
    return XNB_OK;
  }

  uint64_t entry_off(uint64_t i) const { return get<uint64_t>(table.data(), i * kChunkItemBytes); }

  int read_all(int64_t cap, void* const out[8], int64_t* n_out) {
    if (static_cast<uint64_t>(cap) < info.n_particles)
      return set_error(XNB_ERR_ARG, "xnb_dump_read: " + std::to_string(info.n_particles) +
                                        " particles do not fit the arrays");
    const Zlib& z = zlib();
    int64_t at = 0;
    std::vector<uint8_t> comp, raw;
    for (uint64_t i = 0; i < info.chunk_count; ++i) {
      const uint64_t off = entry_off(i);
      const uint32_t bytes = get<uint32_t>(table.data(), i * kChunkItemBytes + 8);
      const int32_t np = get<int32_t>(table.data(), i * kChunkItemBytes + 12);
      if (bytes == 0 && np == 0) continue;
      const size_t n = static_cast<size_t>(np < 0 ? -static_cast<int64_t>(np) : np);
      const ChunkLayout L = chunk_layout(sizes, n);
      // A chunk is stored raw when its stored size equals its raw size
      // (sim_dump_reader.h:216-262). The raw size of n particles is the field
      // arrays' storage, taken as 8-byte padded; a file whose writer did not pad
      // the last array stores `unpadded` bytes raw, and such a chunk is told from
      // a compressed one of the same size by whether it inflates.
      size_t comp_size, raw_size;
      int mode;  // 0 raw, 1 compressed, 2 raw or compressed
      if (np > 0) {  // bytes = stored size; raw size from the particle count
        comp_size = bytes;
        raw_size = L.padded;
        mode = bytes == L.padded ? 0 : (bytes == L.unpadded ? 2 : 1);
      } else {  // optional data follows: bytes = raw size, stored size from the next offset
        if (i + 1 >= info.chunk_count) return set_error(XNB_ERR_IO, "xnb_dump_read: chunk table missing its end");
        raw_size = bytes;
        comp_size = static_cast<size_t>(entry_off(i + 1) - off);
        mode = comp_size == raw_size ? 0 : 1;
        if (raw_size < L.unpadded) return set_error(XNB_ERR_IO, "xnb_dump_read: chunk smaller than its particles");
      }
      // bounds before any allocation: the stored bytes lie in the file, and
      // inflation cannot exceed deflate's largest ratio (1032:1)
      if (off + comp_size > file.total_size() || raw_size > 1032 * comp_size + 1024 ||
          (mode == 0 && raw_size != comp_size))
        return set_error(XNB_ERR_IO, "xnb_dump_read: chunk #" + std::to_string(i) + " exceeds the file");
      comp.resize(comp_size);
      if (!file.read(off, comp.data(), comp.size())) return set_error(XNB_ERR_IO, "xnb_dump_read: short chunk");
      bool inflated = false;
      if (mode != 0 && z.ok) {
        raw.assign(raw_size, 0);
        unsigned long got = static_cast<unsigned long>(raw.size());
        inflated = z.uncompress(raw.data(), &got, comp.data(), static_cast<unsigned long>(comp.size())) == 0 &&
                   got >= L.unpadded;
      }
      if (!inflated) {
        if (mode == 1) {
          return set_error(XNB_ERR_IO, z.ok ? "xnb_dump_read: decompression failed in chunk #" + std::to_string(i)
                                            : std::string("xnb_dump_read: compressed chunk and no zlib (libz.so.1)"));
        }
        raw.swap(comp);
      }
      for (size_t k = 0; k < names.size(); ++k) {
        for (int f = 0; f < 8; ++f) {
          if (names[k] != kDumpFields[f].name || !out[f]) continue;
          std::memcpy(static_cast<uint8_t*>(out[f]) + static_cast<size_t>(at) * sizes[k], raw.data() + L.offset[k],
                      n * sizes[k]);
        }
      }
      at += static_cast<int64_t>(n);
    }
    *n_out = at;
    return XNB_OK;
  }
};

}  // namespace

int xnb_dump_read_info(const char* filename, xnb_dump_info* info) {
  if (!info) return set_error(XNB_ERR_ARG, "xnb_dump_read_info: info required");
  try {
    Reader r;
    const int rc = r.open(filename);
    if (rc) return rc;
    *info = r.info;
    return XNB_OK;
  } catch (const std::exception& e) {
    return set_error(XNB_ERR_IO, std::string("xnb_dump_read_info: ") + e.what());
  }
}

int xnb_dump_read(const char* filename, int64_t cap, double* rx, double* ry, double* rz, double* vx, double* vy,
                  double* vz, uint64_t* id, uint8_t* type, int64_t* n_out, xnb_dump_info* info) {
  if (!n_out || cap < 0 || !rx || !ry || !rz)
    return set_error(XNB_ERR_ARG, "xnb_dump_read: positions and n_out required");
  try {
    Reader r;
    int rc = r.open(filename);
    if (rc) return rc;
    const uint64_t n = r.info.n_particles;
    if (static_cast<uint64_t>(cap) < n)
      return set_error(XNB_ERR_ARG, "xnb_dump_read: " + std::to_string(n) + " particles do not fit the arrays");
    // fields absent from the file read as zero
    void* const outs[8] = {rx, ry, rz, vx, vy, vz, id, type};
    for (int f = 3; f < 8; ++f)
      if (outs[f] && !(r.info.field_mask & (1u << f))) std::memset(outs[f], 0, n * kDumpFields[f].size);
    rc = r.read_all(cap, outs, n_out);
    if (rc) return rc;
    if (info) *info = r.info;
    return XNB_OK;
  } catch (const std::exception& e) {
    return set_error(XNB_ERR_IO, std::string("xnb_dump_read: ") + e.what());
  }
}

}  // extern "C"
