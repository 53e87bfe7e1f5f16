/*
 * xnb_dump.h -- dump/restart files in the reference's .dump format.
 *
 * One process writes and reads the files that exaNBody's write_dump /
 * read_dump operators exchange through MPI-IO (src/io/write_dump.cpp:39-44,
 * src/io/read_dump.cpp:38-45; format in src/io/include/exanb/io/sim_dump_io.h,
 * sim_dump_writer.h:104-480, sim_dump_reader.h:47-395; file parts and zlib
 * chunks in src/io/lib/mpi_file_io.cpp):
 *   * a SimDumpHeader of 5456 bytes: version 1.3 (1003), the field table (names
 *     of at most 31 characters, element sizes), the tuple size, particle count,
 *     time step, physical time, the Domain (248 bytes) and the offsets of the
 *     optional header, chunk table and particle data;
 *   * the optional header (empty here, as NullDumpOptionalFilter writes);
 *   * the chunk table: chunk_count entries {u64 offset, u32 bytes, i32
 *     particles}, sorted by offset, trailing entries {file size, 0, 0};
 *   * the chunks: per chunk, the particle fields as consecutive arrays
 *     (rx, ry, rz, vx, vy, vz, id, type: the field order of the write_dump /
 *     read_dump operators), zlib compress2 at the requested level, stored raw
 *     when the level is 0 or compression does not shrink them;
 *   * the logical file split into parts of max_part_size bytes named
 *     `file`, `file.1`, `file.2`, ...; a reader takes the split size from the
 *     size of `file`.
 * Version 1.2 and older files (Domain_legacy_v1_2, src/io/include/exanb/io/
 * domain_legacy_v1.2.h) are converted on read as SimDumpHeader::post_process does.
 *
 * zlib is loaded at run time (libz.so.1); without it only level-0 files can be
 * written and only raw chunks read (xnb_dump_zlib_available).
 * Errors return XNB_ERR_ARG or XNB_ERR_IO with a message in
 * xnb_last_error_string(); no call aborts on a malformed file.
 */
#ifndef XNB_DUMP_H
#define XNB_DUMP_H

#include <stdint.h>

#include "xnb_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define XNB_ERR_IO (-6) /* file missing, short, malformed or not writable */

#define XNB_DUMP_VERSION 1003 /* XNB_IO_MAKE_VERSION_NUMBER(1,3) */

/* Domain flag bits (core/include/exanb/core/domain.h:33-43) */
#define XNB_DOMAIN_PERIODIC_X (1u << 0)
#define XNB_DOMAIN_PERIODIC_Y (1u << 1)
#define XNB_DOMAIN_PERIODIC_Z (1u << 2)
#define XNB_DOMAIN_MIRROR_X_MIN (1u << 3)
#define XNB_DOMAIN_MIRROR_X_MAX (1u << 4)
#define XNB_DOMAIN_MIRROR_Y_MIN (1u << 5)
#define XNB_DOMAIN_MIRROR_Y_MAX (1u << 6)
#define XNB_DOMAIN_MIRROR_Z_MIN (1u << 7)
#define XNB_DOMAIN_MIRROR_Z_MAX (1u << 8)
#define XNB_DOMAIN_EXPANDABLE (1u << 16)
#define XNB_DOMAIN_XFORM_IDENTITY (1u << 17)

/* Fields present in a file (xnb_dump_info.field_mask) */
#define XNB_DUMP_F_RX (1u << 0)
#define XNB_DUMP_F_RY (1u << 1)
#define XNB_DUMP_F_RZ (1u << 2)
#define XNB_DUMP_F_VX (1u << 3)
#define XNB_DUMP_F_VY (1u << 4)
#define XNB_DUMP_F_VZ (1u << 5)
#define XNB_DUMP_F_ID (1u << 6)
#define XNB_DUMP_F_TYPE (1u << 7)

/* The reference's Domain (domain.h:96-105): bounds, grid dimensions, cell size,
 * transform and its inverse, transform scales, flag bits. */
typedef struct xnb_dump_domain {
  double bmin[3];
  double bmax[3];
  int64_t grid_dims[3];
  double cell_size;
  double xform[9]; /* row-major */
  double inv_xform[9];
  double xform_min_scale;
  double xform_max_scale;
  uint32_t flags;
} xnb_dump_domain;

typedef struct xnb_dump_info {
  uint64_t version;
  uint64_t n_particles;
  uint64_t timestep;
  double physical_time;
  uint64_t tuple_size;
  uint64_t chunk_count;  /* chunk table entries */
  uint64_t data_chunks;  /* non-empty entries */
  uint64_t file_bytes;   /* logical size over all parts */
  uint64_t part_size;    /* split size (size of the first part) */
  int32_t n_fields;
  uint32_t field_mask;   /* XNB_DUMP_F_* of the fields present */
  xnb_dump_domain domain;
} xnb_dump_info;

/* 1 when zlib could be loaded (compressed chunks readable and writable). */
int xnb_dump_zlib_available(void);

/* A domain with identity transform, the given bounds, grid and cell size, and
 * the flags (XNB_DOMAIN_*; the identity bit is added). */
void xnb_dump_domain_init(xnb_dump_domain* d, const double bmin[3], const double bmax[3], const int64_t dims[3],
                          double cell_size, uint32_t flags);

/* Writes n particles in the order given (write_dump writes interior cells in
 * grid order, each cell's particles in storage order). vx..type may be NULL
 * (zeros; id NULL = 0, 1, 2, ...). With cell_counts (n_cells entries summing to
 * n) a chunk is closed at the first cell boundary at or after chunk_particles
 * particles, as each writer thread does (sim_dump_writer.h:262-341); otherwise
 * every chunk_particles particles. chunk_particles <= 0: 65536.
 * compression_level: 0 (raw) .. 9, -1 zlib default; the reference's default is 6.
 * max_part_size <= 0: 128 GiB (MpiIO::DEFAULT_MAX_FILE_SIZE). threads <= 0: all
 * hardware threads compress chunks. */
int xnb_dump_write(const char* filename, const xnb_dump_domain* domain, uint64_t timestep, double physical_time,
                   int64_t n, const double* rx, const double* ry, const double* rz, const double* vx,
                   const double* vy, const double* vz, const uint64_t* id, const uint8_t* type,
                   const int64_t* cell_counts, int64_t n_cells, int32_t compression_level, int64_t max_part_size,
                   int64_t chunk_particles, int32_t threads);

/* Header, domain and chunk table of a file (no particle data read). */
int xnb_dump_read_info(const char* filename, xnb_dump_info* info);

/* All particles in file order into arrays of cap entries (any of vx..type may
 * be NULL; fields absent from the file read as 0). *n_out = particles read.
 * info may be NULL. XNB_ERR_ARG when the file holds more than cap particles. */
int xnb_dump_read(const char* filename, int64_t cap, double* rx, double* ry, double* rz, double* vx, double* vy,
                  double* vz, uint64_t* id, uint8_t* type, int64_t* n_out, xnb_dump_info* info);

/* write_dump for one resident system: its particles in storage order, with
 * the system's domain (bounds, grid, cell size, periodic in x, y, z;
 * expandable unless cleared in extra_flags_clear). Synchronises. */
int xnb_system_write_dump(xnb_batch* b, int32_t sys, const char* filename, uint64_t timestep, double physical_time,
                          int32_t compression_level, int64_t max_part_size, uint32_t extra_flags_clear,
                          void* stream);

/* Particle types of one system in storage order. Synchronises. */
int xnb_system_download_types(xnb_batch* b, int32_t sys, uint8_t* type, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* XNB_DUMP_H */
