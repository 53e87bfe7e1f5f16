// The reference's chunk-neighbour stream format (chunk size 1) and its checker,
// shared by the device kernels (xnb_stream.cu) and a host test compiled with g++
// (tests/test_stream_check.py).
//
// Format, per cell with na > 0 particles (chunk_neighbors_execute.h:249-398,
// decoded by chunknbh_stream_info, chunk_neighbors.h:166-182):
//   * T in {0, 1, 2} offset tables of u32 stored as u16 pairs, (na*T + 1)*2 u16
//     when T >= 1: table 1 holds, for particle p, the start of its sub-stream
//     relative to the end of the tables plus T (so that stream[0] = T and
//     stream[1] = 0 identify the tables), and entry na closes it with the total
//     length plus T; table 2 holds per particle the number of its neighbours that
//     precede it in grid order ((cell_b, p_b) < (cell_a, p_a)).
//   * per particle: the number of neighbour cells G, then G groups of
//     (encoded relative cell, count, count particle indices), cells in increasing
//     encoding order, particle indices increasing within a cell.
// A relative cell (di, dj, dk) in [-15, 15]^3 is encoded in 5-bit fields as
// ((dk + 16) << 10) | ((dj + 16) << 5) | (di + 16) (chunk_neighbors.h:137-151).
// Particle indices of a ghost (periodic image) cell count only the owner cell's
// particles that pass the ghost filter, in the owner's order.
#pragma once

#include <cstdint>

#ifndef __CUDACC__
#define XNB_SHD inline
#else
#define XNB_SHD __host__ __device__ __forceinline__
#endif

namespace xnb {

XNB_SHD uint16_t encode_cell_rel(int di, int dj, int dk) {
  return static_cast<uint16_t>((((dk + 16) << 5 | (dj + 16)) << 5) | (di + 16));
}

// Inverse of encode_cell_rel; false unless every component is in [-1, 1] (one
// layer of neighbour cells, the only layout this library builds).
XNB_SHD bool decode_cell_rel(uint16_t e, int& di, int& dj, int& dk) {
  di = static_cast<int>(e & 31u) - 16;
  dj = static_cast<int>((e >> 5) & 31u) - 16;
  dk = static_cast<int>((e >> 10) & 31u) - 16;
  return (e >> 15) == 0u && di >= -1 && di <= 1 && dj >= -1 && dj <= 1 && dk >= -1 && dk <= 1;
}

// Violation counts of verify_chunk_neighbors (particle_neighbors/verify_chunk_neighbors.cpp:58-168)
// plus the checks a decoder needs: format (tables, lengths, reads past the
// stream), order (cells not increasing, indices not increasing within a cell,
// second-table mismatch), self (a particle listing itself), range (cell outside
// the 27-cell block or index past the cell's size), far (listed pair not within
// 0 < d2 <= nbh^2), missing (listed count differs from an exhaustive search).
struct StreamCounts {
  unsigned long long format, order, self, range, far, missing;
};

// Checks one cell's stream s[0, len) with na particles and T offset tables.
// View supplies, for the cell being checked:
//   uint32_t size_of(int di, int dj, int dk)           particles of the neighbour (or ghost) cell
//   bool pair_d2(uint32_t pa, int di, int dj, int dk, uint32_t pb, double& d2)
//                                                       FP64 squared distance of the pair (pb < size)
//   uint32_t exhaustive_count(uint32_t pa)             neighbours of pa by an exhaustive search
//   double nbh2
// Every read of s is bounded by len and every particle index by size_of before
// the view uses it, so a corrupted stream only raises counts.
template <class View>
XNB_SHD void verify_cell_stream(const View& v, const uint16_t* s, uint64_t len, uint32_t na, int T, StreamCounts& c) {
  if (na == 0) {
    if (len != 0) ++c.format;
    return;
  }
  const uint64_t table = T >= 1 ? (static_cast<uint64_t>(na) * static_cast<uint64_t>(T) + 1u) * 2u : 0u;
  if (table > len) {
    ++c.format;
    return;
  }
  const uint16_t* body = s + table;
  const uint64_t blen = len - table;
  auto table_u32 = [&](uint64_t idx) -> uint32_t {
    return static_cast<uint32_t>(s[idx * 2]) | (static_cast<uint32_t>(s[idx * 2 + 1]) << 16);
  };
  if (T >= 1 && table_u32(na) != blen + static_cast<uint64_t>(T)) ++c.format;
  uint64_t p = 0;  // sequential cursor (T == 0) or the particle's start
  for (uint32_t pa = 0; pa < na; ++pa) {
    if (T >= 1) {
      const uint32_t o = table_u32(pa);
      if (o < static_cast<uint32_t>(T) || static_cast<uint64_t>(o - T) > blen) {
        ++c.format;
        continue;
      }
      if (static_cast<uint64_t>(o - T) != p) ++c.format;  // sub-streams are contiguous, in particle order
      p = o - T;
    }
    if (p >= blen) {
      ++c.format;
      return;
    }
    const uint32_t groups = body[p++];
    uint32_t listed = 0, lower = 0;
    int last_enc = -1;
    bool broken = false;
    for (uint32_t g = 0; g < groups && !broken; ++g) {
      if (p + 2 > blen) {
        ++c.format;
        broken = true;
        break;
      }
      const uint16_t enc = body[p++];
      const uint32_t cnt = body[p++];
      int di, dj, dk;
      const bool ok_cell = decode_cell_rel(enc, di, dj, dk);
      if (!ok_cell) ++c.range;
      if (static_cast<int>(enc) <= last_enc) ++c.order;
      last_enc = enc;
      const uint32_t size = ok_cell ? v.size_of(di, dj, dk) : 0u;
      const int rel = dk * 9 + dj * 3 + di;  // < 0: the cell precedes cell a in grid order
      int last_pb = -1;
      for (uint32_t q = 0; q < cnt; ++q) {
        if (p >= blen) {
          ++c.format;
          broken = true;
          break;
        }
        const uint32_t pb = body[p++];
        ++listed;
        if (static_cast<int>(pb) <= last_pb) ++c.order;
        last_pb = static_cast<int>(pb);
        if (!ok_cell || pb >= size) {
          ++c.range;
          continue;
        }
        if (rel < 0 || (rel == 0 && pb < pa)) ++lower;
        if (rel == 0 && pb == pa) {
          ++c.self;
          continue;
        }
        double d2 = 0.0;
        if (!v.pair_d2(pa, di, dj, dk, pb, d2) || !(d2 > 0.0 && d2 <= v.nbh2)) ++c.far;
      }
    }
    if (broken) return;
    if (T == 2 && table_u32(static_cast<uint64_t>(na) + 1u + pa) != lower) ++c.order;
    const uint32_t want = v.exhaustive_count(pa);
    c.missing += want > listed ? want - listed : listed - want;
  }
  if (p != blen) ++c.format;
}

}  // namespace xnb
