// Rebuild-path kernels: move/rebin with periodic wrap, AMR in-cell ordering,
// backup_r, and the cell-grid neighbour build; plus the device scan they use.
#include "xnb_build_common.cuh"
#include "xnb_launch.cuh"

namespace xnb {

namespace {

using namespace build;
constexpr uint32_t kMoverBit = 0x80000000u;


// sub_grid_size (amr/include/exanb/amr/amr_grid_algorithm.h:66-78): the largest
// side s with s^3 <= n/density (1 below side 2, capped at 16), computed from the
// same double n/density the reference feeds to cbrt.
__device__ __forceinline__ int sub_grid_side(uint32_t n, double density) {
  if (n == 0) return 0;
  const double x = __ddiv_rn(static_cast<double>(n), density);
  if (x < 8.0) return 1;
  int s = 2;
  while (s < 16 && static_cast<double>((s + 1) * (s + 1) * (s + 1)) <= x) ++s;
  return s;
}

// ---------------------------------------------------------------------------
// K_r1: destination cell of each particle of a rebuilding system.
// move_particles_across_cells (grid_cell_particles/include/exanb/grid_cell_particles/
// move_particles_across_cells.h:115-152): dst = domain_periodic_location(r)
// (core/include/exanb/core/domain.h:160-191, wrapping r by whole cells), and the
// particle leaves its cell when dst differs or it lies >= epsilon outside dst's bounds.
__global__ void __launch_bounds__(256)
    k_rebin_dest(uint32_t n_part, const SysDesc* __restrict__ sys, SysState* st, DevArrays a) {
  if (*a.any_rebuild == 0) return;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_part; i += gridDim.x * blockDim.x) {
    const uint32_t c = a.pcell[i];
    if (c == kInvalid) continue;
    const uint32_t s = a.cell_sys[c];
    if (!sys_flagged(st, s)) continue;
    const SysDesc& S = sys[s];
    int ci, cj, ck;
    cell_ijk(S, c - S.cell_base, ci, cj, ck);
    {
      // FP32 pre-decision from the position mirror: a particle whose quotient lies
      // farther than q_margin_f from a cell boundary, inside the grid, gets the
      // reference's cell without the FP64 division, and lies strictly inside it
      // (distance to the cell bounds 0, no wrapping).
      const float4 pq = a.pf[i];
      const float qv[3] = {pq.x * S.inv_cell_f, pq.y * S.inv_cell_f, pq.z * S.inv_cell_f};
      int lf[3];
      bool sure = true;
      for (int ax = 0; ax < 3; ++ax) {
        const float fl = floorf(qv[ax]);
        const float fr = qv[ax] - fl;
        sure = sure && fr > S.q_margin_f && fr < 1.0f - S.q_margin_f && fl >= 0.0f &&
               fl < static_cast<float>(S.dims[ax]);
        lf[ax] = static_cast<int>(fl);
      }
      if (sure) {
        if (lf[0] == ci && lf[1] == cj && lf[2] == ck) {
          a.pdest[i] = c;
        } else {
          const int dd[3] = {pmod_i(lf[0] - ci, S.dims[0]), pmod_i(lf[1] - cj, S.dims[1]),
                             pmod_i(lf[2] - ck, S.dims[2])};
          for (int ax = 0; ax < 3; ++ax)
            if (!(dd[ax] == 0 || dd[ax] == 1 || dd[ax] == S.dims[ax] - 1)) atomicOr(&st[s].error, kErrFarMover);
          a.pdest[i] = (S.cell_base + static_cast<uint32_t>((lf[2] * S.dims[1] + lf[1]) * S.dims[0] + lf[0])) |
                       kMoverBit;
        }
        continue;
      }
    }
    const double ro[3] = {a.rx[i], a.ry[i], a.rz[i]};
    double r[3] = {ro[0], ro[1], ro[2]};
    int loc[3];
    bool bad = false;
    for (int ax = 0; ax < 3; ++ax) {
      const double rel = __dsub_rn(r[ax], S.origin[ax]);
      const double q = floor(__ddiv_rn(rel, S.cell_size));
      if (!(fabs(q) < 1.0e9)) {
        bad = true;
        loc[ax] = 0;
        continue;
      }
      int l = static_cast<int>(q);
      if (l < 0 || l >= S.dims[ax]) {
        const int old = l;
        l = pmod_i(l, S.dims[ax]);
        r[ax] = __dadd_rn(r[ax], __dmul_rn(static_cast<double>(l - old), S.cell_size));
      }
      loc[ax] = l;
    }
    if (bad) {
      atomicOr(&st[s].error, kErrCellIndex);
      a.pdest[i] = c;
      continue;
    }
    // min_distance2_between(ro, cell_bounds(dst)) >= epsilon_cell_size2 (grid.h:60,89-90; geometry.h:137-153)
    double d[3];
    for (int ax = 0; ax < 3; ++ax) {
      const double lo = cell_lo(S, ax, loc[ax]);
      const double hi = cell_lo(S, ax, loc[ax] + 1);
      d[ax] = 0.0;
      if (ro[ax] < lo) d[ax] = __dsub_rn(lo, ro[ax]);
      else if (ro[ax] > hi) d[ax] = __dsub_rn(ro[ax], hi);
    }
    const double md2 = norm2_rn(d[0], d[1], d[2]);
    const double eps = __dmul_rn(0x1p-48, S.cell_size);
    const bool same = (loc[0] == ci && loc[1] == cj && loc[2] == ck);
    const bool mover = !same || md2 >= __dmul_rn(eps, eps);
    const uint32_t dst = S.cell_base + static_cast<uint32_t>((loc[2] * S.dims[1] + loc[1]) * S.dims[0] + loc[0]);
    if (mover) {
      // arrivals are gathered from the 26 neighbouring cells only
      const int dd[3] = {pmod_i(loc[0] - ci, S.dims[0]), pmod_i(loc[1] - cj, S.dims[1]), pmod_i(loc[2] - ck, S.dims[2])};
      for (int ax = 0; ax < 3; ++ax)
        if (!(dd[ax] == 0 || dd[ax] == 1 || dd[ax] == S.dims[ax] - 1)) atomicOr(&st[s].error, kErrFarMover);
      a.rx[i] = r[0];
      a.ry[i] = r[1];
      a.rz[i] = r[2];
    }
    a.pdest[i] = mover ? (dst | kMoverBit) : c;
  }
}

// ---------------------------------------------------------------------------
// K_r2: per source cell, compaction of the staying particles and list of movers.
// The hole left by a mover is filled with the current last particle, scanning
// from the top (move_particles_across_cells.h:186-207).
__global__ void __launch_bounds__(128)
    k_rebin_compact(uint32_t n_cells, const SysDesc* __restrict__ sys, const SysState* __restrict__ st,
                    DevArrays a) {
  if (*a.any_rebuild == 0) return;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < n_cells; c += warps) {
    const uint32_t s = a.cell_sys[c];
    if (s == kInvalid || !sys_flagged(st, s)) continue;
    const uint32_t start = a.cell_start[c];
    const uint32_t n = a.cell_n[c];
    // movers, in particle order, via ballots
    uint32_t nmov = 0;
    for (uint32_t q0 = 0; q0 < n; q0 += 32) {
      const uint32_t q = q0 + lane;
      const bool mv = q < n && (a.pdest[start + q] & kMoverBit);
      const unsigned m = __ballot_sync(0xffffffffu, mv);
      if (mv) a.mover_list[start + nmov + __popc(m & lanemask_lt())] = start + q;
      if (q < n) a.plocal[start + q] = mv ? kInvalid : q;
      nmov += __popc(m);
    }
    __syncwarp();
    if (lane == 0) {
      uint32_t ncur = n;
      for (int q = static_cast<int>(n) - 1; q >= 0; --q) {
        if (a.plocal[start + q] == kInvalid) {
          if (static_cast<uint32_t>(q) + 1 < ncur) a.plocal[start + q] = a.plocal[start + ncur - 1];
          --ncur;
        }
      }
      a.cell_stay[c] = ncur;
      a.cell_nmov[c] = nmov;
    }
  }
}

// The (up to) 27 source cells around destination cell c, sorted by global cell
// index, duplicates removed: arrivals are appended in (source cell, source
// index) order, the order one thread of the reference's OpenMP loop produces.
struct SrcInfo {
  uint32_t src;    // source cell (kInvalid if unused / duplicate)
  uint32_t rank;   // position in sorted order
  uint32_t count;  // movers from src into c
  uint32_t offset; // exclusive prefix of counts in sorted order
};

__device__ __forceinline__ SrcInfo arrivals_of(const SysDesc& S, const DevArrays& a, uint32_t c, uint32_t lane) {
  int ci, cj, ck;
  cell_ijk(S, c - S.cell_base, ci, cj, ck);
  uint32_t src = kInvalid;
  if (lane < 27) {
    const int di = static_cast<int>(lane % 3) - 1, dj = static_cast<int>((lane / 3) % 3) - 1,
              dk = static_cast<int>(lane / 9) - 1;
    const int ni = pmod_i(ci + di, S.dims[0]), nj = pmod_i(cj + dj, S.dims[1]), nk = pmod_i(ck + dk, S.dims[2]);
    src = S.cell_base + static_cast<uint32_t>((nk * S.dims[1] + nj) * S.dims[0] + ni);
  }
  uint32_t rank = 0;
  bool dup = false;
  for (uint32_t m = 0; m < 27; ++m) {
    const uint32_t o = __shfl_sync(0xffffffffu, src, m);
    if (lane < 27) {
      if (o < src) ++rank;
      if (o == src && m < lane) dup = true;
    }
  }
  uint32_t count = 0;
  if (lane < 27 && !dup) {
    const uint32_t st0 = a.cell_start[src];
    const uint32_t nm = a.cell_nmov[src];
    for (uint32_t m = 0; m < nm; ++m) {
      const uint32_t p = a.mover_list[st0 + m];
      if ((a.pdest[p] & ~kMoverBit) == c) ++count;
    }
  }
  if (dup) src = kInvalid;
  // offset = sum of counts of lanes with smaller rank
  uint32_t offset = 0;
  for (uint32_t m = 0; m < 27; ++m) {
    const uint32_t rm = __shfl_sync(0xffffffffu, rank, m);
    const uint32_t cm = __shfl_sync(0xffffffffu, count, m);
    if (rm < rank) offset += cm;
  }
  return SrcInfo{src, rank, count, offset};
}

// K_r3: new particle count of every cell (flagged systems: stayers + arrivals).
__global__ void __launch_bounds__(128)
    k_rebin_count(uint32_t n_cells, const SysDesc* __restrict__ sys, const SysState* __restrict__ st, DevArrays a) {
  if (*a.any_rebuild == 0) return;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < n_cells; c += warps) {
    const uint32_t s = a.cell_sys[c];
    if (s == kInvalid) {
      if (lane == 0) a.cell_cnt[c] = 0;
      continue;
    }
    if (!sys_flagged(st, s)) {
      if (lane == 0) a.cell_cnt[c] = a.cell_n[c];
      continue;
    }
    const SrcInfo si = arrivals_of(sys[s], a, c, lane);
    uint32_t tot = si.count;
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
    if (lane == 0) a.cell_cnt[c] = a.cell_stay[c] + tot;
  }
}

// K_r5: gather stayers then arrivals of each destination cell into the scratch arrays.
__global__ void __launch_bounds__(128)
    k_rebin_scatter(uint32_t n_cells, const SysDesc* __restrict__ sys, const SysState* __restrict__ st,
                    DevArrays a) {
  if (*a.any_rebuild == 0) return;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < n_cells; c += warps) {
    const uint32_t s = a.cell_sys[c];
    if (s == kInvalid || !sys_flagged(st, s)) continue;
    const SysDesc& S = sys[s];
    const uint32_t ns = S.part_base + static_cast<uint32_t>(a.cell_scan[c] - a.cell_scan[S.cell_base]);
    const uint32_t start = a.cell_start[c];
    const uint32_t stay = a.cell_stay[c];
    for (uint32_t q = lane; q < stay; q += 32) {
      const uint32_t src = start + a.plocal[start + q];
      const uint32_t dst = ns + q;
      a.t_rx[dst] = a.rx[src]; a.t_ry[dst] = a.ry[src]; a.t_rz[dst] = a.rz[src];
      a.t_vx[dst] = a.vx[src]; a.t_vy[dst] = a.vy[src]; a.t_vz[dst] = a.vz[src];
      a.t_fx[dst] = a.fx[src]; a.t_fy[dst] = a.fy[src]; a.t_fz[dst] = a.fz[src];
      a.t_id[dst] = a.id[src];
      a.t_ptype[dst] = a.ptype[src];
    }
    const SrcInfo si = arrivals_of(S, a, c, lane);
    if (si.src != kInvalid && si.count > 0) {
      const uint32_t st0 = a.cell_start[si.src];
      const uint32_t nm = a.cell_nmov[si.src];
      uint32_t k = 0;
      for (uint32_t m = 0; m < nm; ++m) {
        const uint32_t p = a.mover_list[st0 + m];
        if ((a.pdest[p] & ~kMoverBit) != c) continue;
        const uint32_t dst = ns + stay + si.offset + k++;
        a.t_rx[dst] = a.rx[p]; a.t_ry[dst] = a.ry[p]; a.t_rz[dst] = a.rz[p];
        a.t_vx[dst] = a.vx[p]; a.t_vy[dst] = a.vy[p]; a.t_vz[dst] = a.vz[p];
        a.t_fx[dst] = a.fx[p]; a.t_fy[dst] = a.fy[p]; a.t_fz[dst] = a.fz[p];
        a.t_id[dst] = a.id[p];
        a.t_ptype[dst] = a.ptype[p];
      }
    }
  }
}

// K_r6: final in-cell order (rebuild_amr's stable sort by sub-cell,
// amr_grid_algorithm.h:131-374, when the cell is dense enough for a sub-grid),
// cell table update, and backup_r (io/backup_r.cpp:56-79).
__global__ void __launch_bounds__(128)
    k_rebin_finalize(uint32_t n_cells, const SysDesc* __restrict__ sys, SysState* st, DevArrays a) {
  if (*a.any_rebuild == 0) return;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < n_cells; c += warps) {
    const uint32_t s = a.cell_sys[c];
    if (s == kInvalid || !sys_flagged(st, s)) continue;
    const SysDesc& S = sys[s];
    const uint32_t ns = S.part_base + static_cast<uint32_t>(a.cell_scan[c] - a.cell_scan[S.cell_base]);
    const uint32_t n = a.cell_cnt[c];
    int ci, cj, ck;
    // the FP64 division of sub_grid_side only for counts that can give a side > 1
    // (a warp-wide FP64 instruction costs the same for one lane as for 32)
    const int side = (S.amr_enabled && n >= S.amr_min_n) ? sub_grid_side(n, S.sub_grid_density) : 1;
    // backup_r runs afterwards in k_backup, one thread per particle
    if (lane == 0) a.cside[c] = static_cast<uint8_t>(side);
    if (side > 1) {
      cell_ijk(S, c - S.cell_base, ci, cj, ck);
      const double lo[3] = {cell_lo(S, 0, ci), cell_lo(S, 1, cj), cell_lo(S, 2, ck)};
      // sub-cell key of each particle (Grid::particle_pcoord, grid.h:184-190), kept in pdest
      for (uint32_t q = lane; q < n; q += 32) {
        const double r[3] = {a.t_rx[ns + q], a.t_ry[ns + q], a.t_rz[ns + q]};
        int key = 0;
        int sidx[3];
        for (int ax = 0; ax < 3; ++ax) {
          const double pc = __ddiv_rn(__dsub_rn(r[ax], lo[ax]), S.cell_size);
          long long v = __double2ll_rz(__dmul_rn(pc, static_cast<double>(side)));
          v = v < 0 ? 0 : (v > side - 1 ? side - 1 : v);
          sidx[ax] = static_cast<int>(v);
        }
        key = (sidx[2] * side + sidx[1]) * side + sidx[0];
        a.pdest[ns + q] = static_cast<uint32_t>(key);
      }
      __syncwarp();
      for (uint32_t q = lane; q < n; q += 32) {
        const uint32_t kq = a.pdest[ns + q];
        uint32_t rank = 0;
        for (uint32_t p = 0; p < n; ++p) {
          const uint32_t kp = a.pdest[ns + p];
          rank += (kp < kq) || (kp == kq && p < q);
        }
        a.plocal[ns + q] = rank;
      }
      __syncwarp();
    }
    for (uint32_t q = lane; q < n; q += 32) {
      const uint32_t src = ns + q;
      const uint32_t dst = ns + (side > 1 ? a.plocal[ns + q] : q);
      const double x = a.t_rx[src], y = a.t_ry[src], z = a.t_rz[src];
      a.rx[dst] = x; a.ry[dst] = y; a.rz[dst] = z;
      a.vx[dst] = a.t_vx[src]; a.vy[dst] = a.t_vy[src]; a.vz[dst] = a.t_vz[src];
      a.fx[dst] = a.t_fx[src]; a.fy[dst] = a.t_fy[src]; a.fz[dst] = a.t_fz[src];
      a.id[dst] = a.t_id[src];
      a.ptype[dst] = a.t_ptype[src];
      float4 mhi, mlo;
      make_pf2(S, x, y, z, mhi, mlo);
      a.pf[dst] = mhi;
      a.pflo[dst] = mlo;
      a.pcell[dst] = c;
      if (side > 1) a.skey[dst] = static_cast<uint16_t>(a.pdest[src]);
    }
    if (lane == 0) {
      a.cell_start[c] = ns;
      a.cell_n[c] = n;
      atomicMax(&st[s].max_cell, n);
    }
  }
}

// backup_r alone (io/backup_r.cpp:42-79) for flagged systems. EXACT = false
// (the FP64 and mixed paths) keeps the backup position itself instead of its
// 32-bit cell-relative encoding: the displacement trigger then differs from the
// reference's by the encoding's quantum (cell_size / 2^32) at most.
template <bool EXACT>
__global__ void __launch_bounds__(256)
    k_backup(uint32_t n_part, const SysDesc* __restrict__ sys, SysState* st, DevArrays a) {
  if (*a.any_rebuild == 0) return;
  if constexpr (!EXACT) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_part; i += gridDim.x * blockDim.x) {
      const uint32_t c = a.pcell[i];
      if (c == kInvalid || !sys_flagged(st, a.cell_sys[c])) continue;
      const double x = a.rx[i], y = a.ry[i], z = a.rz[i];
      a.rbx[i] = x;
      a.rby[i] = y;
      a.rbz[i] = z;
      a.rbf[i] = make_pf(sys[a.cell_sys[c]], x, y, z);
    }
  } else {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_part; i += gridDim.x * blockDim.x) {
    const uint32_t c = a.pcell[i];
    if (c == kInvalid) continue;
    const uint32_t s = a.cell_sys[c];
    if (!sys_flagged(st, s)) continue;
    const SysDesc& S = sys[s];
    int ci, cj, ck;
    cell_ijk(S, c - S.cell_base, ci, cj, ck);
    const double lo[3] = {cell_lo(S, 0, ci), cell_lo(S, 1, cj), cell_lo(S, 2, ck)};
    const uint32_t bx = encode_u32(a.rx[i], lo[0], S.cell_size, S.inv_cell);
    const uint32_t by = encode_u32(a.ry[i], lo[1], S.cell_size, S.inv_cell);
    const uint32_t bz = encode_u32(a.rz[i], lo[2], S.cell_size, S.inv_cell);
    a.bkx[i] = bx; a.bky[i] = by; a.bkz[i] = bz;
    a.rbx[i] = restore_u32(bx, lo[0], S.cell_size);
    a.rby[i] = restore_u32(by, lo[1], S.cell_size);
    a.rbz[i] = restore_u32(bz, lo[2], S.cell_size);
    a.rbf[i] = make_pf(S, a.rbx[i], a.rby[i], a.rbz[i]);
  }
  }
}

// backup_r done for the flagged systems; after a rebin their sub-cell keys
// (k_rebin_finalize) also describe the current positions
__global__ void k_arm(int nsys, SysState* st, const unsigned int* any, bool rebinned) {
  if (*any == 0) return;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys && st[s].rebuild) {
    st[s].rebuild_armed = 1;
    if (rebinned) st[s].keys_fresh = 1;
  }
}

// ---------------------------------------------------------------------------
// chunk_neighbors_execute (particle_neighbors/include/exanb/particle_neighbors/
// chunk_neighbors_execute.h:110-244, 286-372): for each particle of cell a, the
// particles of the 27 cells around a (periodic images included) with
// (cell_a != cell_b || p_a != p_b) && 0 < d2 <= nbh_dist^2, d2 = norm2(r_a - r_b),
// in (cell_enc, p_b) order. Ghost particles outside the partner block enlarged
// by ghost_dist are not candidates (update_ghosts_comm_scheme.cpp:462-469).
//
// Candidates are staged in shared memory as float4 (FP32 position relative to
// the system origin, entry bits in .w); lanes test 32 candidates at a time
// against one particle of the cell and a ballot keeps the hits in order. The FP32 distance decides whenever it lies farther than a
// proven error bound from the threshold; otherwise the reference's FP64 d2 (and
// the FP64 ghost filter) decide, so the pair set is bit-exact.
// Writes one particle's finished list: the buffered entries in full lines, its
// count, lower-half length and slot start.
__device__ __forceinline__ void finish_particle(const DevArrays& a, uint32_t* seg, const uint32_t* sbuf, bool buffered,
                                                uint32_t i, uint32_t base, uint32_t slot, uint32_t cursor,
                                                uint32_t half, bool first_round, uint32_t lane) {
  if (buffered) {
    __syncwarp();
    const uint32_t nw = min(cursor, slot);
    for (uint32_t q = lane; q < nw; q += 32) seg[base + q] = sbuf[q];
    __syncwarp();
  }
  if (lane == 0) {
    a.nbr_cnt[i] = cursor;
    a.nbr_half[i] = half;
    if (first_round) a.nbr_start[i] = base;
  }
}

// One block per cell, for the cells listed by k_neighbors_warp as too large for
// it (a.nbr_wide). The block stages the cell's candidates (up to `cap` per
// round) once in shared memory for all its warps; warp w takes the cell's
// particles w, w + 4, ... two at a time, so each candidate load serves two
// tests. Each particle's hits go into its fixed slot of S.list_slot entries at
// (i - part_base) * list_slot: no count pass, scan or second traversal. When the
// cell's candidates fit one round and the slot fits the warp's list buffers
// (lbuf entries each), a particle's hits are gathered in shared memory and its
// list leaves in full 128-byte lines; otherwise each ballot's hits are stored
// directly. A particle with more hits than the slot holds keeps its true count,
// writes nothing past the slot and flags the system (kErrListOverflow); max_nbr
// records the largest count for resizing.
// 64 registers (8 blocks of 128 per SM): measured faster than the 90-register
// schedule despite a few spills.
__global__ void __launch_bounds__(128, 8)
    k_neighbors(uint32_t n_cells, const SysDesc* __restrict__ sys, SysState* st, DevArrays a, int cap, int lbuf) {
  if (*a.any_rebuild == 0) return;
  extern __shared__ float4 stage_all[];
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t wib = threadIdx.x >> 5;
  const uint32_t nwarp = blockDim.x >> 5;
  float4* srel = stage_all;
  uint32_t* sbuf0 = reinterpret_cast<uint32_t*>(stage_all + cap) + static_cast<size_t>(wib) * 2 * lbuf;
  uint32_t* sbuf1 = sbuf0 + lbuf;
  const unsigned lt = lanemask_lt();
  uint32_t acc_s = kInvalid, acc_max = 0;
  unsigned long long acc_sum = 0;
  const uint32_t n_wide = min(*a.nbr_wide_n, n_cells);
  for (uint32_t it = blockIdx.x; it < n_wide; it += gridDim.x) {
    // every condition below depends on the cell only: the block stays together
    const uint32_t c = a.nbr_wide[it];
    const uint32_t s = a.cell_sys[c];
    if (s == kInvalid || !sys_flagged(st, s)) continue;
    const uint32_t na = a.cell_n[c];
    if (na == 0) continue;
    if (s != acc_s) {
      if (lane == 0) flush_list_stats(st, sys, acc_s, acc_max, acc_sum);
      acc_s = s;
      acc_max = 0;
      acc_sum = 0;
    }
    const SysDesc& S = sys[s];
    const uint32_t sa = a.cell_start[c];
    int ci, cj, ck;
    cell_ijk(S, c - S.cell_base, ci, cj, ck);

    // group table: lane g < 27 describes neighbour cell g in (dk, dj, di) order
    uint32_t g_start = 0, g_n = 0, g_code = kImageCenter;
    if (lane < 27) {
      const int di = static_cast<int>(lane % 3) - 1, dj = static_cast<int>((lane / 3) % 3) - 1,
                dk = static_cast<int>(lane / 9) - 1;
      int n3[3] = {ci + di, cj + dj, ck + dk};
      int img[3];
      for (int ax = 0; ax < 3; ++ax) {
        img[ax] = 1;
        if (n3[ax] < 0) { n3[ax] += S.dims[ax]; img[ax] = 0; }
        else if (n3[ax] >= S.dims[ax]) { n3[ax] -= S.dims[ax]; img[ax] = 2; }
      }
      const uint32_t src = S.cell_base + static_cast<uint32_t>((n3[2] * S.dims[1] + n3[1]) * S.dims[0] + n3[0]);
      g_start = a.cell_start[src];
      g_n = a.cell_n[src];
      g_code = static_cast<uint32_t>(img[0] + 3 * img[1] + 9 * img[2]);
    }
    uint32_t g_off = g_n;  // inclusive scan over lanes
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t v = __shfl_up_sync(0xffffffffu, g_off, off);
      if (lane >= static_cast<uint32_t>(off)) g_off += v;
    }
    const uint32_t ncand = __shfl_sync(0xffffffffu, g_off, 26);
    g_off -= g_n;
    float4 own = make_float4(0.f, 0.f, 0.f, 0.f);
    if (na <= 32 && lane < na) own = a.pf[sa + lane];
    // candidates before cell a's own group come first (groups g < 13), then cell a
    const uint32_t off_self = __shfl_sync(0xffffffffu, g_off, 13);

    const float nb_hi = S.nbh2_f + S.nbh_margin_f;
    const float nb_lo = S.nbh2_f - S.nbh_margin_f;
    const float nb_zero = S.nbh_margin_f;
    const uint32_t slot = S.list_slot;
    uint32_t* const seg = a.nbr + S.list_base;
    const bool buffered = ncand <= static_cast<uint32_t>(cap) && slot <= static_cast<uint32_t>(lbuf);

    for (uint32_t c0 = 0; c0 < ncand; c0 += static_cast<uint32_t>(cap)) {
      const uint32_t c1 = min(ncand, c0 + static_cast<uint32_t>(cap));
      const uint32_t m = c1 - c0;
      const uint32_t mpad = (m + 31u) & ~31u;  // <= cap (a multiple of 32)
      __syncthreads();  // the previous round's readers are done with srel
      // every thread of the block stages candidates t, t + blockDim, ...; the group
      // of candidate u is the last g with g_off[g] <= u (binary search over lanes
      // 0..26; empty groups share their successor's offset and are skipped by it)
      for (uint32_t t0 = 0; t0 < mpad; t0 += blockDim.x) {
        const uint32_t t = t0 + threadIdx.x;
        const uint32_t u = c0 + t;
        uint32_t g = 0;
        for (uint32_t step = 16; step > 0; step >>= 1) {
          const uint32_t probe = g + step;
          const uint32_t po = __shfl_sync(0xffffffffu, g_off, probe < 27u ? probe : 26u);
          if (probe < 27u && po <= u) g = probe;
        }
        const uint32_t gs = __shfl_sync(0xffffffffu, g_start, g);
        const uint32_t go = __shfl_sync(0xffffffffu, g_off, g);
        const uint32_t gc = __shfl_sync(0xffffffffu, g_code, g);
        if (t < m) {
          srel[t] = stage_candidate(S, a, gs + (u - go), gc);
        } else if (t < mpad) {
          // padding up to a whole ballot: unreachable dummies, so the test needs no bound check
          srel[t] = make_float4(1.0e18f, 1.0e18f, 1.0e18f, __uint_as_float(kInvalid));
        }
      }
      __syncthreads();
      const bool last_round = c1 == ncand;
      for (uint32_t pa = wib; pa < na; pa += 2 * nwarp) {
        const uint32_t pb = pa + nwarp;  // second particle of the pair
        const bool two = pb < na;
        const uint32_t i0 = sa + pa, i1 = sa + (two ? pb : pa);
        float4 p0, p1;
        if (na <= 32) {
          p0.x = __shfl_sync(0xffffffffu, own.x, pa);
          p0.y = __shfl_sync(0xffffffffu, own.y, pa);
          p0.z = __shfl_sync(0xffffffffu, own.z, pa);
          const uint32_t src1 = two ? pb : pa;
          p1.x = __shfl_sync(0xffffffffu, own.x, src1);
          p1.y = __shfl_sync(0xffffffffu, own.y, src1);
          p1.z = __shfl_sync(0xffffffffu, own.z, src1);
        } else {
          p0 = a.pf[i0];
          p1 = a.pf[i1];
        }
        // entries taken before candidate index lower_end form the lower half
        const uint32_t low0 = off_self + pa, low1 = off_self + (two ? pb : pa);
        const uint32_t self0 = ((i0 - S.part_base) << 5) | static_cast<uint32_t>(kImageCenter);
        const uint32_t self1 = ((i1 - S.part_base) << 5) | static_cast<uint32_t>(kImageCenter);
        const uint32_t base0 = (i0 - S.part_base) * slot;  // the host keeps npart * slot below 2^32
        const uint32_t base1 = (i1 - S.part_base) * slot;
        uint32_t cur0 = 0, half0 = 0, cur1 = 0, half1 = 0;
        if (c0 > 0) {
          cur0 = a.nbr_cnt[i0];
          half0 = a.nbr_half[i0];
          cur1 = a.nbr_cnt[i1];
          half1 = a.nbr_half[i1];
        }
        const uint32_t start0 = cur0, start1 = cur1;
        uint32_t sv0 = 0, sv1 = 0;  // lane k keeps the ballots of the round's k-th step (<= 32 steps)
        for (uint32_t t0 = 0; t0 < mpad; t0 += 32) {
          const float4 b = srel[t0 + lane];
          const uint32_t ent = __float_as_uint(b.w);
          const bool amb = (ent & kAmbiguousBit) != 0;
          const float ax = p0.x - b.x, ay = p0.y - b.y, az = p0.z - b.z;
          const float bx = p1.x - b.x, by = p1.y - b.y, bz = p1.z - b.z;
          const float d0 = fmaf(ax, ax, fmaf(ay, ay, az * az));
          const float d1 = fmaf(bx, bx, fmaf(by, by, bz * bz));
          bool hit0 = d0 < nb_lo && d0 > nb_zero && !amb;
          bool hit1 = two && d1 < nb_lo && d1 > nb_zero && !amb;
          const bool may0 = !hit0 && d0 <= nb_hi && ent != self0;
          const bool may1 = two && !hit1 && d1 <= nb_hi && ent != self1;
          if (__any_sync(0xffffffffu, may0 || may1)) {
            if (may0) hit0 = exact_neighbor_test(S, a, i0, ent);
            if (may1) hit1 = exact_neighbor_test(S, a, i1, ent);
          }
          const unsigned m0 = __ballot_sync(0xffffffffu, hit0);
          const unsigned m1 = __ballot_sync(0xffffffffu, hit1);
          const uint32_t e = ent & ~kAmbiguousBit;
          const uint32_t q0 = cur0 + __popc(m0 & lt);
          const uint32_t q1 = cur1 + __popc(m1 & lt);
          if (hit0 && q0 < slot) {
            if (buffered) sbuf0[q0] = e;
            else seg[base0 + q0] = e;
          }
          if (hit1 && q1 < slot) {
            if (buffered) sbuf1[q1] = e;
            else seg[base1 + q1] = e;
          }
          if ((t0 >> 5) == lane) {
            sv0 = m0;
            sv1 = m1;
          }
          cur0 += __popc(m0);
          cur1 += __popc(m1);
        }
        // the lower half ends at candidate lower_end: hits of the earlier rounds
        // plus, from the kept ballots, this round's hits below it
        const uint32_t w0 = low0 - c0, w1 = low1 - c0;
        if (w0 < m) {
          const uint32_t v = lane < (w0 >> 5) ? __popc(sv0)
                                             : (lane == (w0 >> 5) ? __popc(sv0 & ((1u << (w0 & 31u)) - 1u)) : 0u);
          half0 = start0 + __reduce_add_sync(0xffffffffu, v);
        }
        if (w1 < m) {
          const uint32_t v = lane < (w1 >> 5) ? __popc(sv1)
                                             : (lane == (w1 >> 5) ? __popc(sv1 & ((1u << (w1 & 31u)) - 1u)) : 0u);
          half1 = start1 + __reduce_add_sync(0xffffffffu, v);
        }
        finish_particle(a, seg, sbuf0, buffered, i0, base0, slot, cur0, half0, c0 == 0, lane);
        if (two) finish_particle(a, seg, sbuf1, buffered, i1, base1, slot, cur1, half1, c0 == 0, lane);
        if (last_round) {
          acc_max = max(acc_max, cur0);
          acc_sum += cur0;
          if (two) {
            acc_max = max(acc_max, cur1);
            acc_sum += cur1;
          }
        }
      }
    }
  }
  if (lane == 0) flush_list_stats(st, sys, acc_s, acc_max, acc_sum);
}

// ---------------------------------------------------------------------------
// Warp-per-cell form of the same build, for every cell whose candidates fit the
// warp's stage (cap); the others are appended to a.nbr_wide for k_neighbors.
// Each warp stages its cell's candidates itself (no block barrier), then tests
// kWarpP particles per staged load: lanes hold 32 candidates, and a ballot per
// particle appends its hits in order straight to the particle's list slot
// (an entry past the slot lands on its last word; the count flags the
// overflow). Two rare cases leave the fast test through
// warp-uniform branches: a chunk holding a candidate whose ghost filter is
// undecided in FP32, and an FP32 distance inside the error band around nbh^2
// (both then take the reference's FP64 decision, as in k_neighbors).
// Six particles per staged load fit 96 registers (8 bytes spilled), so 5 blocks
// of 4 warps stay resident per SM (5 x 40 KB of stage at cap 640); eight per
// load need 126 registers and hold 4 blocks, and take 13% longer per rebuild.
constexpr int kWarpP = 6;  // particles tested per staged candidate load in the warp-per-cell build

__global__ void __launch_bounds__(128, 5)
    k_neighbors_warp(uint32_t n_cells, const SysDesc* __restrict__ sys, SysState* st, DevArrays a, int cap,
                     bool prune, bool half_form) {
  if (*a.any_rebuild == 0) return;
  extern __shared__ float4 stage_w[];
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t wib = threadIdx.x >> 5;
  const uint32_t nwarp = blockDim.x >> 5;
  float4* srel = stage_w + static_cast<size_t>(wib) * cap;
  __shared__ uint32_t sink[4][kWarpP];  // hits of systems without list slots (blocks of 4 warps)
  const unsigned lt = lanemask_lt();
  uint32_t acc_s = kInvalid, acc_max = 0;
  unsigned long long acc_sum = 0;
  const uint32_t nw_all = gridDim.x * nwarp;
  for (uint32_t c = blockIdx.x * nwarp + wib; c < n_cells; c += nw_all) {
    const uint32_t s = a.cell_sys[c];
    if (s == kInvalid || !sys_flagged(st, s)) continue;
    if (half_form && !st[s].half_bad) continue;  // built by the half-shell kernels
    const uint32_t na = a.cell_n[c];
    if (na == 0) continue;
    if (prune && a.cside[c] >= 2 && st[s].keys_fresh) {
      if (lane == 0) a.nbr_sub[atomicAdd(a.nbr_sub_n, 1u)] = c;
      continue;
    }
    const SysDesc& S = sys[s];
    const uint32_t sa = a.cell_start[c];
    int ci, cj, ck;
    cell_ijk(S, c - S.cell_base, ci, cj, ck);

    // group table: lane g < 27 describes neighbour cell g in (dk, dj, di) order
    uint32_t g_start = 0, g_n = 0, g_code = kImageCenter;
    if (lane < 27) {
      const int di = static_cast<int>(lane % 3) - 1, dj = static_cast<int>((lane / 3) % 3) - 1,
                dk = static_cast<int>(lane / 9) - 1;
      int n3[3] = {ci + di, cj + dj, ck + dk};
      int img[3];
      for (int ax = 0; ax < 3; ++ax) {
        img[ax] = 1;
        if (n3[ax] < 0) { n3[ax] += S.dims[ax]; img[ax] = 0; }
        else if (n3[ax] >= S.dims[ax]) { n3[ax] -= S.dims[ax]; img[ax] = 2; }
      }
      const uint32_t src = S.cell_base + static_cast<uint32_t>((n3[2] * S.dims[1] + n3[1]) * S.dims[0] + n3[0]);
      g_start = a.cell_start[src];
      g_n = a.cell_n[src];
      g_code = static_cast<uint32_t>(img[0] + 3 * img[1] + 9 * img[2]);
    }
    uint32_t g_off = g_n;  // inclusive scan over lanes
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t v = __shfl_up_sync(0xffffffffu, g_off, off);
      if (lane >= static_cast<uint32_t>(off)) g_off += v;
    }
    const uint32_t ncand = __shfl_sync(0xffffffffu, g_off, 26);
    g_off -= g_n;
    const uint32_t slot = S.list_slot;
    if (ncand > static_cast<uint32_t>(cap)) {
      if (lane == 0) a.nbr_wide[atomicAdd(a.nbr_wide_n, 1u)] = c;
      continue;
    }
    if (s != acc_s) {
      if (lane == 0) flush_list_stats(st, sys, acc_s, acc_max, acc_sum);
      acc_s = s;
      acc_max = 0;
      acc_sum = 0;
    }
    const uint32_t off_self = __shfl_sync(0xffffffffu, g_off, 13);
    float4 own = make_float4(0.f, 0.f, 0.f, 0.f);
    if (na <= 32 && lane < na) own = a.pf[sa + lane];

    // stage: candidate u belongs to the last group g with g_off[g] <= u; four
    // candidates per lane are located and loaded before any is converted
    const uint32_t mpad = (ncand + 31u) & ~31u;
    for (uint32_t t0 = 0; t0 < mpad; t0 += 128u) {
      float4 pb[4];
      uint32_t jj[4], gcs[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const uint32_t u = t0 + 32u * k + lane;
        uint32_t g = 0;
#pragma unroll
        for (uint32_t step = 16; step > 0; step >>= 1) {
          const uint32_t probe = g + step;
          const uint32_t po = __shfl_sync(0xffffffffu, g_off, probe < 27u ? probe : 26u);
          if (probe < 27u && po <= u) g = probe;
        }
        const uint32_t gs = __shfl_sync(0xffffffffu, g_start, g);
        const uint32_t go = __shfl_sync(0xffffffffu, g_off, g);
        gcs[k] = __shfl_sync(0xffffffffu, g_code, g);
        jj[k] = gs + (u - go);
        pb[k] = u < ncand ? __ldg(a.pf + jj[k]) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const uint32_t u = t0 + 32u * k + lane;
        if (u < ncand) srel[u] = stage_from(S, pb[k], jj[k], gcs[k]);
        else if (u < mpad) srel[u] = make_float4(1.0e18f, 1.0e18f, 1.0e18f, __uint_as_float(kInvalid));
      }
    }
    __syncwarp();

    const float nb_hi = S.nbh2_f + S.nbh_margin_f;
    const float nb_lo = S.nbh2_f - S.nbh_margin_f;
    const float nb_zero = S.nbh_margin_f;
    uint32_t* const seg = a.nbr + S.list_base;
    for (uint32_t p0 = 0; p0 < na; p0 += kWarpP) {
      // particles past the cell's end sit at -1e18: never within reach of a
      // candidate (real ones, or the +1e18 dummies), so they need no test
      float px[kWarpP], py[kWarpP], pz[kWarpP];
      uint32_t cur[kWarpP], half[kWarpP];
#pragma unroll
      for (int k = 0; k < kWarpP; ++k) {
        const uint32_t pk = p0 + k;
        float4 q;
        if (na <= 32) {
          q.x = __shfl_sync(0xffffffffu, own.x, pk & 31u);
          q.y = __shfl_sync(0xffffffffu, own.y, pk & 31u);
          q.z = __shfl_sync(0xffffffffu, own.z, pk & 31u);
        } else {
          q = pk < na ? a.pf[sa + pk] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        const bool valid = pk < na;
        px[k] = valid ? q.x : -1.0e18f;
        py[k] = valid ? q.y : -1.0e18f;
        pz[k] = valid ? q.z : -1.0e18f;
        cur[k] = 0;
        half[k] = 0;
      }
      const uint32_t i0 = sa + p0;
      const uint32_t self0 = ((i0 - S.part_base) << 5) | static_cast<uint32_t>(kImageCenter);
      const uint32_t low0 = off_self + p0;
      // hits go straight to the particles' slots (consecutive particles, stride
      // slot); a system without slots yet (the sizing build) only counts, its
      // hits landing in the warp's sink
      uint32_t* const pslot = slot ? seg + static_cast<size_t>(i0 - S.part_base) * slot : sink[wib];
      const uint32_t pstride = slot ? slot : 1u;
      for (uint32_t t0 = 0; t0 < mpad; t0 += 32) {
        const float4 b = srel[t0 + lane];
        const uint32_t ent = __float_as_uint(b.w);
        // the particles' own entries (lower-half ends) sit at stage indices low0 + k
        const bool self_chunk = t0 < low0 + kWarpP && low0 < t0 + 32u;
        // entries in [kAmbiguousBit, kInvalid): ghost filter undecided in FP32
        if (__any_sync(0xffffffffu, ent - kAmbiguousBit < kInvalid - kAmbiguousBit)) {
          if (self_chunk)
            nbr_chunk<kWarpP, true, true>(S, a, b, px, py, pz, i0, self0, t0, low0, nb_lo, nb_hi, nb_zero, lt, pslot,
                                          pstride, cur, half);
          else
            nbr_chunk<kWarpP, true, false>(S, a, b, px, py, pz, i0, self0, t0, low0, nb_lo, nb_hi, nb_zero, lt, pslot,
                                           pstride, cur, half);
        } else if (self_chunk) {
          nbr_chunk<kWarpP, false, true>(S, a, b, px, py, pz, i0, self0, t0, low0, nb_lo, nb_hi, nb_zero, lt, pslot,
                                         pstride, cur, half);
        } else {
          nbr_chunk<kWarpP, false, false>(S, a, b, px, py, pz, i0, self0, t0, low0, nb_lo, nb_hi, nb_zero, lt, pslot,
                                          pstride, cur, half);
        }
      }
#pragma unroll
      for (int k = 0; k < kWarpP; ++k) {
        const uint32_t pk = p0 + k;
        if (pk < na) {
          const uint32_t i = sa + pk;
          if (lane == 0) {
            a.nbr_cnt[i] = cur[k];
            a.nbr_half[i] = half[k];
            a.nbr_start[i] = (i - S.part_base) * slot;  // the host keeps npart * slot below 2^32
          }
          acc_max = max(acc_max, cur[k]);
          acc_sum += cur[k];
        }
      }
    }
  }
  if (lane == 0) flush_list_stats(st, sys, acc_s, acc_max, acc_sum);
}

// Clears the per-build list statistics of the flagged systems.
__global__ void k_nbr_reset(int nsys, SysState* st, const unsigned int* any, unsigned int* wide_n,
                            unsigned int* sub_n) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *wide_n = 0;
    *sub_n = 0;
  }
  if (*any == 0) return;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys || !st[s].rebuild) return;
  st[s].list_used = 0;
  st[s].max_nbr = 0;
  st[s].lists_fresh = 1;  // the build that follows reads the current positions
  st[s].compact_bad = 0;
  st[s].half_bad = 0;
}

// ---------------------------------------------------------------------------
// Exclusive scan, u32 -> u64, three phases (tile sums, scan of sums, tiles).
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr uint32_t kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const uint32_t* __restrict__ in, uint32_t n,
                                                              unsigned long long* sums, const unsigned int* gate) {
  if (gate && *gate == 0) return;
  __shared__ unsigned long long red[kScanThreads / 32];
  const uint32_t base = blockIdx.x * kScanTile;
  unsigned long long v = 0;
  for (int k = 0; k < kScanItems; ++k) {
    const uint32_t idx = base + threadIdx.x + k * kScanThreads;
    if (idx < n) v += in[idx];
  }
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < kScanThreads / 32; ++w) t += red[w];
    sums[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(1024) k_scan_sums(unsigned long long* sums, uint32_t nb, const unsigned int* gate) {
  if (gate && *gate == 0) return;
  __shared__ unsigned long long carry_s;
  __shared__ unsigned long long wsum[32];
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  for (uint32_t b0 = 0; b0 < nb; b0 += 1024) {
    const uint32_t b = b0 + threadIdx.x;
    const unsigned long long x = b < nb ? sums[b] : 0ull;
    unsigned long long inc = x;
    const uint32_t lane = threadIdx.x & 31;
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, inc, off);
      if (lane >= static_cast<uint32_t>(off)) inc += y;
    }
    if (lane == 31) wsum[threadIdx.x >> 5] = inc;
    __syncthreads();
    if (threadIdx.x < 32) {
      unsigned long long w = wsum[threadIdx.x];
      unsigned long long wi = w;
      for (int off = 1; off < 32; off <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, wi, off);
        if (threadIdx.x >= static_cast<uint32_t>(off)) wi += y;
      }
      wsum[threadIdx.x] = wi - w;
    }
    __syncthreads();
    const unsigned long long carry = carry_s;
    if (b < nb) sums[b] = carry + wsum[threadIdx.x >> 5] + inc - x;
    __syncthreads();
    if (threadIdx.x == 1023) carry_s = carry + wsum[31] + inc;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_final(const uint32_t* __restrict__ in, uint32_t n,
                                                              const unsigned long long* __restrict__ sums,
                                                              unsigned long long* out, const unsigned int* gate) {
  if (gate && *gate == 0) return;
  __shared__ unsigned long long wsum[kScanThreads / 32];
  const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  unsigned long long loc[kScanItems];
  unsigned long long t = 0;
  for (int k = 0; k < kScanItems; ++k) {
    const uint32_t idx = base + k;
    loc[k] = idx < n ? in[idx] : 0ull;
    t += loc[k];
  }
  const uint32_t lane = threadIdx.x & 31;
  unsigned long long inc = t;
  for (int off = 1; off < 32; off <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, inc, off);
    if (lane >= static_cast<uint32_t>(off)) inc += y;
  }
  if (lane == 31) wsum[threadIdx.x >> 5] = inc;
  __syncthreads();
  unsigned long long wpre = 0;
  for (uint32_t w = 0; w < (threadIdx.x >> 5); ++w) wpre += wsum[w];
  unsigned long long run = sums[blockIdx.x] + wpre + inc - t;
  for (int k = 0; k < kScanItems; ++k) {
    const uint32_t idx = base + k;
    if (idx < n) out[idx] = run;
    run += loc[k];
    if (idx + 1 == n) out[n] = run;
  }
}

inline int warp_grid(uint32_t n_items, int warps_per_block, int sm_count) {
  long long want = (static_cast<long long>(n_items) + warps_per_block - 1) / warps_per_block;
  const long long cap = static_cast<long long>(sm_count) * 16;
  if (want > cap) want = cap;
  return static_cast<int>(want < 1 ? 1 : want);
}

inline int thread_grid(uint32_t n, int threads, int sm_count) {
  long long want = (static_cast<long long>(n) + threads - 1) / threads;
  const long long cap = static_cast<long long>(sm_count) * 8;
  if (want > cap) want = cap;
  return static_cast<int>(want < 1 ? 1 : want);
}

}  // namespace

size_t scan_scratch_elems(uint32_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

int launch_scan_u32_to_u64(const uint32_t* in, unsigned long long* out, uint32_t n, unsigned long long* scratch,
                           cudaStream_t stream, const unsigned int* gate) {
  if (n == 0) {
    cudaMemsetAsync(out, 0, sizeof(unsigned long long), stream);
    return 0;
  }
  const uint32_t nb = (n + kScanTile - 1) / kScanTile;
  k_scan_tiles<<<nb, kScanThreads, 0, stream>>>(in, n, scratch, gate);
  k_scan_sums<<<1, 1024, 0, stream>>>(scratch, nb, gate);
  k_scan_final<<<nb, kScanThreads, 0, stream>>>(in, n, scratch, out, gate);
  return 3;
}

int launch_rebin(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, cudaStream_t stream,
                 bool exact_backup) {
  if (ex.n_part == 0 || ex.n_cells == 0) return 0;
  k_rebin_dest<<<thread_grid(ex.n_part, 256, ex.sm_count), 256, 0, stream>>>(ex.n_part, sys, st, a);
  const int wg = warp_grid(ex.n_cells, 4, ex.sm_count);
  k_rebin_compact<<<wg, 128, 0, stream>>>(ex.n_cells, sys, st, a);
  k_rebin_count<<<wg, 128, 0, stream>>>(ex.n_cells, sys, st, a);
  const int ns = launch_scan_u32_to_u64(a.cell_cnt, a.cell_scan, ex.n_cells, a.scan_blocks, stream, a.any_rebuild);
  k_rebin_scatter<<<wg, 128, 0, stream>>>(ex.n_cells, sys, st, a);
  k_rebin_finalize<<<wg, 128, 0, stream>>>(ex.n_cells, sys, st, a);
  if (exact_backup) k_backup<true><<<thread_grid(ex.n_part, 256, ex.sm_count), 256, 0, stream>>>(ex.n_part, sys, st, a);
  else k_backup<false><<<thread_grid(ex.n_part, 256, ex.sm_count), 256, 0, stream>>>(ex.n_part, sys, st, a);
  k_arm<<<(ex.nsys + 127) / 128, 128, 0, stream>>>(ex.nsys, st, a.any_rebuild, true);
  return 7 + ns;
}

int launch_backup(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, cudaStream_t stream) {
  if (ex.n_part == 0) return 0;
  k_backup<true><<<thread_grid(ex.n_part, 256, ex.sm_count), 256, 0, stream>>>(ex.n_part, sys, st, a);
  k_arm<<<(ex.nsys + 127) / 128, 128, 0, stream>>>(ex.nsys, st, a.any_rebuild, false);
  return 2;
}

int launch_neighbors(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, int cap, int lbuf,
                     cudaStream_t stream, int form, bool prune) {
  if (ex.n_cells == 0) return 0;
  const size_t smem = static_cast<size_t>(cap) * sizeof(float4) + static_cast<size_t>(4) * 2 * lbuf * sizeof(uint32_t);
  // warp-per-cell form: the stage alone (hits go straight to the slots)
  const size_t smem_w = 4 * static_cast<size_t>(cap) * sizeof(float4);
  // per-device attributes: set them on the current device every time (host calls, no GPU work)
  cudaFuncSetAttribute(k_neighbors, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
  cudaFuncSetAttribute(k_neighbors_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_neighbors_warp, 128, smem_w) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const long long want_w = (static_cast<long long>(ex.n_cells) + 3) / 4;
  const int grid_w = static_cast<int>(std::max(1ll, std::min(want_w, static_cast<long long>(per_sm) * ex.sm_count)));
  k_nbr_reset<<<(ex.nsys + 127) / 128, 128, 0, stream>>>(ex.nsys, st, a.any_rebuild, a.nbr_wide_n, a.nbr_sub_n);
  // half-shell form: masks first; systems it cannot take go through the warp-per-cell build
  const bool half = form == kBuildHalf && a.nmask != nullptr;
  const int nh = half ? launch_neighbors_half_test(ex, sys, st, a, stream) : 0;
  if (form == kBuildRows) launch_neighbors_rows(ex, sys, st, a, stream, prune);
  else k_neighbors_warp<<<grid_w, 128, smem_w, stream>>>(ex.n_cells, sys, st, a, cap, prune, half);
  const int ne = half ? launch_neighbors_half_emit(ex, sys, st, a, stream) : 0;
  // dense cells (sub-grid side >= 2), before the block-per-cell build, which takes the ones it passes on
  const int nsub = prune ? launch_neighbors_sub(ex, sys, st, a, cap, stream) : 0;
  k_neighbors<<<warp_grid(ex.n_cells, 1, ex.sm_count), 128, smem, stream>>>(ex.n_cells, sys, st, a, cap, lbuf);
  // compact entries for the staged force traversal
  const int nc = ex.force_form == kForceStaged ? launch_compact_lists(ex, sys, st, a, stream) : 0;
  return 3 + nh + ne + nsub + nc;
}

}  // namespace xnb
