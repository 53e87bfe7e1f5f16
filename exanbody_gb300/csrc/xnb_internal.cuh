// Internal definitions shared by the xnb CUDA translation units.
//
// Device data model (one "batch" holds one or many independent periodic systems):
//   * particles of all systems are packed in one SoA set of arrays, system after
//     system, and inside a system cell after cell (cells in the reference's linear
//     order (k*Dj+j)*Di+i, grid_algorithm.h:84-91), inside a cell in the
//     reference's in-cell order;
//   * cell_start[c] .. cell_start[c+1] is cell c's particle range (global index);
//   * there are no ghost cells in memory: a neighbour entry carries a periodic
//     image code and the image position x + (+-1.0)*(max-min) is recomputed where
//     it is needed, which is the same rounding as the reference's ghost copy
//     (ghosts_comm_scheme.h:76-80);
//   * neighbour lists are per particle, in the reference's stream order
//     (cell_enc, p_b) (chunk_neighbors_execute.h:308), as u32 entries
//     (local particle index << 5) | image code, in one list segment per system.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "xnb_pair.cuh"
#include "xnb_widen.h"

namespace xnb {

// the reference roundings shared with the public pair-functor API
using pair::image_coord;
using pair::image_coord_f;
using pair::norm2_rn;

constexpr int kImageCenter = 13;  // image code of the unshifted image: (0+1) + 3*(0+1) + 9*(0+1)

enum ErrorBits : uint32_t {
  kErrListOverflow = 1u << 0,   // neighbour list segment too small
  kErrFarMover = 1u << 1,       // a particle moved further than one cell between rebuilds
  kErrCellIndex = 1u << 2,      // a particle outside the periodic domain grid
  kErrStage = 1u << 3,          // staging capacity exceeded (programming error)
};

// Per-system constants, device resident (SysDesc[nsys]).
struct SysDesc {
  double origin[3];
  double extent[3];
  double period[3];      // extent - origin: the ghost image offset (rmax - rmin)
  double outer_lo[3];    // ghost particle filter bounds: block bounds -/+ ghost_dist
  double outer_hi[3];
  double cell_size;
  double rcut2;          // rcut*rcut (compute_cell_particle_pairs.h:145)
  double nbh2;           // (rcut+rcut_inc)^2 (chunk_neighbors_execute.h:75-76)
  double max_displ2;     // (rcut_inc/2)^2 (nbh_dist.cpp:48, particle_displ_over.cu:111)
  double epsilon, sigma, e_shift;
  double mass;
  double dt;
  double dt_full, dt_sq_half, dt_half;  // dt*1.0, (dt*dt)*0.5, dt*0.5 (push_vec3_2nd_order.h:87-88)
  double sub_grid_density;
  uint32_t amr_min_n;    // smallest cell count n with fl(n / sub_grid_density) >= 8: below it the sub-grid side is 1
  float nbh2_f, nbh_margin_f;  // FP32 prefilter of the neighbour test and its proven error margin
  float rc2_f, rc_margin_f;    // same for the force cutoff test (mixed path)
  float sig2_f, eps24_f, eps4_f, e_shift_f;
  // FP32 copies used by the prefilters: positions are kept as float offsets
  // from the origin (DevArrays::pf); image offsets and ghost-filter bounds in the
  // same frame; pre_margin_f bounds |d2_f32 - d2_f64| for the force prefilter.
  float period_f[3];
  float outer_lo_f[3], outer_hi_f[3];
  float pre_margin_f, filter_margin_f;
  float inv_cell_f, q_margin_f;  // FP32 cell-index pre-decision: 1/cell_size and its proven margin (cells)
  // FP32 pre-decision of the displacement trigger: |d|^2 from the FP32 mirrors of
  // the position and of its backup is above trig_hi_f only when the FP64 |d|^2
  // reaches max_displ2, below trig_lo_f only when it does not
  float trig_lo_f, trig_hi_f;
  float sub_reach_f;             // nbh_dist / cell_size widened by 1e-5: reach of the sub-cell box test (cells)
  float lo_step_f, lo_inv_f;     // quantum of the residual packed in DevArrays::pf.w (ulp(X)/1024) and its inverse
  int32_t packed_lo;             // 1: the mixed traversal reads the packed residuals (X < 1024); 0: DevArrays::pflo
  double inv_cell;               // fl(1/cell_size): reciprocal pre-decision of the backup encoding
  double m24eps, eps4, sig2, eps24;  // -24*eps, 4*eps (lennard_jones.cu:54-55), sigma^2, 24*eps
  int32_t dims[3];
  int32_t divide_by_mass;
  int32_t amr_enabled;
  int32_t origin_zero;  // origin is (+0, +0, +0): x - origin is x itself, no subtraction needed
  int32_t far_coords;   // coordinates beyond 4 periods: image coordinates x +- period round coarser than
                        // the displacements they form (the Newton FP64 traversal then evaluates each
                        // reaction across an image from the partner's own side)
  uint32_t cell_base, ncells;
  uint32_t part_base, npart;
  uint64_t list_base;  // first entry of the system's list segment
  uint32_t list_slot;  // entries reserved per particle: particle i's list starts at (i - part_base) * list_slot
};

// Per-system mutable state, device resident (SysState[nsys]).
struct SysState {
  unsigned long long moved;     // particles over the displacement threshold (this step)
  unsigned long long list_used; // entries of the current neighbour lists (sum of counts)
  uint32_t rebuild;             // 1 when the rebuild path must run for this system
  uint32_t error;               // ErrorBits
  uint32_t max_cell;            // largest cell occupancy after the last rebin
  uint32_t rebuild_armed;        // 1 once backup_r has run (the trigger needs a backup)
  uint32_t max_nbr;              // largest per-particle list count of the last build
  uint32_t lists_fresh;          // 1 from a neighbour build until positions next change
  uint32_t compact_bad;          // the last build's lists could not be compacted (staged force traversal)
  uint32_t keys_fresh;           // 1 from a rebin until positions next change: the sub-cell keys fit them
  uint32_t half_bad;             // the half-shell build met a cell of more than 64 particles (this build)
  unsigned long long rebuilds;
};

// All device arrays of a batch (pointers into HBM).
struct DevArrays {
  double *rx, *ry, *rz, *vx, *vy, *vz, *fx, *fy, *fz, *pe;
  float4* pf;                      // FP32 hi part of (x - origin, y - origin, z - origin), refreshed with r;
                                   // .w packs the three residuals as 10-bit multiples of lo_step_f (lo_field)
  float4* pflo;                    // FP32 residual (x - origin) - hi, so hi + lo carries ~48 bits
  unsigned int* any_rebuild;       // number of systems flagged for the rebuild path this step
  uint64_t* id;
  uint8_t* ptype;                  // particle type (field::type), 0 unless set
  uint32_t* pcell;                 // global cell of each particle
  uint32_t *bkx, *bky, *bkz;       // backup_r u32 encoding (backup_r.h:36-51)
  double *rbx, *rby, *rbz;         // the same backup restored once per rebuild (restore_u32_double)
  float4* rbf;                     // FP32 hi part of (backup - origin), for the trigger's pre-decision
  // rebin scratch
  double *t_rx, *t_ry, *t_rz, *t_vx, *t_vy, *t_vz, *t_fx, *t_fy, *t_fz;
  uint64_t* t_id;
  uint8_t* t_ptype;
  uint32_t* pdest;                 // destination cell (rebin) / scratch
  uint32_t* plocal;                // new in-cell slot of staying particles
  uint32_t* mover_list;            // per source cell, its movers (global index), in the cell's own range
  // cells
  uint32_t* cell_start;            // first particle of each cell (global index)
  uint32_t* cell_n;                // particles in each cell
  uint32_t* cell_sys;              // system of each cell
  unsigned long long* cell_scan;   // per-cell exclusive scan scratch (ncells + 1)
  uint32_t* cell_cnt;              // per-cell scratch counts
  uint32_t* cell_stay;             // staying particles per cell
  uint32_t* cell_nmov;             // movers leaving each cell
  // neighbour lists
  uint32_t* nbr_start;             // per particle, relative to its system segment ((i - part_base) * list_slot)
  uint32_t* nbr_cnt;               // per particle
  uint32_t* nbr_half;              // per particle: entries before it in the reference order
                                   // ((cell_b, p_b) < (cell_a, p_a)), the Newton half list
  uint32_t* nbr;                   // all segments
  uint16_t* nbr16;                 // compact entries (g << 11) | p_b beside nbr (staged force traversal; or null)
  uint4* seg;                      // cell segments of the staged force traversal: first cell, cells, system
  uint32_t* nbr_wide;              // cells whose candidates or slot exceed the warp-per-cell build's buffers
  unsigned int* nbr_wide_n;        // number of them (reset by each build)
  uint32_t* nbr_sub;               // dense cells (sub-grid side >= 2) for the sub-cell pruned build
  unsigned int* nbr_sub_n;         // number of them (reset by each build)
  uint16_t* skey;                  // sub-cell key of each particle of a cell with side >= 2 (k_rebin_finalize)
  uint8_t* cside;                  // sub-grid side of each cell at the last rebin (1: no sub-grid)
  uint64_t* nmask;                 // half-shell build: per group g, per particle, its bits of cell g's particles
  uint64_t nmask_stride;           // particles per group plane of nmask (the particle capacity)
  // scan scratch
  unsigned long long* scan_blocks;
};

// ----------------------------------------------------------------------------
// Exact FP64 helpers: the reference's arithmetic written with explicit rounding
// so the compiler cannot contract to FMA (norm2_rn and image_coord come from the
// pair-functor header).

// restore_u32_double (core/include/exanb/core/backup_r.h:31-34)
__device__ __forceinline__ double restore_u32(uint32_t x, double o, double r) {
  return __dadd_rn(o, __dmul_rn(__dmul_rn(static_cast<double>(x), r), 0x1p-32));
}

// encode_double_u32 (core/include/exanb/core/backup_r.h:36-51). The quotient
// (x - o) * 2^32 / r is first formed with the reciprocal rinv = fl(1/r): that
// product lies within 2 ulp of the correctly rounded quotient, so when it is more
// than 2^-18 (>= 4 ulp below 2^32) away from an integer both truncate to the same
// value and the FP64 division is skipped; otherwise (and outside [0, 2^32)) the
// division decides. The +-1 correction below is the reference's.
__device__ __forceinline__ uint32_t encode_u32(double x, double o, double r, double rinv) {
  const double xo = __dsub_rn(x, o);
  const double X = __dmul_rn(xo, 4294967296.0);  // exact (power of two)
  const double qa = __dmul_rn(X, rinv);
  const double t = trunc(qa);
  const double fr = __dsub_rn(qa, t);
  long long a;
  if (qa >= 1.0 && qa < 4294967295.0 && fr > 0x1p-18 && fr < 1.0 - 0x1p-18) {
    a = static_cast<long long>(t);
  } else {
    a = __double2ll_rz(__ddiv_rn(X, r));
  }
  a = a < 0 ? 0 : a;
  a = a > 4294967295LL ? 4294967295LL : a;
  const uint32_t xa = static_cast<uint32_t>(a);
  const uint32_t xb = xa - 1u;
  const uint32_t xc = xa + 1u;
  const double ea = fabs(__dsub_rn(restore_u32(xa, o, r), x));
  const double eb = fabs(__dsub_rn(restore_u32(xb, o, r), x));
  const double ec = fabs(__dsub_rn(restore_u32(xc, o, r), x));
  if (eb < ea) return xb;
  if (ec < ea) return xc;
  return xa;
}

// Grid::cell_position for a domain cell index (core/include/exanb/core/grid.h:114-117)
__device__ __forceinline__ double cell_lo(const SysDesc& s, int axis, int dloc) {
  return __dadd_rn(s.origin[axis], __dmul_rn(static_cast<double>(dloc), s.cell_size));
}

__device__ __forceinline__ void cell_ijk(const SysDesc& s, uint32_t local_cell, int& i, int& j, int& k) {
  i = static_cast<int>(local_cell % static_cast<uint32_t>(s.dims[0]));
  const uint32_t r = local_cell / static_cast<uint32_t>(s.dims[0]);
  j = static_cast<int>(r % static_cast<uint32_t>(s.dims[1]));
  k = static_cast<int>(r / static_cast<uint32_t>(s.dims[1]));
}

__device__ __forceinline__ int pmod_i(int i, int n) { return ((i % n) + n) % n; }

// fl32(x) and fl64(f) on the integer pipes (xnb_widen.h): the same bits as the
// hardware conversions, which would occupy the FP64 pipe
__device__ __forceinline__ float narrow_f64(double x) {
  return __uint_as_float(narrow_f64_bits(static_cast<uint64_t>(__double_as_longlong(x))));
}
__device__ __forceinline__ double widen_f32(float f);

// The residual of each axis, packed into the fourth word of the mirror: a
// signed 10-bit multiple of lo_step_f = ulp(X) / 1024, where X bounds
// |x - origin| for every particle of the system (the residual is at most
// ulp(X) / 2: the multiple fits [-512, 512] and is clamped to [-511, 511], so
// the packed residual is within lo_step_f of the FP32 one). Rounded to nearest
// by the 1.5 * 2^23 addition (|lo * inv| <= 512); lo * inv is exact (inv a power
// of two).
__device__ __forceinline__ uint32_t lo_code(float lo, float inv) {
  int q = __float_as_int(fmaf(lo, inv, 12582912.0f)) - 0x4B400000;
  q = max(-511, min(511, q));
  return static_cast<uint32_t>(q) & 1023u;
}
// signed 10-bit field k (0: x, 1: y, 2: z) of a packed residual word
__device__ __forceinline__ int lo_field(uint32_t w, int k) { return static_cast<int>(w << (22 - 10 * k)) >> 22; }
// small integer |d| < 2^22 to FP32 on the FP32 pipe (exact)
__device__ __forceinline__ float small_int_f(int d) { return __int_as_float(0x4B400000 + d) - 12582912.0f; }

// FP32 position relative to the system origin, as stored in DevArrays::pf (its
// residuals packed in .w), and the residual (DevArrays::pflo): hi = fl32(x - o),
// lo = fl32((x - o) - hi). Only the two subtractions per coordinate use the FP64
// pipe.
__device__ __forceinline__ float4 make_pf(const SysDesc& s, double x, double y, double z) {
  if (s.origin_zero) return make_float4(narrow_f64(x), narrow_f64(y), narrow_f64(z), 0.f);
  return make_float4(narrow_f64(x - s.origin[0]), narrow_f64(y - s.origin[1]), narrow_f64(z - s.origin[2]), 0.f);
}
__device__ __forceinline__ void make_pf2(const SysDesc& s, double x, double y, double z, float4& hi, float4& lo) {
  double rx = x, ry = y, rz = z;
  if (!s.origin_zero) {
    rx = x - s.origin[0];
    ry = y - s.origin[1];
    rz = z - s.origin[2];
  }
  hi = make_float4(narrow_f64(rx), narrow_f64(ry), narrow_f64(rz), 0.f);
  lo = make_float4(narrow_f64(rx - widen_f32(hi.x)), narrow_f64(ry - widen_f32(hi.y)), narrow_f64(rz - widen_f32(hi.z)),
                   0.f);
  hi.w = __uint_as_float(lo_code(lo.x, s.lo_inv_f) | (lo_code(lo.y, s.lo_inv_f) << 10) |
                         (lo_code(lo.z, s.lo_inv_f) << 20));
}

__device__ __forceinline__ double widen_f32(float f) {
  return __longlong_as_double(static_cast<long long>(widen_f32_bits(__float_as_uint(f))));
}
__device__ __forceinline__ double widen_f32_fast(float f) {
  return __longlong_as_double(static_cast<long long>(widen_f32_fast_bits(__float_as_uint(f))));
}

}  // namespace xnb
