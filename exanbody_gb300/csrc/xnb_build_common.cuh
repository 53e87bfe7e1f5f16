// Pieces shared by the neighbour-build kernels (xnb_build_kernels.cu: the
// lane-per-candidate and block-per-cell builds; xnb_build_rows.cu: the
// lane-per-particle build with bulk-copied rows).
//
// chunk_neighbors_execute (particle_neighbors/include/exanb/particle_neighbors/
// chunk_neighbors_execute.h:110-244, 286-372): for each particle of cell a, the
// particles of the 27 cells around a (periodic images included) with
// (cell_a != cell_b || p_a != p_b) && 0 < d2 <= nbh_dist^2, d2 = norm2(r_a - r_b),
// in (cell_enc, p_b) order. Ghost particles outside the partner block enlarged
// by ghost_dist are not candidates (update_ghosts_comm_scheme.cpp:462-469).
// Candidates are staged as FP32 positions relative to the system origin; the FP32
// distance decides whenever it lies farther than a proven error bound from the
// threshold, otherwise the reference's FP64 d2 (and FP64 ghost filter) decide,
// so the pair set is bit-exact.
#pragma once

#include "xnb_internal.cuh"

namespace xnb {
namespace build {

constexpr uint32_t kInvalid = 0xFFFFFFFFu;

__device__ __forceinline__ bool sys_flagged(const SysState* st, uint32_t s) { return st[s].rebuild != 0; }

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

constexpr uint32_t kAmbiguousBit = 0x80000000u;  // entry flag: ghost filter undecided in FP32

__device__ __forceinline__ float4 stage_from(const SysDesc& S, const float4 pb, uint32_t j, uint32_t gc) {
  float4 rb;
  rb.x = image_coord_f(pb.x, S.period_f[0], static_cast<int>(gc % 3u));
  rb.y = image_coord_f(pb.y, S.period_f[1], static_cast<int>((gc / 3u) % 3u));
  rb.z = image_coord_f(pb.z, S.period_f[2], static_cast<int>(gc / 9u));
  uint32_t ent = ((j - S.part_base) << 5) | gc;
  if (gc != static_cast<uint32_t>(kImageCenter)) {
    const float fm = S.filter_margin_f;
    const float v[3] = {rb.x, rb.y, rb.z};
    bool out = false, amb = false;
    for (int ax = 0; ax < 3; ++ax) {
      if (v[ax] < S.outer_lo_f[ax] - fm || v[ax] > S.outer_hi_f[ax] + fm) out = true;
      else if (v[ax] < S.outer_lo_f[ax] + fm || v[ax] > S.outer_hi_f[ax] - fm) amb = true;
    }
    if (out) {
      ent = kInvalid;
      rb.x = rb.y = rb.z = 1.0e18f;  // never within reach: the test needs no validity check
    } else if (amb) {
      ent |= kAmbiguousBit;
    }
  }
  rb.w = __uint_as_float(ent);
  return rb;
}

__device__ __forceinline__ float4 stage_candidate(const SysDesc& S, const DevArrays& a, uint32_t j, uint32_t gc) {
  return stage_from(S, a.pf[j], j, gc);
}

// The reference's FP64 decision for one (particle i, candidate entry) pair.
static __device__ __noinline__ bool exact_neighbor_test(const SysDesc& S, const DevArrays& a, uint32_t i, uint32_t ent) {
  const uint32_t e = ent & ~kAmbiguousBit;
  const uint32_t j = S.part_base + (e >> 5);
  const uint32_t gc = e & 31u;
  const double xb = image_coord(a.rx[j], S.period[0], static_cast<int>(gc % 3u));
  const double yb = image_coord(a.ry[j], S.period[1], static_cast<int>((gc / 3u) % 3u));
  const double zb = image_coord(a.rz[j], S.period[2], static_cast<int>(gc / 9u));
  bool keep = true;
  if (gc != static_cast<uint32_t>(kImageCenter))
    keep = xb >= S.outer_lo[0] && xb <= S.outer_hi[0] && yb >= S.outer_lo[1] && yb <= S.outer_hi[1] &&
           zb >= S.outer_lo[2] && zb <= S.outer_hi[2];
  const double d2 = norm2_rn(__dsub_rn(a.rx[i], xb), __dsub_rn(a.ry[i], yb), __dsub_rn(a.rz[i], zb));
  return keep && d2 > 0.0 && d2 <= S.nbh2;
}

// Lane-per-candidate chunk test shared by the warp-per-cell build
// (xnb_build_kernels.cu) and the sub-cell pruned build (xnb_build_sub.cu):
// lanes hold 32 staged candidates, NP particles are tested against them, and
// a ballot per particle appends its hits in candidate order to sbuf[k * lbuf + ...]
// (an entry past lbuf - 1 lands on the last word). t0 and low0 are positions in
// the candidate sequence: the particles' own entries sit at low0 + k.
constexpr int kNbrP = 4;  // particles tested per staged candidate load (even: FP32x2 pairs)

template <int NP, bool AMB, bool SELF>
__device__ __forceinline__ void nbr_chunk(const SysDesc& S, const DevArrays& a, const float4 b, const float (&px)[NP],
                                          const float (&py)[NP], const float (&pz)[NP], uint32_t i0,
                                          uint32_t self0, uint32_t t0, uint32_t low0, float nb_lo, float nb_hi,
                                          float nb_zero, unsigned lt, uint32_t* sbuf, uint32_t lbuf,
                                          uint32_t (&cur)[NP], uint32_t (&half)[NP]) {
  const uint32_t ent = __float_as_uint(b.w);
  const bool amb = AMB && (ent & kAmbiguousBit) != 0;
  bool hit[NP], may[NP];
  bool any_may = false;
  // squared FP32 distances two particles at a time on the packed FP32x2 path:
  // per particle the roundings of fmaf(dx, dx, fmaf(dy, dy, dz * dz)) exactly
  float dd[NP];
  {
    unsigned long long bx2, by2, bz2;
    asm("mov.b64 %0, {%1, %1};" : "=l"(bx2) : "f"(b.x));
    asm("mov.b64 %0, {%1, %1};" : "=l"(by2) : "f"(b.y));
    asm("mov.b64 %0, {%1, %1};" : "=l"(bz2) : "f"(b.z));
#pragma unroll
    for (int k = 0; k < NP; k += 2) {
      unsigned long long x2, y2, z2, dx, dy, dz, d;
      asm("mov.b64 %0, {%1, %2};" : "=l"(x2) : "f"(px[k]), "f"(px[k + 1]));
      asm("mov.b64 %0, {%1, %2};" : "=l"(y2) : "f"(py[k]), "f"(py[k + 1]));
      asm("mov.b64 %0, {%1, %2};" : "=l"(z2) : "f"(pz[k]), "f"(pz[k + 1]));
      asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(dx) : "l"(x2), "l"(bx2));
      asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(dy) : "l"(y2), "l"(by2));
      asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(dz) : "l"(z2), "l"(bz2));
      asm("mul.rn.f32x2 %0, %1, %1;" : "=l"(d) : "l"(dz));
      asm("fma.rn.f32x2 %0, %1, %1, %2;" : "=l"(d) : "l"(dy), "l"(d));
      asm("fma.rn.f32x2 %0, %1, %1, %2;" : "=l"(d) : "l"(dx), "l"(d));
      asm("mov.b64 {%0, %1}, %2;" : "=f"(dd[k]), "=f"(dd[k + 1]) : "l"(d));
    }
  }
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    const float d = dd[k];
    hit[k] = d < nb_lo && d > nb_zero && !amb;
    // the particle's own entry only sits in a SELF chunk (d = 0 there: no hit)
    may[k] = !hit[k] && d <= nb_hi && (!SELF || ent != self0 + (static_cast<uint32_t>(k) << 5));
    any_may |= may[k];
  }
  if (__any_sync(0xffffffffu, any_may)) {
#pragma unroll
    for (int k = 0; k < NP; ++k)
      if (may[k]) hit[k] = exact_neighbor_test(S, a, i0 + k, ent);
  }
  const uint32_t e = AMB ? (ent & ~kAmbiguousBit) : ent;
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    const unsigned m = __ballot_sync(0xffffffffu, hit[k]);
    // entries past the slot land in the buffer's last word, which is never written out
    if (hit[k]) sbuf[k * lbuf + min(cur[k] + __popc(m & lt), lbuf - 1u)] = e;
    if (SELF) {
      const uint32_t w = low0 + static_cast<uint32_t>(k) - t0;
      if (w < 32u) half[k] = cur[k] + __popc(m & ((1u << w) - 1u));
    }
    cur[k] += __popc(m);
  }
}

// Per-warp list statistics, flushed to the system's state when the warp moves
// on to another system's cells and at the end.
__device__ __forceinline__ void flush_list_stats(SysState* st, const SysDesc* sys, uint32_t s, uint32_t mx,
                                                 unsigned long long sum) {
  if (s == kInvalid) return;
  if (mx > sys[s].list_slot) atomicOr(&st[s].error, kErrListOverflow);
  atomicMax(&st[s].max_nbr, mx);
  atomicAdd(&st[s].list_used, sum);
}

}  // namespace build
}  // namespace xnb
