// Lane-per-particle form of the neighbour build (chunk_neighbors), with the
// candidates staged one row of three cells at a time by bulk copies.
//
// One warp per cell; lane l owns particles l and l + 32 of the cell. The 27
// neighbour cells are visited as 9 rows (dk, dj) of three x-adjacent cells
// (di = -1, 0, +1), which keeps the reference's (cell_enc, p_b) candidate
// order. Each cell of a row is one contiguous range of the FP32 position
// mirrors (16 bytes per particle), so one lane moves a row into shared memory
// with up to three cp.async.bulk copies completing on an mbarrier; the copy of
// the next row is in flight while the warp tests the current one. The warp then
// applies the periodic image and ghost filter to the row (stage_from) into
// structure-of-arrays form, and every lane tests its particle against four
// candidates per iteration: the four x (then y, z) arrive in one shared load
// and the squared distances of two candidates at a time run on the packed
// FP32x2 pipe. A lane appends its hits, in order, to its particle's buffer in
// shared memory; the warp writes the buffers out to the particles' list slots
// when one may fill up and at the end of the cell. Near the cutoff the FP32
// distance is undecided and the reference's FP64 test decides (warp-uniform
// branch), as it does for candidates whose ghost filter is undecided in FP32
// and for the iterations that hold the particles' own entries (self exclusion
// and the lower-half length).
//
// Cells with more than 64 particles or a row of more than kRowCap candidates
// are appended to a.nbr_wide for the block-per-cell build (xnb_build_kernels.cu).
#include "xnb_build_common.cuh"
#include "xnb_launch.cuh"

namespace xnb {

namespace {

using namespace build;

constexpr int kRowCap = 128;                   // candidates of one row staged at once
constexpr int kBufDepth = 32;                  // entries buffered per particle (16 each for two per lane)
constexpr int kBufStride = kBufDepth + 1;      // odd stride: the warp's flush reads are conflict-free
constexpr uint32_t kNoEntry = 0x7FFFFFFFu;     // staged padding / filtered candidate (never a real entry)
constexpr uint32_t kWaitLimit = 1u << 22;      // mbarrier polls before a copy counts as lost

struct __align__(16) RowsWarp {
  float4 raw[2][kRowCap];                      // bulk-copied mirrors of a row (two in flight)
  float xs[kRowCap], ys[kRowCap], zs[kRowCap]; // the row staged: image applied, relative to the origin
  uint32_t ws[kRowCap];                        // entries ((index << 5) | code [| kAmbiguousBit]) or kNoEntry
  uint32_t buf[32 * kBufStride];               // per-lane list buffers
  unsigned long long bar[2];
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void bar_init(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void bar_expect(unsigned long long* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ bool bar_try(unsigned long long* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for a phase of a row barrier: false when the copy never landed.
__device__ __forceinline__ bool bar_wait(unsigned long long* bar, uint32_t parity) {
  for (uint32_t it = 0; it < kWaitLimit; ++it)
    if (bar_try(bar, parity)) return true;
  return false;
}

// Row r (0..8) of cell (ci, cj, ck): lanes 0..2 describe its cells di = -1, 0, +1
// (start, count, image code); the cell of lane g is group 3r + g of the 27.
__device__ __forceinline__ void row_groups(const SysDesc& S, const DevArrays& a, int ci, int cj, int ck, int r,
                                           uint32_t lane, uint32_t& g_start, uint32_t& g_n, uint32_t& g_code) {
  g_start = 0;
  g_n = 0;
  g_code = kImageCenter;
  if (lane < 3) {
    int n3[3] = {ci + static_cast<int>(lane) - 1, cj + (r % 3) - 1, ck + (r / 3) - 1};
    int img[3];
    for (int ax = 0; ax < 3; ++ax) {
      img[ax] = 1;
      if (n3[ax] < 0) {
        n3[ax] += S.dims[ax];
        img[ax] = 0;
      } else if (n3[ax] >= S.dims[ax]) {
        n3[ax] -= S.dims[ax];
        img[ax] = 2;
      }
    }
    const uint32_t src = S.cell_base + static_cast<uint32_t>((n3[2] * S.dims[1] + n3[1]) * S.dims[0] + n3[0]);
    g_start = a.cell_start[src];
    g_n = a.cell_n[src];
    g_code = static_cast<uint32_t>(img[0] + 3 * img[1] + 9 * img[2]);
  }
}

// Lane 0 starts the bulk copies of a row's mirrors into raw[buf]; the row's
// candidate count comes back (0 copies complete the phase at once).
__device__ __forceinline__ uint32_t issue_row(RowsWarp& w, int bufi, const DevArrays& a, uint32_t g_start,
                                              uint32_t g_n, uint32_t lane) {
  const uint32_t n0 = __shfl_sync(0xffffffffu, g_n, 0), n1 = __shfl_sync(0xffffffffu, g_n, 1),
                 n2 = __shfl_sync(0xffffffffu, g_n, 2);
  const uint32_t s0 = __shfl_sync(0xffffffffu, g_start, 0), s1 = __shfl_sync(0xffffffffu, g_start, 1),
                 s2 = __shfl_sync(0xffffffffu, g_start, 2);
  const uint32_t total = n0 + n1 + n2;
  if (lane == 0 && total <= static_cast<uint32_t>(kRowCap)) {
    // the generic-proxy reads of this buffer (two rows ago) are ordered before the copy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    bar_expect(&w.bar[bufi], total * 16u);
    if (n0) bulk_copy(&w.raw[bufi][0], a.pf + s0, n0 * 16u, &w.bar[bufi]);
    if (n1) bulk_copy(&w.raw[bufi][n0], a.pf + s1, n1 * 16u, &w.bar[bufi]);
    if (n2) bulk_copy(&w.raw[bufi][n0 + n1], a.pf + s2, n2 * 16u, &w.bar[bufi]);
  }
  return total;
}

// Writes out the buffered entries of every particle of the cell (pending counts
// in ptr - rbase, in words) to their list slots, entries past the slot dropped.
template <int PPL>
__device__ __forceinline__ void flush_lists(RowsWarp& w, uint32_t* seg, uint32_t na, uint32_t first_local,
                                            uint32_t slot, uint32_t lane, uint32_t (&ptr)[PPL],
                                            const uint32_t (&rbase)[PPL], uint32_t (&written)[PPL]) {
  __syncwarp();
  uint32_t pend[PPL];
#pragma unroll
  for (int q = 0; q < PPL; ++q) pend[q] = ptr[q] - rbase[q];
  for (uint32_t p = 0; p < na; ++p) {
    const uint32_t owner = p & 31u;
    const bool second = PPL == 2 && p >= 32u;
    const uint32_t cnt = __shfl_sync(0xffffffffu, second ? pend[PPL - 1] : pend[0], owner);
    if (cnt == 0) continue;
    const uint32_t wr = __shfl_sync(0xffffffffu, second ? written[PPL - 1] : written[0], owner);
    const uint32_t from = owner * kBufStride + (second ? kBufDepth / 2 : 0u);
    if (lane < cnt && wr + lane < slot) seg[(first_local + p) * slot + wr + lane] = w.buf[from + lane];
  }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < PPL; ++q) {
    written[q] += pend[q];
    ptr[q] = rbase[q];
  }
}

// Tests the staged row (m candidates, padded to a multiple of 4 with unreachable
// dummies) against the lane's particle(s). self_lo..self_hi: the row-local
// range of the cell's own particles (empty outside the centre row).
template <int PPL>
__device__ __forceinline__ void test_row(RowsWarp& w, const SysDesc& S, const DevArrays& a, uint32_t m,
                                         uint32_t self_lo, uint32_t self_hi, uint32_t lane, const float (&px)[PPL],
                                         const float (&py)[PPL], const float (&pz)[PPL], const uint32_t (&pi)[PPL],
                                         const uint32_t (&pself)[PPL], uint32_t (&ptr)[PPL],
                                         const uint32_t (&rbase)[PPL], uint32_t (&written)[PPL],
                                         uint32_t (&half)[PPL], uint32_t* seg, uint32_t na, uint32_t first_local,
                                         uint32_t slot, float nb_lo, float nb_hi, float nb_zero) {
  constexpr uint32_t kLimit = (PPL == 2 ? kBufDepth / 2 : kBufDepth) - 4;
  unsigned long long ax2[PPL], ay2[PPL], az2[PPL];
#pragma unroll
  for (int q = 0; q < PPL; ++q) {
    asm("mov.b64 %0, {%1, %1};" : "=l"(ax2[q]) : "f"(px[q]));
    asm("mov.b64 %0, {%1, %1};" : "=l"(ay2[q]) : "f"(py[q]));
    asm("mov.b64 %0, {%1, %1};" : "=l"(az2[q]) : "f"(pz[q]));
  }
  for (uint32_t k = 0; k < m; k += 4) {
    bool full = false;
#pragma unroll
    for (int q = 0; q < PPL; ++q) full |= ptr[q] - rbase[q] > kLimit;
    if (__any_sync(0xffffffffu, full)) flush_lists<PPL>(w, seg, na, first_local, slot, lane, ptr, rbase, written);
    const float4 X = *reinterpret_cast<const float4*>(&w.xs[k]);
    const float4 Y = *reinterpret_cast<const float4*>(&w.ys[k]);
    const float4 Z = *reinterpret_cast<const float4*>(&w.zs[k]);
    const uint4 W = *reinterpret_cast<const uint4*>(&w.ws[k]);
    const uint32_t ent[4] = {W.x, W.y, W.z, W.w};
    unsigned long long bx01, bx23, by01, by23, bz01, bz23;
    asm("mov.b64 %0, {%1, %2};" : "=l"(bx01) : "f"(X.x), "f"(X.y));
    asm("mov.b64 %0, {%1, %2};" : "=l"(bx23) : "f"(X.z), "f"(X.w));
    asm("mov.b64 %0, {%1, %2};" : "=l"(by01) : "f"(Y.x), "f"(Y.y));
    asm("mov.b64 %0, {%1, %2};" : "=l"(by23) : "f"(Y.z), "f"(Y.w));
    asm("mov.b64 %0, {%1, %2};" : "=l"(bz01) : "f"(Z.x), "f"(Z.y));
    asm("mov.b64 %0, {%1, %2};" : "=l"(bz23) : "f"(Z.z), "f"(Z.w));
    float d[PPL][4];
#pragma unroll
    for (int q = 0; q < PPL; ++q) {
      // per candidate the roundings of fmaf(dx, dx, fmaf(dy, dy, dz * dz))
      unsigned long long dx, dy, dz, s01, s23;
      asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(dz) : "l"(bz01), "l"(az2[q]));
      asm("mul.rn.f32x2 %0, %1, %1;" : "=l"(s01) : "l"(dz));
      asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(dy) : "l"(by01), "l"(ay2[q]));
      asm("fma.rn.f32x2 %0, %1, %1, %2;" : "=l"(s01) : "l"(dy), "l"(s01));
      asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(dx) : "l"(bx01), "l"(ax2[q]));
      asm("fma.rn.f32x2 %0, %1, %1, %2;" : "=l"(s01) : "l"(dx), "l"(s01));
      asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(dz) : "l"(bz23), "l"(az2[q]));
      asm("mul.rn.f32x2 %0, %1, %1;" : "=l"(s23) : "l"(dz));
      asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(dy) : "l"(by23), "l"(ay2[q]));
      asm("fma.rn.f32x2 %0, %1, %1, %2;" : "=l"(s23) : "l"(dy), "l"(s23));
      asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(dx) : "l"(bx23), "l"(ax2[q]));
      asm("fma.rn.f32x2 %0, %1, %1, %2;" : "=l"(s23) : "l"(dx), "l"(s23));
      asm("mov.b64 {%0, %1}, %2;" : "=f"(d[q][0]), "=f"(d[q][1]) : "l"(s01));
      asm("mov.b64 {%0, %1}, %2;" : "=f"(d[q][2]), "=f"(d[q][3]) : "l"(s23));
    }
    bool hit[PPL][4];
    bool und = false;
#pragma unroll
    for (int q = 0; q < PPL; ++q)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        hit[q][j] = d[q][j] < nb_lo && d[q][j] > nb_zero;
        und |= !hit[q][j] && d[q][j] <= nb_hi;
      }
    // warp-uniform: an FP32-undecided distance, a ghost filter undecided in
    // FP32 (the entry's top bit), or the particles' own entries in this group
    const bool amb = ((W.x | W.y | W.z | W.w) & kAmbiguousBit) != 0;
    const bool self_here = k < self_hi && self_lo < k + 4;
    if (__any_sync(0xffffffffu, und) || amb || self_here) {
#pragma unroll
      for (int q = 0; q < PPL; ++q)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const uint32_t idx = k + static_cast<uint32_t>(j);
          if (pi[q] == kInvalid) {
            hit[q][j] = false;
          } else if (self_here && idx == pself[q]) {
            hit[q][j] = false;
            // the particle's own position in (cell_enc, p_b) order: the entries
            // before it are the lower half of the symmetric split
            half[q] = written[q] + (ptr[q] - rbase[q]);
          } else if (d[q][j] <= nb_hi && (!hit[q][j] || (ent[j] & kAmbiguousBit))) {
            hit[q][j] = exact_neighbor_test(S, a, pi[q], ent[j]);
          }
          if (hit[q][j]) {
            w.buf[ptr[q]] = ent[j] & ~kAmbiguousBit;
            ++ptr[q];
          }
        }
    } else {
#pragma unroll
      for (int q = 0; q < PPL; ++q)
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (hit[q][j]) {
            w.buf[ptr[q]] = ent[j];
            ++ptr[q];
          }
    }
  }
}

__device__ __forceinline__ void rows_stats(SysState* st, const SysDesc* sys, uint32_t s, uint32_t mx,
                                           unsigned long long sum, uint32_t lane) {
  for (int off = 16; off > 0; off >>= 1) {
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    sum += __shfl_xor_sync(0xffffffffu, sum, off);
  }
  if (lane == 0) flush_list_stats(st, sys, s, mx, sum);
}

// Processes cell c with PPL particles per lane (na <= 32 * PPL). Returns false
// when a row's copy never completed (the kernel then stops).
template <int PPL>
__device__ __forceinline__ bool rows_cell(RowsWarp& w, const SysDesc& S, SysState* st, const DevArrays& a,
                                          uint32_t c, uint32_t s, uint32_t na, uint32_t sa, int ci, int cj, int ck,
                                          uint32_t lane, uint32_t (&phase)[2], uint32_t first_total,
                                          uint32_t& acc_max, unsigned long long& acc_sum) {
  const float nb_hi = S.nbh2_f + S.nbh_margin_f;
  const float nb_lo = S.nbh2_f - S.nbh_margin_f;
  const float nb_zero = S.nbh_margin_f;
  const uint32_t slot = S.list_slot;
  uint32_t* const seg = a.nbr + S.list_base;
  const uint32_t first_local = sa - S.part_base;
  float px[PPL], py[PPL], pz[PPL];
  uint32_t pi[PPL], ptr[PPL], rbase[PPL], written[PPL], half[PPL], pself[PPL];
#pragma unroll
  for (int q = 0; q < PPL; ++q) {
    const uint32_t p = lane + 32u * q;
    const bool valid = p < na;
    const float4 m = valid ? a.pf[sa + p] : make_float4(-1.0e18f, -1.0e18f, -1.0e18f, 0.f);
    px[q] = m.x;
    py[q] = m.y;
    pz[q] = m.z;
    pi[q] = valid ? sa + p : kInvalid;
    rbase[q] = lane * kBufStride + (q == 1 ? kBufDepth / 2 : 0u);
    ptr[q] = rbase[q];
    written[q] = 0;
    half[q] = 0;
    pself[q] = kInvalid;
  }
  uint32_t total = first_total;  // row 0's copies were started by the caller
  for (int r = 0; r < 9; ++r) {
    const int cur = r & 1;
    // next row's copies go out before this row is staged
    uint32_t next_total = 0;
    if (r < 8) {
      uint32_t gs, gn, gc;
      row_groups(S, a, ci, cj, ck, r + 1, lane, gs, gn, gc);
      next_total = issue_row(w, cur ^ 1, a, gs, gn, lane);
    }
    // this row's groups again, for the staging pass
    uint32_t g_start, g_n, g_code;
    row_groups(S, a, ci, cj, ck, r, lane, g_start, g_n, g_code);
    if (!bar_wait(&w.bar[cur], phase[cur])) {
      // a lost copy: flag the system and wait (bounded) for the other one
      if (lane == 0) atomicOr(&st[s].error, static_cast<uint32_t>(kErrStage));
      if (r < 8) bar_wait(&w.bar[cur ^ 1], phase[cur ^ 1]);
      return false;
    }
    phase[cur] ^= 1u;
    const uint32_t n0 = __shfl_sync(0xffffffffu, g_n, 0), n1 = __shfl_sync(0xffffffffu, g_n, 1);
    const uint32_t c0 = __shfl_sync(0xffffffffu, g_code, 0), c1 = __shfl_sync(0xffffffffu, g_code, 1),
                   c2 = __shfl_sync(0xffffffffu, g_code, 2);
    const uint32_t s0 = __shfl_sync(0xffffffffu, g_start, 0), s1 = __shfl_sync(0xffffffffu, g_start, 1),
                   s2 = __shfl_sync(0xffffffffu, g_start, 2);
    const uint32_t m4 = (total + 3u) & ~3u;
    for (uint32_t u = lane; u < m4; u += 32) {
      if (u < total) {
        const uint32_t g = u < n0 ? 0u : (u < n0 + n1 ? 1u : 2u);
        const uint32_t j = g == 0 ? s0 + u : (g == 1 ? s1 + u - n0 : s2 + u - n0 - n1);
        const uint32_t gc = g == 0 ? c0 : (g == 1 ? c1 : c2);
        const float4 v = stage_from(S, w.raw[cur][u], j, gc);
        const uint32_t e = __float_as_uint(v.w);
        w.xs[u] = v.x;
        w.ys[u] = v.y;
        w.zs[u] = v.z;
        w.ws[u] = e == kInvalid ? kNoEntry : e;
      } else {
        w.xs[u] = 1.0e18f;
        w.ys[u] = 1.0e18f;
        w.zs[u] = 1.0e18f;
        w.ws[u] = kNoEntry;
      }
    }
    __syncwarp();
    uint32_t self_lo = 0, self_hi = 0;  // outside the centre row no candidate is the particle itself
    if (r == 4) {
      // the centre cell is group 1 of the centre row: its particles' own entries
      self_lo = n0;
      self_hi = n0 + na;
#pragma unroll
      for (int q = 0; q < PPL; ++q)
        if (pi[q] != kInvalid) pself[q] = n0 + lane + 32u * q;
    }
    test_row<PPL>(w, S, a, m4, self_lo, self_hi, lane, px, py, pz, pi, pself, ptr, rbase, written, half, seg, na,
                  first_local, slot, nb_lo, nb_hi, nb_zero);
    __syncwarp();
    total = next_total;
  }
  flush_lists<PPL>(w, seg, na, first_local, slot, lane, ptr, rbase, written);
#pragma unroll
  for (int q = 0; q < PPL; ++q) {
    if (pi[q] != kInvalid) {
      const uint32_t i = pi[q];
      a.nbr_cnt[i] = written[q];
      a.nbr_half[i] = half[q];
      a.nbr_start[i] = (i - S.part_base) * slot;  // the host keeps npart * slot below 2^32
      acc_max = max(acc_max, written[q]);
      acc_sum += written[q];
    }
  }
  (void)c;
  return true;
}

__global__ void __launch_bounds__(128)
    k_neighbors_rows(uint32_t n_cells, const SysDesc* __restrict__ sys, SysState* st, DevArrays a, bool prune) {
  if (*a.any_rebuild == 0) return;
  extern __shared__ __align__(16) unsigned char rows_smem[];
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t wib = threadIdx.x >> 5;
  const uint32_t nwarp = blockDim.x >> 5;
  RowsWarp& w = reinterpret_cast<RowsWarp*>(rows_smem)[wib];
  if (lane == 0) {
    bar_init(&w.bar[0]);
    bar_init(&w.bar[1]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  uint32_t phase[2] = {0u, 0u};
  uint32_t acc_s = kInvalid, acc_max = 0;
  unsigned long long acc_sum = 0;
  const uint32_t nw_all = gridDim.x * nwarp;
  for (uint32_t c = blockIdx.x * nwarp + wib; c < n_cells; c += nw_all) {
    const uint32_t s = a.cell_sys[c];
    if (s == kInvalid || !sys_flagged(st, s)) continue;
    const uint32_t na = a.cell_n[c];
    if (na == 0) continue;
    if (prune && a.cside[c] >= 2 && st[s].keys_fresh) {
      if (lane == 0) a.nbr_sub[atomicAdd(a.nbr_sub_n, 1u)] = c;
      continue;
    }
    const SysDesc& S = sys[s];
    int ci, cj, ck;
    cell_ijk(S, c - S.cell_base, ci, cj, ck);
    // every row must fit the stage: the 27 cells' counts, 3 per row
    uint32_t g_n = 0;
    if (lane < 27) {
      int n3[3] = {ci + static_cast<int>(lane % 3) - 1, cj + static_cast<int>((lane / 3) % 3) - 1,
                   ck + static_cast<int>(lane / 9) - 1};
      for (int ax = 0; ax < 3; ++ax) {
        if (n3[ax] < 0) n3[ax] += S.dims[ax];
        else if (n3[ax] >= S.dims[ax]) n3[ax] -= S.dims[ax];
      }
      g_n = a.cell_n[S.cell_base + static_cast<uint32_t>((n3[2] * S.dims[1] + n3[1]) * S.dims[0] + n3[0])];
    }
    uint32_t row_n = g_n + __shfl_down_sync(0xffffffffu, g_n, 1) + __shfl_down_sync(0xffffffffu, g_n, 2);
    const bool row_over = (lane % 3 == 0 && lane < 27 && row_n > static_cast<uint32_t>(kRowCap));
    if (na > 64u || __any_sync(0xffffffffu, row_over)) {
      if (lane == 0) a.nbr_wide[atomicAdd(a.nbr_wide_n, 1u)] = c;
      continue;
    }
    if (s != acc_s) {
      rows_stats(st, sys, acc_s, acc_max, acc_sum, lane);
      acc_s = s;
      acc_max = 0;
      acc_sum = 0;
    }
    uint32_t gs, gn, gc;
    row_groups(S, a, ci, cj, ck, 0, lane, gs, gn, gc);
    const uint32_t first_total = issue_row(w, 0, a, gs, gn, lane);
    const uint32_t sa = a.cell_start[c];
    // the 9 rows alternate between the two buffers: row 0 always starts in buffer 0
    const bool ok = na <= 32u ? rows_cell<1>(w, S, st, a, c, s, na, sa, ci, cj, ck, lane, phase, first_total,
                                             acc_max, acc_sum)
                              : rows_cell<2>(w, S, st, a, c, s, na, sa, ci, cj, ck, lane, phase, first_total,
                                             acc_max, acc_sum);
    if (!ok) return;
  }
  rows_stats(st, sys, acc_s, acc_max, acc_sum, lane);
}

}  // namespace

int launch_neighbors_rows(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, cudaStream_t stream,
                          bool prune) {
  if (ex.n_cells == 0) return 0;
  const size_t smem = 4 * sizeof(RowsWarp);
  cudaFuncSetAttribute(k_neighbors_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_neighbors_rows, 128, smem) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const long long want = (static_cast<long long>(ex.n_cells) + 3) / 4;
  const int grid = static_cast<int>(std::max(1ll, std::min(want, static_cast<long long>(per_sm) * ex.sm_count)));
  k_neighbors_rows<<<grid, 128, smem, stream>>>(ex.n_cells, sys, st, a, prune);
  return 1;
}

}  // namespace xnb
