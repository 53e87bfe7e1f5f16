// Half-shell form of the neighbour build (chunk_neighbors, XNB_BUILD_HALF).
//
// The reference's lists (chunk_neighbors_execute.h:110-244, 286-372) hold, for
// each particle a, the particles b of the 27 cells around a's cell with
// 0 < d2 <= nbh^2 (and the ghost filter on b's image), in (cell_enc, p_b)
// order. The neighbour relation is symmetric in the distance, so each pair of
// cells is visited once here: the warp of cell c takes c itself and the 13
// cells after it in (dk, dj, di) order, and for each pair (p of c, q of the
// other cell) one distance decision gives both
//   - p's bit for q, in p's mask of that neighbour cell (group g), and
//   - q's bit for p, in q's mask of the opposite group 26 - g (where c lies,
//     seen through the opposite periodic image, 26 - code).
// Each direction keeps its own ghost filter (q's image for p, p's image for
// q). A second kernel turns each particle's 27 masks (64 bits: one per
// particle of the neighbour cell) into its list: groups in (dk, dj, di) order,
// set bits in index order, which is the reference's (cell_enc, p_b) order.
// The lower-half length is the count before the particle's own bit.
//
// The FP32 distance decides whenever it lies farther than the proven error
// bound from nbh^2 (the bound is the same for both directions: each FP64 d2
// lies within FP64 rounding of the other, far below the FP32 bound); inside the
// band, and where a ghost filter is undecided in FP32, the reference's FP64
// test decides each direction separately, so both lists are the reference's.
// Cells of at most 64 particles only: a system with a larger cell is flagged
// (SysState::half_bad) and built by the warp-per-cell kernels.
#include <algorithm>

#include "xnb_build_common.cuh"
#include "xnb_launch.cuh"

namespace xnb {

namespace {

using namespace build;

constexpr uint32_t kHalfMaxCell = 64;

// FP32 ghost filter of an image coordinate: 0 inside, 1 outside, 2 undecided
// (the same margins as stage_from).
__device__ __forceinline__ uint32_t filter_f(const SysDesc& S, float x, float y, float z) {
  const float fm = S.filter_margin_f;
  const float v[3] = {x, y, z};
  uint32_t r = 0;
  for (int ax = 0; ax < 3; ++ax) {
    if (v[ax] < S.outer_lo_f[ax] - fm || v[ax] > S.outer_hi_f[ax] + fm) return 1u;
    if (v[ax] < S.outer_lo_f[ax] + fm || v[ax] > S.outer_hi_f[ax] - fm) r = 2u;
  }
  return r;
}

__device__ __forceinline__ void neighbour_cell(const SysDesc& S, int ci, int cj, int ck, int g, uint32_t& src,
                                               uint32_t& code) {
  int n3[3] = {ci + g % 3 - 1, cj + (g / 3) % 3 - 1, ck + g / 9 - 1};
  int img[3];
  for (int ax = 0; ax < 3; ++ax) {
    img[ax] = 1;
    if (n3[ax] < 0) { n3[ax] += S.dims[ax]; img[ax] = 0; }
    else if (n3[ax] >= S.dims[ax]) { n3[ax] -= S.dims[ax]; img[ax] = 2; }
  }
  src = S.cell_base + static_cast<uint32_t>((n3[2] * S.dims[1] + n3[1]) * S.dims[0] + n3[0]);
  code = static_cast<uint32_t>(img[0] + 3 * img[1] + 9 * img[2]);
}

// One warp per cell: the masks of the cell's particles for groups 13..26 (rows)
// and of the 13 later cells' particles for the opposite groups 13..0 (columns).
__global__ void __launch_bounds__(128)
    k_nbr_half_test(uint32_t n_cells, const SysDesc* __restrict__ sys, SysState* st, DevArrays a) {
  if (*a.any_rebuild == 0) return;
  const unsigned full = 0xffffffffu;
  const uint32_t lane = threadIdx.x & 31;
  const size_t mstride = a.nmask_stride;
  const uint32_t nw_all = gridDim.x * (blockDim.x >> 5);
  for (uint32_t c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < n_cells; c += nw_all) {
    const uint32_t s = a.cell_sys[c];
    if (s == kInvalid || !sys_flagged(st, s)) continue;
    const uint32_t na = a.cell_n[c];
    if (na == 0) continue;
    if (na > kHalfMaxCell) {
      if (lane == 0) atomicOr(&st[s].half_bad, 1u);
      continue;
    }
    const SysDesc& S = sys[s];
    const uint32_t sa = a.cell_start[c];
    int ci, cj, ck;
    cell_ijk(S, c - S.cell_base, ci, cj, ck);
    // the cell's own particles: lane p holds p and p + 32 (absent ones far away)
    const float4 far_p = make_float4(-1.0e18f, -1.0e18f, -1.0e18f, 0.f);
    const float4 own0 = lane < na ? a.pf[sa + lane] : far_p;
    const float4 own1 = lane + 32 < na ? a.pf[sa + lane + 32] : far_p;
    const float nb_hi = S.nbh2_f + S.nbh_margin_f;
    const float nb_lo = S.nbh2_f - S.nbh_margin_f;
    const float nb_zero = S.nbh_margin_f;
    for (int g = 13; g < 27; ++g) {
      uint32_t src, code;
      neighbour_cell(S, ci, cj, ck, g, src, code);
      const uint32_t gn = a.cell_n[src];
      if (gn == 0) continue;
      if (gn > kHalfMaxCell) break;  // that cell's warp flags the system
      const uint32_t gs = a.cell_start[src];
      const bool self = g == 13;
      const bool image = code != static_cast<uint32_t>(kImageCenter);
      const int dx = static_cast<int>(code % 3u), dy = static_cast<int>((code / 3u) % 3u),
                dz = static_cast<int>(code / 9u);
      // the column direction sees p through the opposite image: its filter per p
      uint64_t pok = ~0ull, pamb = 0ull;
      if (image) {
        const uint32_t f0 = lane < na ? filter_f(S, image_coord_f(own0.x, S.period_f[0], 2 - dx),
                                                 image_coord_f(own0.y, S.period_f[1], 2 - dy),
                                                 image_coord_f(own0.z, S.period_f[2], 2 - dz))
                                      : 1u;
        const uint32_t f1 = lane + 32 < na ? filter_f(S, image_coord_f(own1.x, S.period_f[0], 2 - dx),
                                                      image_coord_f(own1.y, S.period_f[1], 2 - dy),
                                                      image_coord_f(own1.z, S.period_f[2], 2 - dz))
                                           : 1u;
        pok = static_cast<uint64_t>(__ballot_sync(full, f0 == 0u)) |
              (static_cast<uint64_t>(__ballot_sync(full, f1 == 0u)) << 32);
        pamb = static_cast<uint64_t>(__ballot_sync(full, f0 == 2u)) |
               (static_cast<uint64_t>(__ballot_sync(full, f1 == 2u)) << 32);
      }
      uint64_t row0 = 0ull, row1 = 0ull;  // this lane's particles' masks of group g
      for (uint32_t qs = 0; qs < gn; qs += 32) {
        const uint32_t q = qs + lane;
        const bool qv = q < gn;
        float4 b = qv ? a.pf[gs + q] : make_float4(1.0e18f, 1.0e18f, 1.0e18f, 0.f);
        uint32_t qf = 0u;
        if (image && qv) {
          b.x = image_coord_f(b.x, S.period_f[0], dx);
          b.y = image_coord_f(b.y, S.period_f[1], dy);
          b.z = image_coord_f(b.z, S.period_f[2], dz);
          qf = filter_f(S, b.x, b.y, b.z);
        }
        const bool qok = qv && qf == 0u;
        const bool qamb = qv && qf == 2u;
        uint64_t col = 0ull;
        for (uint32_t p0 = 0; p0 < na; p0 += kNbrP) {
          float px[kNbrP], py[kNbrP], pz[kNbrP];
#pragma unroll
          for (int k = 0; k < kNbrP; ++k) {
            const uint32_t p = p0 + k;
            const bool lo = p < 32u;
            const int sl = static_cast<int>(p & 31u);
            const float x0 = __shfl_sync(full, own0.x, sl), x1 = __shfl_sync(full, own1.x, sl);
            const float y0 = __shfl_sync(full, own0.y, sl), y1 = __shfl_sync(full, own1.y, sl);
            const float z0 = __shfl_sync(full, own0.z, sl), z1 = __shfl_sync(full, own1.z, sl);
            px[k] = lo ? x0 : x1;
            py[k] = lo ? y0 : y1;
            pz[k] = lo ? z0 : z1;
          }
          float dd[kNbrP];
#pragma unroll
          for (int k = 0; k < kNbrP; ++k) {
            const float ex = px[k] - b.x, ey = py[k] - b.y, ez = pz[k] - b.z;
            dd[k] = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
          }
          bool rh[kNbrP], ch[kNbrP], slow[kNbrP];
          bool any_slow = false;
#pragma unroll
          for (int k = 0; k < kNbrP; ++k) {
            const uint32_t p = p0 + k;
            const bool pv = p < na;
            const bool in = dd[k] < nb_lo && dd[k] > nb_zero;
            const bool band = !in && dd[k] <= nb_hi && !(self && q == p);
            const bool po = ((pok >> p) & 1ull) != 0ull;
            const bool pa = ((pamb >> p) & 1ull) != 0ull;
            rh[k] = in && qok;
            ch[k] = !self && in && qv && po;
            slow[k] = qv && pv && (band || (in && (qamb || (!self && pa))));
            any_slow |= slow[k];
          }
          if (__any_sync(full, any_slow)) {
#pragma unroll
            for (int k = 0; k < kNbrP; ++k) {
              if (slow[k]) {
                const uint32_t ip = sa + p0 + k, iq = gs + q;
                rh[k] = exact_neighbor_test(S, a, ip, ((iq - S.part_base) << 5) | code);
                if (!self) ch[k] = exact_neighbor_test(S, a, iq, ((ip - S.part_base) << 5) | (26u - code));
              }
            }
          }
#pragma unroll
          for (int k = 0; k < kNbrP; ++k) {
            const uint32_t p = p0 + k;
            const uint64_t m = static_cast<uint64_t>(__ballot_sync(full, rh[k])) << qs;
            if (lane == (p & 31u)) {
              if (p < 32u) row0 |= m;
              else row1 |= m;
            }
            col |= static_cast<uint64_t>(ch[k] ? 1u : 0u) << (p & 63u);
          }
        }
        if (!self && qv) a.nmask[static_cast<size_t>(26 - g) * mstride + gs + q] = col;
      }
      if (lane < na) a.nmask[static_cast<size_t>(g) * mstride + sa + lane] = row0;
      if (lane + 32 < na) a.nmask[static_cast<size_t>(g) * mstride + sa + lane + 32] = row1;
    }
  }
}

// One warp per cell, one lane per particle: each particle's list from its 27
// masks, with its count, lower-half length and slot start.
__global__ void __launch_bounds__(128)
    k_nbr_half_emit(uint32_t n_cells, const SysDesc* __restrict__ sys, SysState* st, DevArrays a) {
  if (*a.any_rebuild == 0) return;
  const unsigned full = 0xffffffffu;
  const uint32_t lane = threadIdx.x & 31;
  const size_t mstride = a.nmask_stride;
  uint32_t acc_s = kInvalid, acc_max = 0;
  unsigned long long acc_sum = 0;
  const uint32_t nw_all = gridDim.x * (blockDim.x >> 5);
  for (uint32_t c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < n_cells; c += nw_all) {
    const uint32_t s = a.cell_sys[c];
    if (s == kInvalid || !sys_flagged(st, s) || st[s].half_bad) continue;
    const uint32_t na = a.cell_n[c];
    if (na == 0) continue;
    const SysDesc& S = sys[s];
    const uint32_t sa = a.cell_start[c];
    int ci, cj, ck;
    cell_ijk(S, c - S.cell_base, ci, cj, ck);
    uint32_t g_start = 0, g_n = 0, g_code = kImageCenter;
    if (lane < 27) {
      uint32_t src;
      neighbour_cell(S, ci, cj, ck, static_cast<int>(lane), src, g_code);
      g_start = a.cell_start[src];
      g_n = a.cell_n[src];
    }
    if (s != acc_s) {
      if (lane == 0) flush_list_stats(st, sys, acc_s, acc_max, acc_sum);
      acc_s = s;
      acc_max = 0;
      acc_sum = 0;
    }
    const uint32_t slot = S.list_slot;
    uint32_t* const seg = a.nbr + S.list_base;
    for (uint32_t ps = 0; ps < na; ps += 32) {
      const uint32_t p = ps + lane;
      const bool valid = p < na;
      const uint32_t i = sa + p;
      const uint32_t base = (i - S.part_base) * slot;  // the host keeps npart * slot below 2^32
      uint32_t cnt = 0, half = 0;
      for (int g = 0; g < 27; ++g) {
        const uint32_t gn = __shfl_sync(full, g_n, g);
        const uint32_t gs = __shfl_sync(full, g_start, g);
        const uint32_t code = __shfl_sync(full, g_code, g);
        if (gn == 0) continue;
        uint64_t m = valid ? a.nmask[static_cast<size_t>(g) * mstride + i] : 0ull;
        if (g == 13) half = cnt + static_cast<uint32_t>(__popcll(m & ((1ull << (p & 63u)) - 1ull)));
        const uint32_t eb = ((gs - S.part_base) << 5) | code;
        while (m) {
          const uint32_t bit = static_cast<uint32_t>(__ffsll(static_cast<long long>(m)) - 1);
          m &= m - 1ull;
          if (cnt < slot) seg[base + cnt] = eb + (bit << 5);
          ++cnt;
        }
      }
      if (valid) {
        a.nbr_cnt[i] = cnt;
        a.nbr_half[i] = half;
        a.nbr_start[i] = base;
      }
      uint32_t mx = valid ? cnt : 0u;
      unsigned long long sm = valid ? cnt : 0u;
      for (int o = 16; o > 0; o >>= 1) {
        mx = max(mx, __shfl_xor_sync(full, mx, o));
        sm += __shfl_xor_sync(full, sm, o);
      }
      acc_max = max(acc_max, mx);
      acc_sum += sm;
    }
  }
  if (lane == 0) flush_list_stats(st, sys, acc_s, acc_max, acc_sum);
}

inline int warp_blocks(uint32_t n_cells, int sm_count, const void* kern) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, 0) != cudaSuccess || per_sm < 1) per_sm = 1;
  const long long want = (static_cast<long long>(n_cells) + 3) / 4;
  return static_cast<int>(std::max(1ll, std::min(want, static_cast<long long>(per_sm) * sm_count)));
}

}  // namespace

int launch_neighbors_half_test(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a,
                               cudaStream_t stream) {
  if (ex.n_cells == 0) return 0;
  k_nbr_half_test<<<warp_blocks(ex.n_cells, ex.sm_count, reinterpret_cast<const void*>(k_nbr_half_test)), 128, 0,
                    stream>>>(ex.n_cells, sys, st, a);
  return 1;
}

int launch_neighbors_half_emit(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a,
                               cudaStream_t stream) {
  if (ex.n_cells == 0) return 0;
  k_nbr_half_emit<<<warp_blocks(ex.n_cells, ex.sm_count, reinterpret_cast<const void*>(k_nbr_half_emit)), 128, 0,
                    stream>>>(ex.n_cells, sys, st, a);
  return 1;
}

}  // namespace xnb
