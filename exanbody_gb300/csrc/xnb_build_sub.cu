// Sub-cell pruned form of the neighbour build (chunk_neighbors) for dense cells.
//
// chunk_neighbors_execute (particle_neighbors/include/exanb/particle_neighbors/
// chunk_neighbors_execute.h:160-244) takes, for each pair of neighbouring
// cells, only the pairs of AMR sub-cells whose boxes lie within nbh_dist of each
// other (the table of max_distance_sub_cell_pairs, amr/lib/amr_grid_algorithm.cpp:
// 102-218: minimum distance between the two boxes <= max_dist), then orders each
// particle's hits by (cell_enc, p_b). Here each cell's particles are already in
// sub-cell order (k_rebin_finalize), so for the particles of one sub-cell A the
// candidates of the 27 cells around it, restricted to the sub-cells within reach
// of A, form a sequence of index ranges that is itself in (cell_enc, p_b) order.
// The lane-per-candidate chunk test over that sequence writes the same lists as
// the unpruned build: the pruning only leaves out candidates that cannot lie
// within nbh_dist.
//
// Reach: with sub-grid sides sA and sB, both boxes have integer corners on the
// grid of cell_size / (sA sB), so their squared gap in those units is an exact
// integer; it is compared with (sub_reach_f sA sB)^2, sub_reach_f being
// nbh_dist / cell_size widened by 1e-5. A particle lies inside its cell up to
// 2^-48 cell sizes (k_rebin_dest's epsilon) and inside its sub-cell up to the
// rounding of its key, both far inside the widening, so no neighbour is lost.
//
// One block of four warps per dense cell: the block fills the sub-cell start
// tables of the 27 neighbour cells in shared memory from the particles' keys,
// then each warp takes sub-cells A of the cell, lays out A's candidate ranges,
// stages them (`cap` candidates per round) and tests A's particles four at a
// time. Hits go straight to the particles' list slots, counts carry across
// rounds in nbr_cnt / nbr_half. A cell with a neighbour of sub-grid side above 3
// is passed on to the unpruned block-per-cell build.
#include <algorithm>

#include "xnb_build_common.cuh"
#include "xnb_launch.cuh"

namespace xnb {

namespace {

using namespace build;

constexpr int kSubMaxSide = 3;
constexpr int kSubCells = kSubMaxSide * kSubMaxSide * kSubMaxSide;
constexpr int kSubMaxRanges = 27 * ((kSubCells + 1) / 2);  // runs of kept sub-cells: at most 14 per cell

struct SubTables {
  uint32_t start[27][kSubCells + 1];  // first particle of each sub-cell, relative to its cell's first particle
};

struct SubRanges {
  uint32_t first[kSubMaxRanges];    // first particle (global index) of each candidate range
  uint32_t pos[kSubMaxRanges + 1];  // position of each range in the candidate sequence; pos[R] = length
  uint32_t code[kSubMaxRanges];     // periodic image code of the range's cell
};

__host__ __device__ constexpr size_t sub_stage_offset(int nwarp) {
  return (sizeof(SubTables) + static_cast<size_t>(nwarp) * sizeof(SubRanges) + 15) & ~static_cast<size_t>(15);
}

// gap between sub-cell ia of a cell of side sa and sub-cell ib of the cell d
// cells away (side sb), in units of cell_size / (sa sb)
__device__ __forceinline__ int box_gap(int ia, int sa, int d, int ib, int sb) {
  const int alo = ia * sb, ahi = alo + sb;
  const int blo = d * sa * sb + ib * sa, bhi = blo + sa;
  return max(0, max(blo - ahi, alo - bhi));
}

__global__ void __launch_bounds__(128)
    k_neighbors_sub(uint32_t n_cells, const SysDesc* __restrict__ sys, SysState* st, DevArrays a, int cap) {
  if (*a.any_rebuild == 0) return;
  extern __shared__ float4 sub_smem[];
  unsigned char* const base = reinterpret_cast<unsigned char*>(sub_smem);
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t wib = threadIdx.x >> 5;
  const uint32_t nwarp = blockDim.x >> 5;
  SubTables& tb = *reinterpret_cast<SubTables*>(base);
  SubRanges& rg = reinterpret_cast<SubRanges*>(base + sizeof(SubTables))[wib];
  float4* const srel = reinterpret_cast<float4*>(base + sub_stage_offset(static_cast<int>(nwarp))) +
                       static_cast<size_t>(wib) * cap;
  const unsigned full = 0xffffffffu;
  const unsigned lt = lanemask_lt();
  __shared__ uint32_t sink[4][kNbrP];  // hits of systems without list slots (blocks of 4 warps)
  uint32_t acc_s = kInvalid, acc_max = 0;
  unsigned long long acc_sum = 0;
  const uint32_t n_sub = min(*a.nbr_sub_n, n_cells);
  for (uint32_t it = blockIdx.x; it < n_sub; it += gridDim.x) {
    // every condition below depends on the cell only: the block stays together
    const uint32_t c = a.nbr_sub[it];
    const uint32_t s = a.cell_sys[c];
    const SysDesc& S = sys[s];
    const uint32_t sa = a.cell_start[c];
    const int sA = a.cside[c];
    int ci, cj, ck;
    cell_ijk(S, c - S.cell_base, ci, cj, ck);

    // group table: lane g < 27 describes neighbour cell g in (dk, dj, di) order
    uint32_t g_start = 0, g_n = 0, g_code = kImageCenter, g_side = 1;
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
      g_side = a.cside[src];
    }
    if (__reduce_max_sync(full, g_side) > static_cast<uint32_t>(kSubMaxSide) || sA > kSubMaxSide) {
      if (threadIdx.x == 0) a.nbr_wide[atomicAdd(a.nbr_wide_n, 1u)] = c;
      continue;
    }
    if (s != acc_s) {
      if (lane == 0) flush_list_stats(st, sys, acc_s, acc_max, acc_sum);
      acc_s = s;
      acc_max = 0;
      acc_sum = 0;
    }

    // sub-cell start tables: start[g][B] = first particle of cell g with key >= B
    __syncthreads();  // the previous cell's readers are done with the tables
    for (uint32_t g = wib; g < 27; g += nwarp) {
      const uint32_t gs = __shfl_sync(full, g_start, g);
      const uint32_t gn = __shfl_sync(full, g_n, g);
      const uint32_t sd = __shfl_sync(full, g_side, g);
      const uint32_t nsc = sd * sd * sd;
      for (uint32_t B = lane; B <= nsc; B += 32) tb.start[g][B] = B == 0 ? 0u : gn;
      __syncwarp();
      if (sd > 1) {
        // keys ascend within the cell: particle q starts the sub-cells (key[q-1], key[q]]
        for (uint32_t q = lane; q < gn; q += 32) {
          const uint32_t k = a.skey[gs + q];
          const uint32_t from = q > 0 ? static_cast<uint32_t>(a.skey[gs + q - 1]) + 1u : 1u;
          for (uint32_t B = from; B <= k && B < nsc; ++B) tb.start[g][B] = q;
        }
      }
    }
    __syncthreads();

    const float nb_hi = S.nbh2_f + S.nbh_margin_f;
    const float nb_lo = S.nbh2_f - S.nbh_margin_f;
    const float nb_zero = S.nbh_margin_f;
    const uint32_t slot = S.list_slot;
    uint32_t* const seg = a.nbr + S.list_base;
    const uint32_t nA = static_cast<uint32_t>(sA * sA * sA);
    for (uint32_t A = wib; A < nA; A += nwarp) {
      const uint32_t a0 = tb.start[13][A], a1 = tb.start[13][A + 1];
      if (a0 == a1) continue;
      const int iA = static_cast<int>(A) % sA, jA = (static_cast<int>(A) / sA) % sA, kA = static_cast<int>(A) / (sA * sA);

      // A's candidate sequence: per neighbour cell, the runs of kept sub-cells
      // (an empty sub-cell never splits a run), each one index range
      uint32_t R = 0, M = 0, self_pos = 0;
      for (int g = 0; g < 27; ++g) {
        const uint32_t gs = __shfl_sync(full, g_start, g);
        const uint32_t gcode = __shfl_sync(full, g_code, g);
        const int sd = static_cast<int>(__shfl_sync(full, g_side, g));
        const int nsc = sd * sd * sd;
        bool keep = false;
        if (static_cast<int>(lane) < nsc) {
          const int L = static_cast<int>(lane);
          const int gx = box_gap(iA, sA, g % 3 - 1, L % sd, sd);
          const int gy = box_gap(jA, sA, (g / 3) % 3 - 1, (L / sd) % sd, sd);
          const int gz = box_gap(kA, sA, g / 9 - 1, L / (sd * sd), sd);
          const float lim = S.sub_reach_f * static_cast<float>(sA * sd);
          keep = static_cast<float>(gx * gx + gy * gy + gz * gz) <= lim * lim ||
                 tb.start[g][lane] == tb.start[g][lane + 1];
        }
        const unsigned km = __ballot_sync(full, keep);
        const bool first = keep && (lane == 0 || ((km >> (lane - 1)) & 1u) == 0u);
        const unsigned after = ~km & ~((2u << lane) - 1u);  // lanes above this one that are not kept
        const uint32_t last = after ? static_cast<uint32_t>(__ffs(after) - 1) : 32u;  // <= nsc
        uint32_t r0 = 0, len = 0;
        if (first) {
          r0 = tb.start[g][lane];
          len = tb.start[g][last] - r0;
        }
        const bool run = first && len > 0;
        const unsigned rm = __ballot_sync(full, run);
        uint32_t inc = run ? len : 0u;
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t v = __shfl_up_sync(full, inc, o);
          if (lane >= static_cast<uint32_t>(o)) inc += v;
        }
        const uint32_t at = M + inc - len;
        if (run) {
          const uint32_t idx = R + __popc(rm & lt);
          rg.first[idx] = gs + r0;
          rg.pos[idx] = at;
          rg.code[idx] = gcode;
        }
        if (g == 13) {
          // the particles of A themselves: inside the run that holds sub-cell A
          const unsigned mm = __ballot_sync(full, run && lane <= A && A < last);
          self_pos = __shfl_sync(full, at + (a0 - r0), __ffs(mm) - 1);
        }
        R += __popc(rm);
        M += __shfl_sync(full, inc, 31);
      }
      if (lane == 0) rg.pos[R] = M;
      __syncwarp();

      for (uint32_t c0 = 0; c0 < M; c0 += static_cast<uint32_t>(cap)) {
        const uint32_t m = min(M - c0, static_cast<uint32_t>(cap));
        const uint32_t mpad = (m + 31u) & ~31u;  // <= cap (a multiple of 32)
        __syncwarp();  // the previous round's readers are done with srel
        for (uint32_t t = lane; t < mpad; t += 32) {
          if (t < m) {
            const uint32_t u = c0 + t;
            uint32_t lo = 0, hi = R;  // the last range with pos <= u
            while (hi - lo > 1) {
              const uint32_t mid = (lo + hi) >> 1;
              if (rg.pos[mid] <= u) lo = mid;
              else hi = mid;
            }
            srel[t] = stage_candidate(S, a, rg.first[lo] + (u - rg.pos[lo]), rg.code[lo]);
          } else {
            srel[t] = make_float4(1.0e18f, 1.0e18f, 1.0e18f, __uint_as_float(kInvalid));
          }
        }
        __syncwarp();
        const bool first_round = c0 == 0;
        const bool last_round = c0 + m == M;
        for (uint32_t p0 = a0; p0 < a1; p0 += kNbrP) {
          // particles past A's end sit at -1e18: never within reach of a candidate
          float px[kNbrP], py[kNbrP], pz[kNbrP];
          uint32_t cur[kNbrP], half[kNbrP];
#pragma unroll
          for (int k = 0; k < kNbrP; ++k) {
            const uint32_t pk = p0 + k;
            const bool valid = pk < a1;
            const float4 q = valid ? a.pf[sa + pk] : make_float4(0.f, 0.f, 0.f, 0.f);
            px[k] = valid ? q.x : -1.0e18f;
            py[k] = valid ? q.y : -1.0e18f;
            pz[k] = valid ? q.z : -1.0e18f;
            cur[k] = (valid && !first_round) ? a.nbr_cnt[sa + pk] : 0u;
            half[k] = (valid && !first_round) ? a.nbr_half[sa + pk] : 0u;
          }
          const uint32_t i0 = sa + p0;
          const uint32_t self0 = ((i0 - S.part_base) << 5) | static_cast<uint32_t>(kImageCenter);
          const uint32_t low0 = self_pos + (p0 - a0);
          // a system without slots yet (the sizing build) only counts: its hits land in the sink
          uint32_t* const pslot = slot ? seg + static_cast<size_t>(i0 - S.part_base) * slot : sink[wib];
          const uint32_t pstride = slot ? slot : 1u;
          for (uint32_t t0 = 0; t0 < mpad; t0 += 32) {
            const float4 b = srel[t0 + lane];
            const uint32_t ent = __float_as_uint(b.w);
            const uint32_t u0 = c0 + t0;
            const bool self_chunk = u0 < low0 + kNbrP && low0 < u0 + 32u;
            if (__any_sync(full, ent - kAmbiguousBit < kInvalid - kAmbiguousBit)) {
              if (self_chunk)
                nbr_chunk<kNbrP, true, true>(S, a, b, px, py, pz, i0, self0, u0, low0, nb_lo, nb_hi, nb_zero, lt, pslot, pstride,
                                      cur, half);
              else
                nbr_chunk<kNbrP, true, false>(S, a, b, px, py, pz, i0, self0, u0, low0, nb_lo, nb_hi, nb_zero, lt, pslot, pstride,
                                       cur, half);
            } else if (self_chunk) {
              nbr_chunk<kNbrP, false, true>(S, a, b, px, py, pz, i0, self0, u0, low0, nb_lo, nb_hi, nb_zero, lt, pslot, pstride,
                                     cur, half);
            } else {
              nbr_chunk<kNbrP, false, false>(S, a, b, px, py, pz, i0, self0, u0, low0, nb_lo, nb_hi, nb_zero, lt, pslot, pstride,
                                      cur, half);
            }
          }
          __syncwarp();
#pragma unroll
          for (int k = 0; k < kNbrP; ++k) {
            const uint32_t pk = p0 + k;
            if (pk < a1) {
              const uint32_t i = sa + pk;
              if (lane == 0) {
                a.nbr_cnt[i] = cur[k];
                a.nbr_half[i] = half[k];
                if (last_round) a.nbr_start[i] = (i - S.part_base) * slot;
              }
              if (last_round) {
                acc_max = max(acc_max, cur[k]);
                acc_sum += cur[k];
              }
            }
          }
          __syncwarp();
        }
      }
    }
  }
  if (lane == 0) flush_list_stats(st, sys, acc_s, acc_max, acc_sum);
}

}  // namespace

int launch_neighbors_sub(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, int cap,
                         cudaStream_t stream) {
  if (ex.n_cells == 0) return 0;
  const size_t smem = sub_stage_offset(4) + static_cast<size_t>(4) * cap * sizeof(float4);
  cudaFuncSetAttribute(k_neighbors_sub, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_neighbors_sub, 128, smem) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const long long want = static_cast<long long>(ex.n_cells);
  const int grid = static_cast<int>(std::max(1ll, std::min(want, static_cast<long long>(per_sm) * ex.sm_count)));
  k_neighbors_sub<<<grid, 128, smem, stream>>>(ex.n_cells, sys, st, a, cap);
  return 1;
}

}  // namespace xnb
