// Mixed-precision Lennard-Jones traversal over cell segments staged in shared
// memory (XNB_FORCE_STAGED).
//
// The one-thread-per-particle traversal (xnb_step_kernels.cu) gathers every
// neighbour's FP32 mirror (prefilter) and FP64 position and mirrors (marked
// entries) from global memory: at 4M atoms it is bound by the latency and L1
// throughput of those gathers, not by its FP64 work. Here a block takes a
// segment of kSegCells x-adjacent cells of one row and first copies the
// neighbourhood of the whole segment -- 9 rows of kSegCells + 2 cells, the
// periodic images included -- into shared memory (FP64 position and both FP32
// mirrors per particle); its threads then walk their particles' lists reading
// every neighbour from shared memory.
//
// The lists are read in a compact form: per entry (g << 11) | p_b, g the
// neighbour cell in the reference's (dk, dj, di) order and p_b the particle's
// index in that cell, written next to the regular entries by k_nbr_compact
// after each build. Entry order, the FP32 prefilter, the marks and the pair
// body (mixed_pair) are those of the one-thread traversal, so forces,
// energies and velocities are bitwise equal to it. A segment whose
// neighbourhood exceeds the stage, or whose lists could not be compacted (a
// cell of 2048 or more particles), runs the one-thread traversal from global
// memory inside the same kernel.
#include "xnb_launch.cuh"
#include "xnb_lj_pair.cuh"
#include "xnb_traverse.cuh"

namespace xnb {

namespace {

constexpr uint32_t kInvalidF = 0xFFFFFFFFu;
constexpr int kSegCells = kStagedSegCells;     // cells of a segment (x-adjacent, one row)
constexpr int kSlotRow = kSegCells + 2;        // cells of one staged row
constexpr int kSlots = 9 * kSlotRow;           // staged cells
constexpr int kStageCap = 1792;                // staged particles per block
constexpr int kStagedThreads = 160;

struct StagedSmem {
  double x[kStageCap], y[kStageCap], z[kStageCap];
  float4 hi[kStageCap];  // FP32 mirrors, residuals packed in .w
  uint32_t slot_start[kSlots];
  uint32_t slot_base[kSlots + 1];
  uint32_t slot_code[kSlots];
  uint32_t n_stage;
  int fallback;
};

// ---------------------------------------------------------------------------
// Compact entries of the freshly built lists of flagged systems: entry e
// (particle j of the system, periodic image code) becomes (g << 11) | p_b with
// g the neighbour group of the particle's cell (27 groups in (dk, dj, di)
// order, each one cell with one image code) and p_b = j - first particle of
// that cell. The list is sorted by (g, p_b), so the group pointer only moves
// forward. A p_b above 2047 or an entry outside the 27 groups sets
// compact_bad (the staged traversal then reads that system from global memory).
__device__ __forceinline__ void group_of(const SysDesc& S, const DevArrays& a, int ci, int cj, int ck, uint32_t g,
                                         uint32_t& start, uint32_t& n, uint32_t& code) {
  int n3[3] = {ci + static_cast<int>(g % 3u) - 1, cj + static_cast<int>((g / 3u) % 3u) - 1,
               ck + static_cast<int>(g / 9u) - 1};
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
  start = a.cell_start[src];
  n = a.cell_n[src];
  code = static_cast<uint32_t>(img[0] + 3 * img[1] + 9 * img[2]);
}

__global__ void __launch_bounds__(256)
    k_nbr_compact(uint32_t n_part, const SysDesc* __restrict__ sys, SysState* st, DevArrays a, bool all) {
  if (!all && *a.any_rebuild == 0) return;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_part; i += gridDim.x * blockDim.x) {
    const uint32_t c = a.pcell[i];
    if (c == kInvalidF) continue;
    const uint32_t s = a.cell_sys[c];
    if (!all && !st[s].rebuild) continue;
    const SysDesc& S = sys[s];
    const uint32_t cnt = a.nbr_cnt[i];
    if (cnt > S.list_slot) continue;  // overflowed lists are flagged by the build and not used
    int ci, cj, ck;
    cell_ijk(S, c - S.cell_base, ci, cj, ck);
    const uint64_t at = S.list_base + a.nbr_start[i];
    const uint32_t* __restrict__ L = a.nbr + at;
    uint16_t* L16 = a.nbr16 + at;
    uint32_t g = 0, gs, gn, gc;
    group_of(S, a, ci, cj, ck, 0, gs, gn, gc);
    bool bad = false;
    for (uint32_t k = 0; k < cnt; ++k) {
      const uint32_t e = L[k];
      const uint32_t j = S.part_base + (e >> 5);
      const uint32_t code = e & 31u;
      while (!(code == gc && j >= gs && j < gs + gn)) {
        if (++g >= 27u) break;
        group_of(S, a, ci, cj, ck, g, gs, gn, gc);
      }
      if (g >= 27u || j - gs >= 2048u) {
        bad = true;
        break;
      }
      L16[k] = static_cast<uint16_t>((g << 11) | (j - gs));
    }
    if (bad) atomicOr(&st[s].compact_bad, 1u);
  }
}

// ---------------------------------------------------------------------------
// FP32 prefilter of a window over compact entries (the marks of prefilter_window).
__device__ __forceinline__ pair::Marks staged_prefilter(const StagedSmem& sm, const uint16_t* __restrict__ L16,
                                                        uint32_t kw, uint32_t kend, uint32_t m, float4 paf,
                                                        const float (&pfp)[3], float pre_hi) {
  pair::Marks mk{{0u, 0u, 0u, 0u}};
  for (uint32_t kb = kw; kb < kend; kb += 8) {
    const uint4 ev = __ldg(reinterpret_cast<const uint4*>(L16 + kb));
    const uint32_t w[4] = {ev.x, ev.y, ev.z, ev.w};
    uint32_t bits = 0;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const bool valid = kb + static_cast<uint32_t>(t) < kend;
      // past the list's end: entry 0 (a valid slot), never marked
      const uint32_t e = valid ? (w[t >> 1] >> ((t & 1) * 16)) & 0xFFFFu : 0u;
      const uint32_t g = e >> 11;
      const uint32_t slot = (g / 3u) * kSlotRow + m + (g % 3u);
      const uint32_t sidx = sm.slot_base[slot] + (e & 2047u);
      const uint32_t code = sm.slot_code[slot];
      const float4 pbf = sm.hi[sidx];
      float bx = pbf.x, by = pbf.y, bz = pbf.z;
      if (code != pair::kImageCenter) {
        bx = image_coord_f(bx, pfp[0], static_cast<int>(code % 3u));
        by = image_coord_f(by, pfp[1], static_cast<int>((code / 3u) % 3u));
        bz = image_coord_f(bz, pfp[2], static_cast<int>(code / 9u));
      }
      const float ex = bx - paf.x, ey = by - paf.y, ez = bz - paf.z;
      if (valid && fmaf(ex, ex, fmaf(ey, ey, ez * ez)) <= pre_hi) bits |= 1u << t;
    }
    const uint32_t off = kb - kw;
    const uint32_t sh = off & 31u;
    if (off < 32u) mk.w[0] |= bits << sh;
    else if (off < 64u) mk.w[1] |= bits << sh;
    else if (off < 96u) mk.w[2] |= bits << sh;
    else mk.w[3] |= bits << sh;
  }
  return mk;
}

template <bool PE, bool KICK>
__global__ void __launch_bounds__(kStagedThreads, 2)
    k_force_staged(uint32_t n_seg, const SysDesc* __restrict__ sys, const SysState* __restrict__ st, DevArrays a,
                   int sys_only) {
  extern __shared__ __align__(16) unsigned char staged_smem[];
  StagedSmem& sm = *reinterpret_cast<StagedSmem*>(staged_smem);
  const LJForce<kMixed, PE, KICK> f{sys, a};
  const BatchSource src(sys, st, a, sys_only);
  for (uint32_t sg = blockIdx.x; sg < n_seg; sg += gridDim.x) {
    const uint4 seg = a.seg[sg];  // first cell (global), cells, system
    const uint32_t s = seg.z;
    if (sys_only >= 0 && s != static_cast<uint32_t>(sys_only)) continue;
    if (st[s].error) continue;  // uniform over the block
    const SysDesc& S = sys[s];
    int ci0, cj, ck;
    cell_ijk(S, seg.x - S.cell_base, ci0, cj, ck);
    // the staged cells: row r = (dk + 1) * 3 + (dj + 1), column q = di + 1 relative to the segment start
    if (threadIdx.x < kSlots) {
      const int r = static_cast<int>(threadIdx.x) / kSlotRow, q = static_cast<int>(threadIdx.x) % kSlotRow;
      uint32_t start = 0, n = 0, code = pair::kImageCenter;
      if (q <= static_cast<int>(seg.y) + 1) {
        int n3[3] = {ci0 + q - 1, cj + (r % 3) - 1, ck + (r / 3) - 1};
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
        const uint32_t c = S.cell_base + static_cast<uint32_t>((n3[2] * S.dims[1] + n3[1]) * S.dims[0] + n3[0]);
        start = a.cell_start[c];
        n = a.cell_n[c];
        code = static_cast<uint32_t>(img[0] + 3 * img[1] + 9 * img[2]);
      }
      sm.slot_start[threadIdx.x] = start;
      sm.slot_base[threadIdx.x + 1] = n;  // counts, scanned below
      sm.slot_code[threadIdx.x] = code;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t run = 0;
      sm.slot_base[0] = 0;
      for (int q = 1; q <= kSlots; ++q) {
        run += sm.slot_base[q];
        sm.slot_base[q] = run;
      }
      sm.n_stage = run;
      sm.fallback = (run > static_cast<uint32_t>(kStageCap) || st[s].compact_bad) ? 1 : 0;
    }
    __syncthreads();
    const bool staged = !sm.fallback;
    if (staged) {
      const uint32_t ns = sm.n_stage;
      for (uint32_t u = threadIdx.x; u < ns; u += blockDim.x) {
        // slot of staged particle u: the last slot whose base is <= u
        uint32_t lo = 0, hi = kSlots;
        while (hi - lo > 1) {
          const uint32_t mid = (lo + hi) >> 1;
          if (sm.slot_base[mid] <= u) lo = mid;
          else hi = mid;
        }
        const uint32_t j = sm.slot_start[lo] + (u - sm.slot_base[lo]);
        sm.x[u] = __ldg(a.rx + j);
        sm.y[u] = __ldg(a.ry + j);
        sm.z[u] = __ldg(a.rz + j);
        sm.hi[u] = __ldg(a.pf + j);
      }
    }
    __syncthreads();
    // the segment's own particles: one contiguous range of its cells
    const uint32_t c_last = seg.x + seg.y - 1;
    const uint32_t p0 = a.cell_start[seg.x];
    const uint32_t p1 = a.cell_start[c_last] + a.cell_n[c_last];
    for (uint32_t i = p0 + threadIdx.x; i < p1; i += blockDim.x) {
      if (!staged) {
        pair::traverse_particle(src, i, f);
        continue;
      }
      pair::ParticleContext c;
      if (!src.begin(i, false, false, c)) continue;
      typename LJForce<kMixed, PE, KICK>::Acc q;
      f.start(q, c);
      const uint32_t m = a.pcell[i] - seg.x;  // the particle's cell within the segment
      const uint16_t* __restrict__ L16 = a.nbr16 + S.list_base + a.nbr_start[i];
      const uint32_t n = c.n;
      const float pre_hi = S.rc2_f + S.pre_margin_f;
      const float pfp[3] = {S.period_f[0], S.period_f[1], S.period_f[2]};
      for (uint32_t kw = 0; kw < n; kw += 128) {
        pair::Marks mk = staged_prefilter(sm, L16, kw, min(n, kw + 128u), m, c.hi, pfp, pre_hi);
        // two marked entries per iteration, list order kept (b0 < b1), as the
        // one-thread traversal takes them
        uint32_t b0 = 0, b1 = 0;
        bool h0 = pair::next_mark(mk, b0);
        while (h0) {
          const bool h1 = pair::next_mark(mk, b1);
          const uint32_t e0 = L16[kw + b0], e1 = L16[kw + (h1 ? b1 : b0)];
          const uint32_t s0 = (e0 >> 11) / 3u * kSlotRow + m + (e0 >> 11) % 3u;
          const uint32_t s1 = (e1 >> 11) / 3u * kSlotRow + m + (e1 >> 11) % 3u;
          const uint32_t u0 = sm.slot_base[s0] + (e0 & 2047u), u1 = sm.slot_base[s1] + (e1 & 2047u);
          const uint32_t code0 = sm.slot_code[s0], code1 = sm.slot_code[s1];
          // packed residuals only: launch_force keeps batches without them off this kernel
          const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
          mixed_pair<PE, true>(S, code0, sm.x[u0], sm.y[u0], sm.z[u0], sm.hi[u0], z4, c.x, c.y, c.z, c.hi, z4,
                               S.rcut2, q.fx, q.fy, q.fz, q.psum, q.pe);
          if (h1)
            mixed_pair<PE, true>(S, code1, sm.x[u1], sm.y[u1], sm.z[u1], sm.hi[u1], z4, c.x, c.y, c.z, c.hi, z4,
                                 S.rcut2, q.fx, q.fy, q.fz, q.psum, q.pe);
          h0 = h1 && pair::next_mark(mk, b0);
        }
      }
      f.stop(q, c);
    }
    __syncthreads();  // the stage is refilled for the next segment
  }
}

}  // namespace

size_t staged_smem_bytes() { return sizeof(StagedSmem); }

int launch_compact_lists(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a,
                         cudaStream_t stream, bool all) {
  if (ex.n_part == 0 || !a.nbr16) return 0;
  const int threads = 256;
  long long g = (static_cast<long long>(ex.n_part) + threads - 1) / threads;
  const long long cap = static_cast<long long>(ex.sm_count) * 8;
  if (g > cap) g = cap;
  k_nbr_compact<<<static_cast<int>(g < 1 ? 1 : g), threads, 0, stream>>>(ex.n_part, sys, st, a, all);
  return 1;
}

int launch_force_staged(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, bool with_pe,
                        bool second_half, int sys_only, cudaStream_t stream) {
  if (ex.n_seg == 0) return 0;
  const size_t smem = sizeof(StagedSmem);
  const int grid = static_cast<int>(std::min<long long>(ex.n_seg, static_cast<long long>(ex.sm_count) * 2));
#define XNB_STAGED(PE_, K_)                                                                                   \
  cudaFuncSetAttribute(k_force_staged<PE_, K_>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)); \
  k_force_staged<PE_, K_><<<grid, kStagedThreads, smem, stream>>>(ex.n_seg, sys, st, a, sys_only);
  if (with_pe && second_half) {
    XNB_STAGED(true, true)
  } else if (with_pe) {
    XNB_STAGED(true, false)
  } else if (second_half) {
    XNB_STAGED(false, true)
  } else {
    XNB_STAGED(false, false)
  }
#undef XNB_STAGED
  return 1;
}

}  // namespace xnb
