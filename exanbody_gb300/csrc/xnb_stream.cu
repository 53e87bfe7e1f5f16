// Reference-format chunk-neighbour streams from the per-particle lists, and the
// verify_chunk_neighbors checker over such streams (format in xnb_stream.h).
#include "xnb_launch.cuh"
#include "xnb_stream.h"

namespace xnb {

namespace {

constexpr uint32_t kInvalid = 0xFFFFFFFFu;

__device__ __forceinline__ unsigned lanemask_le_u() {
  unsigned m;
  asm volatile("mov.u32 %0, %%lanemask_le;" : "=r"(m));
  return m;
}

// The reference's ghost filter (update_ghosts_comm_scheme.cpp:462-469; is_inside,
// geometry.h:198-203): the image of owner particle q under image code gc lies in
// the partner block enlarged by ghost_dist.
__device__ bool ghost_keeps(const SysDesc& S, const DevArrays& a, uint32_t q, uint32_t gc) {
  const double x = image_coord(a.rx[q], S.period[0], static_cast<int>(gc % 3u));
  const double y = image_coord(a.ry[q], S.period[1], static_cast<int>((gc / 3u) % 3u));
  const double z = image_coord(a.rz[q], S.period[2], static_cast<int>(gc / 9u));
  return x >= S.outer_lo[0] && x <= S.outer_hi[0] && y >= S.outer_lo[1] && y <= S.outer_hi[1] &&
         z >= S.outer_lo[2] && z <= S.outer_hi[2];
}

// Index of owner particle j inside the ghost cell of image gc: the kept particles
// of j's cell that precede it (ghost cells hold the kept ones in the owner's order).
__device__ uint32_t ghost_rank(const SysDesc& S, const DevArrays& a, uint32_t j, uint32_t gc) {
  uint32_t r = 0;
  for (uint32_t q = a.cell_start[a.pcell[j]]; q < j; ++q) r += ghost_keeps(S, a, q, gc) ? 1u : 0u;
  return r;
}

// Relative cell (di, dj, dk) of list entry e seen from the cell (ci, cj, ck), and
// the entry's particle index in that (interior or ghost) cell.
__device__ void entry_cell(const SysDesc& S, const DevArrays& a, uint32_t e, int ci, int cj, int ck, bool want_pb,
                           uint16_t& enc, uint32_t& pb) {
  const uint32_t j = S.part_base + (e >> 5);
  const uint32_t gc = e & 31u;
  int oi, oj, ok;
  cell_ijk(S, a.pcell[j] - S.cell_base, oi, oj, ok);
  const int di = oi - ci + (static_cast<int>(gc % 3u) - 1) * S.dims[0];
  const int dj = oj - cj + (static_cast<int>((gc / 3u) % 3u) - 1) * S.dims[1];
  const int dk = ok - ck + (static_cast<int>(gc / 9u) - 1) * S.dims[2];
  enc = encode_cell_rel(di, dj, dk);
  pb = 0;
  if (want_pb)
    pb = gc == static_cast<uint32_t>(kImageCenter) ? j - a.cell_start[a.pcell[j]] : ghost_rank(S, a, j, gc);
}

// WRITE = false: stream length of every cell of system sid into cell_len.
// WRITE = true: the streams, cell lc at out + cell_off[lc]. One warp per cell;
// lanes take 32 list entries of a particle at a time, a ballot marks where the
// encoded cell changes and fixes each entry's place in the sub-stream.
template <bool WRITE>
__global__ void __launch_bounds__(128)
    k_stream(uint32_t sid, const SysDesc* __restrict__ sys, DevArrays a, int T, uint32_t* cell_len,
             const unsigned long long* __restrict__ cell_off, uint16_t* out_all, unsigned int* errors) {
  const SysDesc& S = sys[sid];
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  const unsigned le = lanemask_le_u();
  for (uint32_t lc = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); lc < S.ncells; lc += warps) {
    const uint32_t c = S.cell_base + lc;
    const uint32_t na = a.cell_n[c];
    const uint32_t sa = a.cell_start[c];
    if (na == 0) {
      if (!WRITE && lane == 0) cell_len[lc] = 0;
      continue;
    }
    int ci, cj, ck;
    cell_ijk(S, lc, ci, cj, ck);
    const uint32_t table = T >= 1 ? (na * static_cast<uint32_t>(T) + 1u) * 2u : 0u;
    uint16_t* out = WRITE ? out_all + cell_off[lc] : nullptr;
    uint32_t pos = table;  // where the next particle's sub-stream starts
    for (uint32_t pa = 0; pa < na; ++pa) {
      const uint32_t i = sa + pa;
      const uint32_t n = a.nbr_cnt[i];
      const uint32_t* __restrict__ L = a.nbr + S.list_base + a.nbr_start[i];
      if (WRITE && lane == 0 && T >= 1) {
        const uint32_t o = pos - table + static_cast<uint32_t>(T);
        out[pa * 2] = static_cast<uint16_t>(o);
        out[pa * 2 + 1] = static_cast<uint16_t>(o >> 16);
        if (T == 2) {
          const uint32_t h = a.nbr_half[i];
          out[(na + 1 + pa) * 2] = static_cast<uint16_t>(h);
          out[(na + 1 + pa) * 2 + 1] = static_cast<uint16_t>(h >> 16);
        }
      }
      uint32_t groups = 0;
      int carry = -1;  // encoded cell of the previous entry (none yet)
      bool open = false;
      uint32_t open_hdr = 0, open_k = 0;  // the last group, still counting
      for (uint32_t k0 = 0; k0 < n; k0 += 32) {
        const uint32_t k = k0 + lane;
        const bool valid = k < n;
        uint16_t enc = 0;
        uint32_t pb = 0;
        if (valid) entry_cell(S, a, L[k], ci, cj, ck, WRITE, enc, pb);
        int prev = __shfl_up_sync(0xffffffffu, static_cast<int>(enc), 1);
        if (lane == 0) prev = carry;
        const bool flag = valid && static_cast<int>(enc) != prev;
        const unsigned fm = __ballot_sync(0xffffffffu, flag);
        if (WRITE) {
          if (valid) {
            if (pb > 0xFFFFu) atomicOr(errors, 1u);
            const uint32_t gi = groups + __popc(fm & le) - 1u;
            out[pos + 1 + 2 * (gi + 1) + k] = static_cast<uint16_t>(pb);
            if (flag) {
              const uint32_t hdr = pos + 1 + 2 * gi + k;
              out[hdr] = enc;
              const unsigned above = fm & ~le;
              if (above) out[hdr + 1] = static_cast<uint16_t>(static_cast<uint32_t>(__ffs(above) - 1) - lane);
            }
          }
          // the group left open by the previous 32 entries ends at this chunk's first change
          if (open && fm && lane == 0) out[open_hdr + 1] = static_cast<uint16_t>(k0 + (__ffs(fm) - 1) - open_k);
        }
        if (fm) {
          const uint32_t last = 31u - static_cast<uint32_t>(__clz(fm));
          open = true;
          open_k = k0 + last;
          open_hdr = pos + 1 + 2 * (groups + static_cast<uint32_t>(__popc(fm)) - 1u) + open_k;
        }
        groups += static_cast<uint32_t>(__popc(fm));
        carry = __shfl_sync(0xffffffffu, static_cast<int>(enc), 31);
      }
      if (WRITE && lane == 0) {
        if (open) out[open_hdr + 1] = static_cast<uint16_t>(n - open_k);
        out[pos] = static_cast<uint16_t>(groups);
      }
      pos += 1 + 2 * groups + n;
    }
    if (WRITE && lane == 0 && T >= 1) {
      const uint32_t o = pos - table + static_cast<uint32_t>(T);
      out[na * 2] = static_cast<uint16_t>(o);
      out[na * 2 + 1] = static_cast<uint16_t>(o >> 16);
    }
    if (!WRITE && lane == 0) cell_len[lc] = pos;
  }
}

// What verify_cell_stream needs about one cell, read from the device arrays.
struct CellView {
  const SysDesc* S;
  const DevArrays* a;
  uint32_t sa;
  int ci, cj, ck;
  double nbh2;

  // neighbour cell of the relative offset: source cell and image code
  __device__ void source(int di, int dj, int dk, uint32_t& src, uint32_t& gc) const {
    int n3[3] = {ci + di, cj + dj, ck + dk};
    int img[3];
    for (int ax = 0; ax < 3; ++ax) {
      img[ax] = 1;
      if (n3[ax] < 0) { n3[ax] += S->dims[ax]; img[ax] = 0; }
      else if (n3[ax] >= S->dims[ax]) { n3[ax] -= S->dims[ax]; img[ax] = 2; }
    }
    src = S->cell_base + static_cast<uint32_t>((n3[2] * S->dims[1] + n3[1]) * S->dims[0] + n3[0]);
    gc = static_cast<uint32_t>(img[0] + 3 * img[1] + 9 * img[2]);
  }
  __device__ uint32_t size_of(int di, int dj, int dk) const {
    uint32_t src, gc;
    source(di, dj, dk, src, gc);
    const uint32_t s0 = a->cell_start[src], n = a->cell_n[src];
    if (gc == static_cast<uint32_t>(kImageCenter)) return n;
    uint32_t k = 0;
    for (uint32_t q = s0; q < s0 + n; ++q) k += ghost_keeps(*S, *a, q, gc) ? 1u : 0u;
    return k;
  }
  __device__ bool pair_d2(uint32_t pa, int di, int dj, int dk, uint32_t pb, double& d2) const {
    uint32_t src, gc;
    source(di, dj, dk, src, gc);
    const uint32_t s0 = a->cell_start[src], n = a->cell_n[src];
    uint32_t q = kInvalid;
    if (gc == static_cast<uint32_t>(kImageCenter)) {
      if (pb < n) q = s0 + pb;
    } else {
      uint32_t k = 0;
      for (uint32_t t = s0; t < s0 + n; ++t) {
        if (!ghost_keeps(*S, *a, t, gc)) continue;
        if (k == pb) {
          q = t;
          break;
        }
        ++k;
      }
    }
    if (q == kInvalid) return false;
    const uint32_t i = sa + pa;
    const double xb = image_coord(a->rx[q], S->period[0], static_cast<int>(gc % 3u));
    const double yb = image_coord(a->ry[q], S->period[1], static_cast<int>((gc / 3u) % 3u));
    const double zb = image_coord(a->rz[q], S->period[2], static_cast<int>(gc / 9u));
    d2 = norm2_rn(__dsub_rn(xb, a->rx[i]), __dsub_rn(yb, a->ry[i]), __dsub_rn(zb, a->rz[i]));
    return true;
  }
  // FP64 search of the 27-cell block with the ghost filter, independent of the
  // FP32 staging of the neighbour build
  __device__ uint32_t exhaustive_count(uint32_t pa) const {
    const uint32_t i = sa + pa;
    const double xa = a->rx[i], ya = a->ry[i], za = a->rz[i];
    uint32_t cnt = 0;
    for (int dk = -1; dk <= 1; ++dk)
      for (int dj = -1; dj <= 1; ++dj)
        for (int di = -1; di <= 1; ++di) {
          uint32_t src, gc;
          source(di, dj, dk, src, gc);
          const uint32_t s0 = a->cell_start[src], n = a->cell_n[src];
          for (uint32_t q = s0; q < s0 + n; ++q) {
            if (gc == static_cast<uint32_t>(kImageCenter)) {
              if (q == i) continue;
            } else if (!ghost_keeps(*S, *a, q, gc)) {
              continue;
            }
            const double xb = image_coord(a->rx[q], S->period[0], static_cast<int>(gc % 3u));
            const double yb = image_coord(a->ry[q], S->period[1], static_cast<int>((gc / 3u) % 3u));
            const double zb = image_coord(a->rz[q], S->period[2], static_cast<int>(gc / 9u));
            const double d2 = norm2_rn(__dsub_rn(xb, xa), __dsub_rn(yb, ya), __dsub_rn(zb, za));
            if (d2 > 0.0 && d2 <= nbh2) ++cnt;
          }
        }
    return cnt;
  }
};

// One thread per cell of system sid: decodes and checks its stream.
__global__ void __launch_bounds__(128)
    k_stream_verify(uint32_t sid, const SysDesc* __restrict__ sys, DevArrays a, int T, const uint16_t* __restrict__ stream,
                    uint64_t stream_len, const unsigned long long* __restrict__ cell_off, unsigned long long* counts) {
  const SysDesc& S = sys[sid];
  for (uint32_t lc = blockIdx.x * blockDim.x + threadIdx.x; lc < S.ncells; lc += gridDim.x * blockDim.x) {
    const uint32_t c = S.cell_base + lc;
    CellView v;
    v.S = &S;
    v.a = &a;
    v.sa = a.cell_start[c];
    cell_ijk(S, lc, v.ci, v.cj, v.ck);
    v.nbh2 = S.nbh2;
    const unsigned long long o0 = cell_off[lc], o1 = cell_off[lc + 1];
    StreamCounts k{0, 0, 0, 0, 0, 0};
    if (o1 < o0 || o1 > stream_len) {
      k.format = 1;
    } else {
      verify_cell_stream(v, stream + o0, o1 - o0, a.cell_n[c], T, k);
    }
    const unsigned long long vals[6] = {k.format, k.order, k.self, k.range, k.far, k.missing};
    for (int q = 0; q < 6; ++q)
      if (vals[q]) atomicAdd(counts + q, vals[q]);
  }
}

}  // namespace

int launch_stream_lengths(uint32_t sid, uint32_t ncells, const SysDesc* sys, const DevArrays& a, int T,
                          uint32_t* cell_len, int sm_count, cudaStream_t stream) {
  const long long want = (static_cast<long long>(ncells) + 3) / 4;
  const int g = static_cast<int>(want < 1 ? 1 : (want > sm_count * 16LL ? sm_count * 16LL : want));
  k_stream<false><<<g, 128, 0, stream>>>(sid, sys, a, T, cell_len, nullptr, nullptr, nullptr);
  return 1;
}

int launch_stream_write(uint32_t sid, uint32_t ncells, const SysDesc* sys, const DevArrays& a, int T,
                        const unsigned long long* cell_off, uint16_t* out, unsigned int* errors, int sm_count,
                        cudaStream_t stream) {
  const long long want = (static_cast<long long>(ncells) + 3) / 4;
  const int g = static_cast<int>(want < 1 ? 1 : (want > sm_count * 16LL ? sm_count * 16LL : want));
  k_stream<true><<<g, 128, 0, stream>>>(sid, sys, a, T, nullptr, cell_off, out, errors);
  return 1;
}

int launch_stream_verify(uint32_t sid, uint32_t ncells, const SysDesc* sys, const DevArrays& a, int T,
                         const uint16_t* stream_data, uint64_t stream_len, const unsigned long long* cell_off,
                         unsigned long long* counts, int sm_count, cudaStream_t stream) {
  const long long want = (static_cast<long long>(ncells) + 127) / 128;
  const int g = static_cast<int>(want < 1 ? 1 : (want > sm_count * 16LL ? sm_count * 16LL : want));
  k_stream_verify<<<g, 128, 0, stream>>>(sid, sys, a, T, stream_data, stream_len, cell_off, counts);
  return 1;
}

}  // namespace xnb
