// Allocation-free variant of the neighbour build (chunk_neighbors) for one system.
//
// Some callers cannot allocate device memory at the point where they need a
// neighbour list: a host framework that owns every device allocation through
// its own pool (as the reference's onika allocators do) and forbids plugins to
// call cudaMalloc mid-step, or a time-stepping loop that must not stall on the
// device-wide synchronisation cudaFree can impose. This file gives them a build
// that takes only caller-owned inputs and outputs and keeps its scratch in one
// file-scope device array.
//
// Limits: at most kMaxParticles particles and kMaxCells cells per call, and at
// most 2^32 - 1 list entries (entry positions are 32-bit). The array (about
// 5.3 MB) is part of the library image, so every GPU that loads the library
// holds it until the process exits.
//
// Sharing: every call uses the same array. Calls whose kernels overlap on the
// GPU (different streams, or different host threads on one device) race on it
// and must be serialised by the caller. Nothing in the array has to start at
// zero: every scratch word a call reads is written earlier in the same call.
//
// Set-up: the first call on a device looks up the array's device address with
// cudaGetSymbolAddress while that device is current and caches it; make that
// first call before any stream capture begins on the device. Each call ends by
// copying the entry total to the host and synchronising its stream.
#include <cstdio>
#include <mutex>
#include <string>

#include "xnb_launch.cuh"

namespace xnb {

namespace {

constexpr uint32_t kMaxParticles = 1u << 20;  // 1,048,576
constexpr uint32_t kMaxCells = 1u << 17;      // 131,072
constexpr uint32_t kInvalidS = 0xFFFFFFFFu;
constexpr int kStageCap = 640;

// scratch layout (bytes): per-particle fill cursor | per-cell totals | per-cell
// offsets (u64, kMaxCells + 1) | scan tile sums (u64)
constexpr size_t kCursorBytes = sizeof(uint32_t) * kMaxParticles;
constexpr size_t kTotalsBytes = sizeof(uint32_t) * kMaxCells;
constexpr size_t kOffsetsBytes = sizeof(unsigned long long) * (kMaxCells + 1);
constexpr size_t kBlocksElems = kMaxCells / 2048 + 16;
constexpr size_t kBlocksBytes = sizeof(unsigned long long) * kBlocksElems;
constexpr size_t kCursorOff = 0;
constexpr size_t kTotalsOff = kCursorOff + kCursorBytes;
constexpr size_t kOffsetsOff = kTotalsOff + kTotalsBytes;
constexpr size_t kBlocksOff = kOffsetsOff + kOffsetsBytes;
constexpr size_t kScratchBytes = kBlocksOff + kBlocksBytes;

static __device__ __align__(256) unsigned char g_nbr_scratch[kScratchBytes];

__device__ __forceinline__ unsigned lanemask_lt_s() {
  unsigned m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Same candidate order, FP32 prefilter with proven margin and FP64 decision as
// the batch neighbour build (xnb_build_kernels.cu), for one system whose
// particles are given in cell order with local cell_start offsets.
template <bool FILL>
__global__ void __launch_bounds__(128)
    k_neighbors_static(SysDesc S, const double* __restrict__ rx, const double* __restrict__ ry,
                       const double* __restrict__ rz, const uint32_t* __restrict__ cell_start,
                       const uint32_t* __restrict__ cell_n, uint32_t* __restrict__ nbr, uint32_t* __restrict__ nbr_start,
                       uint32_t* __restrict__ nbr_cnt, unsigned long long cap, unsigned char* scratch) {
  extern __shared__ unsigned char smem_s[];
  uint32_t* cursor_g = reinterpret_cast<uint32_t*>(scratch + kCursorOff);
  uint32_t* totals = reinterpret_cast<uint32_t*>(scratch + kTotalsOff);
  const unsigned long long* offsets = reinterpret_cast<const unsigned long long*>(scratch + kOffsetsOff);
  const uint32_t n_cells = S.ncells;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t wib = threadIdx.x >> 5;
  float4* srel = reinterpret_cast<float4*>(smem_s) + static_cast<size_t>(wib) * kStageCap;
  uint32_t* sent = reinterpret_cast<uint32_t*>(reinterpret_cast<float4*>(smem_s) + static_cast<size_t>(blockDim.x >> 5) * kStageCap) +
                   static_cast<size_t>(wib) * kStageCap;
  if (FILL && offsets[n_cells] > cap) return;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t c = blockIdx.x * (blockDim.x >> 5) + wib; c < n_cells; c += warps) {
    const uint32_t sa = cell_start[c];
    const uint32_t na = cell_n[c];
    if (na == 0) {
      if (!FILL && lane == 0) totals[c] = 0;
      continue;
    }
    int ci, cj, ck;
    cell_ijk(S, c, ci, cj, ck);
    const double o[3] = {cell_lo(S, 0, ci), cell_lo(S, 1, cj), cell_lo(S, 2, ck)};
    if (FILL) {
      uint32_t run = static_cast<uint32_t>(offsets[c]);
      for (uint32_t q0 = 0; q0 < na; q0 += 32) {
        const uint32_t q = q0 + lane;
        const uint32_t cnt = q < na ? nbr_cnt[sa + q] : 0;
        uint32_t inc = cnt;
        for (int off = 1; off < 32; off <<= 1) {
          const uint32_t v = __shfl_up_sync(0xffffffffu, inc, off);
          if (lane >= static_cast<uint32_t>(off)) inc += v;
        }
        if (q < na) {
          nbr_start[sa + q] = run + inc - cnt;
          cursor_g[sa + q] = run + inc - cnt;
        }
        run += __shfl_sync(0xffffffffu, inc, 31);
      }
      __syncwarp();
    }
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
      const uint32_t src = static_cast<uint32_t>((n3[2] * S.dims[1] + n3[1]) * S.dims[0] + n3[0]);
      g_start = cell_start[src];
      g_n = cell_n[src];
      g_code = static_cast<uint32_t>(img[0] + 3 * img[1] + 9 * img[2]);
    }
    uint32_t g_off = g_n;
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t v = __shfl_up_sync(0xffffffffu, g_off, off);
      if (lane >= static_cast<uint32_t>(off)) g_off += v;
    }
    const uint32_t ncand = __shfl_sync(0xffffffffu, g_off, 26);
    g_off -= g_n;
    const float nb_hi = S.nbh2_f + S.nbh_margin_f;
    const float nb_lo = S.nbh2_f - S.nbh_margin_f;
    const float nb_zero = S.nbh_margin_f;
    uint32_t cell_total = 0;
    for (uint32_t c0 = 0; c0 < ncand; c0 += kStageCap) {
      const uint32_t c1 = min(ncand, c0 + static_cast<uint32_t>(kStageCap));
      for (int g = 0; g < 27; ++g) {
        const uint32_t gs = __shfl_sync(0xffffffffu, g_start, g);
        const uint32_t gn = __shfl_sync(0xffffffffu, g_n, g);
        const uint32_t go = __shfl_sync(0xffffffffu, g_off, g);
        const uint32_t gc = __shfl_sync(0xffffffffu, g_code, g);
        if (go + gn <= c0 || go >= c1) continue;
        for (uint32_t q = lane; q < gn; q += 32) {
          const uint32_t t = go + q;
          if (t < c0 || t >= c1) continue;
          const uint32_t j = gs + q;
          const double xb = image_coord(rx[j], S.period[0], static_cast<int>(gc % 3u));
          const double yb = image_coord(ry[j], S.period[1], static_cast<int>((gc / 3u) % 3u));
          const double zb = image_coord(rz[j], S.period[2], static_cast<int>(gc / 9u));
          bool keep = true;
          if (gc != static_cast<uint32_t>(kImageCenter))
            keep = xb >= S.outer_lo[0] && xb <= S.outer_hi[0] && yb >= S.outer_lo[1] && yb <= S.outer_hi[1] &&
                   zb >= S.outer_lo[2] && zb <= S.outer_hi[2];
          srel[t - c0] = make_float4(static_cast<float>(__dsub_rn(xb, o[0])), static_cast<float>(__dsub_rn(yb, o[1])),
                                     static_cast<float>(__dsub_rn(zb, o[2])), 0.f);
          sent[t - c0] = keep ? ((j << 5) | gc) : kInvalidS;
        }
      }
      __syncwarp();
      const uint32_t m = c1 - c0;
      for (uint32_t pa = 0; pa < na; ++pa) {
        const uint32_t i = sa + pa;
        const double xa = rx[i], ya = ry[i], za = rz[i];
        const float ax = static_cast<float>(__dsub_rn(xa, o[0]));
        const float ay = static_cast<float>(__dsub_rn(ya, o[1]));
        const float az = static_cast<float>(__dsub_rn(za, o[2]));
        const uint32_t self_ent = (i << 5) | static_cast<uint32_t>(kImageCenter);
        uint32_t cnt = 0, cursor = 0;
        if (FILL) cursor = cursor_g[i];
        for (uint32_t t0 = 0; t0 < m; t0 += 32) {
          const uint32_t t = t0 + lane;
          bool hit = false;
          uint32_t ent = kInvalidS;
          if (t < m) {
            ent = sent[t];
            if (ent != kInvalidS && ent != self_ent) {
              const float4 b = srel[t];
              const float dx = ax - b.x, dy = ay - b.y, dz = az - b.z;
              const float d2f = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
              if (d2f > nb_hi) {
                hit = false;
              } else if (d2f < nb_lo && d2f > nb_zero) {
                hit = true;
              } else {
                const uint32_t j = ent >> 5;
                const uint32_t gc = ent & 31u;
                const double xb = image_coord(rx[j], S.period[0], static_cast<int>(gc % 3u));
                const double yb = image_coord(ry[j], S.period[1], static_cast<int>((gc / 3u) % 3u));
                const double zb = image_coord(rz[j], S.period[2], static_cast<int>(gc / 9u));
                const double d2 = norm2_rn(__dsub_rn(xa, xb), __dsub_rn(ya, yb), __dsub_rn(za, zb));
                hit = d2 > 0.0 && d2 <= S.nbh2;
              }
            }
          }
          const unsigned mask = __ballot_sync(0xffffffffu, hit);
          if (FILL) {
            if (hit) nbr[cursor + __popc(mask & lanemask_lt_s())] = ent;
            cursor += __popc(mask);
          } else {
            cnt += __popc(mask);
          }
        }
        if (lane == 0) {
          if (FILL) cursor_g[i] = cursor;
          else nbr_cnt[i] = (c0 == 0 ? 0u : nbr_cnt[i]) + cnt;
        }
        cell_total += cnt;
      }
      __syncwarp();
    }
    if (!FILL && lane == 0) totals[c] = cell_total;
  }
}

std::mutex g_setup_mutex;
void* g_scratch_ptr[64] = {};  // device address of g_nbr_scratch, per device ordinal

}  // namespace

int launch_neighbors_static(const SysDesc& S_in, uint64_t ncells, uint64_t n, const double* rx, const double* ry,
                            const double* rz, const uint32_t* cell_start, const uint32_t* cell_n, uint32_t* nbr,
                            uint64_t cap, uint32_t* nbr_start, uint32_t* nbr_cnt, unsigned long long* total_out,
                            cudaStream_t stream, std::string* err) {
  if (n > kMaxParticles || ncells > kMaxCells) {
    *err = "chunk_neighbors without allocation: at most " + std::to_string(kMaxParticles) + " particles and " +
           std::to_string(kMaxCells) + " cells per call (got " + std::to_string(n) + " particles, " +
           std::to_string(ncells) + " cells)";
    return -1;
  }
  SysDesc S = S_in;
  S.ncells = static_cast<uint32_t>(ncells);
  S.npart = static_cast<uint32_t>(n);
  // entry positions are 32-bit: a total above 2^32 - 1 reports as a capacity error
  if (cap > 0xFFFFFFFFull) cap = 0xFFFFFFFFull;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) {
    *err = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
    return -2;
  }
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_nbr_scratch);
      if (e != cudaSuccess) {
        *err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
        return -2;
      }
      g_scratch_ptr[dev] = p;
    }
    base = g_scratch_ptr[dev];
  }
  auto failed = [&](const char* what, cudaError_t ce) {
    *err = std::string("chunk_neighbors without allocation: ") + what + ": " + cudaGetErrorString(ce);
    return -2;
  };
  unsigned char* scratch = static_cast<unsigned char*>(base);
  int sm = 1;
  e = cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return failed("cudaDeviceGetAttribute", e);
  const size_t smem = static_cast<size_t>(4) * kStageCap * (sizeof(float4) + sizeof(uint32_t));
  e = cudaFuncSetAttribute(k_neighbors_static<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return failed("cudaFuncSetAttribute", e);
  e = cudaFuncSetAttribute(k_neighbors_static<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return failed("cudaFuncSetAttribute", e);
  long long want = (static_cast<long long>(S.ncells) + 3) / 4;
  const long long capb = static_cast<long long>(sm) * 16;
  const int grid = static_cast<int>(want < 1 ? 1 : (want > capb ? capb : want));
  k_neighbors_static<false><<<grid, 128, smem, stream>>>(S, rx, ry, rz, cell_start, cell_n, nbr, nbr_start, nbr_cnt,
                                                         cap, scratch);
  e = cudaGetLastError();
  if (e != cudaSuccess) return failed("count pass launch", e);
  launch_scan_u32_to_u64(reinterpret_cast<const uint32_t*>(scratch + kTotalsOff),
                         reinterpret_cast<unsigned long long*>(scratch + kOffsetsOff), S.ncells,
                         reinterpret_cast<unsigned long long*>(scratch + kBlocksOff), stream);
  e = cudaGetLastError();
  if (e != cudaSuccess) return failed("offset scan launch", e);
  k_neighbors_static<true><<<grid, 128, smem, stream>>>(S, rx, ry, rz, cell_start, cell_n, nbr, nbr_start, nbr_cnt,
                                                        cap, scratch);
  e = cudaGetLastError();
  if (e != cudaSuccess) return failed("fill pass launch", e);
  e = cudaMemcpyAsync(total_out, scratch + kOffsetsOff + sizeof(unsigned long long) * S.ncells,
                      sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream);
  if (e != cudaSuccess) return failed("cudaMemcpyAsync", e);
  e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return failed("cudaStreamSynchronize", e);
  return 0;
}

}  // namespace xnb
