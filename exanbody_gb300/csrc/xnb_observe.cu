// On-device observables: simulation_stats reductions and id-sampled particle
// values (check_values), so logging and checks need no full host copy.
#include "xnb_launch.cuh"

namespace xnb {

namespace {

constexpr uint32_t kInvalid = 0xFFFFFFFFu;

// Per-block partial results; the second kernel folds them in block order, so
// the sums do not depend on scheduling.
struct StatsPart {
  double ke, pe, vmin, vmax, amin, amax;
  unsigned long long n;
};

__device__ __forceinline__ void fold(StatsPart& x, const StatsPart& y) {
  x.ke += y.ke;
  x.pe += y.pe;
  x.vmin = fmin(x.vmin, y.vmin);
  x.vmax = fmax(x.vmax, y.vmax);
  x.amin = fmin(x.amin, y.amin);
  x.amax = fmax(x.amax, y.amax);
  x.n += y.n;
}

// ComputeSimulationStatistics (debug/simulation_stats.cpp:60-124) over the
// particles of system sid: sum of dot(v, v) * 1.0 (the reference's mass), particle
// count, extremes of |v| and |f|, and the sum of the per-particle energies.
__global__ void __launch_bounds__(256)
    k_stats_blocks(uint32_t sid, const SysDesc* __restrict__ sys, DevArrays a, StatsPart* parts) {
  const SysDesc& S = sys[sid];
  StatsPart m{0.0, 0.0, 1.0e308, 0.0, 1.0e308, 0.0, 0ull};
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < S.npart; q += gridDim.x * blockDim.x) {
    const uint32_t i = S.part_base + q;
    if (a.pcell[i] == kInvalid) continue;
    const double vx = a.vx[i], vy = a.vy[i], vz = a.vz[i];
    const double fx = a.fx[i], fy = a.fy[i], fz = a.fz[i];
    const double v2 = (vx * vx + vy * vy) + vz * vz;
    const double f2 = (fx * fx + fy * fy) + fz * fz;
    m.ke += v2 * 1.0;
    m.pe += a.pe[i];
    const double vn = sqrt(v2), an = sqrt(f2);
    m.vmin = fmin(m.vmin, vn);
    m.vmax = fmax(m.vmax, vn);
    m.amin = fmin(m.amin, an);
    m.amax = fmax(m.amax, an);
    m.n += 1;
  }
  __shared__ StatsPart sh[256];
  sh[threadIdx.x] = m;
  __syncthreads();
  for (uint32_t w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) fold(sh[threadIdx.x], sh[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) parts[blockIdx.x] = sh[0];
}

__global__ void k_stats_final(const StatsPart* parts, int nblocks, StatsPart* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  StatsPart m{0.0, 0.0, 1.0e308, 0.0, 1.0e308, 0.0, 0ull};
  for (int b = 0; b < nblocks; ++b) fold(m, parts[b]);
  *out = m;
}

// Values of the particles whose ids are listed (sorted ascending, n of them):
// out[k*9 ..] = r, f, v of id ids[k]; found[k] = 1 when the id is in the system.
__global__ void __launch_bounds__(256)
    k_sample(uint32_t sid, const SysDesc* __restrict__ sys, DevArrays a, const uint64_t* __restrict__ ids, uint32_t n,
             double* out, int32_t* found) {
  const SysDesc& S = sys[sid];
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < S.npart; q += gridDim.x * blockDim.x) {
    const uint32_t i = S.part_base + q;
    if (a.pcell[i] == kInvalid) continue;
    const uint64_t id = a.id[i];
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (ids[mid] < id) lo = mid + 1;
      else hi = mid;
    }
    if (lo < n && ids[lo] == id) {
      double* o = out + static_cast<size_t>(lo) * 9;
      o[0] = a.rx[i]; o[1] = a.ry[i]; o[2] = a.rz[i];
      o[3] = a.fx[i]; o[4] = a.fy[i]; o[5] = a.fz[i];
      o[6] = a.vx[i]; o[7] = a.vy[i]; o[8] = a.vz[i];
      found[lo] = 1;
    }
  }
}

}  // namespace

size_t stats_scratch_bytes() { return (1024 + 1) * sizeof(StatsPart); }

int launch_stats(uint32_t sid, uint32_t npart, const SysDesc* sys, const DevArrays& a, void* scratch, int sm_count,
                 cudaStream_t stream) {
  long long want = (static_cast<long long>(npart) + 255) / 256;
  const long long cap = sm_count * 4LL < 1024 ? sm_count * 4LL : 1024;
  const int g = static_cast<int>(want < 1 ? 1 : (want > cap ? cap : want));
  auto* parts = static_cast<StatsPart*>(scratch);
  k_stats_blocks<<<g, 256, 0, stream>>>(sid, sys, a, parts);
  k_stats_final<<<1, 32, 0, stream>>>(parts, g, parts + 1024);
  return 2;
}

int copy_stats(void* scratch, double* out6, unsigned long long* count_out, cudaStream_t stream) {
  StatsPart m;
  if (cudaMemcpyAsync(&m, static_cast<StatsPart*>(scratch) + 1024, sizeof(m), cudaMemcpyDeviceToHost, stream) !=
      cudaSuccess)
    return -1;
  if (cudaStreamSynchronize(stream) != cudaSuccess) return -1;
  out6[0] = m.ke;
  out6[1] = m.pe;
  out6[2] = m.vmin;
  out6[3] = m.vmax;
  out6[4] = m.amin;
  out6[5] = m.amax;
  *count_out = m.n;
  return 0;
}

int launch_sample(uint32_t sid, uint32_t npart, const SysDesc* sys, const DevArrays& a, const uint64_t* ids,
                  uint32_t n, double* out, int32_t* found, int sm_count, cudaStream_t stream) {
  long long want = (static_cast<long long>(npart) + 255) / 256;
  const long long cap = sm_count * 8LL;
  const int g = static_cast<int>(want < 1 ? 1 : (want > cap ? cap : want));
  k_sample<<<g, 256, 0, stream>>>(sid, sys, a, ids, n, out, found);
  return 1;
}

}  // namespace xnb
