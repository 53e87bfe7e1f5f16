// A pair potential written the way a user of the library writes one: against
// include/xnb_pair.cuh and include/xnb_gpu.h alone, built into its own shared
// library, run over a resident system's neighbour lists (xnb_system_pair_view).
//
// Morse potential V(r) = D (exp(-2a(r - r0)) - 2 exp(-a(r - r0))), shifted to 0
// at rcut: f_a += (dV/dr / r) (r_b - r_a), dV/dr = 2aD (e1 - e2), e1 = exp(-a(r - r0)),
// e2 = e1^2, and 0.5 (V(r) - V(rcut)) per pair as the particle's energy.
//
//   morse_force(view, D, alpha, r0, rcut, mode, stream)
//     mode 0: buffer-less functor (per pair, full lists)
//     mode 1: compute-buffer functor (the same pairs handed over 16 at a time)
//     mode 2: symmetric functor (lower half lists, reactions by atomics)
//   returns 0, or a cudaError_t / -1 for a cutoff above the lists' distance.
#include <cuda_runtime.h>

#include "xnb_pair.cuh"

namespace {

using xnb::pair::PairData;
using xnb::pair::ParticleContext;

struct MorseCore {
  double D, alpha, r0, rc2, e_shift;
  float pre_hi;
  double *fx, *fy, *fz, *pe;

  struct Acc {
    double fx, fy, fz, pe;
  };
  __device__ double rcut2(const ParticleContext&) const { return rc2; }
  __device__ float prefilter_hi(const ParticleContext&) const { return pre_hi; }
  __device__ bool start(Acc& q, const ParticleContext&) const {
    q.fx = q.fy = q.fz = q.pe = 0.0;
    return true;
  }
  // force factor (dV/dr) / r and the pair's energy share
  __device__ void terms(const PairData& p, double& s, double& en) const {
    const double r = sqrt(p.d2);
    const double e1 = exp(-alpha * (r - r0));
    const double e2 = e1 * e1;
    s = 2.0 * alpha * D * (e1 - e2) / r;
    en = 0.5 * (D * (e2 - 2.0 * e1) - e_shift);
  }
  __device__ void pair(Acc& q, const ParticleContext&, const PairData& p) const {
    double s, en;
    terms(p, s, en);
    q.fx += s * p.dx;
    q.fy += s * p.dy;
    q.fz += s * p.dz;
    q.pe += en;
  }
  __device__ void stop(Acc& q, const ParticleContext& c) const {
    fx[c.i] = q.fx;
    fy[c.i] = q.fy;
    fz[c.i] = q.fz;
    pe[c.i] = q.pe;
  }
};

struct MorseBuffered : MorseCore {
  __device__ void buffer(Acc& q, const ParticleContext& c, int n, const PairData* buf) const {
    for (int k = 0; k < n; ++k) pair(q, c, buf[k]);
  }
};

struct MorseSymmetric : MorseCore {
  // each pair once (lower half): a keeps +f, b receives -f; energies split evenly
  __device__ void pair(Acc& q, const ParticleContext&, const PairData& p) const {
    double s, en;
    terms(p, s, en);
    const double gx = s * p.dx, gy = s * p.dy, gz = s * p.dz;
    q.fx += gx;
    q.fy += gy;
    q.fz += gz;
    q.pe += en;
    atomicAdd(fx + p.j, -gx);
    atomicAdd(fy + p.j, -gy);
    atomicAdd(fz + p.j, -gz);
    atomicAdd(pe + p.j, en);
  }
  __device__ void stop(Acc& q, const ParticleContext& c) const {
    atomicAdd(fx + c.i, q.fx);
    atomicAdd(fy + c.i, q.fy);
    atomicAdd(fz + c.i, q.fz);
    atomicAdd(pe + c.i, q.pe);
  }
};

}  // namespace

namespace xnb {
namespace pair {
template <>
struct ComputePairTraits<MorseBuffered> : DefaultPairTraits {
  static constexpr bool BufferLessCompatible = false;
  static constexpr bool ComputeBufferCompatible = true;
  static constexpr int ComputeBufferSize = 16;
};
template <>
struct ComputePairTraits<MorseSymmetric> : DefaultPairTraits {
  static constexpr bool Symmetric = true;
};
}  // namespace pair
}  // namespace xnb

extern "C" int morse_force(const xnb_pair_view* v, double D, double alpha, double r0, double rcut, int mode,
                           void* stream) {
  if (!v || !(rcut > 0.0) || rcut > v->nbh_dist) return -1;
  MorseCore m;
  m.D = D;
  m.alpha = alpha;
  m.r0 = r0;
  m.rc2 = rcut * rcut;
  const double ec1 = exp(-alpha * (rcut - r0));
  m.e_shift = D * (ec1 * ec1 - 2.0 * ec1);
  m.pre_hi = xnb::pair::prefilter_bound(*v, rcut);
  m.fx = v->fx;
  m.fy = v->fy;
  m.fz = v->fz;
  m.pe = v->pe;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (mode == 0) {
    e = xnb::pair::traverse_pairs(*v, m, st);
  } else if (mode == 1) {
    MorseBuffered b;
    static_cast<MorseCore&>(b) = m;
    e = xnb::pair::traverse_pairs(*v, b, st);
  } else {
    // the reactions land on any particle: clear the outputs first
    const size_t bytes = static_cast<size_t>(v->n_particles) * sizeof(double);
    e = cudaMemsetAsync(v->fx, 0, bytes, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(v->fy, 0, bytes, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(v->fz, 0, bytes, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(v->pe, 0, bytes, st);
    MorseSymmetric y;
    static_cast<MorseCore&>(y) = m;
    if (e == cudaSuccess) e = xnb::pair::traverse_pairs(*v, y, st);
  }
  return static_cast<int>(e);
}
