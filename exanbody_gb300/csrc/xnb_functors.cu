// Pair functors other than Lennard-Jones over the same per-particle lists,
// written against the pair-functor API (include/xnb_pair.cuh) and run through
// its FP32-prefiltered traversal.
//
// gravitational_force (contribs/pi/gravitational_force.cu:42-141) is a
// buffer-less functor: compute_cell_particle_pairs calls it per stream entry
// inside rcut (compute_cell_particle_pairs_impl_default.h:186-205) and it adds
// straight onto the particle's force field:
//   r = sqrt(d2), inv_r = 1/r, e = -G m_a m_b inv_r, de = G m_a m_b inv_r inv_r,
//   de *= w / r (w = 1), f_a += de * dr, dr = r_b - r_a,
// with m_a, m_b the masses of the particles' types.
#include "xnb_launch.cuh"
#include "xnb_traverse.cuh"

namespace xnb {

namespace {

constexpr uint32_t kInvalid = 0xFFFFFFFFu;

// P = kFp64Exact: the functor's operations and roundings, bit-identical to the
// CPU restatement. P = kFp64: same pairs, 1/r^3 from one correctly rounded
// square root and one division, FMA accumulation. A pair-functor API functor
// (include/xnb_pair.cuh): buffer-less, called per pair within gp.rcut.
template <int P, bool PE>
struct GravForce {
  DevArrays a;
  GravParams gp;
  bool accumulate;
  unsigned int* flags;
  struct Acc {
    double fx, fy, fz, pe, ma;
  };

  __device__ __forceinline__ double rcut2(const pair::ParticleContext&) const { return gp.rcut2; }
  __device__ __forceinline__ float prefilter_hi(const pair::ParticleContext&) const { return gp.pre_hi_f; }
  __device__ __forceinline__ bool start(Acc& q, const pair::ParticleContext& c) const {
    const uint32_t ta = a.ptype[c.i];
    if (ta >= static_cast<uint32_t>(gp.ntypes)) {
      atomicOr(flags, 1u);
      return false;
    }
    q.ma = gp.mass[ta];
    q.fx = accumulate ? a.fx[c.i] : 0.0;
    q.fy = accumulate ? a.fy[c.i] : 0.0;
    q.fz = accumulate ? a.fz[c.i] : 0.0;
    q.pe = 0.0;
    return true;
  }
  __device__ __forceinline__ void pair(Acc& q, const pair::ParticleContext&, const pair::PairData& p) const {
    const uint32_t tb = a.ptype[p.j];
    if (tb >= static_cast<uint32_t>(gp.ntypes)) {
      atomicOr(flags, 1u);
      return;
    }
    const double mb = gp.mass[tb];
    if (P == kFp64Exact) {
      const double r = __dsqrt_rn(p.d2);
      const double inv_r = __ddiv_rn(1.0, r);
      double de = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(gp.G, q.ma), mb), inv_r), inv_r);
      de = __dmul_rn(de, __ddiv_rn(1.0, r));
      q.fx = __dadd_rn(q.fx, __dmul_rn(de, p.dx));
      q.fy = __dadd_rn(q.fy, __dmul_rn(de, p.dy));
      q.fz = __dadd_rn(q.fz, __dmul_rn(de, p.dz));
      if (PE) {
        const double en = __dmul_rn(__dmul_rn(__dmul_rn(-gp.G, q.ma), mb), inv_r);
        q.pe = __dadd_rn(q.pe, __dmul_rn(0.5, en));
      }
    } else {
      const double r = sqrt(p.d2);
      const double inv_r3 = 1.0 / (p.d2 * r);
      const double gm = gp.G * q.ma * mb;
      const double de = gm * inv_r3;
      q.fx = fma(de, p.dx, q.fx);
      q.fy = fma(de, p.dy, q.fy);
      q.fz = fma(de, p.dz, q.fz);
      if (PE) q.pe -= 0.5 * gm / r;
    }
  }
  __device__ __forceinline__ void stop(Acc& q, const pair::ParticleContext& c) const {
    a.fx[c.i] = q.fx;
    a.fy[c.i] = q.fy;
    a.fz[c.i] = q.fz;
    if (PE) a.pe[c.i] = accumulate ? a.pe[c.i] + q.pe : q.pe;
  }
};

template <int P, bool PE>
__global__ void __launch_bounds__(128) k_grav(uint32_t n_part, BatchSource src, GravForce<P, PE> f) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_part) pair::traverse_particle(src, i, f);
}

// field::type of the particles whose ids are listed (sorted ascending, n of
// them); matched counts the particles of system sid that were found.
__global__ void __launch_bounds__(256)
    k_set_types(uint32_t sid, const SysDesc* __restrict__ sys, DevArrays a, const uint64_t* __restrict__ ids,
                const uint8_t* __restrict__ types, uint32_t n, unsigned long long* matched) {
  const SysDesc& S = sys[sid];
  unsigned long long mine = 0;
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
      a.ptype[i] = types[lo];
      ++mine;
    }
  }
  for (int off = 16; off > 0; off >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, off);
  if ((threadIdx.x & 31) == 0 && mine) atomicAdd(matched, mine);
}

}  // namespace

int launch_set_types(uint32_t sid, uint32_t npart, const SysDesc* sys, const DevArrays& a, const uint64_t* ids,
                     const uint8_t* types, uint32_t n, unsigned long long* matched, int sm_count, cudaStream_t stream) {
  const long long want = (static_cast<long long>(npart) + 255) / 256;
  const int g = static_cast<int>(want < 1 ? 1 : (want > sm_count * 8LL ? sm_count * 8LL : want));
  k_set_types<<<g, 256, 0, stream>>>(sid, sys, a, ids, types, n, matched);
  return 1;
}

int launch_gravity(const Extent& ex, const SysDesc* sys, const SysState* st, const DevArrays& a, int precision,
                   bool with_pe, bool accumulate, int sys_only, const GravParams& gp, unsigned int* flags,
                   cudaStream_t stream) {
  if (ex.n_part == 0) return 0;
  const int threads = 128;
  const int g = static_cast<int>((static_cast<long long>(ex.n_part) + threads - 1) / threads);
  const BatchSource src(sys, st, a, sys_only);
  if (precision == kFp64Exact) {
    if (with_pe) k_grav<kFp64Exact, true><<<g, threads, 0, stream>>>(ex.n_part, src, {a, gp, accumulate, flags});
    else k_grav<kFp64Exact, false><<<g, threads, 0, stream>>>(ex.n_part, src, {a, gp, accumulate, flags});
  } else {
    if (with_pe) k_grav<kFp64, true><<<g, threads, 0, stream>>>(ex.n_part, src, {a, gp, accumulate, flags});
    else k_grav<kFp64, false><<<g, threads, 0, stream>>>(ex.n_part, src, {a, gp, accumulate, flags});
  }
  return 1;
}

}  // namespace xnb
