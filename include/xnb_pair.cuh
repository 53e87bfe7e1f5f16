/*
 * xnb_pair.cuh -- device-side pair-functor API over the neighbour lists that
 * libxnb_gpu builds (include/xnb_gpu.h). Header-only; needs nothing but the CUDA
 * toolkit and xnb_gpu.h, so a potential compiled against include/ alone runs
 * over a resident system's lists (xnb_system_pair_view).
 *
 * The reference plugs pair potentials into compute_cell_particle_pairs
 * (compute/include/exanb/compute/compute_cell_particle_pairs.h:119-245): a
 * functor, described by a ComputePairTraits specialisation
 * (compute/include/exanb/compute/compute_pair_traits.h:28-74), is called for
 * every neighbour b of particle a with dr = r_b - r_a (the periodic image
 * applied) and d2 = norm2(dr) when 0 < d2 <= rcut^2, in the list's
 * (cell_enc, p_b) order (compute_cell_particle_pairs_impl_default.h:148-238),
 * either per pair as it goes (buffer-less) or once per particle over a
 * buffer of its neighbours (compute buffer). The same contract here:
 *
 *   * one GPU thread per particle walks the particle's list in order, so a
 *     functor accumulating into registers sums in the reference's order and
 *     needs no atomics;
 *   * the list is read in windows of 128 entries; an FP32 prefilter over the
 *     particles' FP32 position mirrors marks the entries that may lie within
 *     the functor's cutoff (rcut^2 plus a proven bound on the FP32 error, see
 *     prefilter_bound); only marked entries are gathered in FP64, so the pair
 *     set is exactly the FP64 one;
 *   * dr and d2 are formed with the reference's roundings (no contraction:
 *     dr = fl(r_b - r_a) per axis, d2 = (dx*dx + dy*dy) + dz*dz).
 *
 * A functor F is a copyable struct with
 *     struct Acc { ... };                                  per-particle state
 *     __device__ double rcut2(const ParticleContext&) const;     cutoff^2
 *     __device__ float prefilter_hi(const ParticleContext&) const; FP32 bound (>= rcut^2)
 *     __device__ bool start(Acc&, const ParticleContext&) const;   false: skip the particle
 *     __device__ void pair(Acc&, const ParticleContext&, const PairData&) const;   buffer-less
 *     __device__ void buffer(Acc&, const ParticleContext&, int n, const PairData*) const;  compute buffer
 *     __device__ void entry(Acc&, const ParticleContext&, const RawEntry&) const;  raw entries
 *     __device__ void stop(Acc&, const ParticleContext&) const;
 *     __device__ void combine(Acc&, const Acc&) const;   (lane groups: add a partial state)
 * and a ComputePairTraits<F> specialisation (derived from DefaultPairTraits)
 * choosing which of pair / buffer / entry the traversal calls:
 *   BufferLessCompatible  pair() per neighbour within the cutoff (default);
 *   ComputeBufferCompatible (and not BufferLessCompatible)  buffer() with up to
 *                         ComputeBufferSize neighbours at a time, in order
 *                         (several calls for a longer neighbourhood);
 *   RawEntries            entry() per prefiltered list entry with the gathered
 *                         FP64 position and FP32 mirrors, before any cutoff test:
 *                         the functor forms its own displacement (used by the
 *                         library's mixed-precision Lennard-Jones);
 *   Symmetric             only the lower half of each list (the reference's
 *                         symmetric split, impl_default.h:181): each pair is
 *                         seen once and the functor adds the reaction to b
 *                         itself (atomics);
 *   GatherMirrors         also gather the FP32 residual mirrors (RawEntries);
 *   EntriesPerIteration   1 or 2 (RawEntries): marked entries whose gathers are
 *                         in flight together.
 * stop() writes the particle's results (the functor holds its output pointers).
 */
#ifndef XNB_PAIR_CUH
#define XNB_PAIR_CUH

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "xnb_gpu.h"

namespace xnb {
namespace pair {

// Image code of the unshifted periodic image ((0+1) + 3*(0+1) + 9*(0+1)); a list
// entry is (particle index within its system << 5) | image code, digit d of the
// code (x: code % 3, y: code / 3 % 3, z: code / 9) meaning a shift of d - 1 periods.
constexpr uint32_t kImageCenter = 13;

// ---------------------------------------------------------------------------
// Traits (compute_pair_traits.h:28-74: ComputePairTraits<void> holds the defaults).
struct DefaultPairTraits {
  static constexpr bool BufferLessCompatible = true;
  static constexpr bool ComputeBufferCompatible = false;
  static constexpr int ComputeBufferSize = 32;
  static constexpr bool CudaCompatible = true;
  static constexpr bool Symmetric = false;
  static constexpr bool RawEntries = false;
  static constexpr bool GatherMirrors = false;
  static constexpr int EntriesPerIteration = 1;
};
template <class F>
struct ComputePairTraits : DefaultPairTraits {};

// ---------------------------------------------------------------------------
// What a functor sees.
struct ParticleContext {
  uint32_t i;         // the particle: index into the arrays the traversal reads
  uint32_t sys;       // its system (0 for a single-system view)
  uint32_t pbase;     // index of the system's first particle: entry e names pbase + (e >> 5)
  double x, y, z;     // FP64 position of the particle
  float4 hi, lo;      // its FP32 mirrors (lo: zero unless GatherMirrors)
  double period[3];   // periodic image offsets of its system
  float period_f[3];
  const uint32_t* list;  // the walked part of its list
  uint32_t n;
};

struct PairData {
  double dx, dy, dz;  // r_b - r_a, the periodic image applied
  double d2;          // (dx*dx + dy*dy) + dz*dz
  uint32_t j;         // index of b
  uint32_t code;      // image code of the entry
};

struct RawEntry {
  uint32_t e;         // the list entry
  uint32_t j;         // index of b
  double xb, yb, zb;  // FP64 position of b (its own image: the functor applies the code)
  float4 hb, lb;      // FP32 mirrors of b (lb: zero unless GatherMirrors)
};

// ---------------------------------------------------------------------------
// Reference roundings.
__device__ __forceinline__ double norm2_rn(double x, double y, double z) {
  return __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
}

// apply_coord_modifier (mpi/include/exanb/mpi/ghosts_comm_scheme.h:76-80): x + (+-1.0)*(rmax - rmin)
// for a shifted axis (digit d of the image code: 0 = -1, 1 = none, 2 = +1).
__device__ __forceinline__ double image_coord(double x, double period, int d) {
  return d == 1 ? x : __dadd_rn(x, __dmul_rn(d == 2 ? 1.0 : -1.0, period));
}
__device__ __forceinline__ float image_coord_f(float x, float period, int d) {
  return d == 1 ? x : (d == 2 ? x + period : x - period);
}

// ---------------------------------------------------------------------------
// FP32 prefilter bound. The mirrors are fl32(x - origin) with |x - origin| <=
// X = P + nbh (P the largest period, nbh the lists' distance: particles stay
// within the skin of the domain between rebuilds); an image adds fl32(period).
// One axis of an FP32 difference is then within D = (3X + 2P + R) u 1.01 of
// the FP64 one for pairs within distance R (u = 2^-24), and the FP32 squared
// distance within 2 sqrt(3) R D + 3 D^2 + 4 u (R^2 + 1) of the FP64 d2. The
// prefilter threshold is rcut^2 + 4 x that bound at R = rcut, rounded up to FP32.
__host__ __device__ inline double fp32_d2_error_bound(double max_period, double nbh, double R) {
  const double u = 5.9604644775390625e-08;  // 2^-24
  const double X = max_period + nbh;
  const double D = (3.0 * X + 2.0 * max_period + R) * u * 1.01;
  return 2.0 * 1.7320508075688772 * R * D + 3.0 * D * D + 4.0 * u * (R * R + 1.0);
}
__host__ __device__ inline float prefilter_bound(double max_period, double nbh, double rcut) {
  const double t = rcut * rcut + 4.0 * fp32_d2_error_bound(max_period, nbh, rcut);
  float f = static_cast<float>(t);
  if (static_cast<double>(f) < t) f = nextafterf(f, 2.0f * f + 1.0f);
  return f;
}

// ---------------------------------------------------------------------------
// Windowed FP32 prefilter: bit k - kw of the mask words is set for each entry of
// [kw, kend) (at most 128) whose FP32 distance to the particle may lie within
// the bound; unmarked entries are provably beyond it. Entries are read 8 at a
// time with two 16-byte loads (lists start on 32-byte boundaries and slots are
// multiples of 8 entries) and the 8 mirror gathers are independent, so they are
// in flight together. Positions past kend gather the particle's own mirror.
struct Marks {
  uint32_t w[4];
};

// With lanes > 1 the caller is lane `sub` of a group sharing the particle and
// marks only the 8-entry blocks kw + 8 (sub + lanes k) of the window.
__device__ __forceinline__ Marks prefilter_window(const uint32_t* __restrict__ L, uint32_t kw, uint32_t kend,
                                                  const float4* __restrict__ pf, uint32_t pbase, uint32_t self_e,
                                                  float4 paf, float pfx, float pfy, float pfz, float pre_hi,
                                                  uint32_t sub = 0, uint32_t lanes = 1) {
  Marks m{{0u, 0u, 0u, 0u}};
  for (uint32_t kb = kw + 8u * sub; kb < kend; kb += 8u * lanes) {
    const uint4 ea = __ldg(reinterpret_cast<const uint4*>(L + kb));
    const uint4 eb = __ldg(reinterpret_cast<const uint4*>(L + kb + 4));
    const uint32_t ev[8] = {ea.x, ea.y, ea.z, ea.w, eb.x, eb.y, eb.z, eb.w};
    uint32_t bits = 0;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const bool valid = kb + static_cast<uint32_t>(t) < kend;
      const uint32_t e = valid ? ev[t] : self_e;
      const uint32_t code = e & 31u;
      const float4 pbf = __ldg(pf + pbase + (e >> 5));
      float bx = pbf.x, by = pbf.y, bz = pbf.z;
      if (code != kImageCenter) {
        bx = image_coord_f(bx, pfx, static_cast<int>(code % 3u));
        by = image_coord_f(by, pfy, static_cast<int>((code / 3u) % 3u));
        bz = image_coord_f(bz, pfz, static_cast<int>(code / 9u));
      }
      const float ex = bx - paf.x, ey = by - paf.y, ez = bz - paf.z;
      if (valid && fmaf(ex, ex, fmaf(ey, ey, ez * ez)) <= pre_hi) bits |= 1u << t;
    }
    const uint32_t off = kb - kw;
    const uint32_t sh = off & 31u;
    if (off < 32u) m.w[0] |= bits << sh;
    else if (off < 64u) m.w[1] |= bits << sh;
    else if (off < 96u) m.w[2] |= bits << sh;
    else m.w[3] |= bits << sh;
  }
  return m;
}

// Next marked entry of a window in list order (offset into the window), or false.
__device__ __forceinline__ bool next_mark(Marks& m, uint32_t& b) {
  if (m.w[0]) {
    b = static_cast<uint32_t>(__ffs(m.w[0]) - 1);
    m.w[0] &= m.w[0] - 1u;
  } else if (m.w[1]) {
    b = 32u + static_cast<uint32_t>(__ffs(m.w[1]) - 1);
    m.w[1] &= m.w[1] - 1u;
  } else if (m.w[2]) {
    b = 64u + static_cast<uint32_t>(__ffs(m.w[2]) - 1);
    m.w[2] &= m.w[2] - 1u;
  } else if (m.w[3]) {
    b = 96u + static_cast<uint32_t>(__ffs(m.w[3]) - 1);
    m.w[3] &= m.w[3] - 1u;
  } else {
    return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
// The walk of one particle's list. Src provides the particle's context
// (begin) and the arrays gathered by list entry (rx, ry, rz, pf, pflo).
template <class F, class Src>
__device__ __forceinline__ void traverse_particle(const Src& src, uint32_t i, const F& f) {
  using T = ComputePairTraits<F>;
  static_assert(T::CudaCompatible, "the functor is not marked CudaCompatible");
  static_assert(T::RawEntries || T::BufferLessCompatible || T::ComputeBufferCompatible,
                "the functor must take pairs, a compute buffer or raw entries");
  static_assert(T::EntriesPerIteration == 1 || (T::RawEntries && T::EntriesPerIteration == 2),
                "two entries per iteration only for raw-entry functors");
  ParticleContext c;
  if (!src.begin(i, T::Symmetric, T::GatherMirrors, c)) return;
  typename F::Acc acc;
  if (!f.start(acc, c)) return;
  const float pre_hi = f.prefilter_hi(c);
  const uint32_t self_e = ((c.i - c.pbase) << 5) | kImageCenter;
  const uint32_t n = c.n;
  const uint32_t* __restrict__ L = c.list;
  if constexpr (T::RawEntries) {
    for (uint32_t kw = 0; kw < n; kw += 128) {
      Marks mk = prefilter_window(L, kw, min(n, kw + 128u), src.pf, c.pbase, self_e, c.hi, c.period_f[0],
                                  c.period_f[1], c.period_f[2], pre_hi);
      if constexpr (T::EntriesPerIteration == 2) {
        // two marked entries per iteration: their list entries, then their
        // gathers, are in flight together; list order is kept (b0 < b1)
        uint32_t b0 = 0, b1 = 0;
        bool h0 = next_mark(mk, b0);
        while (h0) {
          const bool h1 = next_mark(mk, b1);
          RawEntry r0, r1;
          r0.e = __ldg(L + kw + b0);
          r1.e = __ldg(L + kw + (h1 ? b1 : b0));
          r0.j = c.pbase + (r0.e >> 5);
          r1.j = c.pbase + (r1.e >> 5);
          r0.xb = __ldg(src.rx + r0.j);
          r0.yb = __ldg(src.ry + r0.j);
          r0.zb = __ldg(src.rz + r0.j);
          r1.xb = __ldg(src.rx + r1.j);
          r1.yb = __ldg(src.ry + r1.j);
          r1.zb = __ldg(src.rz + r1.j);
          r0.hb = __ldg(src.pf + r0.j);
          r0.lb = T::GatherMirrors ? __ldg(src.pflo + r0.j) : make_float4(0.f, 0.f, 0.f, 0.f);
          r1.hb = __ldg(src.pf + r1.j);
          r1.lb = T::GatherMirrors ? __ldg(src.pflo + r1.j) : make_float4(0.f, 0.f, 0.f, 0.f);
          f.entry(acc, c, r0);
          if (h1) f.entry(acc, c, r1);
          h0 = h1 && next_mark(mk, b0);
        }
      } else {
        uint32_t b;
        while (next_mark(mk, b)) {
          RawEntry r;
          r.e = __ldg(L + kw + b);
          r.j = c.pbase + (r.e >> 5);
          r.xb = __ldg(src.rx + r.j);
          r.yb = __ldg(src.ry + r.j);
          r.zb = __ldg(src.rz + r.j);
          r.hb = __ldg(src.pf + r.j);
          r.lb = T::GatherMirrors ? __ldg(src.pflo + r.j) : make_float4(0.f, 0.f, 0.f, 0.f);
          f.entry(acc, c, r);
        }
      }
    }
  } else {
    constexpr bool kBuffered = !T::BufferLessCompatible;
    constexpr int kBuf = kBuffered ? T::ComputeBufferSize : 1;
    PairData buf[kBuf];
    int nb = 0;
    const double rc2 = f.rcut2(c);
    for (uint32_t kw = 0; kw < n; kw += 128) {
      Marks mk = prefilter_window(L, kw, min(n, kw + 128u), src.pf, c.pbase, self_e, c.hi, c.period_f[0],
                                  c.period_f[1], c.period_f[2], pre_hi);
      uint32_t b;
      while (next_mark(mk, b)) {
        const uint32_t e = __ldg(L + kw + b);
        const uint32_t j = c.pbase + (e >> 5);
        const uint32_t code = e & 31u;
        double xb = __ldg(src.rx + j), yb = __ldg(src.ry + j), zb = __ldg(src.rz + j);
        if (code != kImageCenter) {
          xb = image_coord(xb, c.period[0], static_cast<int>(code % 3u));
          yb = image_coord(yb, c.period[1], static_cast<int>((code / 3u) % 3u));
          zb = image_coord(zb, c.period[2], static_cast<int>(code / 9u));
        }
        PairData p;
        p.dx = __dsub_rn(xb, c.x);
        p.dy = __dsub_rn(yb, c.y);
        p.dz = __dsub_rn(zb, c.z);
        p.d2 = norm2_rn(p.dx, p.dy, p.dz);
        if (p.d2 > 0.0 && p.d2 <= rc2) {
          p.j = j;
          p.code = code;
          if constexpr (kBuffered) {
            buf[nb++] = p;
            if (nb == kBuf) {
              f.buffer(acc, c, nb, buf);
              nb = 0;
            }
          } else {
            f.pair(acc, c, p);
          }
        }
      }
    }
    if constexpr (kBuffered) {
      if (nb > 0) f.buffer(acc, c, nb, buf);
    }
  }
  f.stop(acc, c);
}

// ---------------------------------------------------------------------------
// The same walk with LANES threads per particle (2, 4 or 8 consecutive lanes
// of a warp): lane `sub` of the group takes the 8-entry blocks sub, sub +
// LANES, ... of every window, in list order, and the partial states are
// combined in a fixed order (F::combine, a shuffle tree within the group), so
// results are reproducible from run to run; they agree with the one-lane walk
// to rounding. Every lane of the warp must call it (the shuffles span the
// warp): `active` is false for lanes past the last particle. Raw-entry and
// buffer-less functors; stop() runs on the group's first lane.
template <int LANES, class F, class Src>
__device__ __forceinline__ void traverse_particle_lanes(const Src& src, uint32_t i, bool active, const F& f) {
  using T = ComputePairTraits<F>;
  static_assert(LANES == 2 || LANES == 4 || LANES == 8, "2, 4 or 8 lanes per particle");
  static_assert(T::RawEntries || T::BufferLessCompatible, "lane groups take raw entries or buffer-less pairs");
  static_assert(sizeof(typename F::Acc) % 4 == 0, "the per-particle state is combined 32 bits at a time");
  const uint32_t sub = threadIdx.x & (LANES - 1);
  ParticleContext c;
  typename F::Acc acc{};
  bool ok = active && src.begin(i, T::Symmetric, T::GatherMirrors, c);
  if (ok) ok = f.start(acc, c);
  if (ok) {
    const float pre_hi = f.prefilter_hi(c);
    const uint32_t self_e = ((c.i - c.pbase) << 5) | kImageCenter;
    const uint32_t n = c.n;
    const uint32_t* __restrict__ L = c.list;
    const double rc2 = T::RawEntries ? 0.0 : f.rcut2(c);
    for (uint32_t kw = 0; kw < n; kw += 128) {
      Marks mk = prefilter_window(L, kw, min(n, kw + 128u), src.pf, c.pbase, self_e, c.hi, c.period_f[0],
                                  c.period_f[1], c.period_f[2], pre_hi, sub, LANES);
      uint32_t b;
      while (next_mark(mk, b)) {
        const uint32_t e = __ldg(L + kw + b);
        const uint32_t j = c.pbase + (e >> 5);
        if constexpr (T::RawEntries) {
          RawEntry r;
          r.e = e;
          r.j = j;
          r.xb = __ldg(src.rx + j);
          r.yb = __ldg(src.ry + j);
          r.zb = __ldg(src.rz + j);
          r.hb = __ldg(src.pf + j);
          r.lb = T::GatherMirrors ? __ldg(src.pflo + j) : make_float4(0.f, 0.f, 0.f, 0.f);
          f.entry(acc, c, r);
        } else {
          const uint32_t code = e & 31u;
          double xb = __ldg(src.rx + j), yb = __ldg(src.ry + j), zb = __ldg(src.rz + j);
          if (code != kImageCenter) {
            xb = image_coord(xb, c.period[0], static_cast<int>(code % 3u));
            yb = image_coord(yb, c.period[1], static_cast<int>((code / 3u) % 3u));
            zb = image_coord(zb, c.period[2], static_cast<int>(code / 9u));
          }
          PairData p;
          p.dx = __dsub_rn(xb, c.x);
          p.dy = __dsub_rn(yb, c.y);
          p.dz = __dsub_rn(zb, c.z);
          p.d2 = norm2_rn(p.dx, p.dy, p.dz);
          if (p.d2 > 0.0 && p.d2 <= rc2) {
            p.j = j;
            p.code = code;
            f.pair(acc, c, p);
          }
        }
      }
    }
  }
  // fixed-order tree over the group: lane sub takes lane sub + off's partial
  constexpr int kWords = static_cast<int>(sizeof(typename F::Acc) / 4);
#pragma unroll
  for (int off = LANES / 2; off > 0; off >>= 1) {
    typename F::Acc other;
    uint32_t* ow = reinterpret_cast<uint32_t*>(&other);
    const uint32_t* aw = reinterpret_cast<const uint32_t*>(&acc);
#pragma unroll
    for (int w = 0; w < kWords; ++w) ow[w] = __shfl_down_sync(0xffffffffu, aw[w], off, LANES);
    if (ok && sub < static_cast<uint32_t>(off)) f.combine(acc, other);
  }
  if (ok && sub == 0) f.stop(acc, c);
}

// ---------------------------------------------------------------------------
// One system seen through its public view (xnb_system_pair_view).
struct ViewSource {
  const double* __restrict__ rx;
  const double* __restrict__ ry;
  const double* __restrict__ rz;
  const float4* __restrict__ pf;
  const float4* __restrict__ pflo;
  const uint32_t* __restrict__ nbr;
  const uint32_t* __restrict__ nbr_start;
  const uint32_t* __restrict__ nbr_count;
  const uint32_t* __restrict__ nbr_half;
  uint32_t n_particles;
  double period[3];
  float period_f[3];

  __host__ explicit ViewSource(const xnb_pair_view& v)
      : rx(v.rx), ry(v.ry), rz(v.rz), pf(static_cast<const float4*>(v.mirror)),
        pflo(static_cast<const float4*>(v.mirror_lo)), nbr(v.nbr), nbr_start(v.nbr_start), nbr_count(v.nbr_count),
        nbr_half(v.nbr_half), n_particles(static_cast<uint32_t>(v.n_particles)) {
    for (int a = 0; a < 3; ++a) {
      period[a] = v.period[a];
      period_f[a] = static_cast<float>(v.period[a]);
    }
  }

  __device__ __forceinline__ bool begin(uint32_t i, bool symmetric, bool want_lo, ParticleContext& c) const {
    c.i = i;
    c.sys = 0;
    c.pbase = 0;
    c.x = rx[i];
    c.y = ry[i];
    c.z = rz[i];
    c.hi = pf[i];
    c.lo = want_lo ? pflo[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int a = 0; a < 3; ++a) {
      c.period[a] = period[a];
      c.period_f[a] = period_f[a];
    }
    c.list = nbr + nbr_start[i];
    c.n = symmetric ? nbr_half[i] : nbr_count[i];
    return true;
  }
};

template <class F>
__global__ void __launch_bounds__(128) traverse_view_kernel(ViewSource src, F f) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < src.n_particles; i += gridDim.x * blockDim.x)
    traverse_particle(src, i, f);
}

// Runs functor f over every particle of the viewed system on `stream` (one
// thread per particle, `threads` per block, a multiple of 32 up to 128).
// Returns the launch status; the lists must be current (xnb_chunk_neighbors or
// a step since the last position change).
template <class F>
inline cudaError_t traverse_pairs(const xnb_pair_view& v, const F& f, cudaStream_t stream, int threads = 128) {
  if (v.n_particles <= 0) return cudaSuccess;
  if (threads <= 0 || threads > 128 || threads % 32) return cudaErrorInvalidValue;
  const long long blocks = (v.n_particles + threads - 1) / threads;
  traverse_view_kernel<F><<<static_cast<unsigned>(blocks), threads, 0, stream>>>(ViewSource(v), f);
  return cudaGetLastError();
}

// The FP32 prefilter threshold for a functor cutoff rcut on this view
// (rcut must not exceed the lists' nbh_dist).
inline float prefilter_bound(const xnb_pair_view& v, double rcut) {
  return prefilter_bound(v.max_period, v.nbh_dist, rcut);
}

}  // namespace pair
}  // namespace xnb

#endif  // XNB_PAIR_CUH
