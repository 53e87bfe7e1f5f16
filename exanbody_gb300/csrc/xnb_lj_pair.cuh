// Pieces of the Lennard-Jones pair body shared by the force traversals
// (xnb_step_kernels.cu: one thread per particle over global memory;
// xnb_force_staged.cu: cell segments staged in shared memory).
#pragma once

#include "xnb_launch.cuh"
#include "xnb_traverse.cuh"

namespace xnb {

// ---------------------------------------------------------------------------
// Double-precision reciprocal of d > 0 from an FP32 seed refined by two
// Newton-Raphson steps y <- y + y*(1 - d*y) in FP64, not correctly rounded.
// The seed stays off the FP64 pipe: d is truncated to binary32 by moving its
// exponent (re-biased by -896) and the top 23 fraction bits with one funnel
// shift, the exponent field clamped to [1, 252] so that the FP32 reciprocal is
// a positive normal, which widens back by the inverse bit move. For d in
// [2^-126, 2^126) the seed (truncation, then the hardware FP32 reciprocal,
// within 1 ulp) is within 2^-22 of 1/d, and the two steps take the error to
// 2^-44, then below the FP64 rounding.
__device__ __forceinline__ double rcp_nr(double d) {
  const int hi = min(max(__double2hiint(d) - 0x38000000, 0x00100000), 0x0fcfffff);
  const float s = __uint_as_float(__funnelshift_l(static_cast<uint32_t>(__double2loint(d)), static_cast<uint32_t>(hi), 3));
  float rf;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(s));
  const uint32_t r = __float_as_uint(rf);
  double y = __hiloint2double(static_cast<int>((r >> 3) + 0x38000000u), static_cast<int>(r << 29));
  double e = fma(-d, y, 1.0);
  y = fma(y, e, y);
  e = fma(-d, y, 1.0);
  return fma(y, e, y);
}

// One marked entry of the mixed path: r^2 in FP32 (the compensated mirror
// difference for an entry in the same periodic image: hi difference plus the
// difference of the residuals packed in .w; the FP64 displacement converted for
// an image entry), the cutoff decided in FP32 outside the proven band and in
// FP64 inside it, then the FP32 force factor pd and the FP64 accumulation of
// pd * r_b and pd.
// PACKED = false (batches holding a system of X >= 1024 sigma, whose packed
// residuals are too coarse) takes the gathered residual mirrors lb and pal.
template <bool PE, bool PACKED>
__device__ __forceinline__ void mixed_pair(const SysDesc& S, uint32_t e, double xb, double yb, double zb, float4 hb,
                                           float4 lb, double xa, double ya, double za, float4 paf, float4 pal,
                                           double rcut2, double& fx, double& fy, double& fz, double& psum,
                                           double& pe) {
  const uint32_t code = e & 31u;
  float dxf, dyf, dzf;
  if (code == static_cast<uint32_t>(kImageCenter)) {
    if constexpr (PACKED) {
      // within 2u|d| + 2 lo_step of the FP64 displacement (u = 2^-24), without FP64 work
      const uint32_t wb = __float_as_uint(hb.w), wa = __float_as_uint(paf.w);
      const float q = S.lo_step_f;
      dxf = fmaf(small_int_f(lo_field(wb, 0) - lo_field(wa, 0)), q, hb.x - paf.x);
      dyf = fmaf(small_int_f(lo_field(wb, 1) - lo_field(wa, 1)), q, hb.y - paf.y);
      dzf = fmaf(small_int_f(lo_field(wb, 2) - lo_field(wa, 2)), q, hb.z - paf.z);
    } else {
      // within 2u|d| of the FP64 displacement
      dxf = (hb.x - paf.x) + (lb.x - pal.x);
      dyf = (hb.y - paf.y) + (lb.y - pal.y);
      dzf = (hb.z - paf.z) + (lb.z - pal.z);
    }
  } else {
    xb = image_coord(xb, S.period[0], static_cast<int>(code % 3u));
    yb = image_coord(yb, S.period[1], static_cast<int>((code / 3u) % 3u));
    zb = image_coord(zb, S.period[2], static_cast<int>(code / 9u));
    dxf = narrow_f64(__dsub_rn(xb, xa));
    dyf = narrow_f64(__dsub_rn(yb, ya));
    dzf = narrow_f64(__dsub_rn(zb, za));
  }
  const float r2 = fmaf(dxf, dxf, fmaf(dyf, dyf, dzf * dzf));
  bool in;
  if (r2 > S.rc2_f + S.rc_margin_f) {
    in = false;
  } else if (r2 < S.rc2_f - S.rc_margin_f && r2 > S.rc_margin_f) {
    in = true;
  } else {
    const double d2 = norm2_rn(__dsub_rn(xb, xa), __dsub_rn(yb, ya), __dsub_rn(zb, za));
    in = (d2 > 0.0 && d2 <= rcut2);
  }
  if (in) {
    // FP64 displacement folded into the FP64 accumulation:
    //   sum_b pd_b (r_b - r_a) = sum_b pd_b r_b - r_a sum_b pd_b,
    // so a pair costs 3 DFMA + 1 DADD instead of 3 DADD + 3 DFMA; the
    // subtraction happens once per particle (cancellation error
    // <= ~u_64 |r| sum|pd|, about 1e-12 of |F| at box sizes of 10^3 sigma).
    // The hardware reciprocal (within 1 ulp) is part of the FP32 force magnitude.
    float ir2;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(ir2) : "f"(r2));
    const float s2 = S.sig2_f * ir2;
    const float s6 = s2 * s2 * s2;
    const float pd = S.eps24_f * s6 * fmaf(-2.0f, s6, 1.0f) * ir2;
    const double pdd = widen_f32_fast(pd);  // exact, on the integer pipes
    fx = fma(pdd, xb, fx);
    fy = fma(pdd, yb, fy);
    fz = fma(pdd, zb, fz);
    psum += pdd;
    if (PE) pe += static_cast<double>(0.5f * fmaf(S.eps4_f * s6, s6 - 1.0f, -S.e_shift_f));
  }
}

// ---------------------------------------------------------------------------
// zero_particle_force + lennard_jones_force over the neighbour lists, as a
// functor of the pair-functor API (include/xnb_pair.cuh) run through the batch
// traversal. compute_cell_particle_pairs_cell (compute/include/exanb/compute/
// compute_cell_particle_pairs_impl_default.h:148-238) walks each particle's
// stream in (cell_enc, p_b) order with dr = r_b - r_a and keeps 0 < d2 <= rc^2;
// LennardJonesForceFunctor (contribs/md/lennard_jones/lennard_jones.cu:67-102)
// sums pair_de*dr sequentially and adds the sum onto the zeroed force.
// One thread per particle, full lists: no atomics, fixed summation order.
//   P = kFp64Exact : the functor's own operations and roundings (sqrt, 1/r,
//                    no contraction): bit-identical to the CPU restatement.
//   P = kFp64      : same selection of pairs (exact d2 test), force from
//                    1/d2 by Newton-Raphson, FMA accumulation.
//   P = kMixed     : raw entries (the functor forms the displacement): FP64
//                    displacement and FP64 accumulation; r^2, r^-6 and the
//                    force magnitude in FP32; the cutoff decision is made in
//                    FP32 where a proven margin allows and in FP64 otherwise, so
//                    the pair set is the FP64 one. The displacement is applied
//                    once per particle (sum pd*r_b - r_a*sum pd, all in FP64)
//                    and the FP32 factor is widened on the integer pipes: a
//                    pair costs 3 DFMA + 1 DADD on the FP64 pipe.
template <int P, bool PE, bool KICK, bool PACKED = true>
struct LJForce {
  const SysDesc* __restrict__ sys;
  DevArrays a;
  struct Acc {
    double fx, fy, fz, pe, psum;
  };

  __device__ __forceinline__ double rcut2(const pair::ParticleContext& c) const { return sys[c.sys].rcut2; }
  __device__ __forceinline__ float prefilter_hi(const pair::ParticleContext& c) const {
    const SysDesc& S = sys[c.sys];
    return S.rc2_f + S.pre_margin_f;
  }
  __device__ __forceinline__ bool start(Acc& q, const pair::ParticleContext&) const {
    q.fx = q.fy = q.fz = q.pe = q.psum = 0.0;
    return true;
  }
  __device__ __forceinline__ void pair(Acc& q, const pair::ParticleContext& c, const pair::PairData& p) const {
    const SysDesc& S = sys[c.sys];
    if (P == kFp64Exact) {
      // lj_compute_energy (lennard_jones.cu:46-56) then pair_de *= w / r with w = 1
      const double r = __dsqrt_rn(p.d2);
      const double inv_r = __ddiv_rn(1.0, r);
      const double ratio = __dmul_rn(S.sigma, inv_r);
      const double ratio2 = __dmul_rn(ratio, ratio);
      const double ratio6 = __dmul_rn(__dmul_rn(ratio2, ratio2), ratio2);
      const double ratio12 = __dmul_rn(ratio6, ratio6);
      double de = __dmul_rn(__dmul_rn(S.m24eps, __dsub_rn(__dmul_rn(2.0, ratio12), ratio6)), inv_r);
      de = __dmul_rn(de, inv_r);
      q.fx = __dadd_rn(q.fx, __dmul_rn(de, p.dx));
      q.fy = __dadd_rn(q.fy, __dmul_rn(de, p.dy));
      q.fz = __dadd_rn(q.fz, __dmul_rn(de, p.dz));
      if (PE) {
        const double en = __dmul_rn(S.eps4, __dsub_rn(ratio12, ratio6));
        q.pe = __dadd_rn(q.pe, __dmul_rn(0.5, __dsub_rn(en, S.e_shift)));
      }
    } else {
      const double ir2 = rcp_nr(p.d2);
      const double s2 = S.sig2 * ir2;
      const double s6 = s2 * s2 * s2;
      const double pd = S.eps24 * s6 * fma(-2.0, s6, 1.0) * ir2;
      q.fx = fma(pd, p.dx, q.fx);
      q.fy = fma(pd, p.dy, q.fy);
      q.fz = fma(pd, p.dz, q.fz);
      if (PE) q.pe += 0.5 * fma(S.eps4 * s6, s6 - 1.0, -S.e_shift);
    }
  }
  __device__ __forceinline__ void entry(Acc& q, const pair::ParticleContext& c, const pair::RawEntry& r) const {
    const SysDesc& S = sys[c.sys];
    mixed_pair<PE, PACKED>(S, r.e, r.xb, r.yb, r.zb, r.hb, r.lb, c.x, c.y, c.z, c.hi, c.lo, S.rcut2, q.fx, q.fy,
                           q.fz, q.psum, q.pe);
  }
  __device__ __forceinline__ void combine(Acc& q, const Acc& o) const {
    q.fx += o.fx;
    q.fy += o.fy;
    q.fz += o.fz;
    q.pe += o.pe;
    q.psum += o.psum;
  }
  __device__ __forceinline__ void stop(Acc& q, const pair::ParticleContext& c) const {
    const SysDesc& S = sys[c.sys];
    const uint32_t i = c.i;
    double fx = q.fx, fy = q.fy, fz = q.fz;
    if (P == kMixed) {
      fx = fma(-c.x, q.psum, fx);
      fy = fma(-c.y, q.psum, fy);
      fz = fma(-c.z, q.psum, fz);
    }
    // the force field was zeroed (zero_particle_force.cu:39-46) and receives the
    // sum; 0 + s differs from s only for s = -0, which the exact path keeps
    if (P == kFp64Exact) {
      fx = __dadd_rn(0.0, fx);
      fy = __dadd_rn(0.0, fy);
      fz = __dadd_rn(0.0, fz);
    }
    if (S.divide_by_mass) {
      // divide_force_by_type_scalar (compute/vec3_typescalar_op.cu:156, math_functors.h:140)
      fx = __ddiv_rn(fx, S.mass);
      fy = __ddiv_rn(fy, S.mass);
      fz = __ddiv_rn(fz, S.mass);
    }
    a.fx[i] = fx;
    a.fy[i] = fy;
    a.fz[i] = fz;
    if (PE) a.pe[i] = q.pe;
    if (KICK) {
      // verlet_second_half: push_f_v with dt_scale 0.5 (numerical-scheme.msp:17-18)
      const double h = S.dt_half;
      if (P == kFp64Exact) {
        a.vx[i] = __dadd_rn(a.vx[i], __dmul_rn(fx, h));
        a.vy[i] = __dadd_rn(a.vy[i], __dmul_rn(fy, h));
        a.vz[i] = __dadd_rn(a.vz[i], __dmul_rn(fz, h));
      } else {
        a.vx[i] = fma(fx, h, a.vx[i]);
        a.vy[i] = fma(fy, h, a.vy[i]);
        a.vz[i] = fma(fz, h, a.vz[i]);
      }
    }
  }
};

}  // namespace xnb

namespace xnb {
namespace pair {
// The mixed path takes raw entries (their residuals come packed with the hi
// mirror, so the residual mirrors are gathered only without packing), two per
// iteration (both entries' gathers in flight together; list order unchanged);
// the FP64 paths take the traversal's FP64 pairs within rc.
template <int P, bool PE, bool KICK, bool PACKED>
struct ComputePairTraits<LJForce<P, PE, KICK, PACKED>> : DefaultPairTraits {
  static constexpr bool RawEntries = (P == kMixed);
  static constexpr bool GatherMirrors = (P == kMixed && !PACKED);
  static constexpr int EntriesPerIteration = (P == kMixed) ? 2 : 1;
};
}  // namespace pair
}  // namespace xnb

