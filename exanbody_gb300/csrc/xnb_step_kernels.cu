// Per-step kernels: velocity-Verlet pushes with the displacement trigger, and the
// Lennard-Jones pair-force traversal over the neighbour lists.
#include <algorithm>

#include "xnb_launch.cuh"
#include "xnb_lj_pair.cuh"
#include "xnb_traverse.cuh"

namespace xnb {

namespace {

constexpr uint32_t kInvalid = 0xFFFFFFFFu;

// ---------------------------------------------------------------------------
// push_f_v_r + push_f_v + particle_displ_over, one pass over the particles.
//   push_f_v_r : PushVec3SecondOrderFunctor (defbox/include/exanb/defbox/push_vec3_2nd_order.h:33-38)
//                x += v*dt + f*dt2, dt = dt*scale, dt2 = dt*dt*0.5 (:87-88)
//   push_f_v   : PushVec3FirstOrderFunctor (push_vec3_1st_order.h:32-37), v += f*dt*scale
//   trigger    : ReduceMaxDisplacementFunctor (mpi/particle_displ_over.cu:49-66),
//                norm2(r - restore(backup)) >= max_displ^2, counted per system.
// EXACT=true keeps the reference's two roundings per product/sum (bit-identical
// trajectory); EXACT=false lets the compiler fuse them into FMAs.
// fired (or null): set to 1 when a particle of an armed system is over the
// displacement threshold (the persistent step loop stops there).
template <bool EXACT>
__device__ __forceinline__ void first_half_body(uint32_t n_part, int nsys, const SysDesc* __restrict__ sys,
                                                SysState* __restrict__ st, const DevArrays& a, bool push_r,
                                                bool push_v, bool trigger, double scale_r, double scale_v,
                                                int sys_only, unsigned int* fired) {
  const bool canonical = (scale_r == 1.0 && scale_v == 0.5);
  if (push_r && blockIdx.x == 0) {
    // positions change: lists and sub-cell keys no longer describe them exactly
    for (int s = static_cast<int>(threadIdx.x); s < nsys; s += static_cast<int>(blockDim.x))
      if (sys_only < 0 || s == sys_only) {
        st[s].lists_fresh = 0;
        st[s].keys_fresh = 0;
      }
  }
  // every lane of a warp runs the same number of iterations, so full-warp
  // collectives below see all 32 lanes
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n_part; base += stride) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t c = i < n_part ? a.pcell[i] : kInvalid;
    bool over = false;
    uint32_t s = kInvalid;
    if (c != kInvalid && (sys_only < 0 || a.cell_sys[c] == static_cast<uint32_t>(sys_only))) {
      s = a.cell_sys[c];
      const SysDesc& S = sys[s];
      double dt, dt2, dtv;
      if (canonical) {
        dt = S.dt_full;
        dt2 = S.dt_sq_half;
        dtv = S.dt_half;
      } else {
        dt = __dmul_rn(S.dt, scale_r);
        dt2 = __dmul_rn(__dmul_rn(dt, dt), 0.5);
        dtv = __dmul_rn(S.dt, scale_v);
      }
      double x = a.rx[i], y = a.ry[i], z = a.rz[i];
      double vx = a.vx[i], vy = a.vy[i], vz = a.vz[i];
      const double fx = a.fx[i], fy = a.fy[i], fz = a.fz[i];
      float4 cur_hi;  // FP32 mirror of the position the trigger sees
      if (push_r) {
        if (EXACT) {
          x = __dadd_rn(x, __dadd_rn(__dmul_rn(vx, dt), __dmul_rn(fx, dt2)));
          y = __dadd_rn(y, __dadd_rn(__dmul_rn(vy, dt), __dmul_rn(fy, dt2)));
          z = __dadd_rn(z, __dadd_rn(__dmul_rn(vz, dt), __dmul_rn(fz, dt2)));
        } else {
          // r + v dt + f dt^2/2 as two nested FMAs (two roundings, two FP64 instructions)
          x = fma(fx, dt2, fma(vx, dt, x));
          y = fma(fy, dt2, fma(vy, dt, y));
          z = fma(fz, dt2, fma(vz, dt, z));
        }
        a.rx[i] = x;
        a.ry[i] = y;
        a.rz[i] = z;
        float4 hi, lo;
        make_pf2(S, x, y, z, hi, lo);
        a.pf[i] = hi;
        a.pflo[i] = lo;
        cur_hi = hi;
      } else if (!EXACT && trigger) {
        cur_hi = a.pf[i];
      }
      if (push_v) {
        if (EXACT) {
          vx = __dadd_rn(vx, __dmul_rn(fx, dtv));
          vy = __dadd_rn(vy, __dmul_rn(fy, dtv));
          vz = __dadd_rn(vz, __dmul_rn(fz, dtv));
        } else {
          vx = fma(fx, dtv, vx);
          vy = fma(fy, dtv, vy);
          vz = fma(fz, dtv, vz);
        }
        a.vx[i] = vx;
        a.vy[i] = vy;
        a.vz[i] = vz;
      }
      if (trigger && st[s].rebuild_armed) {
        // FP32 pre-decision from the mirrors, FP64 inside the proven band
        bool decided = false;
        if (!EXACT) {
          const float4 rb = a.rbf[i];
          const float ex = cur_hi.x - rb.x, ey = cur_hi.y - rb.y, ez = cur_hi.z - rb.z;
          const float d2f = fmaf(ez, ez, fmaf(ey, ey, ex * ex));
          if (d2f > S.trig_hi_f) {
            over = true;
            decided = true;
          } else if (d2f < S.trig_lo_f) {
            decided = true;
          }
        }
        if (!decided) {
          const double dx = __dsub_rn(x, a.rbx[i]);
          const double dy = __dsub_rn(y, a.rby[i]);
          const double dz = __dsub_rn(z, a.rbz[i]);
          const double d2 = EXACT ? norm2_rn(dx, dy, dz) : fma(dz, dz, fma(dy, dy, dx * dx));
          over = d2 >= S.max_displ2;
        }
      }
    }
    if (trigger) {
      // warp-aggregated count per system
      const unsigned same = __match_any_sync(0xffffffffu, s);
      const unsigned hits = __ballot_sync(0xffffffffu, over) & same;
      const int leader = __ffs(same) - 1;
      if (s != kInvalid && static_cast<int>(threadIdx.x & 31) == leader && hits) {
        atomicAdd(&st[s].moved, static_cast<unsigned long long>(__popc(hits)));
        if (fired) atomicOr(fired, 1u);
      }
    }
  }
}

template <bool EXACT>
__global__ void __launch_bounds__(256)
    k_first_half(uint32_t n_part, int nsys, const SysDesc* __restrict__ sys, SysState* __restrict__ st, DevArrays a,
                 bool push_r, bool push_v, bool trigger, double scale_r, double scale_v, int sys_only) {
  first_half_body<EXACT>(n_part, nsys, sys, st, a, push_r, push_v, trigger, scale_r, scale_v, sys_only, nullptr);
}

// 72 registers: 7 blocks of 128 threads per SM (measured faster than the
// unconstrained 79 despite a few spilled bytes).
template <int P, bool PE, bool KICK, bool PACKED = true>
__global__ void __maxnreg__(72) k_force(uint32_t n_part, BatchSource src, LJForce<P, PE, KICK, PACKED> f) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_part; i += gridDim.x * blockDim.x)
    pair::traverse_particle(src, i, f);
}

// LANES threads per particle (FP64 and mixed): each takes every LANES-th
// 8-entry block of the particle's list and the partial sums are combined in a
// fixed order, so the result is reproducible (it agrees with the one-lane
// traversal to rounding). The whole warp iterates together: the shuffles of
// the combination span it.
template <int P, bool PE, bool KICK, int LANES>
__global__ void __maxnreg__(72) k_force_lanes(uint32_t n_part, BatchSource src, LJForce<P, PE, KICK> f) {
  const uint64_t total = static_cast<uint64_t>(n_part) * LANES;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t base = static_cast<uint64_t>(blockIdx.x) * blockDim.x; base < total; base += stride) {
    const uint64_t t = base + threadIdx.x;
    pair::traverse_particle_lanes<LANES>(src, static_cast<uint32_t>(t / LANES), t < total, f);
  }
}

// ---------------------------------------------------------------------------
// Newton-third-law form of the same traversal for the FP64 and mixed paths:
// particle a walks only the lower half of its sorted list ((cell_b, p_b) <
// (cell_a, p_a), the reference's symmetric split, compute_cell_particle_pairs_
// impl_default.h:181), keeps f_a in registers and hands -f_pair to b with an FP64
// reduction in L2. Each pair inside rc is evaluated once. The order in which
// reactions arrive varies from run to run, so results agree to rounding, not
// bit for bit; FP64_EXACT always uses the full-list kernel above.
// FAR: instantiated only when a system of the batch lies far from the
// coordinate origin (Extent::far_coords), so the common kernel carries no
// partner-side evaluation.
template <int P, bool PE, bool FAR = false>
__global__ void __launch_bounds__(256)
    k_force_half(uint32_t n_part, const SysDesc* __restrict__ sys, const SysState* __restrict__ st, DevArrays a,
                 int sys_only) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_part; i += gridDim.x * blockDim.x) {
    const uint32_t c = a.pcell[i];
    if (c == kInvalid) continue;
    const uint32_t s = a.cell_sys[c];
    if (sys_only >= 0 && s != static_cast<uint32_t>(sys_only)) continue;
    if (st[s].error) continue;
    const SysDesc& S = sys[s];
    const double xa = a.rx[i], ya = a.ry[i], za = a.rz[i];
    const uint32_t* __restrict__ L = a.nbr + S.list_base + a.nbr_start[i];
    const uint32_t n = a.nbr_half[i];
    const uint32_t pbase = S.part_base;
    const double px = S.period[0], py = S.period[1], pz = S.period[2];
    const double rcut2 = S.rcut2;
    const float4 paf = a.pf[i];
    const float pre_hi = S.rc2_f + S.pre_margin_f;
    const float pfx = S.period_f[0], pfy = S.period_f[1], pfz = S.period_f[2];
    double fx = 0.0, fy = 0.0, fz = 0.0, pe = 0.0;
    uint32_t k = 0;
    for (;;) {
      uint32_t j = 0, code = 0;
      bool found = false;
      while (k < n) {
        const uint32_t e = __ldg(L + k);
        ++k;
        j = pbase + (e >> 5);
        code = e & 31u;
        const float4 pbf = __ldg(a.pf + j);
        float bx = pbf.x, by = pbf.y, bz = pbf.z;
        if (code != static_cast<uint32_t>(kImageCenter)) {
          bx = image_coord_f(bx, pfx, static_cast<int>(code % 3u));
          by = image_coord_f(by, pfy, static_cast<int>((code / 3u) % 3u));
          bz = image_coord_f(bz, pfz, static_cast<int>(code / 9u));
        }
        const float ex = bx - paf.x, ey = by - paf.y, ez = bz - paf.z;
        if (fmaf(ex, ex, fmaf(ey, ey, ez * ez)) <= pre_hi) {
          found = true;
          break;
        }
      }
      if (!found) break;
      const double xbr = __ldg(a.rx + j), ybr = __ldg(a.ry + j), zbr = __ldg(a.rz + j);
      double xb = xbr, yb = ybr, zb = zbr;
      if (code != static_cast<uint32_t>(kImageCenter)) {
        xb = image_coord(xb, px, static_cast<int>(code % 3u));
        yb = image_coord(yb, py, static_cast<int>((code / 3u) % 3u));
        zb = image_coord(zb, pz, static_cast<int>(code / 9u));
      }
      if (FAR && P == kFp64 && code != static_cast<uint32_t>(kImageCenter) && S.far_coords) {
        // Far from the coordinate origin (coordinates beyond 4 periods) the
        // partner's reaction through a periodic image is evaluated as the
        // partner's own full-list traversal would: b sees a through the
        // opposite image (digits 2 - d) and rounds its own image coordinate
        // x_a +- period, whose rounding there exceeds the displacements'
        // resolution and differs from that of x_b -+ period. Each side keeps
        // its own cutoff decision. (A per-system flag: the branch is uniform,
        // and domains near the origin keep the single evaluation.)
        const double xai = image_coord(xa, px, 2 - static_cast<int>(code % 3u));
        const double yai = image_coord(ya, py, 2 - static_cast<int>((code / 3u) % 3u));
        const double zai = image_coord(za, pz, 2 - static_cast<int>(code / 9u));
        const double dxa = __dsub_rn(xb, xa), dya = __dsub_rn(yb, ya), dza = __dsub_rn(zb, za);
        const double dxb = __dsub_rn(xai, xbr), dyb = __dsub_rn(yai, ybr), dzb = __dsub_rn(zai, zbr);
        const double d2a = norm2_rn(dxa, dya, dza);
        const double d2b = norm2_rn(dxb, dyb, dzb);
        if (d2a > 0.0 && d2a <= rcut2) {
          const double ir2 = rcp_nr(d2a);
          const double s2 = S.sig2 * ir2;
          const double s6 = s2 * s2 * s2;
          const double pd = S.eps24 * s6 * fma(-2.0, s6, 1.0) * ir2;
          fx += pd * dxa;
          fy += pd * dya;
          fz += pd * dza;
          if (PE) pe += 0.5 * fma(S.eps4 * s6, s6 - 1.0, -S.e_shift);
        }
        if (d2b > 0.0 && d2b <= rcut2) {
          const double ir2 = rcp_nr(d2b);
          const double s2 = S.sig2 * ir2;
          const double s6 = s2 * s2 * s2;
          const double pd = S.eps24 * s6 * fma(-2.0, s6, 1.0) * ir2;
          atomicAdd(a.fx + j, pd * dxb);
          atomicAdd(a.fy + j, pd * dyb);
          atomicAdd(a.fz + j, pd * dzb);
          if (PE) atomicAdd(a.pe + j, 0.5 * fma(S.eps4 * s6, s6 - 1.0, -S.e_shift));
        }
        continue;
      }
      bool in;
      double pd = 0.0, en = 0.0;
      if (P == kFp64) {
        const double d2 = norm2_rn(__dsub_rn(xb, xa), __dsub_rn(yb, ya), __dsub_rn(zb, za));
        in = d2 > 0.0 && d2 <= rcut2;
        if (in) {
          const double ir2 = rcp_nr(d2);
          const double s2 = S.sig2 * ir2;
          const double s6 = s2 * s2 * s2;
          pd = S.eps24 * s6 * fma(-2.0, s6, 1.0) * ir2;
          if (PE) en = fma(S.eps4 * s6, s6 - 1.0, -S.e_shift);
        }
      } else {
        float dxf, dyf, dzf;
        if (code == static_cast<uint32_t>(kImageCenter)) {
          const float4 hb = __ldg(a.pf + j);
          if (S.packed_lo) {
            const uint32_t wb = __float_as_uint(hb.w), wa = __float_as_uint(paf.w);
            dxf = fmaf(small_int_f(lo_field(wb, 0) - lo_field(wa, 0)), S.lo_step_f, hb.x - paf.x);
            dyf = fmaf(small_int_f(lo_field(wb, 1) - lo_field(wa, 1)), S.lo_step_f, hb.y - paf.y);
            dzf = fmaf(small_int_f(lo_field(wb, 2) - lo_field(wa, 2)), S.lo_step_f, hb.z - paf.z);
          } else {
            const float4 lb = __ldg(a.pflo + j), pal = a.pflo[i];
            dxf = (hb.x - paf.x) + (lb.x - pal.x);
            dyf = (hb.y - paf.y) + (lb.y - pal.y);
            dzf = (hb.z - paf.z) + (lb.z - pal.z);
          }
        } else {
          dxf = narrow_f64(__dsub_rn(xb, xa));
          dyf = narrow_f64(__dsub_rn(yb, ya));
          dzf = narrow_f64(__dsub_rn(zb, za));
        }
        const float r2 = fmaf(dxf, dxf, fmaf(dyf, dyf, dzf * dzf));
        if (r2 > S.rc2_f + S.rc_margin_f) {
          in = false;
        } else if (r2 < S.rc2_f - S.rc_margin_f && r2 > S.rc_margin_f) {
          in = true;
        } else {
          const double d2 = norm2_rn(__dsub_rn(xb, xa), __dsub_rn(yb, ya), __dsub_rn(zb, za));
          in = (d2 > 0.0 && d2 <= rcut2);
        }
        if (in) {
          float ir2;
          asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(ir2) : "f"(r2));
          const float s2 = S.sig2_f * ir2;
          const float s6 = s2 * s2 * s2;
          pd = widen_f32_fast(S.eps24_f * s6 * fmaf(-2.0f, s6, 1.0f) * ir2);
          if (PE) en = static_cast<double>(fmaf(S.eps4_f * s6, s6 - 1.0f, -S.e_shift_f));
        }
      }
      if (in) {
        // FP64 displacement and FP64 pair force; a keeps +f, b receives -f
        const double gx = pd * __dsub_rn(xb, xa);
        const double gy = pd * __dsub_rn(yb, ya);
        const double gz = pd * __dsub_rn(zb, za);
        fx += gx;
        fy += gy;
        fz += gz;
        atomicAdd(a.fx + j, -gx);
        atomicAdd(a.fy + j, -gy);
        atomicAdd(a.fz + j, -gz);
        if (PE) {
          pe += 0.5 * en;
          atomicAdd(a.pe + j, 0.5 * en);
        }
      }
    }
    atomicAdd(a.fx + i, fx);
    atomicAdd(a.fy + i, fy);
    atomicAdd(a.fz + i, fz);
    if (PE) atomicAdd(a.pe + i, pe);
  }
}

// Clears f (and pe) of the selected systems before the reactions arrive.
__global__ void __launch_bounds__(256)
    k_zero_force(uint32_t n_part, const SysState* __restrict__ st, DevArrays a, int sys_only, bool with_pe) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_part; i += gridDim.x * blockDim.x) {
    const uint32_t c = a.pcell[i];
    if (c == kInvalid) continue;
    const uint32_t s = a.cell_sys[c];
    if (sys_only >= 0 && s != static_cast<uint32_t>(sys_only)) continue;
    if (st[s].error) continue;
    a.fx[i] = 0.0;
    a.fy[i] = 0.0;
    a.fz[i] = 0.0;
    if (with_pe) a.pe[i] = 0.0;
  }
}

// After the half-list traversal: divide_force_by_type_scalar and the second-half kick.
__global__ void __launch_bounds__(256)
    k_force_finish(uint32_t n_part, const SysDesc* __restrict__ sys, const SysState* __restrict__ st, DevArrays a,
                   int sys_only, bool kick) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_part; i += gridDim.x * blockDim.x) {
    const uint32_t c = a.pcell[i];
    if (c == kInvalid) continue;
    const uint32_t s = a.cell_sys[c];
    if (sys_only >= 0 && s != static_cast<uint32_t>(sys_only)) continue;
    if (st[s].error) continue;
    const SysDesc& S = sys[s];
    double fx = a.fx[i], fy = a.fy[i], fz = a.fz[i];
    if (S.divide_by_mass) {
      fx = __ddiv_rn(fx, S.mass);
      fy = __ddiv_rn(fy, S.mass);
      fz = __ddiv_rn(fz, S.mass);
      a.fx[i] = fx;
      a.fy[i] = fy;
      a.fz[i] = fz;
    }
    if (kick) {
      const double h = S.dt_half;
      a.vx[i] = fma(fx, h, a.vx[i]);
      a.vy[i] = fma(fy, h, a.vy[i]);
      a.vz[i] = fma(fz, h, a.vz[i]);
    }
  }
}

__global__ void k_mark_rebuild(int nsys, SysState* st, int mode, int sys_only, unsigned int* any) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  if (sys_only >= 0 && s != sys_only) {
    st[s].rebuild = 0;
    return;
  }
  // mode 0: every system (init); mode 1: systems whose trigger fired; mode 2: none
  const uint32_t r = mode == 0 ? 1u : (mode == 1 ? (st[s].moved > 0 ? 1u : 0u) : 0u);
  st[s].rebuild = r;
  if (r) {
    st[s].rebuilds += 1;
    atomicAdd(any, 1u);
  }
}

__global__ void k_clear_moved(int nsys, SysState* st) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) st[s].moved = 0;
}

// One thread per particle: the block scheduler balances the uneven per-particle
// work and the last partial wave is one short block, not a third of the grid.
inline int grid_for(uint32_t n, int threads) {
  const long long g = (static_cast<long long>(n) + threads - 1) / threads;
  return static_cast<int>(g < 1 ? 1 : g);
}

// Grid-stride launch of at most per_sm blocks per SM. The Newton traversal keeps
// it: threads running together then hold particles far apart, so their FP64
// reactions rarely meet on one address (one particle per thread made them
// collide and cost ~25% on GB300).
inline int grid_capped(uint32_t n, int threads, int sm_count, int per_sm) {
  const long long want = (static_cast<long long>(n) + threads - 1) / threads;
  const long long cap = static_cast<long long>(sm_count) * per_sm;
  const long long g = want < cap ? want : cap;
  return static_cast<int>(g < 1 ? 1 : g);
}

template <int P, bool PE, bool KICK>
void force_dispatch(const Extent& ex, const SysDesc* sys, const SysState* st, const DevArrays& a, int sys_only,
                    cudaStream_t stream) {
  const int threads = ex.force_block > 0 ? ex.force_block : 64;
  const BatchSource src(sys, st, a, sys_only);
  if constexpr (P == kMixed) {
    // a batch holding a box of X >= 1024 sigma: residual mirrors gathered, one thread per particle
    if (ex.unpacked) {
      const LJForce<P, PE, KICK, false> fu{sys, a};
      k_force<P, PE, KICK, false><<<grid_for(ex.n_part, threads), threads, 0, stream>>>(ex.n_part, src, fu);
      return;
    }
  }
  const LJForce<P, PE, KICK> f{sys, a};
  // the bit-exact path keeps one thread per particle (the reference's summation order)
  if constexpr (P != kFp64Exact) {
    if (ex.force_lanes == 2) {
      k_force_lanes<P, PE, KICK, 2><<<grid_for(ex.n_part * 2u, threads), threads, 0, stream>>>(ex.n_part, src, f);
      return;
    }
    if (ex.force_lanes == 4) {
      k_force_lanes<P, PE, KICK, 4><<<grid_for(ex.n_part * 4u, threads), threads, 0, stream>>>(ex.n_part, src, f);
      return;
    }
  }
  k_force<P, PE, KICK><<<grid_for(ex.n_part, threads), threads, 0, stream>>>(ex.n_part, src, f);
}


// ---------------------------------------------------------------------------
// Persistent step loop: one cooperative launch advances the batch step after
// step, with a grid barrier between the first half (push_f_v_r, push_f_v,
// trigger) and the forces, and another after the forces. Each phase runs the
// same per-particle code as k_first_half / k_force, so the states are bitwise
// those of xnb_step. The loop stops after the first half of a step whose
// trigger fired (the rebuild path and that step's forces then run as separate
// launches). The trigger flag alternates between two words by step parity:
// every block reads step k's word after the first barrier of step k, and block
// 0 clears the other word during step k's forces, after every block has read it
// at step k - 1 and before step k + 1 sets it.
__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Blocks count in; the last one resets the count and bumps the generation, the
// others poll the generation for at most wait_ns. A wait that runs out records
// the error and returns false (the loop then ends without another barrier).
__device__ bool grid_barrier(StepCtl* ctl, unsigned int nblocks, unsigned long long wait_ns) {
  __syncthreads();
  int ok = 1;
  if (threadIdx.x == 0) {
    const unsigned int gen = ld_acquire_u32(&ctl->generation);
    __threadfence();
    if (atomicAdd(&ctl->arrive, 1u) == nblocks - 1u) {
      atomicExch(&ctl->arrive, 0u);
      __threadfence();
      atomicAdd(&ctl->generation, 1u);
    } else {
      const unsigned long long t0 = global_ns();
      while (ld_acquire_u32(&ctl->generation) == gen) {
        if (global_ns() - t0 > wait_ns) {
          atomicOr(&ctl->error, 1u);
          ok = 0;
          break;
        }
        __nanosleep(100);
      }
    }
    __threadfence();
  }
  return __syncthreads_and(ok) != 0;
}

template <bool EXACT, int P, bool PE, bool PACKED = true>
__global__ void __maxnreg__(72)
    k_steps_persistent(uint32_t n_part, int nsys, const SysDesc* __restrict__ sys, SysState* __restrict__ st,
                       DevArrays a, BatchSource src, LJForce<P, PE, true, PACKED> f, StepCtl* ctl, int max_steps,
                       unsigned int nblocks, unsigned long long wait_ns, bool check) {
  if (check && !grid_barrier(ctl, nblocks + 1u, wait_ns)) return;
  for (int k = 0; k < max_steps; ++k) {
    first_half_body<EXACT>(n_part, nsys, sys, st, a, true, true, true, 1.0, 0.5, -1, &ctl->fired[k & 1]);
    if (!grid_barrier(ctl, nblocks, wait_ns)) return;
    if (ld_acquire_u32(&ctl->fired[k & 1])) {
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctl->steps_done = static_cast<unsigned int>(k);
        ctl->stopped = 1u;
      }
      return;
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_part; i += gridDim.x * blockDim.x)
      pair::traverse_particle(src, i, f);
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->fired[(k + 1) & 1] = 0u;
    if (!grid_barrier(ctl, nblocks, wait_ns)) return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->steps_done = static_cast<unsigned int>(max_steps);
    ctl->stopped = 0u;
  }
}

template <bool EXACT, int P, bool PE, bool PACKED = true>
int persistent_launch(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, StepCtl* ctl,
                      int max_steps, bool check, cudaStream_t stream) {
  auto kern = k_steps_persistent<EXACT, P, PE, PACKED>;
  constexpr int threads = 128;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, 0) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const long long want = (static_cast<long long>(ex.n_part) + threads - 1) / threads;
  const long long cap = static_cast<long long>(per_sm) * ex.sm_count;
  const unsigned int grid = static_cast<unsigned int>(std::max(1ll, std::min(want, cap)));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  // a barrier waits at most 4 s in a run (a phase of the largest batches lasts
  // milliseconds), 20 ms in the timeout check
  const unsigned long long wait_ns = check ? 20000000ull : 4000000000ull;
  LJForce<P, PE, true, PACKED> f{sys, a};
  cudaLaunchKernelEx(&cfg, kern, ex.n_part, ex.nsys, sys, st, a, BatchSource(sys, st, a, -1), f, ctl, max_steps,
                     grid, wait_ns, check);
  return 1;
}
}  // namespace

int launch_first_half(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, bool do_push_r,
                       bool do_push_v, bool do_trigger, double dt_scale_r, double dt_scale_v, bool exact,
                       int sys_only, cudaStream_t stream) {
  if (ex.n_part == 0) return 0;
  const int threads = 256;
  const int g = grid_for(ex.n_part, threads);
  if (exact)
    k_first_half<true><<<g, threads, 0, stream>>>(ex.n_part, ex.nsys, sys, st, a, do_push_r, do_push_v, do_trigger,
                                                  dt_scale_r, dt_scale_v, sys_only);
  else
    k_first_half<false><<<g, threads, 0, stream>>>(ex.n_part, ex.nsys, sys, st, a, do_push_r, do_push_v, do_trigger,
                                                   dt_scale_r, dt_scale_v, sys_only);
  return 1;
}

int launch_force(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, int precision, bool with_pe,
                  bool second_half, int sys_only, cudaStream_t stream, bool newton) {
  if (ex.n_part == 0) return 0;
  if (newton && precision != kFp64Exact) {
    const int threads = 256;
    const int g = grid_capped(ex.n_part, threads, ex.sm_count, 8);
    k_zero_force<<<g, threads, 0, stream>>>(ex.n_part, st, a, sys_only, with_pe);
    if (precision == kFp64) {
      if (ex.far_coords) {
        if (with_pe) k_force_half<kFp64, true, true><<<g, threads, 0, stream>>>(ex.n_part, sys, st, a, sys_only);
        else k_force_half<kFp64, false, true><<<g, threads, 0, stream>>>(ex.n_part, sys, st, a, sys_only);
      } else {
        if (with_pe) k_force_half<kFp64, true><<<g, threads, 0, stream>>>(ex.n_part, sys, st, a, sys_only);
        else k_force_half<kFp64, false><<<g, threads, 0, stream>>>(ex.n_part, sys, st, a, sys_only);
      }
    } else {
      if (with_pe) k_force_half<kMixed, true><<<g, threads, 0, stream>>>(ex.n_part, sys, st, a, sys_only);
      else k_force_half<kMixed, false><<<g, threads, 0, stream>>>(ex.n_part, sys, st, a, sys_only);
    }
    k_force_finish<<<g, threads, 0, stream>>>(ex.n_part, sys, st, a, sys_only, second_half);
    return 3;
  }
  if (precision == kMixed && ex.force_form == kForceStaged && a.nbr16 && a.seg && !ex.unpacked)
    return launch_force_staged(ex, sys, st, a, with_pe, second_half, sys_only, stream);
#define XNB_FORCE_CASE(PP)                                                           \
  if (precision == PP) {                                                             \
    if (with_pe && second_half) force_dispatch<PP, true, true>(ex, sys, st, a, sys_only, stream);   \
    else if (with_pe) force_dispatch<PP, true, false>(ex, sys, st, a, sys_only, stream);            \
    else if (second_half) force_dispatch<PP, false, true>(ex, sys, st, a, sys_only, stream);        \
    else force_dispatch<PP, false, false>(ex, sys, st, a, sys_only, stream);                        \
    return 1;                                                                        \
  }
  XNB_FORCE_CASE(kFp64Exact)
  XNB_FORCE_CASE(kFp64)
  XNB_FORCE_CASE(kMixed)
#undef XNB_FORCE_CASE
  return 0;
}

int launch_mark_rebuild(const Extent& ex, SysState* st, int mode, int sys_only, unsigned int* any,
                        cudaStream_t stream) {
  cudaMemsetAsync(any, 0, sizeof(unsigned int), stream);
  if (ex.nsys == 0) return 0;
  k_mark_rebuild<<<(ex.nsys + 127) / 128, 128, 0, stream>>>(ex.nsys, st, mode, sys_only, any);
  return 1;
}

int launch_clear_moved(const Extent& ex, SysState* st, cudaStream_t stream) {
  if (ex.nsys == 0) return 0;
  k_clear_moved<<<(ex.nsys + 127) / 128, 128, 0, stream>>>(ex.nsys, st);
  return 1;
}

int launch_steps_persistent(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, int precision,
                            bool with_pe, StepCtl* ctl, int max_steps, bool check, cudaStream_t stream) {
  if (ex.n_part == 0) return 0;
  if (precision == kFp64Exact)
    return with_pe ? persistent_launch<true, kFp64Exact, true>(ex, sys, st, a, ctl, max_steps, check, stream)
                   : persistent_launch<true, kFp64Exact, false>(ex, sys, st, a, ctl, max_steps, check, stream);
  if (precision == kFp64)
    return with_pe ? persistent_launch<false, kFp64, true>(ex, sys, st, a, ctl, max_steps, check, stream)
                   : persistent_launch<false, kFp64, false>(ex, sys, st, a, ctl, max_steps, check, stream);
  if (ex.unpacked)
    return with_pe ? persistent_launch<false, kMixed, true, false>(ex, sys, st, a, ctl, max_steps, check, stream)
                   : persistent_launch<false, kMixed, false, false>(ex, sys, st, a, ctl, max_steps, check, stream);
  return with_pe ? persistent_launch<false, kMixed, true>(ex, sys, st, a, ctl, max_steps, check, stream)
                 : persistent_launch<false, kMixed, false>(ex, sys, st, a, ctl, max_steps, check, stream);
}

}  // namespace xnb
