// The pair traversal of the public pair-functor API (include/xnb_pair.cuh) over
// a whole batch: every particle of every (selected) system, each with its
// system's list segment, periodic offsets and mirrors. The Lennard-Jones
// kernels (xnb_step_kernels.cu) and the other pair functors (xnb_functors.cu)
// are functors run through it.
#pragma once

#include "xnb_internal.cuh"

namespace xnb {

using pair::Marks;
using pair::next_mark;
using pair::prefilter_window;

// Particle source of pair::traverse_particle for a batch: skips free slots,
// systems not selected (sys_only >= 0) and systems whose lists failed.
struct BatchSource {
  const SysDesc* __restrict__ sys;
  const SysState* __restrict__ st;
  const double* __restrict__ rx;
  const double* __restrict__ ry;
  const double* __restrict__ rz;
  const float4* __restrict__ pf;
  const float4* __restrict__ pflo;
  const uint32_t* __restrict__ pcell;
  const uint32_t* __restrict__ cell_sys;
  const uint32_t* __restrict__ nbr;
  const uint32_t* __restrict__ nbr_start;
  const uint32_t* __restrict__ nbr_cnt;
  const uint32_t* __restrict__ nbr_half;
  int sys_only;

  __host__ __device__ BatchSource(const SysDesc* s_, const SysState* st_, const DevArrays& a, int sys_only_)
      : sys(s_), st(st_), rx(a.rx), ry(a.ry), rz(a.rz), pf(a.pf), pflo(a.pflo), pcell(a.pcell),
        cell_sys(a.cell_sys), nbr(a.nbr), nbr_start(a.nbr_start), nbr_cnt(a.nbr_cnt), nbr_half(a.nbr_half),
        sys_only(sys_only_) {}

  __device__ __forceinline__ bool begin(uint32_t i, bool symmetric, bool want_lo, pair::ParticleContext& c) const {
    const uint32_t cl = pcell[i];
    if (cl == 0xFFFFFFFFu) return false;
    const uint32_t s = cell_sys[cl];
    if (sys_only >= 0 && s != static_cast<uint32_t>(sys_only)) return false;
    if (st[s].error) return false;  // lists of a failed system are not trusted
    const SysDesc& S = sys[s];
    c.i = i;
    c.sys = s;
    c.pbase = S.part_base;
    c.x = rx[i];
    c.y = ry[i];
    c.z = rz[i];
    c.hi = pf[i];
    c.lo = want_lo ? pflo[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int ax = 0; ax < 3; ++ax) {
      c.period[ax] = S.period[ax];
      c.period_f[ax] = S.period_f[ax];
    }
    c.list = nbr + S.list_base + nbr_start[i];
    c.n = symmetric ? nbr_half[i] : nbr_cnt[i];
    return true;
  }
};

}  // namespace xnb
