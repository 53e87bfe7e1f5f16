// snap_force_generic (contribs/md/snap/include/md/snap/snap_force.h:134-372,
// snap_force_op_coop.hxx:170-405): linear SNAP forces over the per-particle
// neighbour lists, one CTA of kSnapWarps warps per atom.
//
// For atom i (type ti) the environment is the list entries at squared distance
// in (1e-20, ((rad_ti + rad_tj) rcutfac)^2), in list order (snap_force_op_coop.hxx:
// 215-226). Then, in FP64:
//   U_tot = self term (1 on every diagonal) + sum_j wj sfac(r) U(r_ij), where U
//     is built level by level with the recursion of the Wigner U-functions in
//     the Cayley-Klein parameters of r_ij (snap_compute_ui.h:95-150). Only the
//     unique half of each level is computed (rows 2mb < j and the first half
//     of an even j's middle row); the rest follows from
//     U[j-mb][j-ma] = (-1)^(ma+mb) conj(U[mb][ma]). Each warp sums its
//     neighbours into its own partial, and the partials are added in warp order.
//   Y (unique half) = sum over the Z elements of beta_j Z (snap_compute_yi.h:
//     96-160), accumulated in shared memory; the per-atom energy
//     E_i = beta_0 + sum_k beta_k (B_k - bzero_k), B from the same Z elements
//     (snap_compute_bi.h:28-75).
//   For each neighbour j, U and dU/dr_ij are rebuilt level by level and
//     fij = 2 sum_unique w Re(conj(wj (dsfac U u + sfac dU)) Y) (w = 1/2 on an
//     even j's centre, snap_compute_deidrj.h:28-75); f_i += fij, f_j -= fij
//     (snap_force_op_coop.hxx:331-356), the reactions by FP64 atomics.
// Forces are scaled by the energy unit, divided by the mass when the system's
// force chain ends with divide_force_by_type_scalar. The order of the Y and
// reaction additions varies from run to run, so results agree to rounding.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "../../include/xnb_gpu.h"
#include "xnb_snap.cuh"

namespace xnb {

namespace {

constexpr uint32_t kInvalid = 0xFFFFFFFFu;

__host__ __device__ inline int nunique(int j) { return (j & 1) ? ((j + 1) / 2) * (j + 1) : (j / 2) * (j + 1) + j / 2 + 1; }

template <class R>
struct CX {
  R r, i;
};
using C2 = CX<double>;
template <class R>
__device__ __forceinline__ CX<R> cmulc(CX<R> a, CX<R> b) {  // conj(a) * b
  return CX<R>{fma(a.r, b.r, a.i * b.i), fma(a.r, b.i, -(a.i * b.r))};
}
template <class R>
__device__ __forceinline__ CX<R> cmul(CX<R> a, CX<R> b) {
  return CX<R>{fma(a.r, b.r, -(a.i * b.i)), fma(a.r, b.i, a.i * b.r)};
}

// element (r, c) of level L from its unique-half buffer (stride `st` values
// per element, complex at offset `off`)
template <class R>
__device__ __forceinline__ CX<R> level_get(const R* buf, int st, int off, int L, int r, int c) {
  const int idx = r * (L + 1) + c;
  if (idx < nunique(L)) return CX<R>{buf[idx * st + off], buf[idx * st + off + 1]};
  const int k = (L - r) * (L + 1) + (L - c);
  const R s = ((r + c) & 1) ? R(-1) : R(1);
  return CX<R>{s * buf[k * st + off], -s * buf[k * st + off + 1]};
}

// the potential's tables in the compute type
template <class R>
struct Tabs {
  const R *rootpq, *cg, *zbeta, *zener;
};
template <class R>
__device__ __forceinline__ Tabs<R> tabs(const SnapArgs& t);
template <>
__device__ __forceinline__ Tabs<double> tabs<double>(const SnapArgs& t) {
  return Tabs<double>{t.rootpq, t.cg, t.zbeta, t.zener};
}
template <>
__device__ __forceinline__ Tabs<float> tabs<float>(const SnapArgs& t) {
  return Tabs<float>{t.rootpq_f, t.cg_f, t.zbeta_f, t.zener_f};
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Cayley-Klein parameters of r_ij and their derivatives (snap_compute_duidrj.h:75-120).
struct Geo {
  C2 a, b, da[3], db[3];
  double u[3], sfac, dsfac;
};

__device__ __forceinline__ Geo geometry(double x, double y, double z, double rcut, const SnapArgs& t, bool deriv) {
  Geo g;
  const double rsq = fma(x, x, fma(y, y, z * z));
  const double r = sqrt(rsq);
  const double rscale0 = t.rfac0 * M_PI / (rcut - t.rmin0);
  const double theta0 = (r - t.rmin0) * rscale0;
  double sn, cs;
  sincos(theta0, &sn, &cs);
  const double z0 = r * cs / sn;
  const double r0inv = 1.0 / sqrt(fma(r, r, z0 * z0));
  g.a = C2{r0inv * z0, -r0inv * z};
  g.b = C2{r0inv * y, -r0inv * x};
  g.sfac = 1.0;
  g.dsfac = 0.0;
  if (t.switchflag && r > t.rmin0) {
    const double f = M_PI / (rcut - t.rmin0);
    double ss, cc;
    sincos((r - t.rmin0) * f, &ss, &cc);
    g.sfac = 0.5 * (cc + 1.0);
    g.dsfac = -0.5 * ss * f;
  }
  if (deriv) {
    const double rinv = 1.0 / r;
    g.u[0] = x * rinv;
    g.u[1] = y * rinv;
    g.u[2] = z * rinv;
    const double dz0dr = z0 / r - (r * rscale0) * (rsq + z0 * z0) / rsq;
    const double dr0invdr = -(r0inv * r0inv * r0inv) * (r + z0 * dz0dr);
    for (int k = 0; k < 3; ++k) {
      const double dr0 = dr0invdr * g.u[k];
      g.da[k] = C2{dz0dr * g.u[k] * r0inv + z0 * dr0, -z * dr0};
      g.db[k] = C2{y * dr0, -x * dr0};
    }
    g.da[2].i += -r0inv;
    g.db[0].i += -r0inv;
    g.db[1].r += r0inv;
  }
  return g;
}

__global__ void k_snap_zero(uint32_t n_part, const SysDesc* __restrict__ sys, const SysState* __restrict__ st,
                            DevArrays a, int sys_only, bool zero_f, bool zero_pe) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_part) return;
  const uint32_t c = a.pcell[i];
  if (c == kInvalid) return;
  const uint32_t s = a.cell_sys[c];
  if (sys_only >= 0 && s != static_cast<uint32_t>(sys_only)) return;
  if (st[s].error) return;
  if (zero_f) {
    a.fx[i] = 0.0;
    a.fy[i] = 0.0;
    a.fz[i] = 0.0;
  }
  if (zero_pe) a.pe[i] = 0.0;
}

// (row, column) of element `e` of a level with n = j + 1 columns, advanced by
// `step` elements without integer division (its conversion sequence would run
// on the FP64 pipe)
__device__ __forceinline__ void rc_start(int e, int n, int& r, int& c) {
  r = 0;
  c = e;
  while (c >= n) {
    c -= n;
    ++r;
  }
}
__device__ __forceinline__ void rc_step(int step, int n, int& r, int& c) {
  c += step;
  while (c >= n) {
    c -= n;
    ++r;
  }
}

__device__ __forceinline__ bool uq(int j, int r, int c) {
  return r >= 0 && c >= 0 && c <= j && r * (j + 1) + c < nunique(j);
}

// Forward U levels 1..J of one neighbour into its unique-half buffer u (level j
// at ublk[j]); level 0 is set by the caller. Threads slot, slot + lpn, ... of the
// neighbour take the elements of each level; the CTA synchronises between levels.
template <class R>
__device__ __forceinline__ void forward_levels(R* u, bool active, int slot, int lpn, CX<R> a, CX<R> b,
                                               const SnapArgs& t, const R* rootpq) {
  const int J = t.twojmax;
  for (int j = 1; j <= J; ++j) {
    if (active) {
      const int nuj = nunique(j);
      const R* prev = u + 2 * t.ublk[j - 1];
      R* cur = u + 2 * t.ublk[j];
      int mb, ma;
      rc_start(slot, j + 1, mb, ma);
      for (int e = slot; e < nuj; e += lpn, rc_step(lpn, j + 1, mb, ma)) {
        CX<R> v{R(0), R(0)};
        if (ma < j) {
          const CX<R> p = level_get(prev, 2, 0, j - 1, mb, ma);
          const R rp = rootpq[(j - ma) * (J + 1) + (j - mb)];
          const CX<R> q = cmulc(a, p);
          v.r = rp * q.r;
          v.i = rp * q.i;
        }
        if (ma > 0) {
          const CX<R> p = level_get(prev, 2, 0, j - 1, mb, ma - 1);
          const R rp = rootpq[ma * (J + 1) + (j - mb)];
          const CX<R> q = cmulc(b, p);
          v.r = fma(-rp, q.r, v.r);
          v.i = fma(-rp, q.i, v.i);
        }
        cur[2 * e] = v.r;
        cur[2 * e + 1] = v.i;
      }
    }
    __syncthreads();
  }
}

// R: the type of the U, Z, Y and adjoint arithmetic (double, or float for the
// mixed path); geometry, switching and the force sums stay in double.
template <class R>
__global__ void __launch_bounds__(kSnapThreads)
    k_snap(uint32_t n_part, const SysDesc* __restrict__ sys, const SysState* __restrict__ st, DevArrays a,
           SnapArgs t, int group, int sys_only, bool with_pe, unsigned int* flags) {
  extern __shared__ double sm[];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int J = t.twojmax;
  const int lvl_max = nunique(J);
  const int nu = t.nu_unique;
  const Tabs<R> T = tabs<R>(t);
  // shared layout: double part, then the compute-type part
  double* nx = sm;
  double* ny = nx + kSnapMaxNbr;
  double* nz = ny + kSnapMaxNbr;
  double* nspare = nz + kSnapMaxNbr;                                       // (unused double slot)
  uint32_t* nj = reinterpret_cast<uint32_t*>(nspare + kSnapMaxNbr);        // kSnapMaxNbr u32
  uint8_t* nt = reinterpret_cast<uint8_t*>(nj + kSnapMaxNbr);              // kSnapMaxNbr u8
  double* red = nspare + kSnapMaxNbr + kSnapMaxNbr / 2 + kSnapMaxNbr / 8;  // kSnapThreads x 5
  double* misc = red + kSnapThreads * 5;                                    // 8 doubles: fsum[3], wsum[4]
  int* icnt = reinterpret_cast<int*>(misc + 8);                             // 8 ints
  R* nab = reinterpret_cast<R*>(misc + 12);                                // 4 per neighbour: a, b
  R* nsw = nab + 4 * kSnapMaxNbr;                                           // wj sfac per neighbour
  R* utot = nsw + kSnapMaxNbr;                                              // 2 nu_full
  R* yv = utot + 2 * t.nu_full;                                             // 2 nu
  R* uacc = yv + 2 * nu;                                                    // 2 nu
  R* uall = uacc + 2 * nu;                                                  // group x 2 nu
  R* adj = uall + static_cast<size_t>(group) * 2 * nu;                      // group x 2 x 2 lvl_max

  for (uint32_t i = blockIdx.x; i < n_part; i += gridDim.x) {
    const uint32_t c = a.pcell[i];
    if (c == kInvalid) continue;
    const uint32_t s = a.cell_sys[c];
    if (sys_only >= 0 && s != static_cast<uint32_t>(sys_only)) continue;
    if (st[s].error) continue;
    const SysDesc& S = sys[s];
    const uint32_t ti = a.ptype[i];
    if (ti >= static_cast<uint32_t>(t.ntypes)) {
      if (tid == 0) atomicOr(flags, 1u);
      continue;
    }
    const double xa = a.rx[i], ya = a.ry[i], za = a.rz[i];
    const uint32_t* __restrict__ L = a.nbr + S.list_base + a.nbr_start[i];
    const uint32_t n = a.nbr_cnt[i];
    const uint32_t pbase = S.part_base;
    const double radi = t.radelem[ti];
    const double fscale = S.divide_by_mass ? t.energy_unit / S.mass : t.energy_unit;

    // ---- environment, in list order ----
    if (tid == 0) {
      icnt[4] = 0;
      misc[0] = misc[1] = misc[2] = 0.0;
    }
    __syncthreads();
    for (uint32_t base = 0; base < n; base += kSnapThreads) {
      const uint32_t k = base + tid;
      bool keep = false;
      double dx = 0, dy = 0, dz = 0;
      uint32_t j = 0, tj = 0;
      if (k < n) {
        const uint32_t e = __ldg(L + k);
        j = pbase + (e >> 5);
        const uint32_t code = e & 31u;
        double xb = __ldg(a.rx + j), yb = __ldg(a.ry + j), zb = __ldg(a.rz + j);
        if (code != static_cast<uint32_t>(kImageCenter)) {
          xb = image_coord(xb, S.period[0], static_cast<int>(code % 3u));
          yb = image_coord(yb, S.period[1], static_cast<int>((code / 3u) % 3u));
          zb = image_coord(zb, S.period[2], static_cast<int>(code / 9u));
        }
        dx = xb - xa;
        dy = yb - ya;
        dz = zb - za;
        const double d2 = norm2_rn(dx, dy, dz);
        tj = a.ptype[j];
        if (tj >= static_cast<uint32_t>(t.ntypes)) {
          atomicOr(flags, 1u);
        } else {
          const double cij = (radi + t.radelem[tj]) * t.rcutfac;
          keep = d2 < cij * cij && d2 > 1e-20;
        }
      }
      const unsigned bal = __ballot_sync(0xffffffffu, keep);
      if (lane == 0) icnt[w] = __popc(bal);
      __syncthreads();
      int off = icnt[4];
      for (int q = 0; q < w; ++q) off += icnt[q];
      off += __popc(bal & ((1u << lane) - 1u));
      if (keep && off < kSnapMaxNbr) {
        nx[off] = dx;
        ny[off] = dy;
        nz[off] = dz;
        nj[off] = j;
        nt[off] = static_cast<uint8_t>(tj);
      }
      __syncthreads();
      if (tid == 0) icnt[4] += icnt[0] + icnt[1] + icnt[2] + icnt[3];
      __syncthreads();
    }
    const int nn = icnt[4];
    if (nn > kSnapMaxNbr) {
      if (tid == 0) atomicOr(flags, 2u);
      __syncthreads();
      continue;
    }

    // ---- U_tot = self + sum_j wj sfac U_j, neighbours in rounds of `group` ----
    for (int e = tid; e < 2 * nu; e += kSnapThreads) uacc[e] = R(0);
    for (int q0 = 0; q0 < nn; q0 += group) {
      const int gr = min(group, nn - q0);
      const int lpn = kSnapThreads / gr;
      const int g = tid / lpn, slot = tid % lpn;
      const bool active = g < gr;
      R* ug = uall + static_cast<size_t>(active ? g : 0) * 2 * nu;
      if (active && slot == 0) {  // the neighbour's Cayley-Klein parameters, once
        const int q = q0 + g;
        const double rcut = (radi + t.radelem[nt[q]]) * t.rcutfac;
        const Geo geo = geometry(nx[q], ny[q], nz[q], rcut, t, false);
        nab[4 * q] = R(geo.a.r);
        nab[4 * q + 1] = R(geo.a.i);
        nab[4 * q + 2] = R(geo.b.r);
        nab[4 * q + 3] = R(geo.b.i);
        nsw[q] = R(t.wj[nt[q]] * geo.sfac);
        ug[0] = R(1);
        ug[1] = R(0);
      }
      __syncthreads();
      CX<R> ca{R(0), R(0)}, cb{R(0), R(0)};
      if (active) {
        const int q = q0 + g;
        ca = CX<R>{nab[4 * q], nab[4 * q + 1]};
        cb = CX<R>{nab[4 * q + 2], nab[4 * q + 3]};
      }
      forward_levels(ug, active, slot, lpn, ca, cb, t, T.rootpq);
      for (int e = tid; e < nu; e += kSnapThreads) {
        R re = R(0), im = R(0);
        for (int q = 0; q < gr; ++q) {
          const R sw = nsw[q0 + q];
          re = fma(sw, uall[static_cast<size_t>(q) * 2 * nu + 2 * e], re);
          im = fma(sw, uall[static_cast<size_t>(q) * 2 * nu + 2 * e + 1], im);
        }
        uacc[2 * e] += re;
        uacc[2 * e + 1] += im;
      }
      __syncthreads();
    }
    // ---- self term, full matrices ----
    for (int e = tid; e < nu; e += kSnapThreads) {
      int j = 0;
      while (j < J && e >= t.ublk[j + 1]) ++j;
      const int le = e - t.ublk[j];
      const int mb = le / (j + 1), ma = le % (j + 1);
      const R re = uacc[2 * e] + ((mb == ma) ? R(1) : R(0)), im = uacc[2 * e + 1];
      const int f = t.fblk[j] + mb * (j + 1) + ma;
      utot[2 * f] = re;
      utot[2 * f + 1] = im;
      if (!(2 * mb == j && ma == mb)) {
        const int g2 = t.fblk[j] + (j - mb) * (j + 1) + (j - ma);
        const R sg = ((ma + mb) & 1) ? R(-1) : R(1);
        utot[2 * g2] = sg * re;
        utot[2 * g2 + 1] = -sg * im;
      }
      yv[2 * e] = R(0);
      yv[2 * e + 1] = R(0);
    }
    __syncthreads();
    // ---- Y = sum beta_j Z, and the energy ----
    double eloc = 0.0;
    const R* zb = T.zbeta + static_cast<size_t>(ti) * t.nz;
    const R* ze = T.zener + static_cast<size_t>(ti) * t.nz;
    for (int e = tid; e < t.nz; e += kSnapThreads) {
      const SnapZ z = t.z[e];
      const R* cgb = T.cg + z.cg;
      const int j1 = z.j1, j2 = z.j2;
      int jju1 = t.fblk[j1] + (j1 + 1) * z.mb1min;
      int jju2 = t.fblk[j2] + (j2 + 1) * z.mb2max;
      int icgb = z.mb1min * (j2 + 1) + z.mb2max;
      CX<R> zt{R(0), R(0)};
      for (int ib = 0; ib < z.nb; ++ib) {
        CX<R> sa{R(0), R(0)};
        int ma1 = z.ma1min, ma2 = z.ma2max;
        int icga = z.ma1min * (j2 + 1) + z.ma2max;
        for (int ia = 0; ia < z.na; ++ia) {
          const CX<R> p = cmul(CX<R>{utot[2 * (jju1 + ma1)], utot[2 * (jju1 + ma1) + 1]},
                               CX<R>{utot[2 * (jju2 + ma2)], utot[2 * (jju2 + ma2) + 1]});
          sa.r = fma(cgb[icga], p.r, sa.r);
          sa.i = fma(cgb[icga], p.i, sa.i);
          ++ma1;
          --ma2;
          icga += j2;
        }
        zt.r = fma(cgb[icgb], sa.r, zt.r);
        zt.i = fma(cgb[icgb], sa.i, zt.i);
        jju1 += j1 + 1;
        jju2 -= j2 + 1;
        icgb += j2;
      }
      atomicAdd(&yv[2 * z.y], zb[e] * zt.r);
      atomicAdd(&yv[2 * z.y + 1], zb[e] * zt.i);
      if (with_pe && ze[e] != R(0)) {
        const CX<R> u{utot[2 * z.uf], utot[2 * z.uf + 1]};
        eloc += static_cast<double>(ze[e] * cmulc(u, zt).r);
      }
    }
    if (with_pe) {
      eloc = warp_sum(eloc);
      if (lane == 0) misc[4 + w] = eloc;
    }
    __syncthreads();
    if (with_pe && tid == 0) {
      double es = t.e0[ti];
      for (int q = 0; q < kSnapWarps; ++q) es += misc[4 + q];
      a.pe[i] = es * t.energy_unit;
    }

    // ---- forces by reverse mode: F = sum_e w Re(conj(U_e) Y_e) per neighbour,
    //      dF/da and dF/db from the adjoint w Y propagated down the levels ----
    for (int q0 = 0; q0 < nn; q0 += group) {
      const int gr = min(group, nn - q0);
      const int lpn = kSnapThreads / gr;
      const int g = tid / lpn, slot = tid % lpn;
      const bool active = g < gr;
      R* ug = uall + static_cast<size_t>(active ? g : 0) * 2 * nu;
      R* adj0 = adj + static_cast<size_t>(active ? g : 0) * 4 * lvl_max;
      R* adj1 = adj0 + 2 * lvl_max;
      CX<R> ca{R(0), R(0)}, cb{R(0), R(0)};
      if (active) {
        const int q = q0 + g;
        ca = CX<R>{nab[4 * q], nab[4 * q + 1]};
        cb = CX<R>{nab[4 * q + 2], nab[4 * q + 3]};
        if (nn > group && slot == 0) {  // U of this round's neighbours was overwritten
          ug[0] = R(1);
          ug[1] = R(0);
        }
      }
      if (nn > group) {
        __syncthreads();
        forward_levels(ug, active, slot, lpn, ca, cb, t, T.rootpq);
      }
      R F = R(0), gar = R(0), gai = R(0), gbr = R(0), gbi = R(0);
      // seed the top level
      if (active) {
        const int nuJ = nunique(J);
        for (int e = slot; e < nuJ; e += lpn) {
          const R wgt = ((J & 1) == 0 && e == nuJ - 1) ? R(0.5) : R(1);
          adj0[2 * e] = wgt * yv[2 * (t.ublk[J] + e)];
          adj0[2 * e + 1] = wgt * yv[2 * (t.ublk[J] + e) + 1];
        }
      }
      __syncthreads();
      R* A = adj0;
      R* Nx = adj1;
      for (int j = J; j >= 1; --j) {
        const int Lv = j - 1;
        if (active) {
          const int nuj = nunique(j);
          const R* uj = ug + 2 * t.ublk[j];
          const R* ul = ug + 2 * t.ublk[Lv];
          const R* yj = yv + 2 * t.ublk[j];
          int mb, ma;
          rc_start(slot, j + 1, mb, ma);
          for (int e = slot; e < nuj; e += lpn, rc_step(lpn, j + 1, mb, ma)) {
            const R wgt = ((j & 1) == 0 && e == nuj - 1) ? R(0.5) : R(1);
            F = fma(wgt, fma(uj[2 * e], yj[2 * e], uj[2 * e + 1] * yj[2 * e + 1]), F);
            const R Gr = A[2 * e], Gi = A[2 * e + 1];
            if (ma < j) {
              const CX<R> p = level_get(ul, 2, 0, Lv, mb, ma);
              const R rp = T.rootpq[(j - ma) * (J + 1) + (j - mb)];
              gar = fma(rp, fma(Gr, p.r, Gi * p.i), gar);
              gai = fma(rp, fma(Gr, p.i, -(Gi * p.r)), gai);
            }
            if (ma > 0) {
              const CX<R> p = level_get(ul, 2, 0, Lv, mb, ma - 1);
              const R rp = T.rootpq[ma * (J + 1) + (j - mb)];
              gbr = fma(-rp, fma(Gr, p.r, Gi * p.i), gbr);
              gbi = fma(-rp, fma(Gr, p.i, -(Gi * p.r)), gbi);
            }
          }
          // adjoint of level j-1 by gathering its readers in level j
          const int nul = nunique(Lv);
          const R* yl = yv + 2 * t.ublk[Lv];
          int r, cc;
          rc_start(slot, Lv + 1, r, cc);
          for (int u = slot; u < nul; u += lpn, rc_step(lpn, Lv + 1, r, cc)) {
            const R wgt = ((Lv & 1) == 0 && u == nul - 1) ? R(0.5) : R(1);
            R accr = wgt * yl[2 * u], acci = wgt * yl[2 * u + 1];
            if (uq(j, r, cc)) {
              const int k = r * (j + 1) + cc;
              const R rp = T.rootpq[(j - cc) * (J + 1) + (j - r)];
              const CX<R> m = cmul(ca, CX<R>{A[2 * k], A[2 * k + 1]});
              accr = fma(rp, m.r, accr);
              acci = fma(rp, m.i, acci);
            }
            if (cc + 1 <= j && uq(j, r, cc + 1)) {
              const int k = r * (j + 1) + cc + 1;
              const R rp = T.rootpq[(cc + 1) * (J + 1) + (j - r)];
              const CX<R> m = cmul(cb, CX<R>{A[2 * k], A[2 * k + 1]});
              accr = fma(-rp, m.r, accr);
              acci = fma(-rp, m.i, acci);
            }
            const int r2 = Lv - r, c2 = Lv - cc;
            if (!(r2 == r && c2 == cc) && !uq(Lv, r2, c2)) {
              R tr = R(0), tim = R(0);
              if (uq(j, r2, c2)) {
                const int k = r2 * (j + 1) + c2;
                const R rp = T.rootpq[(j - c2) * (J + 1) + (j - r2)];
                const CX<R> m = cmul(ca, CX<R>{A[2 * k], A[2 * k + 1]});
                tr = rp * m.r;
                tim = rp * m.i;
              }
              if (c2 + 1 <= j && uq(j, r2, c2 + 1)) {
                const int k = r2 * (j + 1) + c2 + 1;
                const R rp = T.rootpq[(c2 + 1) * (J + 1) + (j - r2)];
                const CX<R> m = cmul(cb, CX<R>{A[2 * k], A[2 * k + 1]});
                tr = fma(-rp, m.r, tr);
                tim = fma(-rp, m.i, tim);
              }
              const R sg = ((r2 + c2) & 1) ? R(-1) : R(1);
              accr = fma(sg, tr, accr);
              acci = fma(-sg, tim, acci);
            }
            Nx[2 * u] = accr;
            Nx[2 * u + 1] = acci;
          }
        }
        __syncthreads();
        R* tmp = A;
        A = Nx;
        Nx = tmp;
      }
      if (active && slot == 0) F += R(0.5) * yv[0];  // level 0: U = 1, centre weight 1/2
      red[tid * 5 + 0] = active ? static_cast<double>(F) : 0.0;
      red[tid * 5 + 1] = static_cast<double>(gar);
      red[tid * 5 + 2] = static_cast<double>(gai);
      red[tid * 5 + 3] = static_cast<double>(gbr);
      red[tid * 5 + 4] = static_cast<double>(gbi);
      __syncthreads();
      if (tid < gr) {
        const int q = q0 + tid;
        double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        for (int sl = 0; sl < lpn; ++sl)
          for (int k = 0; k < 5; ++k) v[k] += red[(tid * lpn + sl) * 5 + k];
        const double rcut = (radi + t.radelem[nt[q]]) * t.rcutfac;
        const Geo geo = geometry(nx[q], ny[q], nz[q], rcut, t, true);
        const double wjq = t.wj[nt[q]];
        double f[3];
        for (int k = 0; k < 3; ++k) {
          const double dF = v[1] * geo.da[k].r + v[2] * geo.da[k].i + v[3] * geo.db[k].r + v[4] * geo.db[k].i;
          f[k] = 2.0 * fscale * wjq * (geo.dsfac * geo.u[k] * v[0] + geo.sfac * dF);
        }
        const uint32_t j = nj[q];
        atomicAdd(a.fx + j, -f[0]);
        atomicAdd(a.fy + j, -f[1]);
        atomicAdd(a.fz + j, -f[2]);
        atomicAdd(&misc[0], f[0]);
        atomicAdd(&misc[1], f[1]);
        atomicAdd(&misc[2], f[2]);
      }
      __syncthreads();
    }
    if (tid == 0) {
      atomicAdd(a.fx + i, misc[0]);
      atomicAdd(a.fy + i, misc[1]);
      atomicAdd(a.fz + i, misc[2]);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Host tables. Clebsch-Gordan coefficients by Racah's closed formula with
// exact integer factorials in long double.
long double lfact(int n) {
  long double r = 1.0L;
  for (int k = 2; k <= n; ++k) r *= k;
  return r;
}

double clebsch(int j1, int j2, int j, int m1, int m2) {
  const int a2 = 2 * m1 - j1, b2 = 2 * m2 - j2, c2 = a2 + b2;
  if (c2 < -j || c2 > j) return 0.0;
  const long double tri =
      lfact((j1 + j2 - j) / 2) * lfact((j1 - j2 + j) / 2) * lfact((-j1 + j2 + j) / 2) / lfact((j1 + j2 + j) / 2 + 1);
  const long double pre = sqrtl((j + 1) * tri * lfact((j1 + a2) / 2) * lfact((j1 - a2) / 2) * lfact((j2 + b2) / 2) *
                                lfact((j2 - b2) / 2) * lfact((j + c2) / 2) * lfact((j - c2) / 2));
  long double sum = 0.0L;
  const int kmin = std::max(0, std::max(-(j - j2 + a2) / 2, -(j - j1 - b2) / 2));
  const int kmax = std::min((j1 + j2 - j) / 2, std::min((j1 - a2) / 2, (j2 + b2) / 2));
  for (int k = kmin; k <= kmax; ++k) {
    const long double den = lfact(k) * lfact((j1 + j2 - j) / 2 - k) * lfact((j1 - a2) / 2 - k) *
                            lfact((j2 + b2) / 2 - k) * lfact((j - j2 + a2) / 2 + k) * lfact((j - j1 - b2) / 2 + k);
    sum += ((k & 1) ? -1.0L : 1.0L) / den;
  }
  return static_cast<double>(pre * sum);
}

}  // namespace

int snap_build(const xnb_snap_params& p, int device, SnapArgs& t, std::vector<void*>& allocs, std::string& err) {
  const int J = p.twojmax;
  if (J < 0 || J > kSnapMaxTwoJ) {
    err = "twojmax must be in [0, 10]";
    return XNB_ERR_ARG;
  }
  if (p.chemflag || p.bnormflag || p.quadraticflag || p.switchinnerflag) {
    err = "only linear SNAP with chemflag, bnormflag, quadraticflag and switchinnerflag off is supported";
    return XNB_ERR_ARG;
  }
  if (p.ntypes < 1 || p.ntypes > kSnapMaxTypes || !p.coeff) {
    err = "1 to 16 particle types with coefficients";
    return XNB_ERR_ARG;
  }
  std::memset(&t, 0, sizeof(t));
  t.twojmax = J;
  t.ntypes = p.ntypes;
  t.switchflag = p.switchflag != 0;
  t.rcutfac = p.rcutfac;
  t.rfac0 = p.rfac0;
  t.rmin0 = p.rmin0;
  t.energy_unit = p.energy_unit;
  for (int k = 0; k < p.ntypes; ++k) {
    t.radelem[k] = p.radelem[k];
    t.wj[k] = p.wj[k];
  }
  int nu = 0, nf = 0;
  for (int j = 0; j <= J; ++j) {
    t.ublk[j] = nu;
    t.fblk[j] = nf;
    nu += nunique(j);
    nf += (j + 1) * (j + 1);
  }
  t.ublk[J + 1] = nu;
  t.fblk[J + 1] = nf;
  t.nu_unique = nu;
  t.nu_full = nf;
  // coefficient order (sna.cpp:236-259) and Clebsch-Gordan blocks (sna.cpp:194-205)
  struct Tri {
    int j1, j2, j;
  };
  std::vector<Tri> bl;
  std::vector<double> cg;
  std::vector<int> cgoff;  // by (j1, j2, j)
  cgoff.assign((J + 1) * (J + 1) * (J + 1), -1);
  for (int j1 = 0; j1 <= J; ++j1)
    for (int j2 = 0; j2 <= j1; ++j2)
      for (int j = j1 - j2; j <= std::min(J, j1 + j2); j += 2) {
        if (j >= j1) bl.push_back({j1, j2, j});
        cgoff[(j1 * (J + 1) + j2) * (J + 1) + j] = static_cast<int>(cg.size());
        for (int m1 = 0; m1 <= j1; ++m1)
          for (int m2 = 0; m2 <= j2; ++m2) cg.push_back(clebsch(j1, j2, j, m1, m2));
      }
  const int ncoeff = static_cast<int>(bl.size());
  if (p.ncoeffall != ncoeff + 1) {
    err = "coefficient count " + std::to_string(p.ncoeffall) + " does not match twojmax (expected " +
          std::to_string(ncoeff + 1) + ")";
    return XNB_ERR_ARG;
  }
  auto bindex = [&](int a, int b, int c) {
    for (int k = 0; k < ncoeff; ++k)
      if (bl[k].j1 == a && bl[k].j2 == b && bl[k].j == c) return k;
    return -1;
  };
  // Z elements of the unique half, with the beta multipliers (snap_compute_yi.h:133-158)
  std::vector<SnapZ> zs;
  std::vector<double> mult;  // multiplicity * (j1+1)/(j+1)
  std::vector<int> kb;       // coefficient of the multiplier
  std::vector<int> ecoef;    // coefficient for the energy (canonical entries) or -1
  std::vector<double> ew;    // 2 w of the energy sum
  for (int j1 = 0; j1 <= J; ++j1)
    for (int j2 = 0; j2 <= j1; ++j2)
      for (int j = j1 - j2; j <= std::min(J, j1 + j2); j += 2)
        for (int mb = 0; 2 * mb <= j; ++mb)
          for (int ma = 0; ma <= j; ++ma) {
            if (2 * mb == j && ma > mb) continue;
            SnapZ z{};
            z.j1 = static_cast<uint8_t>(j1);
            z.j2 = static_cast<uint8_t>(j2);
            z.j = static_cast<uint8_t>(j);
            const int ma1min = std::max(0, (2 * ma - j - j2 + j1) / 2);
            const int ma2max = (2 * ma - j - (2 * ma1min - j1) + j2) / 2;
            const int na = std::min(j1, (2 * ma - j + j2 + j1) / 2) - ma1min + 1;
            const int mb1min = std::max(0, (2 * mb - j - j2 + j1) / 2);
            const int mb2max = (2 * mb - j - (2 * mb1min - j1) + j2) / 2;
            const int nb = std::min(j1, (2 * mb - j + j2 + j1) / 2) - mb1min + 1;
            z.ma1min = static_cast<uint8_t>(ma1min);
            z.ma2max = static_cast<uint8_t>(ma2max);
            z.na = static_cast<uint8_t>(std::max(0, na));
            z.mb1min = static_cast<uint8_t>(mb1min);
            z.mb2max = static_cast<uint8_t>(mb2max);
            z.nb = static_cast<uint8_t>(std::max(0, nb));
            z.y = static_cast<uint16_t>(t.ublk[j] + mb * (j + 1) + ma);
            z.uf = static_cast<uint16_t>(t.fblk[j] + mb * (j + 1) + ma);
            z.cg = static_cast<uint32_t>(cgoff[(j1 * (J + 1) + j2) * (J + 1) + j]);
            double m;
            int k;
            if (j >= j1) {
              k = bindex(j1, j2, j);
              m = (j1 == j) ? ((j2 == j) ? 3.0 : 2.0) : 1.0;
            } else if (j >= j2) {
              k = bindex(j, j2, j1);
              m = (j2 == j) ? 2.0 : 1.0;
            } else {
              k = bindex(j2, j, j1);
              m = 1.0;
            }
            if (j1 > j) m *= (j1 + 1) / (j + 1.0);
            zs.push_back(z);
            mult.push_back(m);
            kb.push_back(k);
            ecoef.push_back(j >= j1 ? bindex(j1, j2, j) : -1);
            ew.push_back((2 * mb == j && ma == mb) ? 1.0 : 2.0);
          }
  // order the Z elements by their work (na x nb terms), largest first: the
  // threads of a warp then run loops of similar length
  {
    std::vector<int> perm(zs.size());
    for (size_t e = 0; e < perm.size(); ++e) perm[e] = static_cast<int>(e);
    std::stable_sort(perm.begin(), perm.end(),
                     [&](int x, int y) { return zs[x].na * zs[x].nb > zs[y].na * zs[y].nb; });
    std::vector<SnapZ> zs2(zs.size());
    std::vector<double> mult2(zs.size()), ew2(zs.size());
    std::vector<int> kb2(zs.size()), ec2(zs.size());
    for (size_t e = 0; e < perm.size(); ++e) {
      zs2[e] = zs[perm[e]];
      mult2[e] = mult[perm[e]];
      kb2[e] = kb[perm[e]];
      ec2[e] = ecoef[perm[e]];
      ew2[e] = ew[perm[e]];
    }
    zs.swap(zs2);
    mult.swap(mult2);
    kb.swap(kb2);
    ecoef.swap(ec2);
    ew.swap(ew2);
  }
  t.nz = static_cast<int>(zs.size());
  std::vector<double> zbeta(static_cast<size_t>(p.ntypes) * t.nz), zener(zbeta.size());
  for (int ty = 0; ty < p.ntypes; ++ty) {
    const double* c = p.coeff + static_cast<size_t>(ty) * p.ncoeffall;
    double e0 = c[0];
    if (p.bzeroflag)
      for (int k = 0; k < ncoeff; ++k) e0 -= c[1 + k] * (bl[k].j + 1);  // bzero_j = wself^3 (j+1)
    t.e0[ty] = e0;
    for (int e = 0; e < t.nz; ++e) {
      zbeta[static_cast<size_t>(ty) * t.nz + e] = mult[e] * c[1 + kb[e]];
      zener[static_cast<size_t>(ty) * t.nz + e] = ecoef[e] >= 0 ? ew[e] * c[1 + ecoef[e]] : 0.0;
    }
  }
  std::vector<double> rootpq((J + 1) * (J + 1), 0.0);
  for (int a = 1; a <= J; ++a)
    for (int b = 1; b <= J; ++b) rootpq[a * (J + 1) + b] = std::sqrt(static_cast<double>(a) / b);
  // upload
  if (cudaSetDevice(device) != cudaSuccess) {
    err = "cudaSetDevice failed";
    return XNB_ERR_CUDA;
  }
  auto up = [&](const void* src, size_t bytes, const void** dst) -> bool {
    void* d = nullptr;
    if (cudaMalloc(&d, std::max<size_t>(bytes, 16)) != cudaSuccess) return false;
    allocs.push_back(d);
    if (bytes && cudaMemcpy(d, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) return false;
    *dst = d;
    return true;
  };
  auto f32 = [](const std::vector<double>& v) { return std::vector<float>(v.begin(), v.end()); };
  const std::vector<float> rootpq_f = f32(rootpq), cg_f = f32(cg), zbeta_f = f32(zbeta), zener_f = f32(zener);
  if (!up(rootpq.data(), rootpq.size() * 8, reinterpret_cast<const void**>(&t.rootpq)) ||
      !up(cg.data(), cg.size() * 8, reinterpret_cast<const void**>(&t.cg)) ||
      !up(zs.data(), zs.size() * sizeof(SnapZ), reinterpret_cast<const void**>(&t.z)) ||
      !up(zbeta.data(), zbeta.size() * 8, reinterpret_cast<const void**>(&t.zbeta)) ||
      !up(zener.data(), zener.size() * 8, reinterpret_cast<const void**>(&t.zener)) ||
      !up(rootpq_f.data(), rootpq_f.size() * 4, reinterpret_cast<const void**>(&t.rootpq_f)) ||
      !up(cg_f.data(), cg_f.size() * 4, reinterpret_cast<const void**>(&t.cg_f)) ||
      !up(zbeta_f.data(), zbeta_f.size() * 4, reinterpret_cast<const void**>(&t.zbeta_f)) ||
      !up(zener_f.data(), zener_f.size() * 4, reinterpret_cast<const void**>(&t.zener_f))) {
    err = "device memory for the SNAP tables";
    return XNB_ERR_NOMEM;
  }
  // shared memory: a double part (environment, reductions) and a compute-type part:
  // U_tot, Y, the U accumulator and, per neighbour of a round, its forward U
  // (unique half of every level) and two adjoint levels; the round size is the
  // largest that keeps a CTA within ~100 KB (two CTAs per SM), at most 32
  const int lvl_max = nunique(J);
  const size_t fixed_d = 4 * kSnapMaxNbr + kSnapMaxNbr / 2 + kSnapMaxNbr / 8 + kSnapThreads * 5 + 12;
  const size_t fixed_r = 5 * kSnapMaxNbr + 2 * t.nu_full + 4 * t.nu_unique;
  const size_t per = 2 * t.nu_unique + 4 * lvl_max;
  // budgets: ~100 KB (two CTAs per SM) for the FP64 kernel, whose FP64 pipe is
  // busy anyway; ~54 KB (four CTAs per SM with the per-CTA reserve) for the FP32 kernel, which needs the
  // warps to hide shared-memory latency
  auto plan = [&](size_t rsize, int& group, size_t& bytes) {
    const size_t budget = (rsize == 8 ? 100 : 54) * 1024, base = fixed_d * 8 + fixed_r * rsize;
    long long grp = budget > base ? static_cast<long long>((budget - base) / (per * rsize)) : 1;
    grp = std::max(1LL, std::min<long long>(grp, kSnapMaxGroup));
    group = static_cast<int>(grp);
    bytes = base + per * rsize * group;
  };
  plan(8, t.group, t.smem_bytes);
  plan(4, t.group_f, t.smem_bytes_f);
  return XNB_OK;
}

template <class R>
void snap_go(const Extent& ex, const SysDesc* sys, const SysState* st, const DevArrays& a, const SnapArgs& t,
             int group, size_t smem, int sys_only, bool with_pe, unsigned int* flags, cudaStream_t stream) {
  cudaFuncSetAttribute(k_snap<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_snap<R>, kSnapThreads, smem);
  long long g = static_cast<long long>(ex.sm_count) * std::max(1, per_sm) * 4;
  if (g > static_cast<long long>(ex.n_part)) g = ex.n_part;
  k_snap<R><<<static_cast<int>(std::max(1LL, g)), kSnapThreads, smem, stream>>>(ex.n_part, sys, st, a, t, group,
                                                                             sys_only, with_pe, flags);
}

int launch_snap(const Extent& ex, const SysDesc* sys, const SysState* st, const DevArrays& a, const SnapArgs& t,
                int sys_only, bool with_pe, bool accumulate, bool mixed, unsigned int* flags, cudaStream_t stream) {
  if (ex.n_part == 0) return 0;
  int launches = 0;
  if (!accumulate || with_pe) {
    const int g = static_cast<int>((static_cast<long long>(ex.n_part) + 255) / 256);
    k_snap_zero<<<g, 256, 0, stream>>>(ex.n_part, sys, st, a, sys_only, !accumulate, with_pe);
    ++launches;
  }
  if (mixed) snap_go<float>(ex, sys, st, a, t, t.group_f, t.smem_bytes_f, sys_only, with_pe, flags, stream);
  else snap_go<double>(ex, sys, st, a, t, t.group, t.smem_bytes, sys_only, with_pe, flags, stream);
  return launches + 1;
}

}  // namespace xnb
