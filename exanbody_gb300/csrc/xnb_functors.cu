// Pair functors other than Lennard-Jones over the same per-particle lists and
// the same FP32-prefiltered traversal (prefilter_window / next_mark).
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
// square root and one division, FMA accumulation.
template <int P, bool PE>
__global__ void __launch_bounds__(128)
    k_grav(uint32_t n_part, const SysDesc* __restrict__ sys, const SysState* __restrict__ st, DevArrays a,
           int sys_only, GravParams gp, bool accumulate, unsigned int* flags) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_part) return;
  const uint32_t c = a.pcell[i];
  if (c == kInvalid) return;
  const uint32_t s = a.cell_sys[c];
  if (sys_only >= 0 && s != static_cast<uint32_t>(sys_only)) return;
  if (st[s].error) return;
  const SysDesc& S = sys[s];
  const uint32_t ta = a.ptype[i];
  if (ta >= static_cast<uint32_t>(gp.ntypes)) {
    atomicOr(flags, 1u);
    return;
  }
  const double ma = gp.mass[ta];
  const double xa = a.rx[i], ya = a.ry[i], za = a.rz[i];
  const uint32_t* __restrict__ L = a.nbr + S.list_base + a.nbr_start[i];
  const uint32_t n = a.nbr_cnt[i];
  const uint32_t pbase = S.part_base;
  const float4 paf = a.pf[i];
  const float pfx = S.period_f[0], pfy = S.period_f[1], pfz = S.period_f[2];
  double fx = accumulate ? a.fx[i] : 0.0, fy = accumulate ? a.fy[i] : 0.0, fz = accumulate ? a.fz[i] : 0.0;
  double pe = 0.0;
  const uint32_t self_e = ((i - pbase) << 5) | static_cast<uint32_t>(kImageCenter);
  for (uint32_t kw = 0; kw < n; kw += 128) {
    Marks mk = prefilter_window(L, kw, min(n, kw + 128u), a.pf, pbase, self_e, paf, pfx, pfy, pfz, gp.pre_hi_f);
    uint32_t b;
    while (next_mark(mk, b)) {
      const uint32_t e = __ldg(L + kw + b);
      const uint32_t j = pbase + (e >> 5);
      const uint32_t code = e & 31u;
      double xb = __ldg(a.rx + j), yb = __ldg(a.ry + j), zb = __ldg(a.rz + j);
      if (code != static_cast<uint32_t>(kImageCenter)) {
        xb = image_coord(xb, S.period[0], static_cast<int>(code % 3u));
        yb = image_coord(yb, S.period[1], static_cast<int>((code / 3u) % 3u));
        zb = image_coord(zb, S.period[2], static_cast<int>(code / 9u));
      }
      const double dx = __dsub_rn(xb, xa), dy = __dsub_rn(yb, ya), dz = __dsub_rn(zb, za);
      const double d2 = norm2_rn(dx, dy, dz);
      if (!(d2 > 0.0 && d2 <= gp.rcut2)) continue;
      const uint32_t tb = a.ptype[j];
      if (tb >= static_cast<uint32_t>(gp.ntypes)) {
        atomicOr(flags, 1u);
        continue;
      }
      const double mb = gp.mass[tb];
      if (P == kFp64Exact) {
        const double r = __dsqrt_rn(d2);
        const double inv_r = __ddiv_rn(1.0, r);
        double de = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(gp.G, ma), mb), inv_r), inv_r);
        de = __dmul_rn(de, __ddiv_rn(1.0, r));
        fx = __dadd_rn(fx, __dmul_rn(de, dx));
        fy = __dadd_rn(fy, __dmul_rn(de, dy));
        fz = __dadd_rn(fz, __dmul_rn(de, dz));
        if (PE) {
          const double en = __dmul_rn(__dmul_rn(__dmul_rn(-gp.G, ma), mb), inv_r);
          pe = __dadd_rn(pe, __dmul_rn(0.5, en));
        }
      } else {
        const double r = sqrt(d2);
        const double inv_r3 = 1.0 / (d2 * r);
        const double gm = gp.G * ma * mb;
        const double de = gm * inv_r3;
        fx = fma(de, dx, fx);
        fy = fma(de, dy, fy);
        fz = fma(de, dz, fz);
        if (PE) pe -= 0.5 * gm / r;
      }
    }
  }
  a.fx[i] = fx;
  a.fy[i] = fy;
  a.fz[i] = fz;
  if (PE) a.pe[i] = accumulate ? a.pe[i] + pe : pe;
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
  if (precision == kFp64Exact) {
    if (with_pe) k_grav<kFp64Exact, true><<<g, threads, 0, stream>>>(ex.n_part, sys, st, a, sys_only, gp, accumulate, flags);
    else k_grav<kFp64Exact, false><<<g, threads, 0, stream>>>(ex.n_part, sys, st, a, sys_only, gp, accumulate, flags);
  } else {
    if (with_pe) k_grav<kFp64, true><<<g, threads, 0, stream>>>(ex.n_part, sys, st, a, sys_only, gp, accumulate, flags);
    else k_grav<kFp64, false><<<g, threads, 0, stream>>>(ex.n_part, sys, st, a, sys_only, gp, accumulate, flags);
  }
  return 1;
}

}  // namespace xnb
