// SNAP (snap_force_generic) on the GPU: tables built on the host and the
// per-atom kernel (xnb_snap.cu).
#pragma once

#include <string>
#include <vector>

#include "xnb_launch.cuh"

struct xnb_snap_params;

namespace xnb {

constexpr int kSnapMaxTwoJ = 10;
constexpr int kSnapMaxTypes = 16;
constexpr int kSnapMaxNbr = 128;  // environment size per atom
constexpr int kSnapWarps = 4;     // warps per atom (one CTA)
constexpr int kSnapThreads = kSnapWarps * 32;
constexpr int kSnapMaxGroup = 32; // neighbours whose U levels are held at once

// One element Z^j_{j1 j2}[mb][ma] on the unique half of U^j (rows 2 mb < j, and
// the first j/2 + 1 elements of an even j's middle row), with the index ranges
// of its Clebsch-Gordan sums: m1 from ma1min (mb1min), m2 from ma2max (mb2max)
// downwards, na (nb) terms (the reference's SNA_ZINDICES, sna.cpp:262-300).
struct SnapZ {
  uint8_t j1, j2, j, ma1min, ma2max, na, mb1min, mb2max, nb, pad;
  uint16_t y;   // unique-layout index of (j, mb, ma): Y and the energy's U
  uint16_t uf;  // full-layout index of (j, mb, ma)
  uint16_t pad2;
  uint32_t cg;  // offset of the (j1, j2, j) Clebsch-Gordan block [m1][m2]
};

struct SnapArgs {
  int twojmax, nz, nu_unique, nu_full, ntypes, switchflag;
  int group, group_f;          // neighbours per round (shared-memory budget), FP64 / FP32 kernels
  int ublk[kSnapMaxTwoJ + 2];  // first unique-layout index of level j
  int fblk[kSnapMaxTwoJ + 2];  // first full-layout index of level j
  double rcutfac, rfac0, rmin0;
  double radelem[kSnapMaxTypes], wj[kSnapMaxTypes];
  double e0[kSnapMaxTypes];    // beta_0 - sum_k beta_k bzero_k per type
  double energy_unit;
  const double* rootpq;        // [(J+1)^2], sqrt(p/q)
  const double* cg;
  const SnapZ* z;              // nz
  const double* zbeta;         // [ntypes][nz] multiplier of Z into Y
  const double* zener;         // [ntypes][nz] 2 w beta_k of canonical entries, else 0
  const float *rootpq_f, *cg_f, *zbeta_f, *zener_f;  // the same tables in FP32 (mixed path)
  size_t smem_bytes, smem_bytes_f;
};

// Host tables for one potential; device arrays are owned by `allocs`.
int snap_build(const xnb_snap_params& p, int device, SnapArgs& t, std::vector<void*>& allocs, std::string& err);

// zero_particle_force (unless accumulate) + snap_force_generic (+ the division by
// the system's mass when it divides) for the systems selected by sys_only.
// mixed: FP32 arithmetic for U, Z, Y and the adjoint (geometry, switching and
// the force sums in FP64).
// flags receives bit 0 for a particle type without coefficients, bit 1 for an
// environment larger than kSnapMaxNbr.
int launch_snap(const Extent& ex, const SysDesc* sys, const SysState* st, const DevArrays& a, const SnapArgs& t,
                int sys_only, bool with_pe, bool accumulate, bool mixed, unsigned int* flags, cudaStream_t stream);

}  // namespace xnb
