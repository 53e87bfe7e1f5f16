// Shared pieces of the pair traversals over the per-particle lists (the
// Lennard-Jones kernels in xnb_step_kernels.cu, the other pair functors in
// xnb_functors.cu).
#pragma once

#include "xnb_internal.cuh"

namespace xnb {

// ---------------------------------------------------------------------------
// FP32 prefilter of a window of up to 128 list entries [kw, kend): bit k - kw of
// the four mask words is set for each entry whose FP32 distance to the particle
// (mirror paf) may lie within rc (pre_hi = rc^2 + proven margin); unmarked
// entries are provably beyond rc. Entries are read 8 at a time with two 16-byte
// loads (each list starts on a 32-byte boundary, its slot is a multiple of 8
// entries) and the 8 position gathers are independent of one another, so they
// are in flight together. Positions past kend gather the particle's own mirror.
struct Marks {
  uint32_t w[4];
};

__device__ __forceinline__ Marks prefilter_window(const uint32_t* __restrict__ L, uint32_t kw, uint32_t kend,
                                                  const float4* __restrict__ pf, uint32_t pbase, uint32_t self_e,
                                                  float4 paf, float pfx, float pfy, float pfz, float pre_hi) {
  Marks m{{0u, 0u, 0u, 0u}};
  for (uint32_t kb = kw; kb < kend; kb += 8) {
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
      if (code != static_cast<uint32_t>(kImageCenter)) {
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

}  // namespace xnb
