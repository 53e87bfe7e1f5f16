// Float <-> double conversions on integer operations, shared by the kernels and
// the host-side check (tests/test_widen.py compiles this header with g++).
#pragma once

#include <cstdint>

#ifndef __CUDACC__
#define XNB_HD inline
#else
#define XNB_HD __host__ __device__ __forceinline__
#endif

namespace xnb {

// Exact IEEE 754 binary32 -> binary64 widening done on the integer pipes, so
// that it costs no FP64 issue slot (GB300 issues FP64 at ~1/74 of the FP32/INT
// rate). The binary64 fields follow from the binary32 ones: sign kept, exponent
// re-biased from 127 to 1023 (+896), the 23 fraction bits placed at the top of
// the 52-bit fraction. A subnormal input m * 2^-149 is normalised first: with
// its leading bit at position 23 - s, m << s has an implicit-one form with the
// exponent field 1 and a re-bias of 896 - s. Zero keeps its sign; inf and NaN
// keep an all-ones exponent and their fraction bits.
XNB_HD uint64_t widen_f32_bits(uint32_t u) {
  uint32_t bias = 896u;
  const uint32_t m = u & 0x007fffffu;
  if ((u & 0x7f800000u) == 0u && m != 0u) {
#ifdef __CUDA_ARCH__
    const uint32_t s = static_cast<uint32_t>(__clz(m)) - 8u;
#else
    uint32_t s = 1u;
    while (!((m << s) & 0x00800000u)) ++s;
#endif
    u = (u & 0x80000000u) | 0x00800000u | ((m << s) & 0x007fffffu);
    bias -= s;
  }
  const uint32_t mag = u & 0x7fffffffu;
  uint32_t hi = (mag >> 3) + (bias << 20);
  if (mag >= 0x7f800000u) hi = (mag >> 3) | 0x7ff00000u;
  if (mag == 0u) hi = 0u;
  hi |= u & 0x80000000u;
  return (static_cast<uint64_t>(hi) << 32) | static_cast<uint64_t>(u << 29);
}

// The same widening with a short path for finite normal inputs and zeros (the
// FP32 pair-force factor of the mixed kernels): the exponent re-bias and the
// fraction move only. Subnormal, infinite and NaN inputs take widen_f32_bits.
XNB_HD uint64_t widen_f32_fast_bits(uint32_t u) {
  if ((u & 0x7f800000u) - 0x00800000u >= 0x7f000000u && (u & 0x7fffffffu) != 0u) return widen_f32_bits(u);
  const uint32_t mag = u & 0x7fffffffu;
  const uint32_t hi = (mag ? (mag >> 3) + 0x38000000u : 0u) | (u & 0x80000000u);
  return (static_cast<uint64_t>(hi) << 32) | static_cast<uint64_t>(u << 29);
}

// IEEE 754 binary64 -> binary32 conversion, round to nearest (ties to even), on
// integer operations (the hardware conversion occupies the FP64 pipe). With
// e the binary64 exponent field, the binary32 exponent field is e - 896; the 52
// fraction bits plus the implicit one are shifted right by 29 (by 29 + 1 - fe
// for a binary32 subnormal result) and rounded on the dropped bits; a carry out
// of the fraction moves into the exponent, and results at or above the largest
// exponent become infinities. Binary64 zeros and subnormals give a signed zero;
// infinities stay infinite and NaNs stay NaN (quiet bit set, top payload kept).
XNB_HD uint32_t narrow_f64_bits(uint64_t b) {
  const uint32_t sign = static_cast<uint32_t>(b >> 32) & 0x80000000u;
  const int e = static_cast<int>((b >> 52) & 0x7ffu);
  const uint64_t m = b & 0x000fffffffffffffull;
  if (e == 0x7ff) return sign | 0x7f800000u | (m ? (0x00400000u | static_cast<uint32_t>(m >> 29)) : 0u);
  if (e == 0) return sign;
  int fe = e - 896;
  int shift = 29;
  if (fe <= 0) {
    shift += 1 - fe;
    fe = 0;
    if (shift > 62) return sign;
  }
  const uint64_t mant = m | (1ull << 52);
  uint64_t q = mant >> shift;
  const uint64_t rem = mant & ((1ull << shift) - 1u);
  const uint64_t half = 1ull << (shift - 1);
  if (rem > half || (rem == half && (q & 1u))) ++q;
  const uint32_t r = fe == 0 ? static_cast<uint32_t>(q)
                             : (static_cast<uint32_t>(fe) << 23) + (static_cast<uint32_t>(q) - (1u << 23));
  if (fe >= 255 || r >= 0x7f800000u) return sign | 0x7f800000u;
  return sign | r;
}

}  // namespace xnb
