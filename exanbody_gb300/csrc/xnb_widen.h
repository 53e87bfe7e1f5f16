// Float-to-double widening on integer operations, shared by the force kernels
// and the host-side check (tests/test_widen.py compiles this header with g++).
#pragma once

#include <cstdint>

#ifndef __CUDACC__
#define XNB_HD inline
#else
#define XNB_HD __host__ __device__ __forceinline__
#endif

namespace xnb {

// Exact IEEE 754 binary32 -> binary64 widening done on the integer pipes, so
// that it costs no FP64 issue slot (GB300 issues FP64 at ~1/40 of the FP32/INT
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


}  // namespace xnb
