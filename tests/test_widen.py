"""The force kernels widen the FP32 pair-force factor to FP64 with integer
operations (exanbody_gb300/csrc/xnb_widen.h). The same header compiled for the
host must agree bit for bit with the C++ float -> double conversion: every
subnormal, every exponent with a stride through the fraction, zeros, infinities
and NaNs (NaN: any NaN with the same sign); its short path for normal inputs
and zeros (widen_f32_fast_bits) must give the same bits as the general one."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "exanbody_gb300", "csrc")

CHECK = r"""
#include <cstdio>
#include <cstring>
#include "xnb_widen.h"
static unsigned long long bad = 0, tested = 0;
static void one(uint32_t u) {
  float f; std::memcpy(&f, &u, 4);
  const double d = static_cast<double>(f);
  uint64_t want; std::memcpy(&want, &d, 8);
  const uint64_t got = xnb::widen_f32_bits(u);
  ++tested;
  if (xnb::widen_f32_fast_bits(u) != got) {  // the short path gives the same bits
    if (bad < 5) std::printf("fast path differs u=%08x\n", u);
    ++bad;
  }
  if ((u & 0x7f800000u) == 0x7f800000u && (u & 0x7fffffu)) {
    const bool ok = (got & 0x7ff0000000000000ull) == 0x7ff0000000000000ull && (got & 0xfffffffffffffull) &&
                    (got >> 63) == (u >> 31);
    bad += !ok;
    return;
  }
  if (got != want) {
    if (bad < 5) std::printf("mismatch u=%08x got=%016llx want=%016llx\n", u, (unsigned long long)got,
                             (unsigned long long)want);
    ++bad;
  }
}
int main() {
  for (uint32_t sign = 0; sign < 2; ++sign) {
    for (uint32_t m = 0; m < (1u << 23); ++m) one((sign << 31) | m);             // zero and every subnormal
    for (uint32_t e = 1; e < 256; ++e)
      for (uint32_t m = 0; m < (1u << 23); m += 61) one((sign << 31) | (e << 23) | m);
    for (uint32_t e = 1; e < 256; ++e) one((sign << 31) | (e << 23) | 0x7fffffu);
  }
  std::printf("tested %llu mismatches %llu\n", tested, bad);
  return bad != 0;
}
"""


def test_widen_matches_cast():
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "widen_check.cpp")
        exe = os.path.join(d, "widen_check")
        with open(src, "w") as f:
            f.write(CHECK)
        subprocess.check_call([gxx, "-O2", "-std=c++17", "-I", CSRC, src, "-o", exe])
        out = subprocess.run([exe], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout + out.stderr
        assert "mismatches 0" in out.stdout


NARROW = r"""
#include <cstdio>
#include <cstring>
#include <random>
#include "xnb_widen.h"
static unsigned long long bad = 0, tested = 0;
static void one(uint64_t b) {
  double d; std::memcpy(&d, &b, 8);
  const float f = static_cast<float>(d);
  uint32_t want; std::memcpy(&want, &f, 4);
  const uint32_t got = xnb::narrow_f64_bits(b);
  ++tested;
  if (d != d) {  // NaN: any NaN with the same sign
    const bool ok = (got & 0x7f800000u) == 0x7f800000u && (got & 0x7fffffu) && (got >> 31) == (b >> 63);
    bad += !ok;
    return;
  }
  if (got != want) {
    if (bad < 5) std::printf("mismatch b=%016llx got=%08x want=%08x\n", (unsigned long long)b, got, want);
    ++bad;
  }
}
int main() {
  std::mt19937_64 rng(2024);
  for (uint64_t sign = 0; sign < 2; ++sign) {
    // every binary64 exponent, with fractions around every rounding boundary of the
    // 29 dropped bits (exact ties, one below, one above) and random fractions
    for (uint64_t e = 0; e < 2048; ++e) {
      const uint64_t base = (sign << 63) | (e << 52);
      for (uint64_t top = 0; top < 64; ++top) {
        const uint64_t hi = (top * 0x1ffffull) << 29;  // spread of kept fraction bits
        for (uint64_t r : {0ull, 1ull, (1ull << 28) - 1, 1ull << 28, (1ull << 28) + 1, (1ull << 29) - 1})
          one(base | ((hi | r) & 0xfffffffffffffull));
      }
      for (int k = 0; k < 200; ++k) one(base | (rng() & 0xfffffffffffffull));
      // binary32-subnormal results need more dropped bits: ties at every shift
      for (int s = 29; s < 63; ++s)
        for (uint64_t r : {(1ull << (s - 1)) - 1, 1ull << (s - 1), (1ull << (s - 1)) + 1, (3ull << (s - 1))})
          one(base | (r & 0xfffffffffffffull));
    }
    for (int k = 0; k < 2000000; ++k) one((sign << 63) | (rng() >> 1));
  }
  std::printf("tested %llu mismatches %llu\n", tested, bad);
  return bad != 0;
}
"""


def test_narrow_matches_cast():
    """binary64 -> binary32 on integer operations equals the C++ conversion
    (round to nearest even) for every exponent, rounding ties at every shift
    (binary32 subnormals included), overflow, zeros, infinities and NaNs."""
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "narrow_check.cpp")
        exe = os.path.join(d, "narrow_check")
        with open(src, "w") as f:
            f.write(NARROW)
        subprocess.check_call([gxx, "-O2", "-std=c++17", "-I", CSRC, src, "-o", exe])
        out = subprocess.run([exe], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout + out.stderr
        assert "mismatches 0" in out.stdout
