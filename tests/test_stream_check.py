"""The chunk-neighbour stream checker (exanbody_gb300/csrc/xnb_stream.h) on the host.

A C++ harness builds a small periodic system, encodes its neighbour streams in the
reference format with an independent brute-force encoder (offset tables 0, 1, 2),
checks that verify_cell_stream reports nothing on them, then corrupts streams at
random (one u16 changed, or the stream cut short or extended) and checks that the
checker never reads out of bounds (AddressSanitizer / UBSan) and flags nearly
every corruption. The GPU runs the same checker in xnb_verify_chunk_neighbors."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "exanbody_gb300", "csrc")

HARNESS = r"""
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>
#include "xnb_stream.h"
using namespace xnb;

struct Sys {
  int D[3];
  double cs, nbh, L[3];
  std::vector<std::vector<double>> x, y, z;  // per interior cell
  int cell(int i, int j, int k) const { return (k * D[1] + j) * D[0] + i; }
  bool keeps(double gx, double gy, double gz) const {
    return gx >= -nbh && gx <= L[0] + nbh && gy >= -nbh && gy <= L[1] + nbh && gz >= -nbh && gz <= L[2] + nbh;
  }
  // members of the (interior or ghost) cell at relative (di, dj, dk) from (ci, cj, ck)
  void members(int ci, int cj, int ck, int di, int dj, int dk, std::vector<double>& mx, std::vector<double>& my,
               std::vector<double>& mz) const {
    int n3[3] = {ci + di, cj + dj, ck + dk};
    double sh[3] = {0, 0, 0};
    bool img = false;
    for (int a = 0; a < 3; ++a) {
      if (n3[a] < 0) { n3[a] += D[a]; sh[a] = -L[a]; img = true; }
      else if (n3[a] >= D[a]) { n3[a] -= D[a]; sh[a] = L[a]; img = true; }
    }
    const int c = cell(n3[0], n3[1], n3[2]);
    mx.clear(); my.clear(); mz.clear();
    for (size_t q = 0; q < x[c].size(); ++q) {
      const double gx = x[c][q] + sh[0], gy = y[c][q] + sh[1], gz = z[c][q] + sh[2];
      if (img && !keeps(gx, gy, gz)) continue;
      mx.push_back(gx); my.push_back(gy); mz.push_back(gz);
    }
  }
};

struct View {
  const Sys* S;
  int ci, cj, ck;
  double nbh2;
  uint32_t size_of(int di, int dj, int dk) const {
    std::vector<double> a, b, c;
    S->members(ci, cj, ck, di, dj, dk, a, b, c);
    return static_cast<uint32_t>(a.size());
  }
  bool pair_d2(uint32_t pa, int di, int dj, int dk, uint32_t pb, double& d2) const {
    std::vector<double> a, b, c;
    S->members(ci, cj, ck, di, dj, dk, a, b, c);
    if (pb >= a.size()) return false;
    const int own = S->cell(ci, cj, ck);
    const double dx = a[pb] - S->x[own][pa], dy = b[pb] - S->y[own][pa], dz = c[pb] - S->z[own][pa];
    d2 = (dx * dx + dy * dy) + dz * dz;
    return true;
  }
  uint32_t exhaustive_count(uint32_t pa) const {
    uint32_t n = 0;
    for (int dk = -1; dk <= 1; ++dk)
      for (int dj = -1; dj <= 1; ++dj)
        for (int di = -1; di <= 1; ++di) {
          std::vector<double> a, b, c;
          S->members(ci, cj, ck, di, dj, dk, a, b, c);
          for (size_t q = 0; q < a.size(); ++q) {
            if (di == 0 && dj == 0 && dk == 0 && q == pa) continue;
            double d2;
            pair_d2(pa, di, dj, dk, static_cast<uint32_t>(q), d2);
            if (d2 > 0.0 && d2 <= nbh2) ++n;
          }
        }
    return n;
  }
};

// independent brute-force encoder of one cell's stream
std::vector<uint16_t> encode(const Sys& S, int ci, int cj, int ck, int T) {
  const int c = S.cell(ci, cj, ck);
  const size_t na = S.x[c].size();
  std::vector<uint16_t> out;
  if (na == 0) return out;
  const size_t table = T >= 1 ? (na * T + 1) * 2 : 0;
  out.assign(table, 0);
  View v{&S, ci, cj, ck, S.nbh * S.nbh};
  for (size_t pa = 0; pa < na; ++pa) {
    const uint32_t off = static_cast<uint32_t>(out.size() - table + T);
    if (T >= 1) { out[pa * 2] = off & 0xFFFF; out[pa * 2 + 1] = off >> 16; }
    const size_t gpos = out.size();
    out.push_back(0);
    uint32_t lower = 0;
    for (int dk = -1; dk <= 1; ++dk)
      for (int dj = -1; dj <= 1; ++dj)
        for (int di = -1; di <= 1; ++di) {
          std::vector<uint16_t> hits;
          const uint32_t n = v.size_of(di, dj, dk);
          for (uint32_t q = 0; q < n; ++q) {
            if (di == 0 && dj == 0 && dk == 0 && q == pa) continue;
            double d2;
            v.pair_d2(static_cast<uint32_t>(pa), di, dj, dk, q, d2);
            if (d2 > 0.0 && d2 <= v.nbh2) hits.push_back(static_cast<uint16_t>(q));
          }
          if (hits.empty()) continue;
          const int rel = dk * 9 + dj * 3 + di;
          for (uint16_t h : hits) if (rel < 0 || (rel == 0 && h < pa)) ++lower;
          ++out[gpos];
          out.push_back(encode_cell_rel(di, dj, dk));
          out.push_back(static_cast<uint16_t>(hits.size()));
          out.insert(out.end(), hits.begin(), hits.end());
        }
    if (T == 2) { out[(na + 1 + pa) * 2] = lower & 0xFFFF; out[(na + 1 + pa) * 2 + 1] = lower >> 16; }
  }
  if (T >= 1) {
    const uint32_t off = static_cast<uint32_t>(out.size() - table + T);
    out[na * 2] = off & 0xFFFF; out[na * 2 + 1] = off >> 16;
  }
  return out;
}

unsigned long long total(const StreamCounts& c) { return c.format + c.order + c.self + c.range + c.far + c.missing; }

int main() {
  std::mt19937_64 rng(12345);
  int bad = 0;
  unsigned long long trials = 0, detected = 0;
  const int shapes[2][3] = {{3, 3, 3}, {2, 3, 4}};
  for (int sh = 0; sh < 2; ++sh) {
    Sys S;
    for (int a = 0; a < 3; ++a) S.D[a] = shapes[sh][a];
    S.cs = 1.0; S.nbh = 0.95;
    for (int a = 0; a < 3; ++a) S.L[a] = S.D[a] * S.cs;
    const int nc = S.D[0] * S.D[1] * S.D[2];
    S.x.resize(nc); S.y.resize(nc); S.z.resize(nc);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    std::uniform_int_distribution<int> np(0, 7);
    for (int k = 0; k < S.D[2]; ++k)
      for (int j = 0; j < S.D[1]; ++j)
        for (int i = 0; i < S.D[0]; ++i) {
          const int c = S.cell(i, j, k), n = np(rng);
          for (int q = 0; q < n; ++q) {
            S.x[c].push_back((i + u(rng)) * S.cs);
            S.y[c].push_back((j + u(rng)) * S.cs);
            S.z[c].push_back((k + u(rng)) * S.cs);
          }
        }
    for (int T = 0; T <= 2; ++T)
      for (int k = 0; k < S.D[2]; ++k)
        for (int j = 0; j < S.D[1]; ++j)
          for (int i = 0; i < S.D[0]; ++i) {
            const int c = S.cell(i, j, k);
            const uint32_t na = static_cast<uint32_t>(S.x[c].size());
            View v{&S, i, j, k, S.nbh * S.nbh};
            const std::vector<uint16_t> good = encode(S, i, j, k, T);
            StreamCounts c0{0, 0, 0, 0, 0, 0};
            verify_cell_stream(v, good.data(), good.size(), na, T, c0);
            if (total(c0)) { std::printf("clean stream flagged: shape %d T %d cell %d\n", sh, T, c); ++bad; }
            if (good.empty()) continue;
            for (int t = 0; t < 60; ++t) {
              std::vector<uint16_t> s = good;
              size_t len = s.size();
              const int kind = static_cast<int>(rng() % 4);
              if (kind == 0) {          // one word set to a random value
                const size_t at = rng() % s.size();
                const uint16_t nv = static_cast<uint16_t>(rng());
                if (nv == s[at]) continue;
                s[at] = nv;
              } else if (kind == 1) {   // one word off by one
                const size_t at = rng() % s.size();
                s[at] = static_cast<uint16_t>(s[at] + ((rng() & 1) ? 1 : -1));
              } else if (kind == 2) {   // cut short
                len = rng() % s.size();
              } else {                  // trailing garbage
                s.push_back(static_cast<uint16_t>(rng()));
                len = s.size();
              }
              // a heap copy of exactly len words, so any read past it is caught
              std::vector<uint16_t> exact(s.begin(), s.begin() + static_cast<long>(len));
              StreamCounts ck{0, 0, 0, 0, 0, 0};
              verify_cell_stream(v, exact.empty() ? nullptr : exact.data(), exact.size(), na, T, ck);
              ++trials;
              if (total(ck)) ++detected;
            }
          }
  }
  std::printf("trials %llu detected %llu bad %d\n", trials, detected, bad);
  return bad != 0 || detected < trials * 97 / 100;
}
"""


def test_stream_checker_on_host():
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "stream_check.cpp")
        exe = os.path.join(d, "stream_check")
        with open(src, "w") as f:
            f.write(HARNESS)
        flags = ["-O1", "-g", "-std=c++17", "-fsanitize=address,undefined", "-fno-sanitize-recover=all"]
        if subprocess.call([gxx, *flags, "-I", CSRC, src, "-o", exe]) != 0:
            # some images lack the sanitizer runtimes: run the same harness unsanitised
            subprocess.check_call([gxx, "-O1", "-std=c++17", "-I", CSRC, src, "-o", exe])
        out = subprocess.run([exe], capture_output=True, text=True, timeout=600)
        assert out.returncode == 0, out.stdout + out.stderr
        assert "bad 0" in out.stdout
