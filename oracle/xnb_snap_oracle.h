/*
 * SNAP (spectral neighbour analysis potential) for the CPU oracle -- test
 * infrastructure only. It restates the linear SNAP model of the reference's
 * snap_force_generic operator (contribs/md/snap/include/md/snap/snap_force.h:
 * 134-372, snap_force_op_coop.hxx:170-405, lib/sna.cpp) from its published
 * definition (Thompson et al., J. Comput. Phys. 285 (2015) 316; adjoint forces
 * of Wood and Thompson, J. Chem. Phys. 148 (2018) 241721), in the reference's
 * index conventions:
 *   * doubled labels: j = 2J, 0 <= ma, mb <= j; U^j is a (j+1) x (j+1) matrix
 *     stored row mb, column ma;
 *   * U^0 = 1, and for rows 2mb <= j
 *       U^j[mb][ma] = sqrt((j-ma)/(j-mb)) conj(a) U^{j-1}[mb][ma]
 *                   - sqrt(ma/(j-mb))     conj(b) U^{j-1}[mb][ma-1]
 *     with the Cayley-Klein parameters a = (z0 - i z)/r0, b = (y - i x)/r0,
 *     z0 = r cot(theta0), theta0 = (r - rmin0) rfac0 pi / (rcut - rmin0),
 *     r0 = sqrt(r^2 + z0^2) (snap_compute_ui.h:95-150); the other rows and the
 *     second half of an even j's middle row from
 *       U^j[j-mb][j-ma] = (-1)^(ma+mb) conj(U^j[mb][ma]);
 *   * Clebsch-Gordan coefficients C^{j m}_{j1 m1 j2 m2} by Racah's formula
 *     (sna.cpp:305-367 uses the equivalent quasi-binomial form of VMK 8.2.1(3));
 *   * Z^j_{j1 j2}[mb][ma] = sum C C U^{j1} U^{j2} over the m1 + m2 = m pairs,
 *     B_{j1 j2 j} = sum over all (mb, ma) of Re(conj(U^j) Z^j_{j1 j2}) for the
 *     triples j1 >= j2, j >= j1 in the reference's coefficient order
 *     (sna.cpp:236-259), E_i = beta_0 + sum_k beta_k (B_k - bzero_k);
 *   * forces through the adjoint Y^j = sum over (j1, j2) of beta_j Z^j_{j1 j2},
 *     beta_j taking the multiplicity and (j1+1)/(j+1) factors of the reference
 *     (snap_compute_yi.h:133-158), and dE_i/dr_ij = 2 sum over the unique half
 *     of Re(conj(dU^j) Y^j) (centre element of an even j weighted 1/2,
 *     snap_compute_deidrj.h:28-75), with the switching function
 *     sfac(r) = (cos(pi (r - rmin0)/(rcut - rmin0)) + 1)/2 and its derivative.
 * The energy uses the full-matrix definition of B and the forces the adjoint
 * form, so the finite-difference test of the forces checks the adjoint's
 * bookkeeping against the energy's definition.
 */
#pragma once

#include <array>
#include <cmath>
#include <complex>
#include <cstdint>
#include <vector>

namespace xo_snap {

using cplx = std::complex<double>;

// complex products written out (std::complex's operator* guards inf/nan through
// a library call, which dominates the oracle's time)
inline cplx cmul(const cplx& a, const cplx& b) {
  return cplx(a.real() * b.real() - a.imag() * b.imag(), a.real() * b.imag() + a.imag() * b.real());
}
inline cplx cmulc(const cplx& a, const cplx& b) {  // conj(a) * b
  return cplx(a.real() * b.real() + a.imag() * b.imag(), a.real() * b.imag() - a.imag() * b.real());
}

struct Spec {
  int twojmax = 0;
  double rcutfac = 0, rfac0 = 0.99363, rmin0 = 0;
  bool switchflag = true, bzeroflag = false, wselfallflag = false;
  int ntypes = 1;
  std::vector<double> radelem, wj;
  int ncoeffall = 0;             // per type, constant term included
  std::vector<double> coeff;     // ntypes * ncoeffall
  double energy_unit = 1.0;      // energies and forces are multiplied by it
};

class Calc {
 public:
  explicit Calc(const Spec& s) : S(s), J(s.twojmax) {
    for (int j1 = 0; j1 <= J; ++j1)
      for (int j2 = 0; j2 <= j1; ++j2)
        for (int j = j1 - j2; j <= std::min(J, j1 + j2); j += 2) {
          triples.push_back({j1, j2, j});
          if (j >= j1) bidx.push_back({j1, j2, j});
        }
    rootpq.assign((J + 1) * (J + 1), 0.0);
    for (int p = 1; p <= J; ++p)
      for (int q = 1; q <= J; ++q) rootpq[p * (J + 1) + q] = std::sqrt(static_cast<double>(p) / q);
    fact.assign(3 * J + 4, 1.0);
    for (size_t k = 1; k < fact.size(); ++k) fact[k] = fact[k - 1] * static_cast<double>(k);
    // Clebsch-Gordan tables per triple, [m1][m2]
    cgt.resize(triples.size());
    for (size_t t = 0; t < triples.size(); ++t) {
      const int j1 = triples[t][0], j2 = triples[t][1], j = triples[t][2];
      cgt[t].assign((j1 + 1) * (j2 + 1), 0.0);
      for (int m1 = 0; m1 <= j1; ++m1)
        for (int m2 = 0; m2 <= j2; ++m2) cgt[t][m1 * (j2 + 1) + m2] = cg(j1, j2, j, m1, m2);
    }
  }

  int ncoeff() const { return static_cast<int>(bidx.size()); }
  double cut(int ti, int tj) const { return (S.radelem[ti] + S.radelem[tj]) * S.rcutfac; }

  // Clebsch-Gordan <j1/2 m1', j2/2 m2' | j/2 m'> in doubled labels with offsets:
  // m1' = (2 m1 - j1)/2 etc., m = (2m1 - j1 + 2m2 - j2 + j)/2.
  double cg(int j1, int j2, int j, int m1, int m2) const {
    const int a2 = 2 * m1 - j1, b2 = 2 * m2 - j2, c2 = a2 + b2;
    if (c2 < -j || c2 > j) return 0.0;
    // Racah: sqrt((j+1) D(j1 j2 j)) sqrt(prod (j_i +- m_i)!) sum_k (-1)^k / (...)
    auto F = [&](int twice) { return fact[twice / 2]; };
    const double tri = F(j1 + j2 - j) * F(j1 - j2 + j) * F(-j1 + j2 + j) / F(j1 + j2 + j + 2);
    const double pre = std::sqrt((j + 1) * tri * F(j1 + a2) * F(j1 - a2) * F(j2 + b2) * F(j2 - b2) * F(j + c2) *
                                 F(j - c2));
    double sum = 0.0;
    for (int k = 0;; ++k) {
      const int t1 = (j1 + j2 - j) / 2 - k, t2 = (j1 - a2) / 2 - k, t3 = (j2 + b2) / 2 - k;
      const int t4 = (j - j2 + a2) / 2 + k, t5 = (j - j1 - b2) / 2 + k;
      if (t1 < 0 || t2 < 0 || t3 < 0) break;
      if (t4 < 0 || t5 < 0) continue;
      const double den = fact[k] * fact[t1] * fact[t2] * fact[t3] * fact[t4] * fact[t5];
      sum += ((k & 1) ? -1.0 : 1.0) / den;
    }
    return pre * sum;
  }

  // U^0..U^J of one neighbour (full matrices) and, if du, their derivatives
  // with respect to the neighbour's relative position, switching included.
  void ulist(double x, double y, double z, double rcut, double wj, std::vector<std::vector<cplx>>& U,
             std::vector<std::array<std::vector<cplx>, 3>>* dU) const {
    const double r = std::sqrt(x * x + y * y + z * z);
    const double rscale0 = S.rfac0 * M_PI / (rcut - S.rmin0);
    const double theta0 = (r - S.rmin0) * rscale0;
    const double z0 = r / std::tan(theta0);
    const double r0inv = 1.0 / std::sqrt(r * r + z0 * z0);
    const cplx a(z0 * r0inv, -z * r0inv), b(y * r0inv, -x * r0inv);
    const double u[3] = {x / r, y / r, z / r};
    // da/dx_k, db/dx_k
    const double dz0dr = z0 / r - (r * rscale0) * (r * r + z0 * z0) / (r * r);
    const double dr0invdr = -std::pow(r0inv, 3) * (r + z0 * dz0dr);
    cplx da[3], db[3];
    for (int k = 0; k < 3; ++k) {
      const double dr0 = dr0invdr * u[k];
      da[k] = cplx(dz0dr * u[k] * r0inv + z0 * dr0, -z * dr0 - (k == 2 ? r0inv : 0.0));
      db[k] = cplx(y * dr0 + (k == 1 ? r0inv : 0.0), -x * dr0 - (k == 0 ? r0inv : 0.0));
    }
    U.assign(J + 1, {});
    if (dU) dU->assign(J + 1, {});
    U[0] = {cplx(1.0, 0.0)};
    if (dU) (*dU)[0] = {std::vector<cplx>{0.0}, std::vector<cplx>{0.0}, std::vector<cplx>{0.0}};
    for (int j = 1; j <= J; ++j) {
      const int n = j + 1, np = j;
      U[j].assign(n * n, cplx(0.0));
      if (dU)
        for (int k = 0; k < 3; ++k) (*dU)[j][k].assign(n * n, cplx(0.0));
      for (int mb = 0; 2 * mb <= j; ++mb)
        for (int ma = 0; ma <= j; ++ma) {
          cplx v(0.0), dv[3] = {0.0, 0.0, 0.0};
          if (ma < j) {
            const double c = rootpq[(j - ma) * (J + 1) + (j - mb)];
            const cplx up = U[j - 1][mb * np + ma];
            v += c * cmulc(a, up);
            if (dU)
              for (int k = 0; k < 3; ++k)
                dv[k] += c * (cmulc(da[k], up) + cmulc(a, (*dU)[j - 1][k][mb * np + ma]));
          }
          if (ma > 0) {
            const double c = rootpq[ma * (J + 1) + (j - mb)];
            const cplx up = U[j - 1][mb * np + ma - 1];
            v -= c * cmulc(b, up);
            if (dU)
              for (int k = 0; k < 3; ++k)
                dv[k] -= c * (cmulc(db[k], up) + cmulc(b, (*dU)[j - 1][k][mb * np + ma - 1]));
          }
          U[j][mb * n + ma] = v;
          if (dU)
            for (int k = 0; k < 3; ++k) (*dU)[j][k][mb * n + ma] = dv[k];
        }
      // the remaining rows, and the second half of an even j's middle row
      for (int mb = 0; 2 * mb <= j; ++mb)
        for (int ma = 0; ma <= j; ++ma) {
          if (2 * mb == j && 2 * ma >= j) continue;  // middle row: sources are its first half
          const double s = ((ma + mb) & 1) ? -1.0 : 1.0;
          U[j][(j - mb) * n + (j - ma)] = s * std::conj(U[j][mb * n + ma]);
          if (dU)
            for (int k = 0; k < 3; ++k) (*dU)[j][k][(j - mb) * n + (j - ma)] = s * std::conj((*dU)[j][k][mb * n + ma]);
        }
    }
    // switching and weight: U <- w sfac U; dU <- w (dsfac U u + sfac dU)
    double sfac = 1.0, dsfac = 0.0;
    if (S.switchflag && r > S.rmin0) {
      const double f = M_PI / (rcut - S.rmin0);
      sfac = 0.5 * (std::cos((r - S.rmin0) * f) + 1.0);
      dsfac = -0.5 * std::sin((r - S.rmin0) * f) * f;
    }
    for (int j = 0; j <= J; ++j)
      for (size_t e = 0; e < U[j].size(); ++e) {
        if (dU)
          for (int k = 0; k < 3; ++k) (*dU)[j][k][e] = wj * (dsfac * U[j][e] * u[k] + sfac * (*dU)[j][k][e]);
        U[j][e] *= wj * sfac;
      }
  }

  // Z^j_{j1 j2}[mb][ma] from the summed U matrices (t: the triple's index).
  cplx zelem(const std::vector<std::vector<cplx>>& Ut, size_t t, int mb, int ma) const {
    const int j1 = triples[t][0], j2 = triples[t][1], j = triples[t][2];
    const std::vector<double>& C = cgt[t];
    // m1 + m2 = m in doubled offsets: m2 = (2m - j - 2m1 + j1 + j2)/2 within [0, j2]
    const int b_lo = std::max(0, (2 * mb - j - j2 + j1) / 2), b_hi = std::min(j1, (2 * mb - j + j2 + j1) / 2);
    const int a_lo = std::max(0, (2 * ma - j - j2 + j1) / 2), a_hi = std::min(j1, (2 * ma - j + j2 + j1) / 2);
    const cplx* U1 = Ut[j1].data();
    const cplx* U2 = Ut[j2].data();
    cplx s(0.0);
    for (int mb1 = b_lo; mb1 <= b_hi; ++mb1) {
      const int mb2 = (2 * mb - j - 2 * mb1 + j1 + j2) / 2;
      const double cb = C[mb1 * (j2 + 1) + mb2];
      cplx row(0.0);
      for (int ma1 = a_lo; ma1 <= a_hi; ++ma1) {
        const int ma2 = (2 * ma - j - 2 * ma1 + j1 + j2) / 2;
        row += C[ma1 * (j2 + 1) + ma2] * cmul(U1[mb1 * (j1 + 1) + ma1], U2[mb2 * (j2 + 1) + ma2]);
      }
      s += cb * row;
    }
    return s;
  }

  // One atom of type ti with neighbours at dr[n] (r_j - r_i, all inside their
  // cutoffs) of types tj[n]. Returns E_i in potential units times energy_unit if
  // want_e (0 otherwise); fills fij[n] = dE_i/d(dr_n) times energy_unit.
  double atom(int ti, const std::vector<std::array<double, 3>>& dr, const std::vector<int>& tj, bool want_e,
              std::vector<std::array<double, 3>>& fij) const {
    const size_t nn = dr.size();
    std::vector<std::vector<cplx>> Ut(J + 1);
    for (int j = 0; j <= J; ++j) {
      Ut[j].assign((j + 1) * (j + 1), cplx(0.0));
      for (int m = 0; m <= j; ++m) Ut[j][m * (j + 1) + m] = 1.0;  // wself (one element)
    }
    std::vector<std::vector<std::vector<cplx>>> Un(nn);
    std::vector<std::vector<std::array<std::vector<cplx>, 3>>> dUn(nn);
    for (size_t q = 0; q < nn; ++q) {
      ulist(dr[q][0], dr[q][1], dr[q][2], cut(ti, tj[q]), S.wj[tj[q]], Un[q], &dUn[q]);
      for (int j = 0; j <= J; ++j)
        for (size_t e = 0; e < Ut[j].size(); ++e) Ut[j][e] += Un[q][j][e];
    }
    const double* beta = S.coeff.data() + static_cast<size_t>(ti) * S.ncoeffall + 1;
    double e = 0.0;
    if (want_e) {
      e = S.coeff[static_cast<size_t>(ti) * S.ncoeffall];
      for (size_t k = 0; k < bidx.size(); ++k) {
        const int j1 = bidx[k][0], j2 = bidx[k][1], j = bidx[k][2];
        const size_t t = triple_index(j1, j2, j);
        double B = 0.0;
        for (int mb = 0; mb <= j; ++mb)
          for (int ma = 0; ma <= j; ++ma)
            B += cmulc(Ut[j][mb * (j + 1) + ma], zelem(Ut, t, mb, ma)).real();
        if (S.bzeroflag) B -= static_cast<double>(j + 1);
        e += beta[k] * B;
      }
      e *= S.energy_unit;
    }
    // Y on the unique half of each U^j
    auto bindex = [&](int a, int b, int c) {
      for (size_t k = 0; k < bidx.size(); ++k)
        if (bidx[k][0] == a && bidx[k][1] == b && bidx[k][2] == c) return static_cast<int>(k);
      return -1;
    };
    std::vector<std::vector<cplx>> Y(J + 1);
    for (int j = 0; j <= J; ++j) Y[j].assign((j + 1) * (j + 1), cplx(0.0));
    for (size_t ti3 = 0; ti3 < triples.size(); ++ti3) {
      const int j1 = triples[ti3][0], j2 = triples[ti3][1], j = triples[ti3][2];
      double bj;
      if (j >= j1) {
        const double bb = beta[bindex(j1, j2, j)];
        bj = (j1 == j) ? ((j2 == j) ? 3.0 * bb : 2.0 * bb) : bb;
      } else if (j >= j2) {
        const double bb = beta[bindex(j, j2, j1)];
        bj = (j2 == j) ? 2.0 * bb : bb;
      } else {
        bj = beta[bindex(j2, j, j1)];
      }
      if (j1 > j) bj *= (j1 + 1) / (j + 1.0);
      for (int mb = 0; 2 * mb <= j; ++mb)
        for (int ma = 0; ma <= j; ++ma) {
          if (2 * mb == j && ma > mb) continue;
          Y[j][mb * (j + 1) + ma] += bj * zelem(Ut, ti3, mb, ma);
        }
    }
    fij.assign(nn, {0.0, 0.0, 0.0});
    for (size_t q = 0; q < nn; ++q) {
      double f[3] = {0.0, 0.0, 0.0};
      for (int j = 0; j <= J; ++j)
        for (int mb = 0; 2 * mb <= j; ++mb)
          for (int ma = 0; ma <= j; ++ma) {
            if (2 * mb == j && ma > mb) continue;
            const double w = (2 * mb == j && ma == mb) ? 0.5 : 1.0;
            const cplx y = Y[j][mb * (j + 1) + ma];
            for (int k = 0; k < 3; ++k) {
              const cplx d = dUn[q][j][k][mb * (j + 1) + ma];
              f[k] += w * (d.real() * y.real() + d.imag() * y.imag());
            }
          }
      for (int k = 0; k < 3; ++k) fij[q][k] = 2.0 * f[k] * S.energy_unit;
    }
    return e;
  }

 private:
  size_t triple_index(int j1, int j2, int j) const {
    for (size_t t = 0; t < triples.size(); ++t)
      if (triples[t][0] == j1 && triples[t][1] == j2 && triples[t][2] == j) return t;
    return 0;
  }
  Spec S;
  int J;
  std::vector<std::array<int, 3>> triples, bidx;
  std::vector<double> rootpq, fact;
  std::vector<std::vector<double>> cgt;
};

}  // namespace xo_snap
