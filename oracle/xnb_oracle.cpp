/*
 * CPU oracle for the exaNBody particle hot path (test infrastructure only; see
 * xnb_oracle.h). Built twice: with -ffp-contract=off as the parity checker, and
 * with OpenMP for the timed CPU baseline. Only tests/, bench.py's CPU-baseline
 * leg and __graft_entry__.smoke() load it.
 *
 * Reference citations are paths inside the exaNBody source tree.
 *
 * Arithmetic conventions where the reference delegates to its absent onika
 * dependency (stated here because they fix the bits):
 *   norm2(v) = (v.x*v.x + v.y*v.y) + v.z*v.z, evaluated left to right, no FMA;
 *   Mat3d(identity) * v == v exactly (1*x + 0*y + 0*z rounds to x);
 *   IJK * double promotes each index to double, then multiplies.
 */
#include "xnb_oracle.h"
#include "xnb_snap_oracle.h"

#include <algorithm>
#include <array>
#include <memory>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct V3 { double x, y, z; };
struct L3 { long i, j, k; };

inline double norm2(double x, double y, double z) { return (x * x + y * y) + z * z; }

struct Cell {
  std::vector<double> rx, ry, rz, vx, vy, vz, fx, fy, fz, pe;
  std::vector<uint64_t> id;
  std::vector<uint8_t> type;  // particle type (field::type); 0 unless set
  size_t size() const { return rx.size(); }
  void clear() {
    rx.clear(); ry.clear(); rz.clear(); vx.clear(); vy.clear(); vz.clear();
    fx.clear(); fy.clear(); fz.clear(); pe.clear(); id.clear(); type.clear();
  }
  void push(double x, double y, double z, double a, double b, double c, double f0, double f1,
            double f2, uint64_t i, uint8_t t = 0) {
    rx.push_back(x); ry.push_back(y); rz.push_back(z);
    vx.push_back(a); vy.push_back(b); vz.push_back(c);
    fx.push_back(f0); fy.push_back(f1); fz.push_back(f2);
    pe.push_back(0.0); id.push_back(i); type.push_back(t);
  }
  void copy_from(size_t dst, const Cell& s, size_t src) {
    rx[dst] = s.rx[src]; ry[dst] = s.ry[src]; rz[dst] = s.rz[src];
    vx[dst] = s.vx[src]; vy[dst] = s.vy[src]; vz[dst] = s.vz[src];
    fx[dst] = s.fx[src]; fy[dst] = s.fy[src]; fz[dst] = s.fz[src];
    pe[dst] = s.pe[src]; id[dst] = s.id[src]; type[dst] = s.type[src];
  }
  void resize(size_t n) {
    rx.resize(n); ry.resize(n); rz.resize(n); vx.resize(n); vy.resize(n); vz.resize(n);
    fx.resize(n); fy.resize(n); fz.resize(n); pe.resize(n); id.resize(n); type.resize(n);
  }
  void swap_p(size_t a, size_t b) {
    std::swap(rx[a], rx[b]); std::swap(ry[a], ry[b]); std::swap(rz[a], rz[b]);
    std::swap(vx[a], vx[b]); std::swap(vy[a], vy[b]); std::swap(vz[a], vz[b]);
    std::swap(fx[a], fx[b]); std::swap(fy[a], fy[b]); std::swap(fz[a], fz[b]);
    std::swap(pe[a], pe[b]); std::swap(id[a], id[b]); std::swap(type[a], type[b]);
  }
};

/* One ghost cell fill (GhostCellSendScheme, ghosts_comm_scheme.h:141-147). */
struct GhostSend {
  long src_cell;
  long dst_cell;
  uint32_t flags;
  std::vector<uint32_t> particle_i;
};

constexpr uint32_t SHIFT_X = 1u << 0, SIDE_X = 1u << 2;
constexpr uint32_t SHIFT_Y = 1u << 3, SIDE_Y = 1u << 5;
constexpr uint32_t SHIFT_Z = 1u << 6, SIDE_Z = 1u << 8;

/* GhostBoundaryModifier::apply_coord_modifier (ghosts_comm_scheme.h:76-81), periodic branch. */
inline double apply_coord_modifier(double x, double rmin, double rmax, uint32_t f) {
  if (f & 1u) return x + ((f & 4u) ? 1.0 : -1.0) * (rmax - rmin);
  return x;
}

/* restore_u32_double / encode_double_u32 (core/include/exanb/core/backup_r.h:31-51). */
inline double restore_u32_double(uint32_t x, double o, double r) {
  return o + (static_cast<double>(x) * r) / static_cast<double>(1ull << 32);
}
inline uint32_t encode_double_u32(double x, double o, double r) {
  const double xo = x - o;
  int64_t a = static_cast<int64_t>((xo * static_cast<double>(1ull << 32)) / r);
  if (a < 0) a = 0;
  if (a > static_cast<int64_t>(UINT32_MAX)) a = static_cast<int64_t>(UINT32_MAX);
  const uint32_t xa = static_cast<uint32_t>(a);
  const uint32_t xb = xa - 1u;
  const uint32_t xc = xa + 1u;
  const double ea = std::fabs(restore_u32_double(xa, o, r) - x);
  const double eb = std::fabs(restore_u32_double(xb, o, r) - x);
  const double ec = std::fabs(restore_u32_double(xc, o, r) - x);
  if (eb < ea) return xb;
  if (ec < ea) return xc;
  return xa;
}

/* encode_cell_index (particle_neighbors/include/exanb/particle_neighbors/chunk_neighbors.h:137-150). */
inline uint16_t encode_cell_index(long di, long dj, long dk) {
  uint16_t c = static_cast<uint16_t>(dk + 16);
  c = static_cast<uint16_t>(c << 5);
  c = static_cast<uint16_t>(c + dj + 16);
  c = static_cast<uint16_t>(c << 5);
  c = static_cast<uint16_t>(c + di + 16);
  return c;
}

/* sub_grid_size (amr/include/exanb/amr/amr_grid_algorithm.h:66-78), MAX 16, no po2 restriction. */
inline long sub_grid_size(size_t n, double avg_density) {
  if (n == 0) return 0;
  const double nbiased = static_cast<double>(n) / avg_density;
  const double side = std::cbrt(nbiased);
  if (side < 2.0) return 1;
  const long iside = static_cast<long>(std::floor(side));
  return std::min(iside, 16L);
}

inline long pmod(long i, long n) { return ((i % n) + n) % n; }

}  // namespace

struct xo_sys {
  xo_params p{};
  long D[3]{};      // domain grid dims
  long G[3]{};      // grid dims including one ghost layer per side
  long gl = 1;
  double nbh_dist = 0, nbh2 = 0, rcut2 = 0, max_displ = 0, ghost_dist = 0;
  double e_shift = 0;
  std::vector<Cell> cells;                       // G cells
  std::vector<std::vector<uint32_t>> backup;     // per grid cell
  std::vector<std::vector<uint16_t>> streams;    // per grid cell (interior filled)
  std::vector<GhostSend> ghosts;
  int64_t rebuilds = 0;
  bool ready = false;
  std::unique_ptr<xo_snap::Calc> snap;  // set: the force chain is snap_force_generic
  bool snap_energy = false;

  long gidx(long i, long j, long k) const { return (k * G[1] + j) * G[0] + i; }
  L3 gloc(long c) const { return L3{c % G[0], (c / G[0]) % G[1], c / (G[0] * G[1])}; }
  bool is_ghost(const L3& l) const {
    return l.i < gl || l.j < gl || l.k < gl || l.i >= G[0] - gl || l.j >= G[1] - gl || l.k >= G[2] - gl;
  }
  /* Grid::cell_position (core/include/exanb/core/grid.h:114-117), offset = -gl. */
  V3 cell_position(const L3& l) const {
    return V3{p.origin[0] + static_cast<double>(l.i - gl) * p.cell_size,
              p.origin[1] + static_cast<double>(l.j - gl) * p.cell_size,
              p.origin[2] + static_cast<double>(l.k - gl) * p.cell_size};
  }
  long interior_to_grid(long c) const {
    const long i = c % D[0], j = (c / D[0]) % D[1], k = c / (D[0] * D[1]);
    return gidx(i + gl, j + gl, k + gl);
  }

  /* domain_periodic_location (core/include/exanb/core/domain.h:160-191); returns the
   * domain cell location and wraps r in place. */
  L3 domain_periodic_location(V3& r) const {
    const double relx = r.x - p.origin[0], rely = r.y - p.origin[1], relz = r.z - p.origin[2];
    L3 loc{static_cast<long>(std::floor(relx / p.cell_size)),
           static_cast<long>(std::floor(rely / p.cell_size)),
           static_cast<long>(std::floor(relz / p.cell_size))};
    if (loc.i < 0 || loc.i >= D[0]) {
      const long old = loc.i;
      loc.i = pmod(loc.i, D[0]);
      r.x += static_cast<double>(loc.i - old) * p.cell_size;
    }
    if (loc.j < 0 || loc.j >= D[1]) {
      const long old = loc.j;
      loc.j = pmod(loc.j, D[1]);
      r.y += static_cast<double>(loc.j - old) * p.cell_size;
    }
    if (loc.k < 0 || loc.k >= D[2]) {
      const long old = loc.k;
      loc.k = pmod(loc.k, D[2]);
      r.z += static_cast<double>(loc.k - old) * p.cell_size;
    }
    return loc;
  }

  /* move_particles_across_cells (grid_cell_particles/include/exanb/grid_cell_particles/
   * move_particles_across_cells.h:104-229), single rank: every destination is an
   * interior cell because domain_periodic_location wraps. Arrivals are appended in
   * (source cell, source index) order, the order one OpenMP thread produces. */
  int move_particles() {
    const size_t n_cells = cells.size();
    std::vector<std::vector<uint32_t>> removed(n_cells);
    struct Mover { long dst; V3 r; long src; uint32_t p; };
    std::vector<std::vector<Mover>> incoming(n_cells);
    const double eps = p.cell_size * (1.0 / static_cast<double>(1ull << 48));
    const double eps2 = eps * eps;
    for (long k = gl; k < G[2] - gl; ++k)
      for (long j = gl; j < G[1] - gl; ++j)
        for (long i = gl; i < G[0] - gl; ++i) {
          const long c = gidx(i, j, k);
          Cell& cell = cells[c];
          for (size_t q = 0; q < cell.size(); ++q) {
            V3 r{cell.rx[q], cell.ry[q], cell.rz[q]};
            const V3 ro = r;
            L3 d = domain_periodic_location(r);
            const L3 dst{d.i + gl, d.j + gl, d.k + gl};
            /* min_distance2_between(ro, cell_bounds(dst)) (core/include/exanb/core/geometry.h:137-153) */
            const V3 lo = cell_position(dst);
            const V3 hi = cell_position(L3{dst.i + 1, dst.j + 1, dst.k + 1});
            double dx = 0, dy = 0, dz = 0;
            if (ro.x < lo.x) dx = lo.x - ro.x; else if (ro.x > hi.x) dx = ro.x - hi.x;
            if (ro.y < lo.y) dy = lo.y - ro.y; else if (ro.y > hi.y) dy = ro.y - hi.y;
            if (ro.z < lo.z) dz = lo.z - ro.z; else if (ro.z > hi.z) dz = ro.z - hi.z;
            const double md2 = dx * dx + dy * dy + dz * dz;
            const bool same = (dst.i == i && dst.j == j && dst.k == k);
            if (!same || md2 >= eps2) {
              const long cj = gidx(dst.i, dst.j, dst.k);
              incoming[cj].push_back(Mover{cj, r, c, static_cast<uint32_t>(q)});
              removed[c].push_back(static_cast<uint32_t>(q));
            }
          }
        }
    // Collect mover payloads before any cell is modified.
    struct Payload { double v[3], f[3], pe; uint64_t id; uint8_t type; };
    std::vector<std::vector<Payload>> pay(n_cells);
    for (size_t c = 0; c < n_cells; ++c) {
      for (const Mover& m : incoming[c]) {
        const Cell& s = cells[m.src];
        pay[c].push_back(Payload{{s.vx[m.p], s.vy[m.p], s.vz[m.p]},
                                 {s.fx[m.p], s.fy[m.p], s.fz[m.p]},
                                 s.pe[m.p],
                                 s.id[m.p],
                                 s.type[m.p]});
      }
    }
    for (size_t c = 0; c < n_cells; ++c) {
      Cell& cell = cells[c];
      const long n0 = static_cast<long>(cell.size());
      const long n_out = static_cast<long>(removed[c].size());
      if (n_out > 0) {
        std::vector<int32_t> pack(n0);
        for (long q = 0; q < n0; ++q) pack[q] = static_cast<int32_t>(q);
        for (uint32_t q : removed[c]) pack[q] = -1;
        long n = n0;
        for (long q = n0 - 1; q >= 0; --q) {
          if (pack[q] == -1) {
            if (q < n - 1) pack[q] = pack[n - 1];
            --n;
          }
        }
        Cell old = cell;
        for (long q = 0; q < n; ++q) {
          if (q != pack[q]) cell.copy_from(static_cast<size_t>(q), old, static_cast<size_t>(pack[q]));
        }
        cell.resize(static_cast<size_t>(n));
      }
      for (size_t m = 0; m < incoming[c].size(); ++m) {
        const Mover& mv = incoming[c][m];
        const Payload& pl = pay[c][m];
        cell.push(mv.r.x, mv.r.y, mv.r.z, pl.v[0], pl.v[1], pl.v[2], pl.f[0], pl.f[1], pl.f[2], pl.id, pl.type);
        cell.pe.back() = pl.pe;
      }
    }
    return 0;
  }

  /* Single-rank migrate_cell_particles leaves inner cells in place and starts
   * ghost cells empty (migrate_cell_particles.h:166-262); ghosts are refilled by
   * ghost_update_all. */
  void clear_ghosts() {
    for (size_t c = 0; c < cells.size(); ++c)
      if (is_ghost(gloc(static_cast<long>(c)))) cells[c].clear();
  }

  /* project_particles_in_sub_grids (amr/include/exanb/amr/amr_grid_algorithm.h:113-375),
   * SUBRES=1, no z-curve: a stable counting sort of each cell's particles by
   * linear sub-cell index. */
  void rebuild_amr() {
    if (!p.amr_enabled) return;
#pragma omp parallel for schedule(dynamic)
    for (long c = 0; c < static_cast<long>(cells.size()); ++c) {
      Cell& cell = cells[c];
      const size_t n = cell.size();
      const long side = sub_grid_size(n, p.sub_grid_density);
      if (side <= 1) continue;
      const L3 l = gloc(c);
      const V3 low = cell_position(l);
      std::vector<long> key(n);
      for (size_t q = 0; q < n; ++q) {
        /* Grid::particle_pcoord (core/include/exanb/core/grid.h:184-190) */
        const double px = (cell.rx[q] - low.x) / p.cell_size;
        const double py = (cell.ry[q] - low.y) / p.cell_size;
        const double pz = (cell.rz[q] - low.z) / p.cell_size;
        long si = static_cast<long>(px * static_cast<double>(side));
        long sj = static_cast<long>(py * static_cast<double>(side));
        long sk = static_cast<long>(pz * static_cast<double>(side));
        si = std::min(std::max(si, 0L), side - 1);
        sj = std::min(std::max(sj, 0L), side - 1);
        sk = std::min(std::max(sk, 0L), side - 1);
        key[q] = (sk * side + sj) * side + si;
      }
      std::vector<size_t> order(n);
      for (size_t q = 0; q < n; ++q) order[q] = q;
      std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return key[a] < key[b]; });
      Cell old = cell;
      for (size_t q = 0; q < n; ++q) cell.copy_from(q, old, order[q]);
    }
  }

  /* PositionBackupNode::execute (io/backup_r.cpp:42-79). */
  void backup_r() {
    backup.assign(cells.size(), {});
#pragma omp parallel for schedule(dynamic)
    for (long c = 0; c < static_cast<long>(cells.size()); ++c) {
      const L3 l = gloc(c);
      if (is_ghost(l)) continue;
      const Cell& cell = cells[c];
      const V3 o = cell_position(l);
      std::vector<uint32_t>& rb = backup[c];
      rb.resize(cell.size() * 3);
      for (size_t q = 0; q < cell.size(); ++q) {
        rb[q * 3 + 0] = encode_double_u32(cell.rx[q], o.x, p.cell_size);
        rb[q * 3 + 1] = encode_double_u32(cell.ry[q], o.y, p.cell_size);
        rb[q * 3 + 2] = encode_double_u32(cell.rz[q], o.z, p.cell_size);
      }
    }
  }

  /* UpdateGhostsCommSchemeNode + partner_comm_scheme for one periodic rank
   * (mpi/update_ghosts_comm_scheme.cpp:127-196, 379-476). Shifts loop k,j,i over
   * {-1,0,1}; inner cells in grid order; particles kept when their shifted
   * position lies inside the partner block enlarged by ghost_dist. */
  void ghost_comm_scheme() {
    ghosts.clear();
    const double bmin[3] = {0.0 * p.cell_size + p.origin[0], 0.0 * p.cell_size + p.origin[1],
                            0.0 * p.cell_size + p.origin[2]};
    const double bmax[3] = {static_cast<double>(D[0]) * p.cell_size + p.origin[0],
                            static_cast<double>(D[1]) * p.cell_size + p.origin[1],
                            static_cast<double>(D[2]) * p.cell_size + p.origin[2]};
    const double omin[3] = {bmin[0] - ghost_dist, bmin[1] - ghost_dist, bmin[2] - ghost_dist};
    const double omax[3] = {bmax[0] + ghost_dist, bmax[1] + ghost_dist, bmax[2] + ghost_dist};
    for (int sk = -1; sk <= 1; ++sk)
      for (int sj = -1; sj <= 1; ++sj)
        for (int si = -1; si <= 1; ++si) {
          if (si == 0 && sj == 0 && sk == 0) continue;
          uint32_t flags = 0;
          if (si == -1) flags |= SHIFT_X;
          if (si == 1) flags |= SHIFT_X | SIDE_X;
          if (sj == -1) flags |= SHIFT_Y;
          if (sj == 1) flags |= SHIFT_Y | SIDE_Y;
          if (sk == -1) flags |= SHIFT_Z;
          if (sk == 1) flags |= SHIFT_Z | SIDE_Z;
          for (long k = 0; k < D[2]; ++k)
            for (long j = 0; j < D[1]; ++j)
              for (long i = 0; i < D[0]; ++i) {
                const long ti = si * D[0] + i, tj = sj * D[1] + j, tk = sk * D[2] + k;
                if (ti < -gl || ti >= D[0] + gl || tj < -gl || tj >= D[1] + gl || tk < -gl || tk >= D[2] + gl)
                  continue;
                GhostSend gs;
                gs.src_cell = gidx(i + gl, j + gl, k + gl);
                gs.dst_cell = gidx(ti + gl, tj + gl, tk + gl);
                gs.flags = flags;
                const Cell& s = cells[gs.src_cell];
                for (size_t q = 0; q < s.size(); ++q) {
                  const double gx = apply_coord_modifier(s.rx[q], p.origin[0], p.extent[0], flags >> 0);
                  const double gy = apply_coord_modifier(s.ry[q], p.origin[1], p.extent[1], flags >> 3);
                  const double gz = apply_coord_modifier(s.rz[q], p.origin[2], p.extent[2], flags >> 6);
                  /* is_inside (core/include/exanb/core/geometry.h:198-203), inclusive bounds */
                  if (gx >= omin[0] && gx <= omax[0] && gy >= omin[1] && gy <= omax[1] && gz >= omin[2] &&
                      gz <= omax[2])
                    gs.particle_i.push_back(static_cast<uint32_t>(q));
                }
                ghosts.push_back(std::move(gs));
              }
        }
  }

  /* ghost_update_all / ghost_update_r through the rank-self loopback
   * (mpi/include/exanb/mpi/grid_update_ghosts.h:63-202, update_ghost_functors.h:170-456). */
  void ghost_update(bool all) {
    for (const GhostSend& gs : ghosts) {
      const Cell& s = cells[gs.src_cell];
      Cell& d = cells[gs.dst_cell];
      if (all) d.resize(gs.particle_i.size());
      for (size_t q = 0; q < gs.particle_i.size(); ++q) {
        const uint32_t pi = gs.particle_i[q];
        d.rx[q] = apply_coord_modifier(s.rx[pi], p.origin[0], p.extent[0], gs.flags >> 0);
        d.ry[q] = apply_coord_modifier(s.ry[pi], p.origin[1], p.extent[1], gs.flags >> 3);
        d.rz[q] = apply_coord_modifier(s.rz[pi], p.origin[2], p.extent[2], gs.flags >> 6);
        if (all) {
          d.vx[q] = s.vx[pi]; d.vy[q] = s.vy[pi]; d.vz[q] = s.vz[pi];
          d.fx[q] = s.fx[pi]; d.fy[q] = s.fy[pi]; d.fz[q] = s.fz[pi];
          d.pe[q] = 0.0; d.id[q] = s.id[pi]; d.type[q] = s.type[pi];
        }
      }
    }
  }

  /* chunk_neighbors_execute (particle_neighbors/include/exanb/particle_neighbors/
   * chunk_neighbors_execute.h:100-412) for inner cells, chunk size 1,
   * build_particle_offset=true, one offset table. The sub-cell pair cache only
   * prunes cell pairs that cannot hold a neighbour, so candidates are taken from
   * the full 27-cell block. */
  int chunk_neighbors() {
    streams.assign(cells.size(), {});
    int err = 0;
#pragma omp parallel for schedule(dynamic) reduction(| : err)
    for (long c = 0; c < static_cast<long>(cells.size()); ++c) {
      const L3 la = gloc(c);
      if (is_ghost(la)) continue;
      const Cell& A = cells[c];
      const size_t na = A.size();
      std::vector<std::vector<std::pair<uint16_t, uint16_t>>> nbh(na);
      for (long bk = la.k - 1; bk <= la.k + 1; ++bk)
        for (long bj = la.j - 1; bj <= la.j + 1; ++bj)
          for (long bi = la.i - 1; bi <= la.i + 1; ++bi) {
            const long cb = gidx(bi, bj, bk);
            const Cell& B = cells[cb];
            const uint16_t enc = encode_cell_index(bi - la.i, bj - la.j, bk - la.k);
            for (size_t pa = 0; pa < na; ++pa)
              for (size_t pb = 0; pb < B.size(); ++pb) {
                const double dx = A.rx[pa] - B.rx[pb];
                const double dy = A.ry[pa] - B.ry[pb];
                const double dz = A.rz[pa] - B.rz[pb];
                const double d2 = norm2(dx, dy, dz);
                /* DefaultNeighborFilterFunc (neighbor_filter_func.h:26-33) */
                if ((cb != c || pa != pb) && d2 > 0.0 && d2 <= nbh2) {
                  if (pb >= 65535) err |= 1;
                  nbh[pa].emplace_back(enc, static_cast<uint16_t>(pb));
                }
              }
          }
      std::vector<uint16_t>& cc = streams[c];
      const long offset_table_size = (na > 0) ? static_cast<long>((na + 1) * 2) : 0;
      if (na > 0) cc.assign(static_cast<size_t>(offset_table_size), 0);
      for (size_t pa = 0; pa < na; ++pa) {
        const uint32_t off = static_cast<uint32_t>(static_cast<long>(cc.size()) - offset_table_size + 1);
        cc[pa * 2 + 0] = static_cast<uint16_t>(off);
        cc[pa * 2 + 1] = static_cast<uint16_t>(off >> 16);
        auto& L = nbh[pa];
        std::sort(L.begin(), L.end());
        L.erase(std::unique(L.begin(), L.end()), L.end());
        const size_t cell_count_idx = cc.size();
        size_t chunk_count_idx = 0;
        uint16_t last_cell = 0;
        cc.push_back(0);
        for (const auto& e : L) {
          if (e.first != last_cell) {
            ++cc[cell_count_idx];
            last_cell = e.first;
            cc.push_back(last_cell);
            chunk_count_idx = cc.size();
            cc.push_back(0);
          }
          ++cc[chunk_count_idx];
          cc.push_back(e.second);
        }
      }
      if (na > 0) {
        const uint32_t off = static_cast<uint32_t>(static_cast<long>(cc.size()) - offset_table_size + 1);
        cc[na * 2 + 0] = static_cast<uint16_t>(off);
        cc[na * 2 + 1] = static_cast<uint16_t>(off >> 16);
      }
    }
    return err ? -3 : 0;
  }

  /* lj_compute_energy (contribs/md/lennard_jones/lennard_jones.cu:46-56). */
  void lj(double r, double& e, double& de) const {
    const double inv_r = 1.0 / r;
    const double ratio = p.sigma * inv_r;
    const double ratio2 = ratio * ratio;
    const double ratio6 = ratio2 * ratio2 * ratio2;
    const double ratio12 = ratio6 * ratio6;
    e = 4. * p.epsilon * (ratio12 - ratio6);
    de = (-24. * p.epsilon * (2. * ratio12 - ratio6)) * inv_r;
  }

  /* zero_particle_force + lennard_jones_force: compute_cell_particle_pairs_cell
   * (compute/include/exanb/compute/compute_cell_particle_pairs_impl_default.h:107-238)
   * decoding the stream (chunk_neighbors.h:172-186) into the per-particle compute
   * buffer, then LennardJonesForceFunctor (lennard_jones.cu:67-102). The potential
   * energy (discarded by the reference) is 0.5*(e - e(rc)) per stream entry. */
  int compute_forces() {
    if (snap) return snap_forces();
    int err = 0;
#pragma omp parallel for schedule(dynamic) reduction(| : err)
    for (long c = 0; c < static_cast<long>(cells.size()); ++c) {
      Cell& A = cells[c];
      const L3 la = gloc(c);
      for (size_t q = 0; q < A.size(); ++q) { A.fx[q] = 0.0; A.fy[q] = 0.0; A.fz[q] = 0.0; A.pe[q] = 0.0; }
      if (is_ghost(la)) continue;
      const size_t na = A.size();
      if (na == 0) continue;
      const uint16_t* base = streams[c].data();
      const uint32_t* offset = nullptr;
      const uint16_t* stream_base = base;
      int32_t shift = 0;
      if (base[0] <= 2 && base[1] == 0) {
        const int ntab = base[0];
        const int tab = ntab >= 1 ? static_cast<int>((na * ntab + 1) * 2) : 0;
        stream_base = base + tab;
        offset = reinterpret_cast<const uint32_t*>(base);
        shift = -ntab;
      }
      std::vector<double> bx, by, bz, b2;
      bx.reserve(256); by.reserve(256); bz.reserve(256); b2.reserve(256);
      for (size_t pa = 0; pa < na; ++pa) {
        const uint16_t* s = stream_base + offset[pa] + shift;
        int groups = *(s++);
        bx.clear(); by.clear(); bz.clear(); b2.clear();
        double epa = 0.0;
        while (groups > 0) {
          const uint16_t enc = *(s++);
          int nch = *(s++);
          const long ri = static_cast<long>(enc & 31) - 16;
          const long rj = static_cast<long>((enc >> 5) & 31) - 16;
          const long rk = static_cast<long>((enc >> 10) & 31) - 16;
          const long cb = c + ((rk * G[1]) + rj) * G[0] + ri;
          const Cell& B = cells[cb];
          --groups;
          while (nch > 0) {
            const unsigned pb = *(s++);
            --nch;
            const double drx = B.rx[pb] - A.rx[pa];
            const double dry = B.ry[pb] - A.ry[pa];
            const double drz = B.rz[pb] - A.rz[pa];
            const double d2 = norm2(drx, dry, drz);
            if (d2 > 0.0 && d2 <= rcut2) {
              bx.push_back(drx); by.push_back(dry); bz.push_back(drz); b2.push_back(d2);
            }
          }
        }
        if (bx.size() >= 256) err |= 1; /* ComputePairBuffer2 capacity (compute_pair_buffer.h:197-208) */
        double tfx = 0.0, tfy = 0.0, tfz = 0.0;
        for (size_t i = 0; i < bx.size(); ++i) {
          const double r = std::sqrt(b2[i]);
          double e = 0.0, de = 0.0;
          lj(r, e, de);
          de *= 1.0 / r;
          tfx += de * bx[i];
          tfy += de * by[i];
          tfz += de * bz[i];
          epa += 0.5 * (e - e_shift);
        }
        A.fx[pa] += tfx;
        A.fy[pa] += tfy;
        A.fz[pa] += tfz;
        A.pe[pa] = epa;
        if (p.divide_by_mass) {
          /* divide_force_by_type_scalar (compute/vec3_typescalar_op.cu:156, math_functors.h:136-141) */
          A.fx[pa] /= p.mass;
          A.fy[pa] /= p.mass;
          A.fz[pa] /= p.mass;
        }
      }
    }
    return err ? -4 : 0;
  }

  /* zero_particle_force { ghost: true } + snap_force_generic + update_force_from_ghost
   * (+ divide_force_by_type_scalar): SnapForceRealT over the per-particle compute
   * buffer (contribs/md/snap/include/md/snap/snap_force.h:290-372): for particle i,
   * the stream entries inside the traversal cutoff whose squared distance lies in
   * (1e-20, ((rad_i + rad_j) rcutfac)^2) (snap_force_op_coop.hxx:215-226) are its
   * environment; f_i += sum fij and f_j -= fij for each (snap_force_op_coop.hxx:
   * 331-356), fij = dE_i/dr_ij. Reactions are applied after all environments, in
   * cell, particle and stream order; ghost particles' forces then go to the
   * particles they copy (update_force_from_ghost). */
  int snap_forces() {
    for (Cell& C : cells)
      for (size_t q = 0; q < C.size(); ++q) { C.fx[q] = 0.0; C.fy[q] = 0.0; C.fz[q] = 0.0; C.pe[q] = 0.0; }
    struct Reac { long cb; uint32_t pb; std::array<double, 3> f; };
    struct AtomOut { double e; std::array<double, 3> f; std::vector<Reac> reac; };
    std::vector<std::vector<AtomOut>> out(cells.size());
    int err = 0;
#pragma omp parallel for schedule(dynamic) reduction(| : err)
    for (long c = 0; c < static_cast<long>(cells.size()); ++c) {
      const L3 la = gloc(c);
      if (is_ghost(la)) continue;
      const Cell& A = cells[c];
      const size_t na = A.size();
      if (na == 0) continue;
      out[c].resize(na);
      const uint16_t* base = streams[c].data();
      const int ntab = base[0];
      const int tab = ntab >= 1 ? static_cast<int>((na * ntab + 1) * 2) : 0;
      const uint16_t* stream_base = base + tab;
      const uint32_t* offset = reinterpret_cast<const uint32_t*>(base);
      std::vector<std::array<double, 3>> dr, fij;
      std::vector<int> tj;
      std::vector<Reac> who;
      for (size_t pa = 0; pa < na; ++pa) {
        const uint16_t* st = stream_base + offset[pa] - ntab;
        int groups = *(st++);
        dr.clear(); tj.clear(); who.clear();
        const int ti = A.type[pa];
        while (groups-- > 0) {
          const uint16_t enc = *(st++);
          int nch = *(st++);
          const long ri = static_cast<long>(enc & 31) - 16;
          const long rj = static_cast<long>((enc >> 5) & 31) - 16;
          const long rk = static_cast<long>((enc >> 10) & 31) - 16;
          const long cb = c + ((rk * G[1]) + rj) * G[0] + ri;
          const Cell& B = cells[cb];
          while (nch-- > 0) {
            const unsigned pb = *(st++);
            const double drx = B.rx[pb] - A.rx[pa];
            const double dry = B.ry[pb] - A.ry[pa];
            const double drz = B.rz[pb] - A.rz[pa];
            const double d2 = norm2(drx, dry, drz);
            if (!(d2 > 0.0 && d2 <= rcut2)) continue;
            const double cij = snap->cut(ti, B.type[pb]);
            if (!(d2 < cij * cij && d2 > 1e-20)) continue;
            dr.push_back({drx, dry, drz});
            tj.push_back(B.type[pb]);
            who.push_back({cb, pb, {0.0, 0.0, 0.0}});
          }
        }
        if (dr.size() >= 256) err |= 1;
        AtomOut& o = out[c][pa];
        o.e = snap->atom(ti, dr, tj, snap_energy, fij);
        o.f = {0.0, 0.0, 0.0};
        for (size_t q = 0; q < fij.size(); ++q) {
          for (int k = 0; k < 3; ++k) o.f[k] += fij[q][k];
          who[q].f = fij[q];
        }
        o.reac = who;
      }
    }
    for (long c = 0; c < static_cast<long>(cells.size()); ++c) {
      Cell& A = cells[c];
      for (size_t pa = 0; pa < out[c].size(); ++pa) {
        const AtomOut& o = out[c][pa];
        A.fx[pa] += o.f[0];
        A.fy[pa] += o.f[1];
        A.fz[pa] += o.f[2];
        A.pe[pa] = o.e;
        for (const Reac& r : o.reac) {
          Cell& B = cells[r.cb];
          B.fx[r.pb] -= r.f[0];
          B.fy[r.pb] -= r.f[1];
          B.fz[r.pb] -= r.f[2];
        }
      }
    }
    for (const GhostSend& gs : ghosts) {
      Cell& owner = cells[gs.src_cell];
      const Cell& g = cells[gs.dst_cell];
      for (size_t q = 0; q < gs.particle_i.size() && q < g.size(); ++q) {
        const uint32_t pi = gs.particle_i[q];
        owner.fx[pi] += g.fx[q];
        owner.fy[pi] += g.fy[q];
        owner.fz[pi] += g.fz[q];
      }
    }
    if (p.divide_by_mass)
      for (long c = 0; c < static_cast<long>(cells.size()); ++c) {
        if (is_ghost(gloc(c))) continue;
        Cell& A = cells[c];
        for (size_t q = 0; q < A.size(); ++q) {
          A.fx[q] /= p.mass;
          A.fy[q] /= p.mass;
          A.fz[q] /= p.mass;
        }
      }
    return err ? -4 : 0;
  }

  /* zero_particle_force + gravitational_force (contribs/pi/gravitational_force.cu:42-
   * 141): the buffer-less functor called per stream entry inside rcut
   * (compute_cell_particle_pairs_impl_default.h:186-205), adding straight onto
   * the zeroed force: r = sqrt(d2), inv_r = 1/r, e = -G m_a m_b inv_r,
   * de = G m_a m_b inv_r inv_r, de *= w / r (w = 1), f_a += de * dr with
   * dr = r_b - r_a; masses from the particle types. Energies (which the
   * reference discards) as 0.5 * e per entry. */
  int gravitational_forces(double Gc, const double* type_mass, int ntypes, double rcut_g) {
    const double rc2 = rcut_g * rcut_g;
    int err = 0;
#pragma omp parallel for schedule(dynamic) reduction(| : err)
    for (long c = 0; c < static_cast<long>(cells.size()); ++c) {
      Cell& A = cells[c];
      const L3 la = gloc(c);
      for (size_t q = 0; q < A.size(); ++q) { A.fx[q] = 0.0; A.fy[q] = 0.0; A.fz[q] = 0.0; A.pe[q] = 0.0; }
      if (is_ghost(la)) continue;
      const size_t na = A.size();
      if (na == 0) continue;
      const uint16_t* base = streams[c].data();
      const uint16_t* stream_base = base + (na + 1) * 2;
      const uint32_t* offset = reinterpret_cast<const uint32_t*>(base);
      for (size_t pa = 0; pa < na; ++pa) {
        const uint16_t* st = stream_base + offset[pa] - 1;
        int groups = *(st++);
        if (A.type[pa] >= ntypes) { err |= 1; continue; }
        const double mass_a = type_mass[A.type[pa]];
        double fx = 0.0, fy = 0.0, fz = 0.0, e_sum = 0.0;
        while (groups > 0) {
          const uint16_t enc = *(st++);
          int nch = *(st++);
          const long ri = static_cast<long>(enc & 31) - 16;
          const long rj = static_cast<long>((enc >> 5) & 31) - 16;
          const long rk = static_cast<long>((enc >> 10) & 31) - 16;
          const Cell& B = cells[c + ((rk * G[1]) + rj) * G[0] + ri];
          --groups;
          while (nch > 0) {
            const unsigned pb = *(st++);
            --nch;
            const double drx = B.rx[pb] - A.rx[pa];
            const double dry = B.ry[pb] - A.ry[pa];
            const double drz = B.rz[pb] - A.rz[pa];
            const double d2 = norm2(drx, dry, drz);
            if (d2 > 0.0 && d2 <= rc2) {
              if (B.type[pb] >= ntypes) { err |= 1; continue; }
              const double mass_b = type_mass[B.type[pb]];
              const double r = std::sqrt(d2);
              const double inv_r = 1.0 / r;
              const double e = -Gc * mass_a * mass_b * inv_r;
              double de = Gc * mass_a * mass_b * inv_r * inv_r;
              de *= 1.0 / r;
              fx += de * drx;
              fy += de * dry;
              fz += de * drz;
              e_sum += 0.5 * e;
            }
          }
        }
        A.fx[pa] = fx;
        A.fy[pa] = fy;
        A.fz[pa] = fz;
        A.pe[pa] = e_sum;
      }
    }
    return err ? -4 : 0;
  }

  /* zero_particle_force + a Morse pair potential as a buffer-less functor over
   * the streams (the reference has no Morse functor; this restates the
   * published form V(r) = D (exp(-2a(r-r0)) - 2 exp(-a(r-r0))) for the
   * pair-functor API test): per stream entry inside rcut, in stream order
   * (compute_cell_particle_pairs_impl_default.h:186-205), with dr = r_b - r_a,
   * e1 = exp(-a(r-r0)), e2 = e1*e1, dV/dr = 2aD(e1 - e2), f_a += (dV/dr / r) dr,
   * and 0.5 (V(r) - V(rcut)) per entry as the particle's energy. */
  int morse_forces(double D, double alpha, double r0, double rcut_m) {
    const double rc2 = rcut_m * rcut_m;
    const double ec1 = std::exp(-alpha * (rcut_m - r0));
    const double e_shift = D * (ec1 * ec1 - 2.0 * ec1);
#pragma omp parallel for schedule(dynamic)
    for (long c = 0; c < static_cast<long>(cells.size()); ++c) {
      Cell& A = cells[c];
      const L3 la = gloc(c);
      for (size_t q = 0; q < A.size(); ++q) { A.fx[q] = 0.0; A.fy[q] = 0.0; A.fz[q] = 0.0; A.pe[q] = 0.0; }
      if (is_ghost(la)) continue;
      const size_t na = A.size();
      if (na == 0) continue;
      const uint16_t* base = streams[c].data();
      const uint16_t* stream_base = base + (na + 1) * 2;
      const uint32_t* offset = reinterpret_cast<const uint32_t*>(base);
      for (size_t pa = 0; pa < na; ++pa) {
        const uint16_t* st = stream_base + offset[pa] - 1;
        int groups = *(st++);
        double fx = 0.0, fy = 0.0, fz = 0.0, e_sum = 0.0;
        while (groups > 0) {
          const uint16_t enc = *(st++);
          int nch = *(st++);
          const long ri = static_cast<long>(enc & 31) - 16;
          const long rj = static_cast<long>((enc >> 5) & 31) - 16;
          const long rk = static_cast<long>((enc >> 10) & 31) - 16;
          const Cell& B = cells[c + ((rk * G[1]) + rj) * G[0] + ri];
          --groups;
          while (nch > 0) {
            const unsigned pb = *(st++);
            --nch;
            const double drx = B.rx[pb] - A.rx[pa];
            const double dry = B.ry[pb] - A.ry[pa];
            const double drz = B.rz[pb] - A.rz[pa];
            const double d2 = norm2(drx, dry, drz);
            if (d2 > 0.0 && d2 <= rc2) {
              const double r = std::sqrt(d2);
              const double e1 = std::exp(-alpha * (r - r0));
              const double e2 = e1 * e1;
              const double s = 2.0 * alpha * D * (e1 - e2) / r;
              fx += s * drx;
              fy += s * dry;
              fz += s * drz;
              e_sum += 0.5 * (D * (e2 - 2.0 * e1) - e_shift);
            }
          }
        }
        A.fx[pa] = fx;
        A.fy[pa] = fy;
        A.fz[pa] = fz;
        A.pe[pa] = e_sum;
      }
    }
    return 0;
  }

  /* type of each particle by id; ghost copies follow their owner */
  int set_types(const uint64_t* ids, const uint8_t* types, int64_t n) {
    std::vector<std::pair<uint64_t, uint8_t>> t(static_cast<size_t>(n));
    for (int64_t q = 0; q < n; ++q) t[static_cast<size_t>(q)] = {ids[q], types[q]};
    std::sort(t.begin(), t.end());
    long matched = 0;
    for (auto& cell : cells)
      for (size_t q = 0; q < cell.size(); ++q) {
        auto it = std::lower_bound(t.begin(), t.end(), std::make_pair(cell.id[q], static_cast<uint8_t>(0)));
        if (it != t.end() && it->first == cell.id[q]) { cell.type[q] = it->second; ++matched; }
      }
    for (const GhostSend& gs : ghosts) {
      const Cell& s = cells[gs.src_cell];
      Cell& d = cells[gs.dst_cell];
      for (size_t q = 0; q < gs.particle_i.size() && q < d.size(); ++q) d.type[q] = s.type[gs.particle_i[q]];
    }
    return static_cast<int>(matched > 0 ? 0 : -1);
  }

  /* PushVec3SecondOrderFunctor (defbox/include/exanb/defbox/push_vec3_2nd_order.h:29-38,
   * :85-88): r += v*dt + f*(dt*dt*0.5), inner cells only. */
  void push_f_v_r(double dt_scale) {
    const double dt = p.dt * dt_scale;
    const double dt2 = dt * dt * 0.5;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < static_cast<long>(cells.size()); ++c) {
      if (is_ghost(gloc(c))) continue;
      Cell& A = cells[c];
      for (size_t q = 0; q < A.size(); ++q) {
        A.rx[q] += A.vx[q] * dt + A.fx[q] * dt2;
        A.ry[q] += A.vy[q] * dt + A.fy[q] * dt2;
        A.rz[q] += A.vz[q] * dt + A.fz[q] * dt2;
      }
    }
  }

  /* PushVec3FirstOrderFunctor (defbox/include/exanb/defbox/push_vec3_1st_order.h:29-38,:79-81). */
  void push_f_v(double dt_scale) {
    const double dt = p.dt * dt_scale;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < static_cast<long>(cells.size()); ++c) {
      if (is_ghost(gloc(c))) continue;
      Cell& A = cells[c];
      for (size_t q = 0; q < A.size(); ++q) {
        A.vx[q] += A.fx[q] * dt;
        A.vy[q] += A.fy[q] * dt;
        A.vz[q] += A.fz[q] * dt;
      }
    }
  }

  /* ReduceMaxDisplacementFunctor (mpi/particle_displ_over.cu:38-66): count of inner
   * particles with norm2(r - restore(backup)) >= max_displ^2. */
  int64_t displ_over() const {
    const double thr2 = max_displ * max_displ;
    int64_t count = 0;
#pragma omp parallel for schedule(static) reduction(+ : count)
    for (long c = 0; c < static_cast<long>(cells.size()); ++c) {
      const L3 l = gloc(c);
      if (is_ghost(l)) continue;
      const Cell& A = cells[c];
      const V3 o = cell_position(l);
      const uint32_t* rb = backup[c].data();
      for (size_t q = 0; q < A.size(); ++q) {
        const double bx = restore_u32_double(rb[q * 3 + 0], o.x, p.cell_size);
        const double by = restore_u32_double(rb[q * 3 + 1], o.y, p.cell_size);
        const double bz = restore_u32_double(rb[q * 3 + 2], o.z, p.cell_size);
        if (norm2(A.rx[q] - bx, A.ry[q] - by, A.rz[q] - bz) >= thr2) ++count;
      }
    }
    return count;
  }

  /* update_particles_full body (update-particles.msp:62-68, 47-53, 42-45). */
  int update_full() {
    int e = move_particles();
    if (e) return e;
    clear_ghosts();
    rebuild_amr();
    backup_r();
    ghost_comm_scheme();
    ghost_update(true);
    e = chunk_neighbors();
    ++rebuilds;
    return e;
  }
};

extern "C" {

xo_sys* xo_create(const xo_params* p) {
  if (!p) return nullptr;
  xo_sys* s = new xo_sys();
  s->p = *p;
  for (int a = 0; a < 3; ++a) {
    s->D[a] = p->dims[a];
    s->G[a] = p->dims[a] + 2;
  }
  s->nbh_dist = p->rcut + p->rcut_inc;           /* nbh_dist.cpp:47 */
  s->max_displ = p->rcut_inc / 2.0;              /* nbh_dist.cpp:48 */
  s->ghost_dist = (p->rcut + p->rcut_inc) / 1.0; /* nbh_dist.cpp:63-65 */
  s->nbh2 = s->nbh_dist * s->nbh_dist;           /* chunk_neighbors_execute.h:75-76 */
  s->rcut2 = p->rcut * p->rcut;                  /* compute_cell_particle_pairs.h:145 */
  const long gl = static_cast<long>(std::ceil(s->ghost_dist / p->cell_size));
  const long gap = static_cast<long>(std::ceil(s->nbh_dist / p->cell_size));
  if (gl != 1 || gap != 1 || p->dims[0] < 2 || p->dims[1] < 2 || p->dims[2] < 2) {
    delete s;
    return nullptr;
  }
  double e = 0, de = 0;
  s->lj(p->rcut, e, de);
  s->e_shift = e;
  s->cells.assign(static_cast<size_t>(s->G[0] * s->G[1] * s->G[2]), Cell{});
  return s;
}

void xo_destroy(xo_sys* s) { delete s; }

int xo_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

int xo_load_flat(xo_sys* s, int64_t n, const double* rx, const double* ry, const double* rz,
                 const double* vx, const double* vy, const double* vz, const uint64_t* id) {
  if (!s) return -1;
  for (auto& c : s->cells) c.clear();
  for (int64_t q = 0; q < n; ++q) {
    V3 r{rx[q], ry[q], rz[q]};
    const L3 d = s->domain_periodic_location(r);
    Cell& c = s->cells[s->gidx(d.i + s->gl, d.j + s->gl, d.k + s->gl)];
    c.push(r.x, r.y, r.z, vx[q], vy[q], vz[q], 0.0, 0.0, 0.0, id[q]);
  }
  s->ready = false;
  return 0;
}

int xo_load_cells(xo_sys* s, const int64_t* cell_counts, const double* rx, const double* ry,
                  const double* rz, const double* vx, const double* vy, const double* vz,
                  const uint64_t* id) {
  if (!s) return -1;
  for (auto& c : s->cells) c.clear();
  int64_t q = 0;
  const long nint = s->D[0] * s->D[1] * s->D[2];
  for (long ci = 0; ci < nint; ++ci) {
    Cell& c = s->cells[s->interior_to_grid(ci)];
    for (int64_t t = 0; t < cell_counts[ci]; ++t, ++q)
      c.push(rx[q], ry[q], rz[q], vx[q], vy[q], vz[q], 0.0, 0.0, 0.0, id[q]);
  }
  s->ready = false;
  return 0;
}

int xo_load_lattice_noise_fcc(xo_sys* s, double a, double sigma) { return xo_load_lattice_noise(s, 2, a, sigma); }

/* generate_particle_lattice (grid_cell_particles/include/exanb/grid_cell_particles/
 * generate_particle_lattice.h:247-388) with deterministic_noise, SC / BCC / FCC
 * basis (lattice_generator.h:140-170), then GaussianNoise on rx,ry,rz
 * (compute/include/exanb/compute/gaussian_noise.h:62-80,150-161). */
int xo_load_lattice_noise(xo_sys* s, int32_t structure, double a, double sigma) {
  if (!s || structure < 0 || structure > 2) return -1;
  for (auto& c : s->cells) c.clear();
  static const double sc[1][3] = {{.5, .5, .5}};
  static const double bcc[2][3] = {{.0, .0, .0}, {.5, .5, .5}};
  static const double fcc[4][3] = {{.0, .0, .0}, {.0, .5, .5}, {.5, .0, .5}, {.5, .5, .0}};
  const double(*basis)[3] = structure == 0 ? sc : structure == 1 ? bcc : fcc;
  const int nbasis = structure == 0 ? 1 : structure == 1 ? 2 : 4;
  const double lo[3] = {s->p.origin[0], s->p.origin[1], s->p.origin[2]};
  const double hi[3] = {s->p.extent[0], s->p.extent[1], s->p.extent[2]};
  const long ist = static_cast<long>(std::floor(lo[0] / a)) - 1, iend = static_cast<long>(std::ceil(hi[0] / a)) + 1;
  const long jst = static_cast<long>(std::floor(lo[1] / a)) - 1, jend = static_cast<long>(std::ceil(hi[1] / a)) + 1;
  const long kst = static_cast<long>(std::floor(lo[2] / a)) - 1, kend = static_cast<long>(std::ceil(hi[2] / a)) + 1;
  /* grid bounds including ghost cells */
  const double gblo[3] = {s->p.origin[0] + static_cast<double>(-1) * s->p.cell_size,
                          s->p.origin[1] + static_cast<double>(-1) * s->p.cell_size,
                          s->p.origin[2] + static_cast<double>(-1) * s->p.cell_size};
  const double gbhi[3] = {s->p.origin[0] + static_cast<double>(s->D[0] + 1) * s->p.cell_size,
                          s->p.origin[1] + static_cast<double>(s->D[1] + 1) * s->p.cell_size,
                          s->p.origin[2] + static_cast<double>(s->D[2] + 1) * s->p.cell_size};
  const uint64_t no_id = ~0ull;
  for (long k = kst; k <= kend; ++k)
    for (long j = jst; j <= jend; ++j)
      for (long i = ist; i <= iend; ++i)
        for (int l = 0; l < nbasis; ++l) {
          const double x = (static_cast<double>(i) + basis[l][0]) * a;
          const double y = (static_cast<double>(j) + basis[l][1]) * a;
          const double z = (static_cast<double>(k) + basis[l][2]) * a;
          /* Grid::locate_cell (grid.h:126-134) */
          const long li = static_cast<long>(std::floor((x - s->p.origin[0]) / s->p.cell_size)) + 1;
          const long lj = static_cast<long>(std::floor((y - s->p.origin[1]) / s->p.cell_size)) + 1;
          const long lk = static_cast<long>(std::floor((z - s->p.origin[2]) / s->p.cell_size)) + 1;
          if (li < 0 || lj < 0 || lk < 0 || li >= s->G[0] || lj >= s->G[1] || lk >= s->G[2]) continue;
          if (!(x >= lo[0] && x <= hi[0] && y >= lo[1] && y <= hi[1] && z >= lo[2] && z <= hi[2])) continue;
          if (!(x >= gblo[0] && x <= gbhi[0] && y >= gblo[1] && y <= gbhi[1] && z >= gblo[2] && z <= gbhi[2])) continue;
          s->cells[s->gidx(li, lj, lk)].push(x, y, z, 0, 0, 0, 0, 0, 0, no_id);
        }
  /* ids: exclusive scan of per-domain-cell counts, starting after max id (0) + 1 */
  const uint64_t first_id = 1;
  uint64_t running = 0;
  for (long k = 0; k < s->D[2]; ++k)
    for (long j = 0; j < s->D[1]; ++j)
      for (long i = 0; i < s->D[0]; ++i) {
        Cell& c = s->cells[s->gidx(i + 1, j + 1, k + 1)];
        for (size_t q = 0; q < c.size(); ++q)
          if (c.id[q] == no_id) c.id[q] = first_id + (running++);
      }
  /* deterministic gaussian noise, one engine seeded per domain cell */
  for (long k = 0; k < s->D[2]; ++k)
    for (long j = 0; j < s->D[1]; ++j)
      for (long i = 0; i < s->D[0]; ++i) {
        const uint64_t dci = static_cast<uint64_t>((k * s->D[1] + j) * s->D[0] + i);
        std::mt19937_64 re;
        re.seed(dci * 1023);
        std::normal_distribution<double> g(0.0, sigma);
        Cell& c = s->cells[s->gidx(i + 1, j + 1, k + 1)];
        for (size_t q = 0; q < c.size(); ++q) {
          c.rx[q] += g(re);
          c.ry[q] += g(re);
          c.rz[q] += g(re);
        }
      }
  /* particles the generator put in ghost cells are not owned; they are dropped */
  s->clear_ghosts();
  s->ready = false;
  return 0;
}

int xo_init(xo_sys* s) {
  if (!s) return -1;
  int e = s->update_full();
  s->rebuilds = 0;
  if (e) return e;
  e = s->compute_forces();
  if (e) return e;
  s->ready = true;
  return 0;
}

int xo_step(xo_sys* s) {
  if (!s || !s->ready) return -1;
  s->push_f_v_r(1.0);
  s->push_f_v(0.5);
  int rebuilt = 0;
  if (s->displ_over() > 0) {
    const int e = s->update_full();
    if (e) return e;
    rebuilt = 1;
  } else {
    s->ghost_update(false);
  }
  const int e = s->compute_forces();
  if (e) return e;
  s->push_f_v(0.5);
  return rebuilt;
}

/* Timing hooks of the CPU baseline, on an initialised state: the force pass
 * alone (zero_particle_force + lennard_jones_force) and the neighbour build alone
 * (chunk_neighbors over the current grid and ghosts). Neither moves particles. */
int xo_compute_forces(xo_sys* s) {
  if (!s || !s->ready) return -1;
  return s->compute_forces();
}

int xo_chunk_neighbors(xo_sys* s) {
  if (!s || !s->ready) return -1;
  return s->chunk_neighbors();
}

int64_t xo_num_particles(const xo_sys* s) {
  int64_t n = 0;
  for (size_t c = 0; c < s->cells.size(); ++c)
    if (!s->is_ghost(s->gloc(static_cast<long>(c)))) n += static_cast<int64_t>(s->cells[c].size());
  return n;
}

int64_t xo_rebuild_count(const xo_sys* s) { return s->rebuilds; }
int64_t xo_num_cells(const xo_sys* s) { return s->D[0] * s->D[1] * s->D[2]; }

int xo_get_particles(const xo_sys* s, double* rx, double* ry, double* rz, double* vx, double* vy,
                     double* vz, double* fx, double* fy, double* fz, uint64_t* id, int32_t* cell,
                     double* pe) {
  int64_t q = 0;
  const long nint = s->D[0] * s->D[1] * s->D[2];
  for (long ci = 0; ci < nint; ++ci) {
    const Cell& c = s->cells[s->interior_to_grid(ci)];
    for (size_t t = 0; t < c.size(); ++t, ++q) {
      if (rx) rx[q] = c.rx[t];
      if (ry) ry[q] = c.ry[t];
      if (rz) rz[q] = c.rz[t];
      if (vx) vx[q] = c.vx[t];
      if (vy) vy[q] = c.vy[t];
      if (vz) vz[q] = c.vz[t];
      if (fx) fx[q] = c.fx[t];
      if (fy) fy[q] = c.fy[t];
      if (fz) fz[q] = c.fz[t];
      if (id) id[q] = c.id[t];
      if (cell) cell[q] = static_cast<int32_t>(ci);
      if (pe) pe[q] = c.pe[t];
    }
  }
  return 0;
}

int xo_get_cell_counts(const xo_sys* s, int64_t* counts) {
  const long nint = s->D[0] * s->D[1] * s->D[2];
  for (long ci = 0; ci < nint; ++ci) counts[ci] = static_cast<int64_t>(s->cells[s->interior_to_grid(ci)].size());
  return 0;
}

// The stream entries of the interior cells [ci0, ci1) as ids, in stream order
// (the decoding of compute_cell_particle_pairs_impl_default.h:148-180).
static int64_t walk_pairs(const xo_sys* s, uint64_t* ida, uint64_t* idb, int32_t* cnt, long ci0 = 0,
                          long ci1 = -1) {
  int64_t k = 0, q = 0;
  const long nint = s->D[0] * s->D[1] * s->D[2];
  if (ci1 < 0 || ci1 > nint) ci1 = nint;
  for (long ci = ci0 < 0 ? 0 : ci0; ci < ci1; ++ci) {
    const long c = s->interior_to_grid(ci);
    const Cell& A = s->cells[c];
    const size_t na = A.size();
    if (na == 0) continue;
    const uint16_t* base = s->streams[c].data();
    const uint32_t* offset = reinterpret_cast<const uint32_t*>(base);
    const uint16_t* sb = base + (na + 1) * 2;
    for (size_t pa = 0; pa < na; ++pa, ++q) {
      const uint16_t* st = sb + offset[pa] - 1;
      int groups = *(st++);
      int32_t n = 0;
      while (groups-- > 0) {
        const uint16_t enc = *(st++);
        int nch = *(st++);
        const long ri = static_cast<long>(enc & 31) - 16;
        const long rj = static_cast<long>((enc >> 5) & 31) - 16;
        const long rk = static_cast<long>((enc >> 10) & 31) - 16;
        const long cb = c + ((rk * s->G[1]) + rj) * s->G[0] + ri;
        while (nch-- > 0) {
          const unsigned pb = *(st++);
          if (ida) ida[k] = A.id[pa];
          if (idb) idb[k] = s->cells[cb].id[pb];
          ++k;
          ++n;
        }
      }
      if (cnt) cnt[q] = n;
    }
  }
  return k;
}

int64_t xo_pair_count(const xo_sys* s) { return walk_pairs(s, nullptr, nullptr, nullptr); }

int xo_get_pairs(const xo_sys* s, uint64_t* id_a, uint64_t* id_b, int32_t* nbh_count) {
  walk_pairs(s, id_a, id_b, nbh_count);
  return 0;
}

int64_t xo_pair_count_cells(const xo_sys* s, int64_t ci0, int64_t ci1) {
  return walk_pairs(s, nullptr, nullptr, nullptr, static_cast<long>(ci0), static_cast<long>(ci1));
}

int xo_get_pairs_cells(const xo_sys* s, int64_t ci0, int64_t ci1, uint64_t* id_b, int32_t* nbh_count) {
  walk_pairs(s, nullptr, id_b, nbh_count, static_cast<long>(ci0), static_cast<long>(ci1));
  return 0;
}

int64_t xo_cell_stream_size(const xo_sys* s, int64_t ci) {
  return static_cast<int64_t>(s->streams[s->interior_to_grid(static_cast<long>(ci))].size());
}

int xo_get_cell_stream(const xo_sys* s, int64_t ci, uint16_t* out) {
  const auto& v = s->streams[s->interior_to_grid(static_cast<long>(ci))];
  std::memcpy(out, v.data(), v.size() * sizeof(uint16_t));
  return 0;
}

int xo_set_types(xo_sys* s, const uint64_t* ids, const uint8_t* types, int64_t n) {
  return s->set_types(ids, types, n);
}

int xo_set_snap(xo_sys* s, int32_t twojmax, double rcutfac, double rfac0, double rmin0, int32_t switchflag,
                int32_t bzeroflag, int32_t ntypes, const double* radelem, const double* wj, int32_t ncoeffall,
                const double* coeff, double energy_unit, int32_t with_energy) {
  if (!s || twojmax < 0 || twojmax > 16 || ntypes < 1 || !radelem || !wj || !coeff) return -1;
  xo_snap::Spec sp;
  sp.twojmax = twojmax;
  sp.rcutfac = rcutfac;
  sp.rfac0 = rfac0;
  sp.rmin0 = rmin0;
  sp.switchflag = switchflag != 0;
  sp.bzeroflag = bzeroflag != 0;
  sp.ntypes = ntypes;
  sp.radelem.assign(radelem, radelem + ntypes);
  sp.wj.assign(wj, wj + ntypes);
  sp.ncoeffall = ncoeffall;
  sp.coeff.assign(coeff, coeff + static_cast<size_t>(ntypes) * ncoeffall);
  sp.energy_unit = energy_unit;
  auto calc = std::make_unique<xo_snap::Calc>(sp);
  if (calc->ncoeff() + 1 != ncoeffall) return -2;
  s->snap = std::move(calc);
  s->snap_energy = with_energy != 0;
  return 0;
}

int xo_gravitational_force(xo_sys* s, double G, const double* type_mass, int32_t ntypes, double rcut) {
  return s->gravitational_forces(G, type_mass, ntypes, rcut);
}

int xo_morse_force(xo_sys* s, double D, double alpha, double r0, double rcut) {
  return s->morse_forces(D, alpha, r0, rcut);
}

int xo_energy(const xo_sys* s, double* ke, double* pe) {
  double k = 0.0, e = 0.0;
  const long nint = s->D[0] * s->D[1] * s->D[2];
  for (long ci = 0; ci < nint; ++ci) {
    const Cell& c = s->cells[s->interior_to_grid(ci)];
    for (size_t t = 0; t < c.size(); ++t) {
      k += 0.5 * s->p.mass * norm2(c.vx[t], c.vy[t], c.vz[t]);
      e += c.pe[t];
    }
  }
  if (ke) *ke = k;
  if (pe) *pe = e;
  return 0;
}

int64_t xo_displ_over_count(const xo_sys* s) { return s->displ_over(); }

}  // extern "C"
