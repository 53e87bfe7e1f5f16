// C ABI (include/xnb_gpu.h) and the host runtime of a batch: device pools,
// system admission, and the launch sequence of the reference's operators.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/xnb_dump.h"
#include "../../include/xnb_gpu.h"
#include "xnb_launch.cuh"
#include "xnb_snap.cuh"

using namespace xnb;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define XCK(call)                                                                              \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) return fail(XNB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// First-fit allocator of index ranges inside one device pool.
struct RangeAlloc {
  uint64_t cap = 0;
  std::map<uint64_t, uint64_t> free_;  // offset -> length
  std::map<uint64_t, uint64_t> used_;  // offset -> length
  void init(uint64_t c) {
    cap = c;
    free_.clear();
    used_.clear();
    if (c) free_[0] = c;
  }
  int64_t alloc(uint64_t n) {
    if (n == 0) n = 1;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        const uint64_t off = it->first, len = it->second;
        free_.erase(it);
        if (len > n) free_[off + n] = len - n;
        used_[off] = n;
        return static_cast<int64_t>(off);
      }
    }
    return -1;
  }
  void release(uint64_t off) {
    auto u = used_.find(off);
    if (u == used_.end()) return;
    uint64_t n = u->second;
    used_.erase(u);
    auto nx = free_.lower_bound(off);
    if (nx != free_.end() && off + n == nx->first) {
      n += nx->second;
      nx = free_.erase(nx);
    }
    if (nx != free_.begin()) {
      auto pv = std::prev(nx);
      if (pv->first + pv->second == off) {
        pv->second += n;
        return;
      }
    }
    free_[off] = n;
  }
  uint64_t high_water() const {
    if (used_.empty()) return 0;
    auto it = std::prev(used_.end());
    return it->first + it->second;
  }
};

struct SysHost {
  bool active = false;
  SysDesc d{};
  double list_factor = 1.3;
  int64_t list_off = -1;
  uint64_t list_cap = 0;
  bool initialised = false;
};

}  // namespace

struct xnb_batch {
  unsigned long long launches = 0;  // kernels enqueued by this batch (for benchmark accounting)
  int device = 0;
  int sm_count = 1;
  xnb_batch_config cfg{};
  int stage_cap = 640;
  int force_block = 64;
  int force_lanes = 1;          // threads per particle of the FP64 / mixed force traversal
  int force_form = kForceThread;  // mixed full-list traversal form (xnb_batch_set_force_form)
  std::vector<uint4> segs;      // cell segments of the staged traversal (host copy of a.seg)
  int build_form = kBuildWarp;  // neighbour-build kernel (xnb_batch_set_build_form)
  int subcell_prune = 1;        // sub-cell pruned build of dense cells after a rebin (xnb_batch_set_subcell_pruning)
  DevArrays a{};
  SysDesc* d_sys = nullptr;
  SysState* d_st = nullptr;
  SysState* h_st = nullptr;  // pinned mirror
  unsigned int* d_flag = nullptr;             // scratch error flag of the stream writer
  unsigned long long* d_counts = nullptr;     // scratch counters of the stream checker
  unsigned char* d_stats = nullptr;           // scratch of the simulation_stats reduction
  StepCtl* d_ctl = nullptr;                   // control block of the persistent step loop
  std::vector<SysHost> sys;
  RangeAlloc parts, cells, lists;
  std::vector<void*> allocs;

  Extent extent() const {
    Extent e;
    e.n_part = static_cast<uint32_t>(parts.high_water());
    e.n_cells = static_cast<uint32_t>(cells.high_water());
    int hw = 0;
    e.far_coords = 0;
    e.unpacked = 0;
    for (size_t s = 0; s < sys.size(); ++s)
      if (sys[s].active) {
        hw = static_cast<int>(s) + 1;
        if (sys[s].d.far_coords) e.far_coords = 1;
        if (!sys[s].d.packed_lo) e.unpacked = 1;
      }
    e.nsys = hw;
    e.sm_count = sm_count;
    e.force_block = force_block;
    e.force_lanes = force_lanes;
    e.force_form = force_form;
    e.n_seg = a.seg ? static_cast<uint32_t>(segs.size()) : 0u;
    return e;
  }
};

struct xnb_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  xnb_batch* batch = nullptr;
  // what the captured launches depend on besides device memory: the batch's
  // work extent and launch configuration at capture
  uint32_t n_part = 0, n_cells = 0;
  int nsys = 0, lbuf = 0, stage_cap = 0, force_block = 0, force_lanes = 0, build_form = 0, far_coords = 0;
  int force_form = 0, subcell_prune = 0;
  uint32_t n_seg = 0;
};

namespace {

template <class T>
int dalloc(xnb_batch* b, T** p, uint64_t n) {
  void* q = nullptr;
  const cudaError_t e = cudaMalloc(&q, std::max<uint64_t>(n, 1) * sizeof(T));
  if (e != cudaSuccess) return fail(XNB_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  b->allocs.push_back(q);
  *p = static_cast<T*>(q);
  return XNB_OK;
}

// domain_periodic_location (core/include/exanb/core/domain.h:160-191) on the host,
// same operations as the device rebin.
void periodic_location(const xnb_lj_params& p, double r[3], int loc[3]) {
  for (int a = 0; a < 3; ++a) {
    const double rel = r[a] - p.origin[a];
    long l = static_cast<long>(std::floor(rel / p.cell_size));
    if (l < 0 || l >= p.dims[a]) {
      const long old = l;
      l = ((l % p.dims[a]) + p.dims[a]) % p.dims[a];
      r[a] += static_cast<double>(l - old) * p.cell_size;
    }
    loc[a] = static_cast<int>(l);
  }
}

int validate(const xnb_lj_params* p) {
  if (!p) return fail(XNB_ERR_ARG, "null params");
  for (int a = 0; a < 3; ++a)
    if (p->dims[a] < 2) return fail(XNB_ERR_ARG, "domain needs at least 2 cells per axis");
  if (!(p->cell_size > 0) || !(p->rcut > 0) || !(p->rcut_inc >= 0)) return fail(XNB_ERR_ARG, "bad cutoffs");
  const double nbh = p->rcut + p->rcut_inc;
  if (std::ceil(nbh / p->cell_size) != 1.0)
    return fail(XNB_ERR_ARG, "cell_size must be >= rcut + rcut_inc (one ghost layer, gap 1)");
  return XNB_OK;
}

// Bound on |d2_f32 - d2_f64| for pairs within distance R in a system of largest
// period P and neighbour distance nbh (the derivation is in make_desc).
double fp32_d2_error(double P, double nbh, double R) {
  const double u = std::ldexp(1.0, -24);
  const double X = P + nbh;
  const double D = (3.0 * X + 2.0 * P + R) * u * 1.01;
  return 2.0 * std::sqrt(3.0) * R * D + 3.0 * D * D + 4.0 * u * (R * R + 1.0);
}

SysDesc make_desc(const xnb_lj_params& p) {
  SysDesc d{};
  for (int a = 0; a < 3; ++a) {
    d.origin[a] = p.origin[a];
    d.extent[a] = p.extent[a];
    d.period[a] = p.extent[a] - p.origin[a];
    d.dims[a] = p.dims[a];
  }
  // +0 only: x - (+0) is x for every x (including -0); x - (-0) would turn -0 into +0
  d.origin_zero = (p.origin[0] == 0.0 && !std::signbit(p.origin[0]) && p.origin[1] == 0.0 &&
                   !std::signbit(p.origin[1]) && p.origin[2] == 0.0 && !std::signbit(p.origin[2]))
                      ? 1
                      : 0;
  {
    double P = 0.0, X = 0.0;
    for (int a = 0; a < 3; ++a) {
      P = std::max(P, std::fabs(p.extent[a] - p.origin[a]));
      X = std::max(X, std::max(std::fabs(p.origin[a]), std::fabs(p.extent[a])));
    }
    d.far_coords = X > 4.0 * P ? 1 : 0;
  }
  d.cell_size = p.cell_size;
  const double ghost_dist = (p.rcut + p.rcut_inc) / 1.0;  // nbh_dist.cpp:63-65
  for (int a = 0; a < 3; ++a) {
    // block_to_bounds(partner_block) enlarged by max_neighbor_distance (update_ghosts_comm_scheme.cpp:402-403)
    const double bmin = 0.0 * p.cell_size + p.origin[a];
    const double bmax = static_cast<double>(p.dims[a]) * p.cell_size + p.origin[a];
    d.outer_lo[a] = bmin - ghost_dist;
    d.outer_hi[a] = bmax + ghost_dist;
  }
  d.rcut2 = p.rcut * p.rcut;
  const double nbh = p.rcut + p.rcut_inc;
  d.nbh2 = nbh * nbh;
  const double max_displ = p.rcut_inc / 2.0;
  d.max_displ2 = max_displ * max_displ;
  {
    // Trigger pre-decision. Each FP32 mirror h = fl32(fl64(x - o)) is within
    // u|X| (1 + 2^-29) of X = x - o, u = 2^-24; positions stay within one cell
    // of the domain between rebuilds, so |X| <= P = max period + cell size. A
    // mirror difference fl32(h_x - h_b) is then within E = u (2P + 1) (1 + 2^-20)
    // of the exact displacement component d_k (|d_k| <= 1 when it matters), and
    // fmaf(dz, dz, fmaf(dy, dy, dx dx)) within 2 sqrt(3) |d| E + 3 E^2 + 3 u |d|^2
    // of |d|^2 (+ u^2 terms). The error grows with |d|, so the bound at
    // |d| = max_displ decides both sides of the threshold; it is doubled and the
    // thresholds are rounded outwards to FP32.
    double P = 0.0;
    for (int a = 0; a < 3; ++a) P = std::max(P, std::fabs(p.extent[a] - p.origin[a]));
    P += p.cell_size;
    const double u = std::ldexp(1.0, -24);
    const double E = u * (2.0 * P + 1.0) * (1.0 + std::ldexp(1.0, -20));
    const double m2 = 2.0 * (2.0 * std::sqrt(3.0) * max_displ * E + 3.0 * E * E + 3.0 * u * d.max_displ2 +
                             4.0 * u * u * d.max_displ2);
    float lo_f = static_cast<float>(d.max_displ2 - m2), hi_f = static_cast<float>(d.max_displ2 + m2);
    if (static_cast<double>(lo_f) > d.max_displ2 - m2) lo_f = std::nextafter(lo_f, -1.0f);
    if (static_cast<double>(hi_f) < d.max_displ2 + m2) hi_f = std::nextafter(hi_f, 2.0f * hi_f + 1.0f);
    d.trig_lo_f = lo_f > 0.0f ? lo_f : 0.0f;
    d.trig_hi_f = hi_f;
  }
  d.epsilon = p.epsilon;
  d.sigma = p.sigma;
  {
    // lj_compute_energy at r = rcut (lennard_jones.cu:46-56)
    const double inv_r = 1.0 / p.rcut;
    const double ratio = p.sigma * inv_r;
    const double ratio2 = ratio * ratio;
    const double ratio6 = ratio2 * ratio2 * ratio2;
    const double ratio12 = ratio6 * ratio6;
    d.e_shift = 4. * p.epsilon * (ratio12 - ratio6);
  }
  d.m24eps = -24. * p.epsilon;
  d.eps4 = 4. * p.epsilon;
  d.eps24 = 24. * p.epsilon;
  d.sig2 = p.sigma * p.sigma;
  d.mass = p.mass;
  d.divide_by_mass = p.divide_by_mass;
  d.amr_enabled = p.amr_enabled;
  d.sub_grid_density = p.sub_grid_density > 0 ? p.sub_grid_density : 6.5;
  {
    // sub_grid_side returns 1 while the rounded quotient n / density stays below
    // 8; the same IEEE division here gives the first count where it does not
    double n0 = std::floor(8.0 * d.sub_grid_density) - 2.0;
    if (!(n0 >= 1.0)) n0 = 1.0;
    uint64_t n = static_cast<uint64_t>(std::min(n0, 4294967295.0));
    while (n < 4294967295ull && static_cast<double>(n) / d.sub_grid_density < 8.0) ++n;
    while (n > 1 && static_cast<double>(n - 1) / d.sub_grid_density >= 8.0) --n;
    d.amr_min_n = static_cast<uint32_t>(n);
  }
  // sub-cell pair pruning: two sub-cell boxes are searched together when their
  // distance, in cells, is at most this (nbh / cell_size rounded up, then
  // widened by 1e-5 so that rounding of positions, keys and images never drops a
  // neighbour)
  d.sub_reach_f = std::nextafter(static_cast<float>(nbh / p.cell_size * (1.0 + 1e-5)), 2.0f);
  d.dt = p.dt;
  d.dt_full = p.dt * 1.0;
  d.dt_sq_half = d.dt_full * d.dt_full * 0.5;
  d.dt_half = p.dt * 0.5;
  d.sig2_f = static_cast<float>(d.sig2);
  d.eps24_f = static_cast<float>(d.eps24);
  d.eps4_f = static_cast<float>(d.eps4);
  d.e_shift_f = static_cast<float>(d.e_shift);
  // Error bounds of the FP32 prefilters (u = 2^-24 unit roundoff). Positions
  // are mirrored as pf = fl32(x - origin) with |x - origin| <= X = max period
  // + nbh (drift allowance); an image coordinate adds fl32(period) (P); so one
  // axis of an FP32 difference is within D = (3X + 2P + R) u (1.01) of the FP64
  // one for pairs within distance R, and |d2_f32 - d2_f64| <=
  // err(R) = 2 sqrt(3) R D + 3 D^2 + 4 u (R^2 + 1). Each margin is 4 err.
  const double u = std::ldexp(1.0, -24);
  double P = 0.0;
  for (int a = 0; a < 3; ++a) P = std::max(P, std::fabs(d.period[a]));
  const double X = P + nbh;
  auto err_at = [&](double R) { return fp32_d2_error(P, nbh, R); };
  d.nbh2_f = static_cast<float>(d.nbh2);
  d.nbh_margin_f = static_cast<float>(4.0 * err_at(nbh));
  d.pre_margin_f = static_cast<float>(4.0 * err_at(p.rcut));
  for (int a = 0; a < 3; ++a) {
    d.period_f[a] = static_cast<float>(d.period[a]);
    d.outer_lo_f[a] = static_cast<float>(d.outer_lo[a] - d.origin[a]);
    d.outer_hi_f[a] = static_cast<float>(d.outer_hi[a] - d.origin[a]);
  }
  // ghost filter compare: coordinate error 2 (X + P) u, bound conversion (X + nbh) u
  d.filter_margin_f = static_cast<float>(4.0 * (2.0 * (X + P) + X + nbh) * u * 1.01);
  //  force cutoff test of the mixed path: each FP32 axis difference is within
  //  2u|d| + delta of the FP64 one (converted, or compensated hi/lo with the
  //  residuals packed to lo_step: delta = 2 lo_step), so
  //  |r2_f32 - d2_f64| <= 6 u d2 + 2 sqrt(3) |d| delta + 3 delta^2; margin = 4x
  //  at rc^2 (+1 absolute guard so tiny d2 also go to FP64).
  {
    int e = 0;
    std::frexp(X, &e);  // X = m 2^e, m in [0.5, 1): ulp_32(X) = 2^(e - 24)
    d.lo_step_f = std::ldexp(1.0f, e - 34);
    d.lo_inv_f = std::ldexp(1.0f, 34 - e);
    // the packed residual's absolute error grows with X: beyond X = 1024 sigma
    // (lo_step 2^-24) the mixed traversal gathers the FP32 residual mirror instead
    d.packed_lo = e <= 10 ? 1 : 0;
  }
  // FP32 cell index of the rebin: the mirror pf = fl32(x - origin) and
  // fl32(1/cell_size) put pf * inv within 3.01 u |q| of the quotient q of the
  // reference's division (|q| <= max dims + 2 before wrapping); a fraction farther
  // than 4 u (max dims + 2) from an integer floors like the division does.
  int dmax = 1;
  for (int a = 0; a < 3; ++a) dmax = std::max(dmax, static_cast<int>(p.dims[a]));
  d.inv_cell_f = static_cast<float>(1.0 / p.cell_size);
  d.q_margin_f = static_cast<float>(4.0 * u * (dmax + 2.0));
  d.inv_cell = 1.0 / p.cell_size;
  d.rc2_f = static_cast<float>(d.rcut2);
  {
    const double delta = d.packed_lo ? 2.0 * static_cast<double>(d.lo_step_f) : 0.0;
    d.rc_margin_f = static_cast<float>(
        4.0 * (6.0 * u * (d.rcut2 + 1.0) + 2.0 * std::sqrt(3.0) * p.rcut * delta + 3.0 * delta * delta));
  }
  return d;
}

int upload_desc(xnb_batch* b, int s, cudaStream_t st) {
  XCK(cudaMemcpyAsync(b->d_sys + s, &b->sys[s].d, sizeof(SysDesc), cudaMemcpyHostToDevice, st));
  return XNB_OK;
}

int check_sys(xnb_batch* b, int32_t s) {
  if (!b) return fail(XNB_ERR_ARG, "null batch");
  if (s == -1) return XNB_OK;
  if (s < 0 || s >= static_cast<int32_t>(b->sys.size()) || !b->sys[s].active) return fail(XNB_ERR_ARG, "bad system id");
  return XNB_OK;
}

int pull_states(xnb_batch* b, cudaStream_t st) {
  const Extent ex = b->extent();
  if (ex.nsys == 0) return XNB_OK;
  XCK(cudaMemcpyAsync(b->h_st, b->d_st, sizeof(SysState) * ex.nsys, cudaMemcpyDeviceToHost, st));
  XCK(cudaStreamSynchronize(st));
  return XNB_OK;
}

// Cell segments of the staged force traversal: every row (j, k) of every
// resident system cut into runs of kStagedSegCells x-adjacent cells; uploaded
// whenever the set of systems changes (and the staged form is allocated).
int upload_segments(xnb_batch* b, cudaStream_t st) {
  b->segs.clear();
  for (size_t q = 0; q < b->sys.size(); ++q) {
    const SysHost& h = b->sys[q];
    if (!h.active) continue;
    const SysDesc& d = h.d;
    for (int k = 0; k < d.dims[2]; ++k)
      for (int j = 0; j < d.dims[1]; ++j)
        for (int i = 0; i < d.dims[0]; i += kStagedSegCells) {
          const uint32_t first = d.cell_base + static_cast<uint32_t>((k * d.dims[1] + j) * d.dims[0] + i);
          const uint32_t n = static_cast<uint32_t>(std::min(kStagedSegCells, d.dims[0] - i));
          b->segs.push_back(make_uint4(first, n, static_cast<uint32_t>(q), 0u));
        }
  }
  if (!b->a.seg || b->segs.empty()) return XNB_OK;
  XCK(cudaMemcpyAsync(b->a.seg, b->segs.data(), b->segs.size() * sizeof(uint4), cudaMemcpyHostToDevice, st));
  XCK(cudaStreamSynchronize(st));
  return XNB_OK;
}

// Per-warp list buffer of the neighbour build: the largest slot of the resident
// systems, rounded up to 32 entries, at most kMaxListBuf (larger slots are
// written without buffering).
constexpr uint32_t kMaxListBuf = 1024;
int list_buf(const xnb_batch* b) {
  uint32_t m = 0;
  for (const SysHost& h : b->sys)
    if (h.active && h.d.list_slot > m) m = h.d.list_slot;
  m = (m + 31) / 32 * 32;
  return static_cast<int>(m > kMaxListBuf ? 0 : m);
}

// (Re)sizes system s's list segment for a largest per-particle count `need`:
// slot = list_factor * max(need, 1.2 x the mean count of a uniform fluid of the
// system's density) + 16 entries, rounded up to 8 (32-byte list starts). The
// density term covers a lattice start whose counts sit below the fluid's.
int size_lists(xnb_batch* b, int s, uint32_t need, cudaStream_t st) {
  SysHost& h = b->sys[s];
  const double vol = std::fabs(h.d.period[0] * h.d.period[1] * h.d.period[2]);
  const double nbh = std::sqrt(h.d.nbh2);
  const double fluid = vol > 0 ? 1.2 * 4.18879020478639 * nbh * nbh * nbh * static_cast<double>(h.d.npart) / vol : 0.0;
  const double base = std::max(static_cast<double>(need), std::ceil(fluid));
  uint64_t slot = static_cast<uint64_t>(std::ceil(base * h.list_factor)) + 16;
  slot = (slot + 7) / 8 * 8;
  if (slot < h.d.list_slot) slot = h.d.list_slot;
  const uint64_t entries = static_cast<uint64_t>(h.d.npart) * slot;
  if (entries >= (1ull << 32)) return fail(XNB_ERR_ARG, "neighbour lists of one system above 2^32 entries");
  if (h.list_off >= 0) b->lists.release(static_cast<uint64_t>(h.list_off));
  // every segment is a multiple of 8 entries, so each list starts on a 32-byte boundary
  const int64_t off = b->lists.alloc(std::max<uint64_t>(entries, 8));
  if (off < 0) {
    h.list_off = -1;
    h.list_cap = 0;
    h.d.list_base = 0;
    h.d.list_slot = 0;
    upload_desc(b, s, st);
    return fail(XNB_ERR_NOMEM, "neighbour list pool exhausted");
  }
  h.list_off = off;
  h.list_cap = entries;
  h.d.list_base = static_cast<uint64_t>(off);
  h.d.list_slot = static_cast<uint32_t>(slot);
  int rc = upload_desc(b, s, st);
  if (rc) return rc;
  // the build against the old slot flagged an overflow: clear it
  const uint32_t err = b->h_st[s].error & ~kErrListOverflow;
  XCK(cudaMemcpyAsync(&b->d_st[s].error, &err, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  b->h_st[s].error = err;
  return XNB_OK;
}

// Neighbour lists for flagged systems, synchronising with the host: one build
// pass; a system without a segment yet (slot 0: the pass only counts) or whose
// largest count outgrew its slot gets a segment sized from that count, and the
// pass runs again. Counts depend only on positions, so the second pass fits.
int neighbors_sync(xnb_batch* b, cudaStream_t st) {
  const Extent ex = b->extent();
  for (int pass = 0; pass < 3; ++pass) {
    b->launches += launch_neighbors(ex, b->d_sys, b->d_st, b->a, b->stage_cap, list_buf(b), st, b->build_form,
                                    b->subcell_prune != 0);
    int rc = pull_states(b, st);
    if (rc) return rc;
    bool again = false;
    for (int s = 0; s < ex.nsys; ++s) {
      SysHost& h = b->sys[s];
      if (!h.active || !b->h_st[s].rebuild) continue;
      const uint32_t need = b->h_st[s].max_nbr;
      if (h.list_off >= 0 && need <= h.d.list_slot) continue;
      rc = size_lists(b, s, need, st);
      if (rc) return rc;
      again = true;
    }
    if (!again) return XNB_OK;
  }
  return fail(XNB_ERR_DEVICE, "neighbour lists did not fit their resized slots");
}

int clear_rebuild(xnb_batch* b, cudaStream_t st) {
  const Extent ex = b->extent();
  b->launches += launch_mark_rebuild(ex, b->d_st, 2, -1, b->a.any_rebuild, st);
  return XNB_OK;
}

// precision argument: base precision in the low bits, XNB_PREC_NEWTON as a flag
int decode_precision(int32_t precision, int* base, bool* newton) {
  *base = precision & 0xF;
  *newton = (precision & XNB_PREC_NEWTON) != 0;
  if (*base < 0 || *base > 2 || (precision & ~(0xF | XNB_PREC_NEWTON)))
    return fail(XNB_ERR_ARG, "bad precision");
  if (*newton && *base == XNB_PREC_FP64_EXACT)
    return fail(XNB_ERR_ARG, "the Newton half-list traversal is not bit-exact: use it with FP64 or MIXED");
  return XNB_OK;
}

int check_launch() {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(XNB_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return XNB_OK;
}

}  // namespace

extern "C" {

const char* xnb_last_error_string(void) { return g_err.c_str(); }
int xnb_version(void) { return 10000; }

int64_t xnb_system_bytes(int64_t n, int64_t ncells, double list_per_particle) {
  // doubles r v f pe, restored backup, rebin scratch (22); ids (2); u32 cell, backup,
  // rebin and list bookkeeping (10); FP32 hi/lo mirrors; types (2); sub-cell key;
  // per cell: u32 tables (6), scan, the two build lists and the sub-grid side
  const int64_t per_part = 22 * 8 + 2 * 8 + 10 * 4 + 3 * 16 + 2 + 2;
  const int64_t per_cell = 4 * 6 + 8 + 4 + 4 + 1;
  return n * per_part + ncells * per_cell + static_cast<int64_t>(static_cast<double>(n) * list_per_particle) * 4;
}

int xnb_batch_create(const xnb_batch_config* cfg, xnb_batch** out) {
  if (!cfg || !out) return fail(XNB_ERR_ARG, "null argument");
  if (cfg->particle_capacity <= 0 || cfg->cell_capacity <= 0 || cfg->list_capacity <= 0 || cfg->max_systems <= 0)
    return fail(XNB_ERR_ARG, "capacities must be positive");
  if (cfg->particle_capacity >= (1ll << 31) || cfg->cell_capacity >= (1ll << 31))
    return fail(XNB_ERR_ARG, "capacity above 2^31");
  XCK(cudaSetDevice(cfg->device));
  xnb_batch* b = new xnb_batch();
  b->device = cfg->device;
  b->cfg = *cfg;
  if (cfg->stage_cap > 0) b->stage_cap = (cfg->stage_cap + 31) / 32 * 32;
  if (cfg->stage_cap > 1024) {
    delete b;
    return fail(XNB_ERR_ARG, "stage_cap above 1024 candidates");
  }
  if (cfg->force_block > 0) {
    if (cfg->force_block % 32 || cfg->force_block > 256) {
      delete b;
      return fail(XNB_ERR_ARG, "force_block must be a multiple of 32 and at most 256");
    }
    b->force_block = cfg->force_block;
  }
  cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, cfg->device);
  const uint64_t P = static_cast<uint64_t>(cfg->particle_capacity);
  const uint64_t Cc = static_cast<uint64_t>(cfg->cell_capacity);
  const uint64_t L = static_cast<uint64_t>(cfg->list_capacity);
  int rc = 0;
  DevArrays& a = b->a;
  double** dbl[] = {&a.rx, &a.ry, &a.rz, &a.vx, &a.vy, &a.vz, &a.fx, &a.fy, &a.fz, &a.pe,
                    &a.rbx, &a.rby, &a.rbz, &a.t_rx, &a.t_ry, &a.t_rz, &a.t_vx, &a.t_vy, &a.t_vz,
                    &a.t_fx, &a.t_fy, &a.t_fz};
  for (double** p : dbl) rc = rc ? rc : dalloc(b, p, P);
  rc = rc ? rc : dalloc(b, &a.id, P);
  rc = rc ? rc : dalloc(b, &a.pf, P);
  rc = rc ? rc : dalloc(b, &a.pflo, P);
  rc = rc ? rc : dalloc(b, &a.rbf, P);
  rc = rc ? rc : dalloc(b, &a.nbr_half, P);
  rc = rc ? rc : dalloc(b, &a.any_rebuild, 4);
  rc = rc ? rc : dalloc(b, &a.t_id, P);
  rc = rc ? rc : dalloc(b, &a.ptype, P);
  rc = rc ? rc : dalloc(b, &a.t_ptype, P);
  uint32_t** u32p[] = {&a.pcell, &a.bkx, &a.bky, &a.bkz, &a.pdest, &a.plocal, &a.mover_list,
                       &a.nbr_start, &a.nbr_cnt};
  for (uint32_t** p : u32p) rc = rc ? rc : dalloc(b, p, P);
  uint32_t** u32c[] = {&a.cell_start, &a.cell_n, &a.cell_sys, &a.cell_cnt, &a.cell_stay, &a.cell_nmov};
  for (uint32_t** p : u32c) rc = rc ? rc : dalloc(b, p, Cc + 1);
  rc = rc ? rc : dalloc(b, &a.cell_scan, Cc + 1);
  rc = rc ? rc : dalloc(b, &a.nbr_wide, Cc + 1);
  rc = rc ? rc : dalloc(b, &a.nbr_wide_n, 1);
  rc = rc ? rc : dalloc(b, &a.nbr_sub, Cc + 1);
  rc = rc ? rc : dalloc(b, &a.nbr_sub_n, 1);
  rc = rc ? rc : dalloc(b, &a.skey, P);
  rc = rc ? rc : dalloc(b, &a.cside, Cc + 1);
  rc = rc ? rc : dalloc(b, &a.scan_blocks, scan_scratch_elems(static_cast<uint32_t>(Cc + 1)) + 8);
  rc = rc ? rc : dalloc(b, &a.nbr, L);
  rc = rc ? rc : dalloc(b, &b->d_sys, static_cast<uint64_t>(cfg->max_systems));
  rc = rc ? rc : dalloc(b, &b->d_st, static_cast<uint64_t>(cfg->max_systems));
  rc = rc ? rc : dalloc(b, &b->d_flag, 1);
  rc = rc ? rc : dalloc(b, &b->d_counts, 8);
  rc = rc ? rc : dalloc(b, &b->d_stats, stats_scratch_bytes());
  rc = rc ? rc : dalloc(b, &b->d_ctl, 1);
  if (!rc && cudaMallocHost(&b->h_st, sizeof(SysState) * cfg->max_systems) != cudaSuccess)
    rc = fail(XNB_ERR_NOMEM, "cudaMallocHost failed");
  if (rc) {
    xnb_batch_destroy(b);
    return rc;
  }
  cudaMemset(a.pcell, 0xFF, P * sizeof(uint32_t));
  cudaMemset(a.cell_sys, 0xFF, (Cc + 1) * sizeof(uint32_t));
  cudaMemset(a.cell_n, 0, (Cc + 1) * sizeof(uint32_t));
  cudaMemset(a.cell_start, 0, (Cc + 1) * sizeof(uint32_t));
  cudaMemset(b->d_st, 0, sizeof(SysState) * cfg->max_systems);
  cudaMemset(a.any_rebuild, 0, sizeof(unsigned int));
  cudaMemset(a.nbr_wide_n, 0, sizeof(unsigned int));
  cudaMemset(a.nbr_sub_n, 0, sizeof(unsigned int));
  cudaMemset(a.cside, 1, Cc + 1);
  if (cudaDeviceSynchronize() != cudaSuccess) {
    xnb_batch_destroy(b);
    return fail(XNB_ERR_CUDA, "initialisation failed");
  }
  b->parts.init(P);
  b->cells.init(Cc);
  b->lists.init(L);
  b->sys.resize(static_cast<size_t>(cfg->max_systems));
  *out = b;
  return XNB_OK;
}

int xnb_batch_destroy(xnb_batch* b) {
  if (!b) return XNB_OK;
  cudaSetDevice(b->device);
  cudaDeviceSynchronize();
  for (void* p : b->allocs) cudaFree(p);
  if (b->h_st) cudaFreeHost(b->h_st);
  delete b;
  return XNB_OK;
}

namespace {
int place_system(xnb_batch* b, const xnb_lj_params* p, int64_t n, const double* rx, const double* ry,
                 const double* rz, const double* vx, const double* vy, const double* vz, const uint64_t* id,
                 const int64_t* cell_counts, int64_t poff, int64_t coff, uint64_t ncells, int slot, cudaStream_t st);
}  // namespace

int xnb_system_add(xnb_batch* b, const xnb_lj_params* p, int64_t n, const double* rx, const double* ry,
                   const double* rz, const double* vx, const double* vy, const double* vz, const uint64_t* id,
                   const int64_t* cell_counts, double list_factor, void* stream, int32_t* sys_out) {
  if (!b || !sys_out) return fail(XNB_ERR_ARG, "null argument");
  int rc = validate(p);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!rx || !ry || !rz || !vx || !vy || !vz || !id))) return fail(XNB_ERR_ARG, "bad particle arrays");
  if (n >= (1ll << 26)) return fail(XNB_ERR_ARG, "a system holds at most 2^26 - 1 particles");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  XCK(cudaSetDevice(b->device));
  int slot = -1;
  for (size_t s = 0; s < b->sys.size(); ++s)
    if (!b->sys[s].active) {
      slot = static_cast<int>(s);
      break;
    }
  if (slot < 0) return fail(XNB_ERR_NOMEM, "no free system slot");
  const uint64_t ncells = static_cast<uint64_t>(p->dims[0]) * p->dims[1] * p->dims[2];
  const int64_t poff = b->parts.alloc(static_cast<uint64_t>(n));
  if (poff < 0) return fail(XNB_ERR_NOMEM, "particle pool exhausted");
  const int64_t coff = b->cells.alloc(ncells);
  if (coff < 0) {
    b->parts.release(static_cast<uint64_t>(poff));
    return fail(XNB_ERR_NOMEM, "cell pool exhausted");
  }
  rc = place_system(b, p, n, rx, ry, rz, vx, vy, vz, id, cell_counts, poff, coff, ncells, slot, st);
  if (rc) {
    b->parts.release(static_cast<uint64_t>(poff));
    b->cells.release(static_cast<uint64_t>(coff));
    return rc;
  }
  SysHost& sh = b->sys[slot];
  sh = SysHost{};
  sh.d = make_desc(*p);
  sh.d.cell_base = static_cast<uint32_t>(coff);
  sh.d.ncells = static_cast<uint32_t>(ncells);
  sh.d.part_base = static_cast<uint32_t>(poff);
  sh.d.npart = static_cast<uint32_t>(n);
  sh.list_factor = list_factor >= 1.0 ? list_factor : 1.3;
  SysState zero{};
  XCK(cudaMemcpyAsync(b->d_st + slot, &zero, sizeof(SysState), cudaMemcpyHostToDevice, st));
  sh.active = true;
  b->h_st[slot] = zero;  // the host mirror may still hold a previous occupant's state
  rc = upload_desc(b, slot, st);
  if (rc) return rc;
  // list slots from the uniform-fluid estimate, so that the first build usually
  // fits in one pass (a larger count regrows them as before); when the pool has
  // no room now, the first build sizes them
  if (size_lists(b, slot, 0, st) != XNB_OK) g_err.clear();
  // the caller's arrays and the host staging are pageable: finish the copies before returning
  XCK(cudaStreamSynchronize(st));
  *sys_out = slot;
  {
    const int urc = upload_segments(b, st);
    if (urc) return urc;
  }
  return XNB_OK;
}

namespace {

// Particles, cell table and mirrors of a new system. Flat input (cell_counts
// NULL) is placed on the device (launch_place); input given per reference cell,
// or a cell too dense for the device pass, is staged on the host.
int place_system(xnb_batch* b, const xnb_lj_params* p, int64_t n, const double* rx, const double* ry,
                 const double* rz, const double* vx, const double* vy, const double* vz, const uint64_t* id,
                 const int64_t* cell_counts, int64_t poff, int64_t coff, uint64_t ncells, int slot, cudaStream_t st) {
  DevArrays& a = b->a;
  if (!cell_counts && n > 0) {
    const size_t nb = static_cast<size_t>(n);
    const double* srcs[6] = {rx, ry, rz, vx, vy, vz};
    double* dsts[6] = {a.t_rx, a.t_ry, a.t_rz, a.t_vx, a.t_vy, a.t_vz};
    for (int k = 0; k < 6; ++k)
      XCK(cudaMemcpyAsync(dsts[k] + poff, srcs[k], nb * sizeof(double), cudaMemcpyHostToDevice, st));
    XCK(cudaMemcpyAsync(a.t_id + poff, id, nb * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    PlaceArgs P{};
    for (int ax = 0; ax < 3; ++ax) {
      P.origin[ax] = p->origin[ax];
      P.dims[ax] = p->dims[ax];
    }
    P.cell_size = p->cell_size;
    P.poff = static_cast<uint32_t>(poff);
    P.coff = static_cast<uint32_t>(coff);
    P.n = static_cast<uint32_t>(n);
    P.ncells = static_cast<uint32_t>(ncells);
    P.sys_slot = static_cast<uint32_t>(slot);
    XCK(cudaMemsetAsync(b->d_flag, 0, sizeof(unsigned int), st));
    b->launches += launch_place(P, a, b->d_flag, b->sm_count, st);
    unsigned int flag = 0;
    XCK(cudaMemcpyAsync(&flag, b->d_flag, sizeof(flag), cudaMemcpyDeviceToHost, st));
    XCK(cudaStreamSynchronize(st));
    int rc = check_launch();
    if (rc) return rc;
    if (flag & 1u) return fail(XNB_ERR_ARG, "a particle position lies outside every representable cell");
    if (!(flag & 2u)) return XNB_OK;
  }
  // Host staging in storage order.
  std::vector<double> h[6];
  for (auto& v : h) v.resize(static_cast<size_t>(n));
  std::vector<uint64_t> hid(static_cast<size_t>(n));
  std::vector<uint32_t> hcell(static_cast<size_t>(n));
  std::vector<uint32_t> cstart(ncells), cn(ncells, 0), csys(ncells, static_cast<uint32_t>(slot));
  if (cell_counts) {
    int64_t q = 0;
    for (uint64_t c = 0; c < ncells; ++c) {
      if (cell_counts[c] < 0) return fail(XNB_ERR_ARG, "negative cell count");
      cn[c] = static_cast<uint32_t>(cell_counts[c]);
      cstart[c] = static_cast<uint32_t>(poff + q);
      for (int64_t t = 0; t < cell_counts[c]; ++t, ++q) {
        if (q >= n) return fail(XNB_ERR_ARG, "cell counts exceed n");
        h[0][q] = rx[q]; h[1][q] = ry[q]; h[2][q] = rz[q];
        h[3][q] = vx[q]; h[4][q] = vy[q]; h[5][q] = vz[q];
        hid[q] = id[q];
        hcell[q] = static_cast<uint32_t>(coff + static_cast<int64_t>(c));
      }
    }
    if (q != n) return fail(XNB_ERR_ARG, "cell counts do not sum to n");
  } else {
    std::vector<uint32_t> pc(static_cast<size_t>(n));
    std::vector<double> wr(static_cast<size_t>(n) * 3);
    for (int64_t q = 0; q < n; ++q) {
      double r[3] = {rx[q], ry[q], rz[q]};
      int loc[3];
      periodic_location(*p, r, loc);
      pc[q] = static_cast<uint32_t>((static_cast<uint64_t>(loc[2]) * p->dims[1] + loc[1]) * p->dims[0] + loc[0]);
      wr[q * 3 + 0] = r[0]; wr[q * 3 + 1] = r[1]; wr[q * 3 + 2] = r[2];
      cn[pc[q]]++;
    }
    uint32_t run = static_cast<uint32_t>(poff);
    for (uint64_t c = 0; c < ncells; ++c) {
      cstart[c] = run;
      run += cn[c];
    }
    std::vector<uint32_t> fillc(ncells, 0);
    for (int64_t q = 0; q < n; ++q) {
      const uint32_t c = pc[q];
      const uint64_t dst = cstart[c] - static_cast<uint64_t>(poff) + fillc[c]++;
      h[0][dst] = wr[q * 3 + 0]; h[1][dst] = wr[q * 3 + 1]; h[2][dst] = wr[q * 3 + 2];
      h[3][dst] = vx[q]; h[4][dst] = vy[q]; h[5][dst] = vz[q];
      hid[dst] = id[q];
      hcell[dst] = static_cast<uint32_t>(coff) + c;
    }
  }
  const size_t nb = static_cast<size_t>(n);
  double* dsts[6] = {a.rx, a.ry, a.rz, a.vx, a.vy, a.vz};
  for (int k = 0; k < 6; ++k)
    if (nb) XCK(cudaMemcpyAsync(dsts[k] + poff, h[k].data(), nb * sizeof(double), cudaMemcpyHostToDevice, st));
  if (nb) {
    XCK(cudaMemcpyAsync(a.id + poff, hid.data(), nb * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    XCK(cudaMemcpyAsync(a.pcell + poff, hcell.data(), nb * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    std::vector<float4> hpf(nb), hlo(nb);
    for (size_t q = 0; q < nb; ++q) {
      const double r0 = h[0][q] - p->origin[0], r1 = h[1][q] - p->origin[1], r2 = h[2][q] - p->origin[2];
      hpf[q] = make_float4(static_cast<float>(r0), static_cast<float>(r1), static_cast<float>(r2), 0.f);
      hlo[q] = make_float4(static_cast<float>(r0 - static_cast<double>(hpf[q].x)),
                           static_cast<float>(r1 - static_cast<double>(hpf[q].y)),
                           static_cast<float>(r2 - static_cast<double>(hpf[q].z)), 0.f);
    }
    XCK(cudaMemcpyAsync(a.pf + poff, hpf.data(), nb * sizeof(float4), cudaMemcpyHostToDevice, st));
    XCK(cudaMemcpyAsync(a.pflo + poff, hlo.data(), nb * sizeof(float4), cudaMemcpyHostToDevice, st));
    XCK(cudaMemsetAsync(a.fx + poff, 0, nb * sizeof(double), st));
    XCK(cudaMemsetAsync(a.fy + poff, 0, nb * sizeof(double), st));
    XCK(cudaMemsetAsync(a.fz + poff, 0, nb * sizeof(double), st));
    XCK(cudaMemsetAsync(a.pe + poff, 0, nb * sizeof(double), st));
    XCK(cudaMemsetAsync(a.nbr_cnt + poff, 0, nb * sizeof(uint32_t), st));
    XCK(cudaMemsetAsync(a.ptype + poff, 0, nb * sizeof(uint8_t), st));
    XCK(cudaMemsetAsync(a.nbr_start + poff, 0, nb * sizeof(uint32_t), st));
  }
  XCK(cudaMemcpyAsync(a.cell_start + coff, cstart.data(), ncells * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  XCK(cudaMemcpyAsync(a.cell_n + coff, cn.data(), ncells * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  XCK(cudaMemcpyAsync(a.cell_sys + coff, csys.data(), ncells * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  // the staging vectors are local: finish the copies before they go
  XCK(cudaStreamSynchronize(st));
  return XNB_OK;
}

}  // namespace

int xnb_system_remove(xnb_batch* b, int32_t s, void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  if (s < 0) return fail(XNB_ERR_ARG, "remove needs one system");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SysHost& h = b->sys[s];
  XCK(cudaMemsetAsync(b->a.pcell + h.d.part_base, 0xFF, static_cast<size_t>(h.d.npart) * sizeof(uint32_t), st));
  XCK(cudaMemsetAsync(b->a.cell_sys + h.d.cell_base, 0xFF, static_cast<size_t>(h.d.ncells) * sizeof(uint32_t), st));
  XCK(cudaMemsetAsync(b->a.cell_n + h.d.cell_base, 0, static_cast<size_t>(h.d.ncells) * sizeof(uint32_t), st));
  SysState zero{};
  XCK(cudaMemcpyAsync(b->d_st + s, &zero, sizeof(SysState), cudaMemcpyHostToDevice, st));
  XCK(cudaStreamSynchronize(st));
  b->parts.release(h.d.part_base);
  b->cells.release(h.d.cell_base);
  if (h.list_off >= 0) b->lists.release(static_cast<uint64_t>(h.list_off));
  h = SysHost{};
  {
    const int urc = upload_segments(b, st);
    if (urc) return urc;
  }
  return XNB_OK;
}

int xnb_system_info_get(xnb_batch* b, int32_t s, xnb_system_info* info, void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  if (s < 0 || !info) return fail(XNB_ERR_ARG, "info needs one system");
  rc = pull_states(b, static_cast<cudaStream_t>(stream));
  if (rc) return rc;
  const SysHost& h = b->sys[s];
  info->n_particles = h.d.npart;
  info->n_cells = h.d.ncells;
  info->list_used = static_cast<int64_t>(b->h_st[s].list_used);
  info->list_cap = static_cast<int64_t>(h.list_cap);
  info->rebuilds = static_cast<int64_t>(b->h_st[s].rebuilds);
  info->error_bits = b->h_st[s].error;
  info->max_cell = b->h_st[s].max_cell;
  info->active = h.active ? 1 : 0;
  info->max_nbr = b->h_st[s].max_nbr;
  return XNB_OK;
}

int xnb_system_download(xnb_batch* b, int32_t s, double* rx, double* ry, double* rz, double* vx, double* vy,
                        double* vz, double* fx, double* fy, double* fz, uint64_t* id, int32_t* cell, double* pe,
                        void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  if (s < 0) return fail(XNB_ERR_ARG, "download needs one system");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const SysHost& h = b->sys[s];
  const size_t n = h.d.npart, o = h.d.part_base;
  double* outs[10] = {rx, ry, rz, vx, vy, vz, fx, fy, fz, pe};
  const double* ins[10] = {b->a.rx, b->a.ry, b->a.rz, b->a.vx, b->a.vy, b->a.vz, b->a.fx, b->a.fy, b->a.fz, b->a.pe};
  for (int k = 0; k < 10; ++k)
    if (outs[k] && n) XCK(cudaMemcpyAsync(outs[k], ins[k] + o, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (id && n) XCK(cudaMemcpyAsync(id, b->a.id + o, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
  std::vector<uint32_t> pc;
  if (cell && n) {
    pc.resize(n);
    XCK(cudaMemcpyAsync(pc.data(), b->a.pcell + o, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  }
  XCK(cudaStreamSynchronize(st));
  if (cell)
    for (size_t q = 0; q < n; ++q) cell[q] = static_cast<int32_t>(pc[q] - h.d.cell_base);
  return XNB_OK;
}

int xnb_system_pairs(xnb_batch* b, int32_t s, uint64_t* id_a, uint64_t* id_b, int32_t* nbh_count, int64_t cap,
                     int64_t* n_out, void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  if (s < 0) return fail(XNB_ERR_ARG, "pairs needs one system");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const SysHost& h = b->sys[s];
  rc = pull_states(b, st);
  if (rc) return rc;
  const size_t n = h.d.npart, o = h.d.part_base;
  std::vector<uint32_t> start(n), cnt(n);
  std::vector<uint64_t> ids(n);
  const uint64_t used = h.list_off >= 0 ? h.list_cap : 0;
  std::vector<uint32_t> list(used);
  if (n) {
    XCK(cudaMemcpyAsync(start.data(), b->a.nbr_start + o, n * 4, cudaMemcpyDeviceToHost, st));
    XCK(cudaMemcpyAsync(cnt.data(), b->a.nbr_cnt + o, n * 4, cudaMemcpyDeviceToHost, st));
    XCK(cudaMemcpyAsync(ids.data(), b->a.id + o, n * 8, cudaMemcpyDeviceToHost, st));
  }
  if (used && h.list_off >= 0)
    XCK(cudaMemcpyAsync(list.data(), b->a.nbr + h.d.list_base, used * 4, cudaMemcpyDeviceToHost, st));
  XCK(cudaStreamSynchronize(st));
  int64_t k = 0;
  for (size_t q = 0; q < n; ++q) {
    if (nbh_count) nbh_count[q] = static_cast<int32_t>(cnt[q]);
    for (uint32_t t = 0; t < cnt[q]; ++t, ++k) {
      if (k < cap) {
        const uint64_t pos = static_cast<uint64_t>(start[q]) + t;
        if (pos >= used) return fail(XNB_ERR_DEVICE, "neighbour entry outside the list segment");
        const uint32_t e = list[pos];
        if (id_a) id_a[k] = ids[q];
        if (id_b) id_b[k] = ids[e >> 5];
      }
    }
  }
  if (n_out) *n_out = k;
  return XNB_OK;
}

// The pairs of a particle range: only that range's counts, starts and list
// block cross to the host (with the system's ids, to translate the entries).
int xnb_system_pairs_range(xnb_batch* b, int32_t s, int64_t first, int64_t count, uint64_t* id_b,
                           int32_t* nbh_count, int64_t cap, int64_t* n_out, void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  if (s < 0) return fail(XNB_ERR_ARG, "pairs needs one system");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const SysHost& h = b->sys[s];
  const int64_t n = h.d.npart;
  if (first < 0 || count < 0 || first + count > n) return fail(XNB_ERR_ARG, "particle range outside the system");
  const size_t o = h.d.part_base + static_cast<size_t>(first), m = static_cast<size_t>(count);
  std::vector<uint32_t> start(m), cnt(m);
  std::vector<uint64_t> ids(static_cast<size_t>(n));
  if (m) {
    XCK(cudaMemcpyAsync(start.data(), b->a.nbr_start + o, m * 4, cudaMemcpyDeviceToHost, st));
    XCK(cudaMemcpyAsync(cnt.data(), b->a.nbr_cnt + o, m * 4, cudaMemcpyDeviceToHost, st));
  }
  if (n) XCK(cudaMemcpyAsync(ids.data(), b->a.id + h.d.part_base, static_cast<size_t>(n) * 8, cudaMemcpyDeviceToHost, st));
  XCK(cudaStreamSynchronize(st));
  const uint64_t used = h.list_off >= 0 ? h.list_cap : 0;
  uint64_t lo = used, hi = 0;
  for (size_t q = 0; q < m; ++q) {
    if (!cnt[q]) continue;
    lo = std::min<uint64_t>(lo, start[q]);
    hi = std::max<uint64_t>(hi, static_cast<uint64_t>(start[q]) + cnt[q]);
  }
  if (hi > used) return fail(XNB_ERR_DEVICE, "neighbour entry outside the list segment");
  std::vector<uint32_t> list(hi > lo ? hi - lo : 0);
  if (!list.empty()) {
    XCK(cudaMemcpyAsync(list.data(), b->a.nbr + h.d.list_base + lo, list.size() * 4, cudaMemcpyDeviceToHost, st));
    XCK(cudaStreamSynchronize(st));
  }
  int64_t k = 0;
  for (size_t q = 0; q < m; ++q) {
    if (nbh_count) nbh_count[q] = static_cast<int32_t>(cnt[q]);
    for (uint32_t t = 0; t < cnt[q]; ++t, ++k) {
      if (k < cap && id_b) {
        const uint32_t e = list[static_cast<uint64_t>(start[q]) + t - lo];
        if ((e >> 5) >= static_cast<uint64_t>(n)) return fail(XNB_ERR_DEVICE, "neighbour entry outside the system");
        id_b[k] = ids[e >> 5];
      }
    }
  }
  if (n_out) *n_out = k;
  return XNB_OK;
}

int xnb_system_energy(xnb_batch* b, int32_t s, double* ke, double* pe, void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  if (s < 0) return fail(XNB_ERR_ARG, "energy needs one system");
  const SysHost& h = b->sys[s];
  const size_t n = h.d.npart;
  std::vector<double> v[3], e(n);
  for (auto& x : v) x.resize(n);
  rc = xnb_system_download(b, s, nullptr, nullptr, nullptr, v[0].data(), v[1].data(), v[2].data(), nullptr, nullptr,
                           nullptr, nullptr, nullptr, e.data(), stream);
  if (rc) return rc;
  double k = 0.0, p = 0.0;
  for (size_t q = 0; q < n; ++q) {
    k += 0.5 * h.d.mass * ((v[0][q] * v[0][q] + v[1][q] * v[1][q]) + v[2][q] * v[2][q]);
    p += e[q];
  }
  if (ke) *ke = k;
  if (pe) *pe = p;
  return XNB_OK;
}

int xnb_init_particles(xnb_batch* b, int32_t s, int32_t precision, void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  int base = 0;
  bool newton = false;
  rc = decode_precision(precision, &base, &newton);
  if (rc) return rc;
  precision = base;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  XCK(cudaSetDevice(b->device));
  const Extent ex = b->extent();
  // init marks every selected system; the counter then starts from zero
  b->launches += launch_mark_rebuild(ex, b->d_st, 0, s, b->a.any_rebuild, st);
  b->launches += launch_rebin(ex, b->d_sys, b->d_st, b->a, st, precision == XNB_PREC_FP64_EXACT);
  rc = neighbors_sync(b, st);
  if (rc) return rc;
  b->launches += launch_force(ex, b->d_sys, b->d_st, b->a, precision, true, false, s, st, newton);
  rc = pull_states(b, st);
  if (rc) return rc;
  for (int q = 0; q < ex.nsys; ++q) {
    if (!b->sys[q].active || !b->h_st[q].rebuild) continue;
    b->h_st[q].rebuilds = 0;
    b->h_st[q].moved = 0;
    b->h_st[q].rebuild = 0;
    XCK(cudaMemcpyAsync(b->d_st + q, b->h_st + q, sizeof(SysState), cudaMemcpyHostToDevice, st));
    b->sys[q].initialised = true;
  }
  XCK(cudaStreamSynchronize(st));
  rc = check_launch();
  if (rc) return rc;
  return xnb_check_errors(b, stream);
}

int xnb_push_f_v_r(xnb_batch* b, int32_t s, double dt_scale, void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  const Extent ex = b->extent();
  b->launches += launch_first_half(ex, b->d_sys, b->d_st, b->a, true, false, false, dt_scale, 0.0, true, s,
                    static_cast<cudaStream_t>(stream));
  return check_launch();
}

int xnb_push_f_v(xnb_batch* b, int32_t s, double dt_scale, void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  const Extent ex = b->extent();
  b->launches += launch_first_half(ex, b->d_sys, b->d_st, b->a, false, true, false, 1.0, dt_scale, true, s,
                    static_cast<cudaStream_t>(stream));
  return check_launch();
}

int xnb_particle_displ_over(xnb_batch* b, int32_t s, int64_t* count_out, void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const Extent ex = b->extent();
  b->launches += launch_clear_moved(ex, b->d_st, st);
  b->launches += launch_first_half(ex, b->d_sys, b->d_st, b->a, false, false, true, 1.0, 0.5, true, s, st);
  rc = pull_states(b, st);
  if (rc) return rc;
  if (count_out) {
    if (s >= 0) {
      count_out[0] = static_cast<int64_t>(b->h_st[s].moved);
    } else {
      for (int q = 0; q < ex.nsys; ++q) count_out[q] = static_cast<int64_t>(b->h_st[q].moved);
    }
  }
  return check_launch();
}

int xnb_update_particles_full(xnb_batch* b, int32_t s, void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const Extent ex = b->extent();
  b->launches += launch_mark_rebuild(ex, b->d_st, 0, s, b->a.any_rebuild, st);
  b->launches += launch_rebin(ex, b->d_sys, b->d_st, b->a, st);
  rc = neighbors_sync(b, st);
  if (rc) return rc;
  clear_rebuild(b, st);
  return check_launch();
}

int xnb_chunk_neighbors(xnb_batch* b, int32_t s, void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const Extent ex = b->extent();
  b->launches += launch_mark_rebuild(ex, b->d_st, 0, s, b->a.any_rebuild, st);
  rc = neighbors_sync(b, st);
  if (rc) return rc;
  clear_rebuild(b, st);
  return check_launch();
}

int xnb_backup_r(xnb_batch* b, int32_t s, void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const Extent ex = b->extent();
  b->launches += launch_mark_rebuild(ex, b->d_st, 0, s, b->a.any_rebuild, st);
  b->launches += launch_backup(ex, b->d_sys, b->d_st, b->a, st);
  clear_rebuild(b, st);
  return check_launch();
}

int xnb_lennard_jones_force(xnb_batch* b, int32_t s, int32_t precision, int32_t with_energy, void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  int base = 0;
  bool newton = false;
  rc = decode_precision(precision, &base, &newton);
  if (rc) return rc;
  const Extent ex = b->extent();
  b->launches += launch_force(ex, b->d_sys, b->d_st, b->a, base, with_energy != 0, false, s,
                              static_cast<cudaStream_t>(stream), newton);
  return check_launch();
}

int xnb_ghost_update_r(xnb_batch* b, int32_t s, void*) { return check_sys(b, s); }

int xnb_step(xnb_batch* b, int32_t nsteps, int32_t precision, int32_t flags, void* stream) {
  if (!b) return fail(XNB_ERR_ARG, "null batch");
  int base = 0;
  bool newton = false;
  int rc0 = decode_precision(precision, &base, &newton);
  if (rc0) return rc0;
  precision = base;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const Extent ex = b->extent();
  const bool exact = precision == XNB_PREC_FP64_EXACT;
  const bool energy = (flags & XNB_STEP_ENERGY) != 0;
  for (int k = 0; k < nsteps; ++k) {
    // verlet_first_half + trigger_move_particles
    b->launches += launch_first_half(ex, b->d_sys, b->d_st, b->a, true, true, true, 1.0, 0.5, exact, -1, st);
    b->launches += launch_mark_rebuild(ex, b->d_st, 1, -1, b->a.any_rebuild, st);
    bool rebuild = true;
    if (flags & XNB_STEP_HOST_SYNC) {
      int rc = pull_states(b, st);
      if (rc) return rc;
      rebuild = false;
      for (int q = 0; q < ex.nsys; ++q)
        if (b->sys[q].active && b->h_st[q].moved > 0) rebuild = true;
    }
    if (rebuild) {
      // update_particles_full
      b->launches += launch_rebin(ex, b->d_sys, b->d_st, b->a, st, exact);
      if (flags & XNB_STEP_HOST_SYNC) {
        int rc = neighbors_sync(b, st);
        if (rc) return rc;
      } else {
        b->launches += launch_neighbors(ex, b->d_sys, b->d_st, b->a, b->stage_cap, list_buf(b), st, b->build_form,
                                        b->subcell_prune != 0);
      }
    }
    // compute_all_forces_energy + verlet_second_half
    b->launches += launch_force(ex, b->d_sys, b->d_st, b->a, precision, energy, true, -1, st, newton);
    b->launches += launch_clear_moved(ex, b->d_st, st);
  }
  return check_launch();
}

int xnb_step_persistent(xnb_batch* b, int32_t nsteps, int32_t precision, int32_t flags, void* stream) {
  if (!b) return fail(XNB_ERR_ARG, "null batch");
  if (nsteps < 0) return fail(XNB_ERR_ARG, "nsteps must be >= 0");
  if (flags & ~(XNB_STEP_HOST_SYNC | XNB_STEP_ENERGY | XNB_STEP_BARRIER_CHECK)) return fail(XNB_ERR_ARG, "bad flags");
  int base = 0;
  bool newton = false;
  int rc = decode_precision(precision, &base, &newton);
  if (rc) return rc;
  if (newton) return fail(XNB_ERR_ARG, "the persistent step loop runs the full-list traversal");
  for (const SysHost& h : b->sys)
    if (h.active && !h.initialised) return fail(XNB_ERR_ARG, "call xnb_init_particles first");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  XCK(cudaSetDevice(b->device));
  const Extent ex = b->extent();
  const bool exact = base == XNB_PREC_FP64_EXACT;
  const bool energy = (flags & XNB_STEP_ENERGY) != 0;
  const bool check = (flags & XNB_STEP_BARRIER_CHECK) != 0;
  int remaining = nsteps;
  while (remaining > 0 || check) {
    XCK(cudaMemsetAsync(b->d_ctl, 0, sizeof(StepCtl), st));
    b->launches += launch_steps_persistent(ex, b->d_sys, b->d_st, b->a, base, energy, b->d_ctl, remaining, check, st);
    rc = check_launch();
    if (rc) return rc;
    StepCtl h{};
    XCK(cudaMemcpyAsync(&h, b->d_ctl, sizeof(StepCtl), cudaMemcpyDeviceToHost, st));
    XCK(cudaStreamSynchronize(st));
    if (h.error) return fail(XNB_ERR_DEVICE, "a grid barrier of the persistent step loop ran out of time");
    if (check) return fail(XNB_ERR_ARG, "the barrier check did not run out");
    remaining -= static_cast<int>(h.steps_done);
    if (h.stopped) {
      // the rest of the step whose trigger fired: rebuild path, forces and kick
      b->launches += launch_mark_rebuild(ex, b->d_st, 1, -1, b->a.any_rebuild, st);
      b->launches += launch_rebin(ex, b->d_sys, b->d_st, b->a, st, exact);
      rc = neighbors_sync(b, st);
      if (rc) return rc;
      b->launches += launch_force(ex, b->d_sys, b->d_st, b->a, base, energy, true, -1, st, false);
      b->launches += launch_clear_moved(ex, b->d_st, st);
      remaining -= 1;
    }
  }
  return check_launch();
}

int xnb_step_graph_create(xnb_batch* b, int32_t nsteps, int32_t precision, int32_t flags, void* stream,
                          xnb_graph** out) {
  if (!b || !out) return fail(XNB_ERR_ARG, "null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (st == nullptr) return fail(XNB_ERR_ARG, "graph capture needs a non-default stream");
  XCK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  const int rc = xnb_step(b, nsteps, precision, flags & ~XNB_STEP_HOST_SYNC, stream);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(st, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return fail(XNB_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
  xnb_graph* G = new xnb_graph();
  G->graph = g;
  G->batch = b;
  const Extent ex = b->extent();
  G->n_part = ex.n_part;
  G->n_cells = ex.n_cells;
  G->nsys = ex.nsys;
  G->far_coords = ex.far_coords;
  G->force_form = ex.force_form;
  G->n_seg = ex.n_seg;
  G->lbuf = list_buf(b);
  G->stage_cap = b->stage_cap;
  G->force_block = b->force_block;
  G->force_lanes = b->force_lanes;
  G->build_form = b->build_form;
  G->subcell_prune = b->subcell_prune;
  const cudaError_t ie = cudaGraphInstantiate(&G->exec, g, 0);
  if (ie != cudaSuccess) {
    cudaGraphDestroy(g);
    delete G;
    return fail(XNB_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(ie));
  }
  *out = G;
  return XNB_OK;
}

int xnb_graph_is_current(const xnb_graph* g) {
  if (!g || !g->batch) return 0;
  const xnb_batch* b = g->batch;
  const Extent ex = b->extent();
  return (ex.n_part == g->n_part && ex.n_cells == g->n_cells && ex.nsys == g->nsys && ex.far_coords == g->far_coords &&
          ex.force_form == g->force_form && ex.n_seg == g->n_seg &&
          list_buf(b) == g->lbuf &&
          b->stage_cap == g->stage_cap && b->force_block == g->force_block && b->force_lanes == g->force_lanes &&
          b->build_form == g->build_form && b->subcell_prune == g->subcell_prune)
             ? 1
             : 0;
}

int xnb_graph_launch(xnb_graph* g, void* stream) {
  if (!g) return fail(XNB_ERR_ARG, "null graph");
  // a graph captured for a smaller extent would skip the particles and cells of
  // systems added beyond it: refuse instead of stepping part of the batch
  if (!xnb_graph_is_current(g))
    return fail(XNB_ERR_ARG, "the batch's extent or launch configuration changed since the graph was captured");
  XCK(cudaGraphLaunch(g->exec, static_cast<cudaStream_t>(stream)));
  return XNB_OK;
}

int xnb_graph_destroy(xnb_graph* g) {
  if (!g) return XNB_OK;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
  return XNB_OK;
}

int xnb_check_errors(xnb_batch* b, void* stream) {
  if (!b) return fail(XNB_ERR_ARG, "null batch");
  int rc = pull_states(b, static_cast<cudaStream_t>(stream));
  if (rc) return rc;
  const Extent ex = b->extent();
  for (int q = 0; q < ex.nsys; ++q) {
    if (!b->sys[q].active) continue;
    const uint32_t e = b->h_st[q].error;
    if (e & kErrListOverflow) return fail(XNB_ERR_CAPACITY, "neighbour list segment overflow in system " + std::to_string(q));
    if (e) return fail(XNB_ERR_DEVICE, "device error bits " + std::to_string(e) + " in system " + std::to_string(q));
  }
  return XNB_OK;
}

int xnb_batch_set_tuning(xnb_batch* b, int32_t stage_cap, int32_t force_block) {
  if (!b) return fail(XNB_ERR_ARG, "null batch");
  if (stage_cap <= 0 || stage_cap > 1024) return fail(XNB_ERR_ARG, "stage_cap must be in 1..1024");
  if (force_block <= 0 || force_block % 32 || force_block > 256)
    return fail(XNB_ERR_ARG, "force_block must be a multiple of 32 and at most 256");
  b->stage_cap = (stage_cap + 31) / 32 * 32;
  b->force_block = force_block;
  return XNB_OK;
}

int xnb_batch_set_force_lanes(xnb_batch* b, int32_t lanes) {
  if (!b) return fail(XNB_ERR_ARG, "null batch");
  if (lanes != 1 && lanes != 2 && lanes != 4) return fail(XNB_ERR_ARG, "force lanes per particle must be 1, 2 or 4");
  b->force_lanes = lanes;
  return XNB_OK;
}

int xnb_batch_set_force_form(xnb_batch* b, int32_t form) {
  if (!b) return fail(XNB_ERR_ARG, "null batch");
  if (form != XNB_FORCE_THREAD && form != XNB_FORCE_STAGED) return fail(XNB_ERR_ARG, "unknown force traversal form");
  if (form == XNB_FORCE_STAGED && b->force_form != kForceStaged) {
    XCK(cudaSetDevice(b->device));
    if (!b->a.nbr16) {
      int rc = dalloc(b, &b->a.nbr16, b->lists.cap);
      if (rc) return rc;
      rc = dalloc(b, &b->a.seg, static_cast<uint64_t>(b->cells.cap) + 1);
      if (rc) return rc;
      rc = upload_segments(b, nullptr);
      if (rc) return rc;
    }
    // the current lists get their compact entries now; later builds write them as they go
    XCK(cudaDeviceSynchronize());
    Extent ex = b->extent();
    ex.force_form = kForceStaged;
    b->launches += launch_compact_lists(ex, b->d_sys, b->d_st, b->a, nullptr, true);
    XCK(cudaDeviceSynchronize());
  }
  b->force_form = form == XNB_FORCE_STAGED ? kForceStaged : kForceThread;
  return check_launch();
}

int xnb_batch_set_build_form(xnb_batch* b, int32_t form) {
  if (!b) return fail(XNB_ERR_ARG, "null batch");
  if (form != XNB_BUILD_ROWS && form != XNB_BUILD_WARP && form != XNB_BUILD_HALF)
    return fail(XNB_ERR_ARG, "unknown neighbour-build form");
  if (form == XNB_BUILD_HALF && !b->a.nmask) {
    XCK(cudaSetDevice(b->device));
    const uint64_t P = static_cast<uint64_t>(b->cfg.particle_capacity);
    int rc = dalloc(b, &b->a.nmask, 27 * P);
    if (rc) return rc;
    b->a.nmask_stride = P;
  }
  b->build_form = form == XNB_BUILD_ROWS ? kBuildRows : (form == XNB_BUILD_WARP ? kBuildWarp : kBuildHalf);
  return XNB_OK;
}

int xnb_batch_set_subcell_pruning(xnb_batch* b, int32_t on) {
  if (!b) return fail(XNB_ERR_ARG, "null batch");
  if (on != 0 && on != 1) return fail(XNB_ERR_ARG, "subcell pruning is 0 or 1");
  b->subcell_prune = on;
  return XNB_OK;
}

int xnb_autotune(xnb_batch* b, int32_t trial_steps, int32_t precision, void* stream, xnb_tuning* out) {
  if (!b || !out) return fail(XNB_ERR_ARG, "null argument");
  if (trial_steps <= 0) return fail(XNB_ERR_ARG, "trial_steps must be positive");
  if (precision != XNB_PREC_FP64 && precision != XNB_PREC_MIXED)
    return fail(XNB_ERR_ARG, "autotune for XNB_PREC_FP64 or XNB_PREC_MIXED");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  XCK(cudaSetDevice(b->device));
  uint64_t atoms = 0;
  for (const SysHost& h : b->sys)
    if (h.active) atoms += h.d.npart;
  if (atoms == 0) return fail(XNB_ERR_ARG, "no resident particles");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  XCK(cudaEventCreate(&e0));
  XCK(cudaEventCreate(&e1));
  int trials = 0;
  auto rate_of = [&](int sc, int fb, int nw, int bf, int fl, int ff, double* rate) -> int {
    int rc = xnb_batch_set_tuning(b, sc, fb);
    if (rc) return rc;
    rc = xnb_batch_set_force_form(b, ff);
    if (rc) return rc;
    rc = xnb_batch_set_build_form(b, bf);
    if (rc) return rc;
    rc = xnb_batch_set_force_lanes(b, fl);
    if (rc) return rc;
    const int32_t prec = precision | (nw ? XNB_PREC_NEWTON : 0);
    rc = xnb_step(b, 1, prec, 0, stream);
    if (rc) return rc;
    if (cudaEventRecord(e0, st) != cudaSuccess) return fail(XNB_ERR_CUDA, "event record");
    rc = xnb_step(b, trial_steps, prec, 0, stream);
    if (rc) return rc;
    if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
      return fail(XNB_ERR_CUDA, "event sync");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    ++trials;
    *rate = static_cast<double>(atoms) * trial_steps / (static_cast<double>(ms) * 1e-3);
    return xnb_check_errors(b, stream);
  };
  // the half-shell build is not searched: it allocates 27 x 8 bytes per particle
  // and measured slower than the lane-per-candidate build
  const int caps[3] = {384, 640, 1024}, blocks[3] = {64, 128, 256}, forms[2] = {XNB_BUILD_ROWS, XNB_BUILD_WARP},
            lanes[3] = {1, 2, 4};
  int best_sc = b->stage_cap, best_fb = b->force_block, best_nw = 0, best_fl = b->force_lanes;
  int best_bf = b->build_form;  // kBuild* and XNB_BUILD_* share their values
  // the batch's force form is kept: the staged form allocates 2 bytes per list
  // entry when switched on, and it measured slower than the one-thread
  // traversal at every size tried
  const int best_ff = b->force_form == kForceStaged ? XNB_FORCE_STAGED : XNB_FORCE_THREAD;
  double best = 0.0;
  int rc = rate_of(best_sc, best_fb, best_nw, best_bf, best_fl, best_ff, &best);
  // coordinate search: one parameter at a time, the others at their best so far
  // (neighbour-build form, the stage cap of the forms that stage whole
  // neighbourhoods, the force block size, threads per particle of the force
  // traversal and the Newton traversal)
  const int nvals[5] = {2, 3, 3, 3, 2};
  for (int pass = 0; pass < 5 && rc == 0; ++pass) {
    // the pass's knob at its value when the pass starts was timed already (the
    // other knobs stay as they are through the pass): it is not timed again
    // after another value of the knob took the lead
    const int timed = pass == 0 ? best_bf : pass == 1 ? best_sc : pass == 2 ? best_fb : pass == 3 ? best_fl : best_nw;
    for (int v = 0; v < nvals[pass] && rc == 0; ++v) {
      int sc = best_sc, fb = best_fb, nw = best_nw, bf = best_bf, fl = best_fl, val = 0;
      if (pass == 0) bf = val = forms[v];
      else if (pass == 1) sc = val = caps[v];
      else if (pass == 2) fb = val = blocks[v];
      else if (pass == 3) fl = val = lanes[v];
      else nw = val = v;
      if (val == timed) continue;
      double r = 0.0;
      rc = rate_of(sc, fb, nw, bf, fl, best_ff, &r);
      if (rc == 0 && r > best) {
        best = r;
        best_sc = sc;
        best_fb = fb;
        best_nw = nw;
        best_bf = bf;
        best_fl = fl;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  rc = xnb_batch_set_tuning(b, best_sc, best_fb);
  if (rc) return rc;
  rc = xnb_batch_set_build_form(b, best_bf);
  if (rc) return rc;
  rc = xnb_batch_set_force_lanes(b, best_fl);
  if (rc) return rc;
  out->force_form = best_ff;
  out->stage_cap = best_sc;
  out->force_block = best_fb;
  out->build_form = best_bf;
  out->force_lanes = best_fl;
  out->newton = best_nw;
  out->trials = trials;
  out->atom_steps_per_s = best;
  return XNB_OK;
}

int xnb_chunk_neighbors_stream(xnb_batch* b, int32_t s, int32_t offset_tables, uint16_t* stream, int64_t cap,
                               uint64_t* cell_offsets, int64_t* total_out, void* cuda_stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  if (s < 0) return fail(XNB_ERR_ARG, "streams are built for one system");
  if (offset_tables < 0 || offset_tables > 2) return fail(XNB_ERR_ARG, "offset_tables must be 0, 1 or 2");
  if (!cell_offsets) return fail(XNB_ERR_ARG, "cell_offsets is required");
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  XCK(cudaSetDevice(b->device));
  rc = pull_states(b, st);
  if (rc) return rc;
  const SysHost& h = b->sys[s];
  if (h.list_off < 0 || !b->h_st[s].lists_fresh)
    return fail(XNB_ERR_ARG, "positions changed since the last neighbour build: call xnb_chunk_neighbors first");
  if (b->h_st[s].error) return fail(XNB_ERR_DEVICE, "the system has device error bits set");
  const uint32_t ncells = h.d.ncells;
  uint32_t* len = b->a.cell_cnt + h.d.cell_base;  // rebin scratch, free outside a step
  auto* off = reinterpret_cast<unsigned long long*>(cell_offsets);
  b->launches += launch_stream_lengths(static_cast<uint32_t>(s), ncells, b->d_sys, b->a, offset_tables, len,
                                       b->sm_count, st);
  b->launches += launch_scan_u32_to_u64(len, off, ncells, b->a.scan_blocks, st);
  unsigned long long total = 0;
  XCK(cudaMemcpyAsync(&total, off + ncells, sizeof(total), cudaMemcpyDeviceToHost, st));
  XCK(cudaStreamSynchronize(st));
  if (total_out) *total_out = static_cast<int64_t>(total);
  if (!stream) return check_launch();
  if (static_cast<int64_t>(total) > cap) return fail(XNB_ERR_CAPACITY, "stream buffer too small");
  XCK(cudaMemsetAsync(b->d_flag, 0, sizeof(unsigned int), st));
  b->launches += launch_stream_write(static_cast<uint32_t>(s), ncells, b->d_sys, b->a, offset_tables, off, stream,
                                     b->d_flag, b->sm_count, st);
  unsigned int flag = 0;
  XCK(cudaMemcpyAsync(&flag, b->d_flag, sizeof(flag), cudaMemcpyDeviceToHost, st));
  XCK(cudaStreamSynchronize(st));
  if (flag) return fail(XNB_ERR_ARG, "a cell holds more than 65535 particles: not representable in the u16 stream");
  return check_launch();
}

int xnb_verify_chunk_neighbors(xnb_batch* b, int32_t s, int32_t offset_tables, const uint16_t* stream,
                               int64_t stream_len, const uint64_t* cell_offsets, int64_t* counts_out,
                               void* cuda_stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  if (s < 0) return fail(XNB_ERR_ARG, "streams are checked for one system");
  if (offset_tables < 0 || offset_tables > 2) return fail(XNB_ERR_ARG, "offset_tables must be 0, 1 or 2");
  if (!stream || !cell_offsets || !counts_out || stream_len < 0) return fail(XNB_ERR_ARG, "null argument");
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  XCK(cudaSetDevice(b->device));
  const SysHost& h = b->sys[s];
  XCK(cudaMemsetAsync(b->d_counts, 0, 6 * sizeof(unsigned long long), st));
  b->launches += launch_stream_verify(static_cast<uint32_t>(s), h.d.ncells, b->d_sys, b->a, offset_tables, stream,
                                      static_cast<uint64_t>(stream_len),
                                      reinterpret_cast<const unsigned long long*>(cell_offsets), b->d_counts,
                                      b->sm_count, st);
  unsigned long long c[6];
  XCK(cudaMemcpyAsync(c, b->d_counts, sizeof(c), cudaMemcpyDeviceToHost, st));
  XCK(cudaStreamSynchronize(st));
  for (int k = 0; k < 6; ++k) counts_out[k] = static_cast<int64_t>(c[k]);
  return check_launch();
}

int xnb_simulation_stats(xnb_batch* b, int32_t s, xnb_sim_stats* out, void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  if (s < 0 || !out) return fail(XNB_ERR_ARG, "simulation_stats needs one system and an output");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  XCK(cudaSetDevice(b->device));
  const SysHost& h = b->sys[s];
  b->launches += launch_stats(static_cast<uint32_t>(s), h.d.npart, b->d_sys, b->a, b->d_stats, b->sm_count, st);
  double v[6];
  unsigned long long n = 0;
  if (copy_stats(b->d_stats, v, &n, st) != 0) return fail(XNB_ERR_CUDA, "simulation_stats copy failed");
  out->particle_count = static_cast<int64_t>(n);
  out->kinetic_sum = v[0];
  out->potential_energy = v[1];
  out->min_vel = v[2];
  out->max_vel = v[3];
  out->min_acc = v[4];
  out->max_acc = v[5];
  return check_launch();
}

int xnb_sample_particles(xnb_batch* b, int32_t s, const uint64_t* ids, int64_t n, double* values, int32_t* found,
                         void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  if (s < 0) return fail(XNB_ERR_ARG, "sampling needs one system");
  if (n < 0 || n > (1 << 24)) return fail(XNB_ERR_ARG, "n must be in [0, 2^24]");
  if (n == 0) return XNB_OK;
  if (!ids || !values || !found) return fail(XNB_ERR_ARG, "null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  XCK(cudaSetDevice(b->device));
  const size_t m = static_cast<size_t>(n);
  std::vector<size_t> order(m);
  for (size_t k = 0; k < m; ++k) order[k] = k;
  std::sort(order.begin(), order.end(), [&](size_t x, size_t y) { return ids[x] < ids[y]; });
  std::vector<uint64_t> sorted(m);
  for (size_t k = 0; k < m; ++k) sorted[k] = ids[order[k]];
  for (size_t k = 1; k < m; ++k)
    if (sorted[k] == sorted[k - 1]) return fail(XNB_ERR_ARG, "ids must be distinct");
  uint64_t* d_ids = nullptr;
  double* d_vals = nullptr;
  int32_t* d_found = nullptr;
  auto release = [&]() {
    if (d_ids) cudaFree(d_ids);
    if (d_vals) cudaFree(d_vals);
    if (d_found) cudaFree(d_found);
  };
  if (cudaMalloc(&d_ids, m * sizeof(uint64_t)) != cudaSuccess || cudaMalloc(&d_vals, m * 9 * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&d_found, m * sizeof(int32_t)) != cudaSuccess) {
    release();
    return fail(XNB_ERR_NOMEM, "sampling buffers");
  }
  std::vector<double> hv(m * 9, 0.0);
  std::vector<int32_t> hf(m, 0);
  bool ok = cudaMemcpyAsync(d_ids, sorted.data(), m * sizeof(uint64_t), cudaMemcpyHostToDevice, st) == cudaSuccess &&
            cudaMemsetAsync(d_found, 0, m * sizeof(int32_t), st) == cudaSuccess;
  if (ok) {
    b->launches += launch_sample(static_cast<uint32_t>(s), b->sys[s].d.npart, b->d_sys, b->a, d_ids,
                                 static_cast<uint32_t>(m), d_vals, d_found, b->sm_count, st);
    ok = cudaMemcpyAsync(hv.data(), d_vals, m * 9 * sizeof(double), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
         cudaMemcpyAsync(hf.data(), d_found, m * sizeof(int32_t), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
         cudaStreamSynchronize(st) == cudaSuccess;
  }
  release();
  if (!ok) return fail(XNB_ERR_CUDA, "sampling failed");
  for (size_t k = 0; k < m; ++k) {
    const size_t dst = order[k];
    found[dst] = hf[k];
    if (hf[k])
      for (int q = 0; q < 9; ++q) values[dst * 9 + q] = hv[k * 9 + q];
  }
  return check_launch();
}

int xnb_system_set_types(xnb_batch* b, int32_t s, const uint64_t* ids, const uint8_t* types, int64_t n,
                         int64_t* matched, void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  if (s < 0) return fail(XNB_ERR_ARG, "types are set for one system");
  if (n < 0 || n > (1 << 24)) return fail(XNB_ERR_ARG, "n must be in [0, 2^24]");
  if (n > 0 && (!ids || !types)) return fail(XNB_ERR_ARG, "null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  XCK(cudaSetDevice(b->device));
  const size_t m = static_cast<size_t>(n);
  std::vector<size_t> order(m);
  for (size_t k = 0; k < m; ++k) order[k] = k;
  std::sort(order.begin(), order.end(), [&](size_t x, size_t y) { return ids[x] < ids[y]; });
  std::vector<uint64_t> sid(m);
  std::vector<uint8_t> sty(m);
  for (size_t k = 0; k < m; ++k) {
    sid[k] = ids[order[k]];
    sty[k] = types[order[k]];
    if (k && sid[k] == sid[k - 1]) return fail(XNB_ERR_ARG, "ids must be distinct");
  }
  uint64_t* d_ids = nullptr;
  uint8_t* d_types = nullptr;
  if (m && (cudaMalloc(&d_ids, m * sizeof(uint64_t)) != cudaSuccess ||
            cudaMalloc(&d_types, m * sizeof(uint8_t)) != cudaSuccess)) {
    if (d_ids) cudaFree(d_ids);
    return fail(XNB_ERR_NOMEM, "type buffers");
  }
  bool ok = cudaMemsetAsync(b->d_counts, 0, sizeof(unsigned long long), st) == cudaSuccess;
  if (ok && m) {
    ok = cudaMemcpyAsync(d_ids, sid.data(), m * sizeof(uint64_t), cudaMemcpyHostToDevice, st) == cudaSuccess &&
         cudaMemcpyAsync(d_types, sty.data(), m, cudaMemcpyHostToDevice, st) == cudaSuccess;
    if (ok)
      b->launches += launch_set_types(static_cast<uint32_t>(s), b->sys[s].d.npart, b->d_sys, b->a, d_ids, d_types,
                                      static_cast<uint32_t>(m), b->d_counts, b->sm_count, st);
  }
  unsigned long long got = 0;
  ok = ok && cudaMemcpyAsync(&got, b->d_counts, sizeof(got), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
       cudaStreamSynchronize(st) == cudaSuccess;
  if (d_ids) cudaFree(d_ids);
  if (d_types) cudaFree(d_types);
  if (!ok) return fail(XNB_ERR_CUDA, "setting types failed");
  if (matched) *matched = static_cast<int64_t>(got);
  return check_launch();
}

int xnb_gravitational_force(xnb_batch* b, int32_t s, double G, const double* type_mass, int32_t ntypes,
                            double rcut, int32_t precision, int32_t flags, void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  if (precision != XNB_PREC_FP64_EXACT && precision != XNB_PREC_FP64)
    return fail(XNB_ERR_ARG, "gravitational_force runs in FP64_EXACT or FP64");
  if (ntypes <= 0 || ntypes > kMaxTypes || !type_mass) return fail(XNB_ERR_ARG, "1 to 16 type masses");
  if (!(rcut > 0.0)) return fail(XNB_ERR_ARG, "rcut must be positive");
  if (flags & ~(XNB_FORCE_ENERGY | XNB_FORCE_ACCUMULATE)) return fail(XNB_ERR_ARG, "bad flags");
  GravParams gp{};
  gp.G = G;
  gp.rcut2 = rcut * rcut;
  gp.ntypes = ntypes;
  for (int t = 0; t < ntypes; ++t) gp.mass[t] = type_mass[t];
  // prefilter threshold: rcut^2 + the largest FP32 error bound of the systems it runs on
  double margin = 0.0;
  for (size_t q = 0; q < b->sys.size(); ++q) {
    const SysHost& h = b->sys[q];
    if (!h.active || (s >= 0 && static_cast<int32_t>(q) != s)) continue;
    const double nbh = std::sqrt(h.d.nbh2);
    if (rcut > nbh) return fail(XNB_ERR_ARG, "rcut above the neighbour distance of the lists");
    double P = 0.0;
    for (int a = 0; a < 3; ++a) P = std::max(P, std::fabs(h.d.period[a]));
    margin = std::max(margin, 4.0 * fp32_d2_error(P, nbh, rcut));
  }
  gp.pre_hi_f = static_cast<float>(gp.rcut2 + margin);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  XCK(cudaSetDevice(b->device));
  XCK(cudaMemsetAsync(b->d_flag, 0, sizeof(unsigned int), st));
  const Extent ex = b->extent();
  b->launches += launch_gravity(ex, b->d_sys, b->d_st, b->a, precision, (flags & XNB_FORCE_ENERGY) != 0,
                                (flags & XNB_FORCE_ACCUMULATE) != 0, s, gp, b->d_flag, st);
  unsigned int flag = 0;
  XCK(cudaMemcpyAsync(&flag, b->d_flag, sizeof(flag), cudaMemcpyDeviceToHost, st));
  XCK(cudaStreamSynchronize(st));
  if (flag & 1u) return fail(XNB_ERR_ARG, "a particle type has no mass");
  return check_launch();
}

int xnb_system_pair_view(xnb_batch* b, int32_t s, xnb_pair_view* out) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  if (s < 0 || !out) return fail(XNB_ERR_ARG, "pair view needs one system and an output");
  const SysHost& h = b->sys[s];
  const size_t o = h.d.part_base;
  xnb_pair_view v{};
  v.n_particles = h.d.npart;
  v.rx = b->a.rx + o;
  v.ry = b->a.ry + o;
  v.rz = b->a.rz + o;
  v.vx = b->a.vx + o;
  v.vy = b->a.vy + o;
  v.vz = b->a.vz + o;
  v.fx = b->a.fx + o;
  v.fy = b->a.fy + o;
  v.fz = b->a.fz + o;
  v.pe = b->a.pe + o;
  v.id = b->a.id + o;
  v.type = b->a.ptype + o;
  v.mirror = b->a.pf + o;
  v.mirror_lo = b->a.pflo + o;
  v.nbr = b->a.nbr + h.d.list_base;
  v.nbr_start = b->a.nbr_start + o;
  v.nbr_count = b->a.nbr_cnt + o;
  v.nbr_half = b->a.nbr_half + o;
  double P = 0.0;
  for (int a = 0; a < 3; ++a) {
    v.origin[a] = h.d.origin[a];
    v.period[a] = h.d.period[a];
    P = std::max(P, std::fabs(h.d.period[a]));
  }
  v.nbh_dist = std::sqrt(h.d.nbh2);
  v.max_period = P;
  v.mass = h.d.mass;
  v.divide_by_mass = h.d.divide_by_mass;
  v.sys = s;
  *out = v;
  return XNB_OK;
}

int64_t xnb_stats_kernel_launches(const xnb_batch* b) { return b ? static_cast<int64_t>(b->launches) : -1; }

}  // extern "C"

struct xnb_snap {
  int device = 0;
  SnapArgs t{};
  std::vector<void*> allocs;
};

extern "C" {

int xnb_snap_create(const xnb_snap_params* p, int32_t device, xnb_snap** out) {
  if (!p || !out) return fail(XNB_ERR_ARG, "xnb_snap_create: params and out required");
  *out = nullptr;
  auto* s = new xnb_snap();
  s->device = device;
  std::string err;
  const int rc = snap_build(*p, device, s->t, s->allocs, err);
  if (rc != XNB_OK) {
    for (void* q : s->allocs) cudaFree(q);
    delete s;
    return fail(rc, "xnb_snap_create: " + err);
  }
  *out = s;
  return XNB_OK;
}

int xnb_snap_destroy(xnb_snap* s) {
  if (!s) return XNB_OK;
  cudaSetDevice(s->device);
  for (void* q : s->allocs) cudaFree(q);
  delete s;
  return XNB_OK;
}

int xnb_snap_force(xnb_batch* b, int32_t s, const xnb_snap* snap, int32_t flags, void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  if (!snap) return fail(XNB_ERR_ARG, "xnb_snap_force: no potential");
  if (snap->device != b->device) return fail(XNB_ERR_ARG, "xnb_snap_force: potential built on another device");
  if (flags & ~(XNB_FORCE_ENERGY | XNB_FORCE_ACCUMULATE | XNB_FORCE_MIXED)) return fail(XNB_ERR_ARG, "bad flags");
  double rad_max = 0.0;
  for (int k = 0; k < snap->t.ntypes; ++k) rad_max = std::max(rad_max, snap->t.radelem[k]);
  const double cut_max = 2.0 * rad_max * snap->t.rcutfac;
  for (size_t q = 0; q < b->sys.size(); ++q) {
    const SysHost& h = b->sys[q];
    if (!h.active || (s >= 0 && static_cast<int32_t>(q) != s)) continue;
    if (cut_max > std::sqrt(h.d.nbh2) * (1.0 + 1e-15))
      return fail(XNB_ERR_ARG, "SNAP cutoff above the neighbour distance of the lists");
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  XCK(cudaSetDevice(b->device));
  XCK(cudaMemsetAsync(b->d_flag, 0, sizeof(unsigned int), st));
  const Extent ex = b->extent();
  b->launches += launch_snap(ex, b->d_sys, b->d_st, b->a, snap->t, s, (flags & XNB_FORCE_ENERGY) != 0,
                             (flags & XNB_FORCE_ACCUMULATE) != 0, (flags & XNB_FORCE_MIXED) != 0, b->d_flag, st);
  unsigned int flag = 0;
  XCK(cudaMemcpyAsync(&flag, b->d_flag, sizeof(flag), cudaMemcpyDeviceToHost, st));
  XCK(cudaStreamSynchronize(st));
  if (flag & 1u) return fail(XNB_ERR_ARG, "a particle type has no SNAP coefficients");
  if (flag & 2u) return fail(XNB_ERR_ARG, "a SNAP environment exceeds 128 neighbours");
  return check_launch();
}

// chunk_neighbors for callers that cannot allocate device memory: only the
// caller's buffers and the library's static scratch array are touched.
int xnb_chunk_neighbors_noalloc(const xnb_lj_params* p, int64_t n, const double* rx, const double* ry,
                                const double* rz, const uint32_t* cell_start, const uint32_t* cell_count,
                                uint32_t* nbr, int64_t nbr_capacity, uint32_t* nbr_start, uint32_t* nbr_count,
                                int64_t* total_out, void* stream) {
  int rc = validate(p);
  if (rc) return rc;
  if (n < 0 || !rx || !ry || !rz || !cell_start || !cell_count || !nbr || !nbr_start || !nbr_count || !total_out ||
      nbr_capacity < 0)
    return fail(XNB_ERR_ARG, "chunk_neighbors without allocation: null buffer or negative size");
  SysDesc d = make_desc(*p);
  d.cell_base = 0;
  d.part_base = 0;
  // the cell count stays 64-bit until the launcher has checked it against its limit
  const uint64_t ncells = static_cast<uint64_t>(p->dims[0]) * static_cast<uint64_t>(p->dims[1]) *
                          static_cast<uint64_t>(p->dims[2]);
  unsigned long long total = 0;
  std::string err;
  const int lr = launch_neighbors_static(d, ncells, static_cast<uint64_t>(n), rx, ry, rz, cell_start, cell_count, nbr,
                                         static_cast<uint64_t>(nbr_capacity), nbr_start, nbr_count, &total,
                                         static_cast<cudaStream_t>(stream), &err);
  if (lr == -1) return fail(XNB_ERR_ARG, err);
  if (lr != 0) return fail(XNB_ERR_CUDA, err);
  *total_out = static_cast<int64_t>(total);
  if (total > static_cast<unsigned long long>(nbr_capacity))
    return fail(XNB_ERR_CAPACITY, "chunk_neighbors without allocation: " + std::to_string(total) +
                                      " entries needed, capacity " + std::to_string(nbr_capacity));
  return XNB_OK;
}

int xnb_system_download_types(xnb_batch* b, int32_t s, uint8_t* type, void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  if (s < 0 || !type) return fail(XNB_ERR_ARG, "download_types needs one system and an output array");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const SysHost& h = b->sys[s];
  if (h.d.npart)
    XCK(cudaMemcpyAsync(type, b->a.ptype + h.d.part_base, h.d.npart, cudaMemcpyDeviceToHost, st));
  XCK(cudaStreamSynchronize(st));
  return XNB_OK;
}

// write_dump (src/io/write_dump.cpp:35-44 over sim_dump_writer.h): the system's
// particles in storage order -- interior cells in linear order, each cell's
// particles in order -- as the writer walks the grid, chunks closed at cell
// boundaries.
int xnb_system_write_dump(xnb_batch* b, int32_t s, const char* filename, uint64_t timestep, double physical_time,
                          int32_t compression_level, int64_t max_part_size, uint32_t extra_flags_clear,
                          void* stream) {
  int rc = check_sys(b, s);
  if (rc) return rc;
  if (s < 0) return fail(XNB_ERR_ARG, "write_dump needs one system");
  const SysHost& h = b->sys[s];
  const size_t n = h.d.npart;
  std::vector<double> r[6];
  for (auto& v : r) v.resize(n);
  std::vector<uint64_t> id(n);
  std::vector<int32_t> cell(n);
  std::vector<uint8_t> type(n);
  rc = xnb_system_download(b, s, r[0].data(), r[1].data(), r[2].data(), r[3].data(), r[4].data(), r[5].data(),
                           nullptr, nullptr, nullptr, id.data(), cell.data(), nullptr, stream);
  if (rc) return rc;
  rc = xnb_system_download_types(b, s, type.data(), stream);
  if (rc) return rc;
  std::vector<int64_t> counts(h.d.ncells, 0);
  for (size_t q = 0; q < n; ++q) {
    if (cell[q] < 0 || static_cast<uint32_t>(cell[q]) >= h.d.ncells)
      return fail(XNB_ERR_DEVICE, "write_dump: a particle has no cell (system in error)");
    ++counts[static_cast<size_t>(cell[q])];
  }
  const int64_t dims[3] = {h.d.dims[0], h.d.dims[1], h.d.dims[2]};
  xnb_dump_domain dom;
  const uint32_t flags = (XNB_DOMAIN_PERIODIC_X | XNB_DOMAIN_PERIODIC_Y | XNB_DOMAIN_PERIODIC_Z |
                          XNB_DOMAIN_EXPANDABLE) & ~extra_flags_clear;
  xnb_dump_domain_init(&dom, h.d.origin, h.d.extent, dims, h.d.cell_size, flags);
  return xnb_dump_write(filename, &dom, timestep, physical_time, static_cast<int64_t>(n), r[0].data(), r[1].data(),
                        r[2].data(), r[3].data(), r[4].data(), r[5].data(), id.data(), type.data(), counts.data(),
                        static_cast<int64_t>(counts.size()), compression_level, max_part_size, 0, 0);
}

}  // extern "C"

namespace xnb {
int set_error(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace xnb
