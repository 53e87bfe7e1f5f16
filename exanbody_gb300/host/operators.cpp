// The hot-path operators under the reference's names, each a thin OperatorNode
// over the C ABI (include/xnb_gpu.h). Input generators (domain, lattice,
// gaussian noise) restate the reference's single-rank behaviour on the host.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <map>
#include <random>
#include <sstream>

#include "xnb_host.hpp"

namespace xnbhost {

Context::~Context() {
  if (snap) xnb_snap_destroy(snap);
  if (batch) xnb_batch_destroy(batch);
}

double Context::get_double(const std::string& k, double dflt) const {
  auto it = slots.find(k);
  return (it == slots.end() || it->second.kind == Node::Null) ? dflt : quantity(it->second);
}
bool Context::get_bool(const std::string& k, bool dflt) const {
  auto it = slots.find(k);
  return (it == slots.end() || it->second.kind == Node::Null) ? dflt : to_bool(it->second);
}
long Context::get_long(const std::string& k, long dflt) const {
  auto it = slots.find(k);
  return (it == slots.end() || it->second.kind == Node::Null) ? dflt : to_long(it->second);
}
void Context::set_bool(const std::string& k, bool v) { slots[k] = Node::make_scalar(v ? "true" : "false"); }
void Context::set_double(const std::string& k, double v) {
  char buf[64];
  std::snprintf(buf, sizeof(buf), "%.17g", v);
  slots[k] = Node::make_scalar(buf);
}

double OperatorNode::param_double(const Context& ctx, const std::string& k, double dflt) const {
  if (const Node* n = local(k)) return quantity(*n);
  return ctx.get_double(k, dflt);
}
bool OperatorNode::param_bool(const Context& ctx, const std::string& k, bool dflt) const {
  if (const Node* n = local(k)) return to_bool(*n);
  return ctx.get_bool(k, dflt);
}

OperatorNodeFactory* OperatorNodeFactory::instance() {
  static OperatorNodeFactory f;
  return &f;
}
void OperatorNodeFactory::register_factory(const std::string& name, Creator c) { m_creators[name] = std::move(c); }
std::unique_ptr<OperatorNode> OperatorNodeFactory::make_operator(const std::string& name) const {
  auto it = m_creators.find(name);
  if (it == m_creators.end()) throw Error("no operator named '" + name + "'");
  auto op = it->second();
  op->set_name(name);
  return op;
}
std::vector<std::string> OperatorNodeFactory::names() const {
  std::vector<std::string> v;
  for (const auto& kv : m_creators) v.push_back(kv.first);
  return v;
}

namespace {

void ck(int rc, const char* what) {
  if (rc != XNB_OK) throw Error(std::string(what) + ": " + xnb_last_error_string());
}

bool gpu_ready(const Context& ctx) { return ctx.batch != nullptr && ctx.sys >= 0; }

// ---------------------------------------------------------------------------
// domain (core/include/exanb/core/domain.h:36-129): periodic cubic-cell grid.
struct DomainOp : OperatorNode {
  std::vector<SlotDecl> slots() const override {
    return {{"cell_size", INPUT, "cubic cell size"}, {"grid_dims", INPUT, "cells per axis"},
            {"bounds", INPUT, "[[xmin,ymin,zmin],[xmax,ymax,zmax]]"}, {"periodic", INPUT, "must be all true"},
            {"domain", OUTPUT, "simulation domain"}};
  }
  void execute(Context& ctx) override {
    const Node* cs = local("cell_size");
    const Node* gd = local("grid_dims");
    const Node* bd = local("bounds");
    if (!cs || !gd || !bd || !gd->is_seq() || !bd->is_seq() || bd->seq.size() != 2)
      throw Error("domain: cell_size, grid_dims and bounds are required");
    if (const Node* per = local("periodic")) {
      for (const auto& p : per->seq)
        if (!to_bool(p)) throw Error("domain: only fully periodic domains are supported");
    }
    if (const Node* xf = local("xform")) {
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
          if (quantity(xf->seq.at(r).seq.at(c)) != (r == c ? 1.0 : 0.0))
            throw Error("domain: only the identity xform is supported");
    }
    if (const Node* ex = local("expandable")) ctx.domain_expandable = to_bool(*ex);
    ctx.params.cell_size = quantity(*cs);
    for (int a = 0; a < 3; ++a) {
      ctx.params.dims[a] = static_cast<int32_t>(to_long(gd->seq.at(a)));
      ctx.params.origin[a] = quantity(bd->seq[0].seq.at(a));
      ctx.params.extent[a] = quantity(bd->seq[1].seq.at(a));
    }
    ctx.domain_set = true;
  }
};

struct NopOp : OperatorNode {
  void execute(Context&) override {}
};

// particle_type_add_properties: { Type: { mass: ..., ... } } -- one particle type here
struct TypePropertiesOp : OperatorNode {
  void execute(Context& ctx) override {
    if (!m_local.is_map() || m_local.map.empty()) return;
    const Node& props = m_local.map.front().second;
    if (const Node* m = props.find("mass")) ctx.mass = quantity(*m);
  }
};

// lattice (grid_cell_particles/include/exanb/grid_cell_particles/generate_particle_lattice.h:247-388):
// FCC sites in (k, j, i, basis) order; a site is kept when it lies inside the
// domain bounds (inclusive) and its cell is an interior cell; ids follow a
// per-domain-cell exclusive scan starting at 1.
struct LatticeOp : OperatorNode {
  void execute(Context& ctx) override {
    if (!ctx.domain_set) throw Error("lattice: domain must come first");
    const Node* st = local("structure");
    // unit-cell bases of lattice_generator.h:140-170
    static const double sc[1][3] = {{.5, .5, .5}};
    static const double bcc[2][3] = {{.0, .0, .0}, {.5, .5, .5}};
    static const double fcc[4][3] = {{.0, .0, .0}, {.0, .5, .5}, {.5, .0, .5}, {.5, .5, .0}};
    if (!st || (st->scalar != "FCC" && st->scalar != "BCC" && st->scalar != "SC"))
      throw Error("lattice: structure SC, BCC or FCC");
    const double(*basis)[3] = st->scalar == "SC" ? sc : st->scalar == "BCC" ? bcc : fcc;
    const int nbasis = st->scalar == "SC" ? 1 : st->scalar == "BCC" ? 2 : 4;
    const Node* sz = local("size");
    if (!sz || !sz->is_seq()) throw Error("lattice: size [a, a, a] required");
    const double a[3] = {quantity(sz->seq.at(0)), quantity(sz->seq.at(1)), quantity(sz->seq.at(2))};
    const auto& p = ctx.params;
    const long D[3] = {p.dims[0], p.dims[1], p.dims[2]};
    const long ncell = D[0] * D[1] * D[2];
    std::vector<std::vector<double>> cx(static_cast<size_t>(ncell)), cy(cx), cz(cx);
    long lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
      lo[d] = static_cast<long>(std::floor(p.origin[d] / a[d])) - 1;
      hi[d] = static_cast<long>(std::ceil(p.extent[d] / a[d])) + 1;
    }
    for (long k = lo[2]; k <= hi[2]; ++k)
      for (long j = lo[1]; j <= hi[1]; ++j)
        for (long i = lo[0]; i <= hi[0]; ++i)
          for (int l = 0; l < nbasis; ++l) {
            const double x = (static_cast<double>(i) + basis[l][0]) * a[0];
            const double y = (static_cast<double>(j) + basis[l][1]) * a[1];
            const double z = (static_cast<double>(k) + basis[l][2]) * a[2];
            if (!(x >= p.origin[0] && x <= p.extent[0] && y >= p.origin[1] && y <= p.extent[1] &&
                  z >= p.origin[2] && z <= p.extent[2]))
              continue;
            const long li = static_cast<long>(std::floor((x - p.origin[0]) / p.cell_size));
            const long lj = static_cast<long>(std::floor((y - p.origin[1]) / p.cell_size));
            const long lk = static_cast<long>(std::floor((z - p.origin[2]) / p.cell_size));
            if (li < 0 || lj < 0 || lk < 0 || li >= D[0] || lj >= D[1] || lk >= D[2]) continue;
            const size_t c = static_cast<size_t>((lk * D[1] + lj) * D[0] + li);
            cx[c].push_back(x);
            cy[c].push_back(y);
            cz[c].push_back(z);
          }
    HostParticles& h = ctx.host;
    h = HostParticles{};
    h.cell_counts.resize(static_cast<size_t>(ncell));
    uint64_t next_id = 1;
    for (size_t c = 0; c < static_cast<size_t>(ncell); ++c) {
      h.cell_counts[c] = static_cast<int64_t>(cx[c].size());
      for (size_t q = 0; q < cx[c].size(); ++q) {
        h.rx.push_back(cx[c][q]);
        h.ry.push_back(cy[c][q]);
        h.rz.push_back(cz[c][q]);
        h.vx.push_back(0.0);
        h.vy.push_back(0.0);
        h.vz.push_back(0.0);
        h.id.push_back(next_id++);
      }
    }
    if (ctx.verbose) std::printf("lattice: %zu particles\n", h.id.size());
  }
};

// gaussian_noise_r (compute/include/exanb/compute/gaussian_noise.h:62-80,150-161)
// with deterministic_noise: one mt19937_64 seeded domain_cell_index*1023 per cell.
struct GaussianNoiseOp : OperatorNode {
  void execute(Context& ctx) override {
    const double sigma = param_double(ctx, "sigma", 1.0);
    if (!ctx.get_bool("deterministic_noise", false))
      throw Error("gaussian_noise_r: only deterministic_noise: true is supported");
    HostParticles& h = ctx.host;
    size_t q = 0;
    for (size_t c = 0; c < h.cell_counts.size(); ++c) {
      std::mt19937_64 re;
      re.seed(static_cast<uint64_t>(c) * 1023u);
      std::normal_distribution<double> g(0.0, sigma);
      for (int64_t t = 0; t < h.cell_counts[c]; ++t, ++q) {
        h.rx[q] += g(re);
        h.ry[q] += g(re);
        h.rz[q] += g(re);
      }
    }
  }
};

struct ReplicateDomainOp : OperatorNode {
  void execute(Context&) override {
    if (const Node* r = local("repeat"))
      for (const auto& x : r->seq)
        if (to_long(x) != 1) throw Error("replicate_domain: only repeat [1,1,1] is supported");
  }
};

// nbh_dist (particle_neighbors/nbh_dist.cpp:45-66)
struct NbhDistOp : OperatorNode {
  void execute(Context& ctx) override {
    const double rcut_max = ctx.get_double("rcut_max", 0.0);
    const double rcut_inc = ctx.get_double("rcut_inc", 0.0);
    ctx.set_double("nbh_dist_lab", rcut_max + rcut_inc);
    ctx.set_double("max_displ", rcut_inc / 2.0);
    ctx.set_double("ghost_dist", (rcut_max + rcut_inc) / 1.0);
  }
};

// init_particles (update-particles.msp:31-36): the host grid goes to the GPU
// (one system of a one-system batch) and is rebinned, sorted, backed up and
// given its neighbour lists. The force chain's parameters come from the deck's
// lennard_jones_force block (read by the runner into `lj.*` slots).
struct InitParticlesOp : OperatorNode {
  void execute(Context& ctx) override {
    if (!ctx.domain_set) throw Error("init_particles: no domain");
    xnb_lj_params& p = ctx.params;
    p.rcut = ctx.get_double("lj.rcut", ctx.get_double("rcut_max", 0.0));
    p.rcut_inc = ctx.get_double("rcut_inc", 0.0);
    p.epsilon = ctx.get_double("lj.epsilon", 1.0);
    p.sigma = ctx.get_double("lj.sigma", 1.0);
    p.dt = ctx.get_double("dt", 0.0);
    p.mass = ctx.mass;
    p.divide_by_mass = ctx.divide_by_mass ? 1 : 0;
    p.amr_enabled = 1;
    p.sub_grid_density = ctx.get_double("sub_grid_density", 6.5);
    HostParticles& h = ctx.host;
    const int64_t n = static_cast<int64_t>(h.id.size());
    int64_t ncell = 1;
    for (int a = 0; a < 3; ++a) ncell *= p.dims[a];
    if (ctx.dry_run) return;
    if (!ctx.batch) {
      xnb_batch_config cfg{};
      cfg.device = 0;
      cfg.max_systems = 1;
      cfg.particle_capacity = n + 64;
      cfg.cell_capacity = ncell + 64;
      const double nb = p.rcut + p.rcut_inc;
      const double rho = static_cast<double>(n) / ((p.extent[0] - p.origin[0]) * (p.extent[1] - p.origin[1]) *
                                                   (p.extent[2] - p.origin[2]));
      cfg.list_capacity = static_cast<int64_t>((2.0 * 4.18879 * nb * nb * nb * rho + 32.0) * static_cast<double>(n)) + 4096;
      ck(xnb_batch_create(&cfg, &ctx.batch), "xnb_batch_create");
    }
    // per-cell input (lattice) or flat input placed by periodic location in
    // input order (read_dump)
    ck(xnb_system_add(ctx.batch, &p, n, h.rx.data(), h.ry.data(), h.rz.data(), h.vx.data(), h.vy.data(),
                      h.vz.data(), h.id.data(), h.cell_counts.empty() ? nullptr : h.cell_counts.data(), 1.3,
                      nullptr, &ctx.sys),
       "xnb_system_add");
    if (std::any_of(h.type.begin(), h.type.end(), [](uint8_t t) { return t != 0; })) {
      int64_t matched = 0;
      ck(xnb_system_set_types(ctx.batch, ctx.sys, h.id.data(), h.type.data(), n, &matched, nullptr),
         "init_particles (types)");
    }
    ck(xnb_update_particles_full(ctx.batch, ctx.sys, nullptr), "init_particles");
  }
};

// push_f_v_r / push_f_v (defbox/include/exanb/defbox/push_vec3_2nd_order.h:85-117,
// push_vec3_1st_order.h:79-106)
struct PushFVROp : OperatorNode {
  void execute(Context& ctx) override {
    const double scale = param_double(ctx, "dt_scale", 1.0);
    if (!ctx.dry_run) ck(xnb_push_f_v_r(ctx.batch, ctx.sys, scale, nullptr), "push_f_v_r");
  }
};
struct PushFVOp : OperatorNode {
  void execute(Context& ctx) override {
    const double scale = param_double(ctx, "dt_scale", 1.0);
    if (!ctx.dry_run) ck(xnb_push_f_v(ctx.batch, ctx.sys, scale, nullptr), "push_f_v");
  }
};

// particle_displ_over (mpi/particle_displ_over.cu:93-177): result = count > 0
struct DisplOverOp : OperatorNode {
  void execute(Context& ctx) override {
    int64_t count = 0;
    if (!ctx.dry_run) ck(xnb_particle_displ_over(ctx.batch, ctx.sys, &count, nullptr), "particle_displ_over");
    ctx.set_bool("result", count > 0);
  }
};

// move_particles (grid_cell_particles/move_particles.cpp:39-48) together with the
// operators the GPU runs in the same pass: migrate_cell_particles, rebuild_amr,
// backup_r, ghost_comm_scheme, ghost_update_all, chunk_neighbors.
struct MoveParticlesOp : OperatorNode {
  void execute(Context& ctx) override {
    if (!ctx.dry_run) ck(xnb_update_particles_full(ctx.batch, ctx.sys, nullptr), "move_particles");
  }
};

struct ChunkNeighborsOp : OperatorNode {
  void execute(Context& ctx) override {
    if (!ctx.dry_run) ck(xnb_chunk_neighbors(ctx.batch, ctx.sys, nullptr), "chunk_neighbors");
  }
};

struct BackupROp : OperatorNode {
  void execute(Context& ctx) override {
    if (!ctx.dry_run) ck(xnb_backup_r(ctx.batch, ctx.sys, nullptr), "backup_r");
  }
};

// zero_particle_force + lennard_jones_force (+ divide_force_by_type_scalar):
// one GPU pass; the zeroing and the division are part of it.
struct LennardJonesOp : OperatorNode {
  void execute(Context& ctx) override {
    if (!ctx.dry_run) ck(xnb_lennard_jones_force(ctx.batch, ctx.sys, ctx.precision, 1, nullptr), "lennard_jones_force");
    ctx.forces_written = true;
  }
};

// zero_particle_force (compute/zero_particle_force.cu:17-53): the force operators
// that follow start from zero (lennard_jones_force zeroes the field itself).
struct ZeroForceOp : OperatorNode {
  void execute(Context& ctx) override { ctx.forces_written = false; }
};

// gravitational_force (contribs/pi/gravitational_force.cu:167-223): slots
// config { G }, rcut; the species mass of particle_type_add_properties for every
// particle (one species here). It adds onto the forces written earlier in the
// step's force block (lennard_jones_force first when both are used), as chained
// force operators add onto the zeroed field.
struct GravityOp : OperatorNode {
  void execute(Context& ctx) override {
    const Node* cfg = local("config");
    const Node* g = cfg ? cfg->find("G") : nullptr;
    if (!g) throw Error("gravitational_force: config { G } required");
    const double G = quantity(*g);
    const Node* rc = local("rcut");
    if (!rc) throw Error("gravitational_force: rcut required");
    const double rcut = quantity(*rc);
    if (ctx.dry_run) return;
    const double mass = ctx.mass;
    const int prec = ctx.precision == XNB_PREC_FP64_EXACT ? XNB_PREC_FP64_EXACT : XNB_PREC_FP64;
    ck(xnb_gravitational_force(ctx.batch, ctx.sys, G, &mass, 1, rcut, prec,
                               XNB_FORCE_ENERGY | (ctx.forces_written ? XNB_FORCE_ACCUMULATE : 0), nullptr),
       "gravitational_force");
    ctx.forces_written = true;
  }
};

// next_time_step: the time step counter and the physical time advance by one step
// snap_force_generic (contribs/md/snap/include/md/snap/snap_force.h:52-372):
// slot parameters { param, coef, nt } naming LAMMPS files (read as
// lib/snap_read_lammps.cpp:30-132 does: `key value` lines over the SnapConfig
// defaults, then `n_materials coefs_per_material`, per material `name radelem
// weight` and one coefficient per line), conv_coef_units (false: coefficients
// stay in eV and forces are converted). Relative file names are taken from the
// deck's directory. Adds onto the forces written earlier in the force block.
struct SnapOp : OperatorNode {
  static std::string resolve(Context& ctx, const std::string& f) {
    return (!f.empty() && f[0] != '/') ? ctx.slots["deck_dir"].scalar + "/" + f : f;
  }
  static void read(const std::string& param, const std::string& coef, xnb_snap_params& p,
                   std::vector<double>& coeffs) {
    std::map<std::string, double> v = {{"rfac0", 0.99363}, {"rmin0", 0.0},      {"rcutfac", 0.0},
                                       {"twojmax", 6.0},    {"nelements", 1.0},  {"bzeroflag", 1.0},
                                       {"switchflag", 1.0}, {"chemflag", 0.0},   {"bnormflag", 0.0},
                                       {"wselfallflag", 0.0}, {"switchinnerflag", 0.0}, {"quadraticflag", 0.0}};
    std::ifstream in(param);
    if (!in.good()) throw Error("snap_force_generic: can't open file '" + param + "'");
    std::string line;
    while (std::getline(in, line)) {
      if (line.empty() || line[0] == '#') continue;
      std::istringstream ls(line);
      std::string key;
      double value = 0.0;
      if (ls >> key >> value && v.count(key)) v[key] = value;
    }
    std::ifstream cf(coef);
    if (!cf.good()) throw Error("snap_force_generic: cannot read file '" + coef + "'");
    int skipped = 0;
    std::getline(cf, line);
    while (cf.good() && (line.empty() || line[0] == '#') && skipped < 100) {
      std::getline(cf, line);
      ++skipped;
    }
    size_t nmat = 0, ncoef = 0;
    std::istringstream(line) >> nmat >> ncoef;
    if (nmat == 0 || nmat > 16 || ncoef == 0) throw Error("snap_force_generic: bad coefficient file '" + coef + "'");
    p = xnb_snap_params{};
    p.twojmax = static_cast<int32_t>(v["twojmax"]);
    p.rcutfac = v["rcutfac"];
    p.rfac0 = v["rfac0"];
    p.rmin0 = v["rmin0"];
    p.switchflag = static_cast<int32_t>(v["switchflag"]);
    p.bzeroflag = static_cast<int32_t>(v["bzeroflag"]);
    p.chemflag = static_cast<int32_t>(v["chemflag"]);
    p.bnormflag = static_cast<int32_t>(v["bnormflag"]);
    p.quadraticflag = static_cast<int32_t>(v["quadraticflag"]);
    p.switchinnerflag = static_cast<int32_t>(v["switchinnerflag"]);
    p.ntypes = static_cast<int32_t>(nmat);
    p.ncoeffall = static_cast<int32_t>(ncoef);
    coeffs.clear();
    for (size_t m = 0; m < nmat; ++m) {
      std::getline(cf, line);
      std::string name;
      double rad = 0.0, w = 1.0;
      std::istringstream(line) >> name >> rad >> w;
      p.radelem[m] = rad;
      p.wj[m] = w;
      for (size_t k = 0; k < ncoef; ++k) {
        std::getline(cf, line);
        double c = 0.0;
        std::istringstream(line) >> c;
        coeffs.push_back(c);
      }
    }
    if (!cf) throw Error("snap_force_generic: coefficient file '" + coef + "' is short");
  }
  void execute(Context& ctx) override {
    const Node* prm = local("parameters");
    const Node* pf = prm ? prm->find("param") : nullptr;
    const Node* cf = prm ? prm->find("coef") : nullptr;
    if (!pf || !cf) throw Error("snap_force_generic: parameters { param, coef } required");
    const bool conv = local("conv_coef_units") && to_bool(*local("conv_coef_units"));
    if (!ctx.snap) {
      xnb_snap_params p{};
      std::vector<double> coeffs;
      read(resolve(ctx, pf->scalar), resolve(ctx, cf->scalar), p, coeffs);
      if (conv) {
        for (double& c : coeffs) c *= quantity("1 eV");
        p.energy_unit = 1.0;
      } else {
        p.energy_unit = quantity("1 eV");
      }
      p.coeff = coeffs.data();
      if (ctx.dry_run) return;
      if (xnb_snap_create(&p, 0, &ctx.snap) != XNB_OK)
        throw Error(std::string("snap_force_generic: ") + xnb_last_error_string());
    }
    if (ctx.dry_run || !gpu_ready(ctx)) return;
    const int32_t fl = XNB_FORCE_ENERGY | (ctx.forces_written ? XNB_FORCE_ACCUMULATE : 0) |
                       (ctx.precision == XNB_PREC_MIXED ? XNB_FORCE_MIXED : 0);
    ck(xnb_snap_force(ctx.batch, ctx.sys, ctx.snap, fl, nullptr), "snap_force_generic");
    ctx.forces_written = true;
  }
};

struct NextTimeStepOp : OperatorNode {
  void execute(Context& ctx) override {
    ++ctx.timestep;
    ctx.physical_time += ctx.get_double("dt", 0.0);
    ctx.set_double("physical_time", ctx.physical_time);
  }
};

struct SimContinueOp : OperatorNode {
  void execute(Context& ctx) override {
    const long end = ctx.get_long("simulation_end_iteration", 0);
    ctx.set_bool("result", ctx.timestep <= end);
  }
};

// message: `message: text` or `message: { mesg: text, endl: bool }`; without a
// text of its own it prints the `mesg` slot (rebound, e.g., to a file name).
struct MessageOp : OperatorNode {
  void execute(Context& ctx) override {
    if (!ctx.verbose) return;
    std::string text;
    bool endl = true;
    if (m_local.is_scalar()) {
      text = m_local.scalar;
    } else {
      if (const Node* m = local("mesg")) text = m->scalar;
      else if (auto it = ctx.slots.find("mesg"); it != ctx.slots.end()) text = it->second.scalar;
      if (const Node* e = local("endl")) endl = to_bool(*e);
    }
    std::printf("%s%s", text.c_str(), endl ? "\n" : "");
  }
};

// timestep_file (logic/timestep_file_name.cpp:30-52): filename = format % timestep
struct TimestepFileOp : OperatorNode {
  void execute(Context& ctx) override {
    const Node* f = m_local.is_scalar() ? &m_local : local("format");
    if (!f) throw Error("timestep_file: format required");
    const std::string& fmt = f->scalar;
    char buf[4096];
    const bool is_long = fmt.find("%l") != std::string::npos;
    const int len = is_long ? std::snprintf(buf, sizeof(buf), fmt.c_str(), ctx.timestep)
                            : std::snprintf(buf, sizeof(buf), fmt.c_str(), static_cast<int>(ctx.timestep));
    if (len < 0 || len >= static_cast<int>(sizeof(buf))) throw Error("timestep_file: bad format '" + fmt + "'");
    ctx.slots["filename"] = Node::make_scalar(buf);
  }
};

// a string slot: the operator's own value, else the global slot, else dflt
std::string slot_string(const Node* local_value, const Context& ctx, const std::string& k, const std::string& dflt) {
  if (local_value) return local_value->scalar;
  auto it = ctx.slots.find(k);
  return (it == ctx.slots.end() || it->second.kind == Node::Null) ? dflt : it->second.scalar;
}

// write_dump (io/write_dump.cpp:35-44, sim_dump_writer.h:518-547): slots filename
// ("output.dump"), compression_level (6), max_part_size (-1 = 128 GiB); the
// time step and physical time of the run.
struct WriteDumpOp : OperatorNode {
  void execute(Context& ctx) override {
    const std::string fn = slot_string(local("filename"), ctx, "filename", "output.dump");
    const long level = local("compression_level") ? to_long(*local("compression_level"))
                                                   : ctx.get_long("compression_level", 6);
    const long mps = local("max_part_size") ? to_long(*local("max_part_size")) : ctx.get_long("max_part_size", -1);
    if (ctx.dry_run || !gpu_ready(ctx)) return;
    ck(xnb_system_write_dump(ctx.batch, ctx.sys, fn.c_str(), static_cast<uint64_t>(ctx.timestep), ctx.physical_time,
                             static_cast<int32_t>(level), mps, ctx.domain_expandable ? 0u : XNB_DOMAIN_EXPANDABLE,
                             nullptr),
       "write_dump");
    if (ctx.verbose) std::printf("write_dump: %s\n", fn.c_str());
  }
};

// read_dump (io/read_dump.cpp:36-45, sim_dump_reader.h:430-456): the domain,
// time step, physical time and particles of a .dump file; the particles go to
// init_particles in file order and are placed in the cells of their periodic
// locations (sim_dump_reader.h:293-352).
struct ReadDumpOp : OperatorNode {
  void execute(Context& ctx) override {
    const std::string fn = slot_string(local("filename"), ctx, "filename", "");
    if (fn.empty()) throw Error("read_dump: filename required");
    xnb_dump_info info{};
    if (xnb_dump_read_info(fn.c_str(), &info) != XNB_OK) throw Error(std::string("read_dump: ") + xnb_last_error_string());
    const xnb_dump_domain& d = info.domain;
    const uint32_t per = XNB_DOMAIN_PERIODIC_X | XNB_DOMAIN_PERIODIC_Y | XNB_DOMAIN_PERIODIC_Z;
    if ((d.flags & per) != per) throw Error("read_dump: only fully periodic domains are supported");
    if (!(d.flags & XNB_DOMAIN_XFORM_IDENTITY)) throw Error("read_dump: only the identity xform is supported");
    for (int a = 0; a < 3; ++a) {
      ctx.params.origin[a] = d.bmin[a];
      ctx.params.extent[a] = d.bmax[a];
      ctx.params.dims[a] = static_cast<int32_t>(d.grid_dims[a]);
    }
    ctx.params.cell_size = d.cell_size;
    ctx.domain_set = true;
    ctx.domain_expandable = (d.flags & XNB_DOMAIN_EXPANDABLE) != 0;
    HostParticles& h = ctx.host;
    h = HostParticles{};
    const size_t n = static_cast<size_t>(info.n_particles);
    h.rx.resize(n);
    h.ry.resize(n);
    h.rz.resize(n);
    h.vx.resize(n);
    h.vy.resize(n);
    h.vz.resize(n);
    h.id.resize(n);
    h.type.resize(n);
    int64_t got = 0;
    if (xnb_dump_read(fn.c_str(), static_cast<int64_t>(n), h.rx.data(), h.ry.data(), h.rz.data(), h.vx.data(),
                      h.vy.data(), h.vz.data(), h.id.data(), h.type.data(), &got, nullptr) != XNB_OK)
      throw Error(std::string("read_dump: ") + xnb_last_error_string());
    ctx.timestep = static_cast<long>(info.timestep);
    ctx.physical_time = info.physical_time;
    ctx.set_double("physical_time", ctx.physical_time);
    if (ctx.verbose) std::printf("read_dump: %s, %lld particles, timestep %ld\n", fn.c_str(), static_cast<long long>(got), ctx.timestep);
  }
};

// simulation_stats (debug/simulation_stats.cpp:60-124), reduced on the GPU; the
// kinetic energy printed is 0.5 * m * sum |v|^2 with the species mass.
struct StatsOp : OperatorNode {
  void execute(Context& ctx) override {
    if (ctx.dry_run || !gpu_ready(ctx)) return;
    xnb_sim_stats st{};
    ck(xnb_simulation_stats(ctx.batch, ctx.sys, &st, nullptr), "simulation_stats");
    const double ke = 0.5 * ctx.params.mass * st.kinetic_sum;
    std::printf("T=%ld n=%lld ke=%.10g pe=%.10g total=%.10g |v|=[%.6g,%.6g] |a|=[%.6g,%.6g]\n", ctx.timestep,
                static_cast<long long>(st.particle_count), ke, st.potential_energy, ke + st.potential_energy,
                st.min_vel, st.max_vel, st.min_acc, st.max_acc);
  }
};

// check_values (debug/check_values.cpp:230-401): L2 norms of the position,
// acceleration and velocity errors over the sampled ids of a golden file
// ([id, rx, ry, rz, ax, ay, az, vx, vy, vz] rows, hex floats), positions compared
// through their periodic image closest to the reference point.
struct CheckValuesOp : OperatorNode {
  void execute(Context& ctx) override {
    const Node* f = local("file");
    if (!f) throw Error("check_values: file required");
    std::string path = f->scalar;
    if (!path.empty() && path[0] != '/') path = ctx.slots["deck_dir"].scalar + "/" + path;
    const Node golden = parse_yaml_file(path);
    const Node* vals = golden.find("values");
    if (!vals || !vals->is_seq()) throw Error("check_values: no values in " + path);
    if (ctx.dry_run) return;
    // only the sampled particles leave the GPU (xnb_sample_particles)
    std::vector<uint64_t> ids;
    for (const auto& row : vals->seq) ids.push_back(static_cast<uint64_t>(to_long(row.seq.at(0))));
    std::vector<double> got(ids.size() * 9);
    std::vector<int32_t> found(ids.size());
    ck(xnb_sample_particles(ctx.batch, ctx.sys, ids.data(), static_cast<int64_t>(ids.size()), got.data(),
                            found.data(), nullptr),
       "check_values sampling");
    const auto& p = ctx.params;
    double er = 0, ea = 0, ev = 0;
    for (size_t q = 0; q < ids.size(); ++q) {
      if (!found[q]) throw Error("check_values: id " + std::to_string(ids[q]) + " not found");
      const Node& row = vals->seq[q];
      double ref[9];
      for (int k = 0; k < 9; ++k) ref[k] = std::strtod(row.seq.at(static_cast<size_t>(k + 1)).scalar.c_str(), nullptr);
      const double* g = got.data() + q * 9;  // r, f, v
      for (int a = 0; a < 3; ++a) {
        const double L = p.extent[a] - p.origin[a];
        double d = g[a] - ref[a];
        d -= L * std::round(d / L);
        er += d * d;
        ea += (g[3 + a] - ref[3 + a]) * (g[3 + a] - ref[3 + a]);
        ev += (g[6 + a] - ref[6 + a]) * (g[6 + a] - ref[6 + a]);
      }
    }
    er = std::sqrt(er);
    ea = std::sqrt(ea);
    ev = std::sqrt(ev);
    const double tp = param_double(ctx, "pos_threshold", 1e-5), ta = param_double(ctx, "acc_threshold", 1e-5),
                 tv = param_double(ctx, "vel_threshold", 1e-5);
    std::printf("** Position error L2 norm = %.6g / %g\n** Acceleration error L2 norm = %.6g / %g\n"
                "** Velocity error L2 norm = %.6g / %g\n",
                er, tp, ea, ta, ev, tv);
    ctx.set_double("check_values.pos", er);
    ctx.set_double("check_values.acc", ea);
    ctx.set_double("check_values.vel", ev);
    if (er > tp || ea > ta || ev > tv) throw Error("check_values: golden values not reproduced");
  }
};

template <class T>
void reg(const char* name) {
  OperatorNodeFactory::instance()->register_factory(name, [] { return std::unique_ptr<OperatorNode>(new T()); });
}

}  // namespace

void register_hot_path_operators() {
  reg<DomainOp>("domain");
  reg<NopOp>("init_rcb_grid");
  reg<NopOp>("particle_types");
  reg<TypePropertiesOp>("particle_type_add_properties");
  reg<LatticeOp>("lattice");
  reg<GaussianNoiseOp>("gaussian_noise_r");
  reg<ReplicateDomainOp>("replicate_domain");
  reg<NbhDistOp>("nbh_dist");
  reg<InitParticlesOp>("init_particles");
  reg<PushFVROp>("push_f_v_r");
  reg<PushFVOp>("push_f_v");
  reg<DisplOverOp>("particle_displ_over");
  reg<MoveParticlesOp>("move_particles");
  reg<ChunkNeighborsOp>("chunk_neighbors");
  reg<BackupROp>("backup_r");
  reg<LennardJonesOp>("lennard_jones_force");
  reg<GravityOp>("gravitational_force");
  reg<ZeroForceOp>("zero_particle_force");
  reg<SnapOp>("snap_force_generic");
  // folded into move_particles / lennard_jones_force on the GPU, or single-rank no-ops
  for (const char* n : {"migrate_cell_particles", "rebuild_amr", "ghost_comm_scheme", "ghost_update_all",
                        "ghost_update_r", "amr_grid_pairs", "resize_particle_locks",
                        "update_force_from_ghost", "divide_force_by_type_scalar", "extend_domain",
                        "simple_cost_model", "load_balance_rcb", "nop", "init_cuda", "mpi_comm_world",
                        "print_grid", "grid_stats", "chunk_neighbors_stats", "dump_data",
                        "memory_stats", "print_log_if_triggered", "dump_data_if_triggered"})
    reg<NopOp>(n);
  reg<NextTimeStepOp>("next_time_step");
  reg<SimContinueOp>("sim_continue");
  reg<MessageOp>("message");
  reg<TimestepFileOp>("timestep_file");
  reg<WriteDumpOp>("write_dump");
  reg<ReadDumpOp>("read_dump");
  reg<StatsOp>("simulation_stats");
  reg<NopOp>("print_simulation_stats");
  reg<CheckValuesOp>("check_values");
}

}  // namespace xnbhost
