// Deck runner and the `xnb-exec` entry point.
//
// The default operator graph below has the block names and order of the
// reference's data/config decks (main-config.msp, compute-loop.msp,
// numerical-scheme.msp, update-particles.msp, dump-data.msp), restated for the GPU operators
// of this library; a user deck overrides or extends blocks by name ('+name'
// appends), sets slot defaults of an operator by a map under its name, and
// chooses the block to run with `simulation:`.
#include <cstdio>
#include <cstring>
#include <set>

#include "xnb_host.hpp"

namespace xnbhost {

namespace {

const char* kDefaultGraph = R"(
simulation: default_simulation
compute_loop_continue: true
deterministic_noise: false
sub_grid_density: 6.5
default_simulation:
  - global
  - input_data
  - nbh_dist
  - first_iteration
  - compute_loop
  - simulation_epilog
  - final_dump
global: {}
input_data: nop
simulation_epilog: nop
final_dump: dump_data_particles
dump_data_particles:
  - timestep_file: "particles_%09d.dump"
  - message: { mesg: "Write " , endl: false }
  - print_dump_file:
      rebind: { mesg: filename }
      body:
        - message: { endl: true }
  - write_dump
first_iteration:
  - init_particles
  - print_grid
  - compute_all_forces_energy
  - simulation_stats
  - print_simulation_stats
  - next_time_step
compute_loop:
  loop: true
  condition: compute_loop_continue
  body:
    - begin_iteration
    - numerical_scheme
    - end_iteration
    - next_time_step
    - compute_loop_stop
compute_loop_stop:
  rebind: { end_at: simulation_end_iteration, result: compute_loop_continue }
  body:
    - sim_continue
begin_iteration: nop
end_iteration: nop
numerical_scheme:
  - verlet_first_half
  - check_and_update_particles
  - compute_all_forces_energy
  - verlet_second_half
verlet_first_half:
  - push_f_v_r: { dt_scale: 1.0 }
  - push_f_v: { dt_scale: 0.5 }
verlet_second_half:
  - push_f_v: { dt_scale: 0.5 }
compute_all_forces_energy:
  - compute_force_prolog
  - compute_force
  - compute_force_epilog
compute_force_prolog: zero_particle_force
compute_force: nop
compute_force_epilog: nop
check_and_update_particles:
  - trigger_move_particles
  - update_particles_full
  - update_particles_fast
trigger_move_particles:
  rebind: { threshold: max_displ, result: trigger_move_particles }
  body:
    - particle_displ_over
update_particles_full:
  condition: trigger_move_particles
  body:
    - move_particles
update_particles_fast:
  condition: not trigger_move_particles
  body:
    - ghost_update_r
)";

const std::set<std::string> kFlowKeys = {"body", "condition", "rebind", "loop", "name", "profiling"};

bool is_flow_map(const Node& n) {
  if (!n.is_map()) return false;
  for (const auto& kv : n.map)
    if (kFlowKeys.count(kv.first)) return true;
  return false;
}

void merge_map(Node& into, const Node& from) {
  if (!from.is_map()) return;
  into.kind = Node::Map;
  for (const auto& kv : from.map) into.set(kv.first, kv.second);
}

bool contains_name(const Node& block, const std::string& name) {
  if (block.is_scalar()) return block.scalar == name;
  if (block.is_seq()) {
    for (const auto& it : block.seq)
      if (contains_name(it, name)) return true;
  }
  if (block.is_map() && !block.map.empty() && !is_flow_map(block))
    for (const auto& kv : block.map)
      if (kv.first == name) return true;
  return false;
}

}  // namespace

void Runner::load_defaults() { load_deck(parse_yaml(kDefaultGraph)); }

void Runner::load_deck(const Node& deck) {
  if (!deck.is_map()) throw Error("a deck is a map of block definitions");
  for (const auto& kv : deck.map) {
    std::string key = kv.first;
    if (key == "configuration") continue;
    if (!key.empty() && key[0] == '+') {
      key = key.substr(1);
      Node& blk = m_blocks[key];
      if (blk.kind == Node::Null) blk.kind = Node::Seq;
      if (blk.is_scalar()) {
        Node s;
        s.kind = Node::Seq;
        s.seq.push_back(blk);
        blk = s;
      }
      if (kv.second.is_seq())
        for (const auto& it : kv.second.seq) blk.seq.push_back(it);
      else
        blk.seq.push_back(kv.second);
      continue;
    }
    // scalar values of slots the graph reads directly (booleans / numbers)
    if (kv.second.is_scalar() && !OperatorNodeFactory::instance()->has(kv.second.scalar) && key != "simulation" &&
        m_blocks.find(kv.second.scalar) == m_blocks.end() && kv.second.scalar != "nop") {
      m_ctx.slots[key] = kv.second;
    }
    m_blocks[key] = kv.second;
  }
  // force-chain settings the GPU system needs at creation
  if (const auto it = m_blocks.find("lennard_jones_force"); it != m_blocks.end() && it->second.is_map()) {
    if (const Node* cfg = it->second.find("config")) {
      if (const Node* e = cfg->find("epsilon")) m_ctx.slots["lj.epsilon"] = *e;
      if (const Node* s = cfg->find("sigma")) m_ctx.slots["lj.sigma"] = *s;
    }
    if (const Node* rc = it->second.find("rcut")) m_ctx.slots["lj.rcut"] = *rc;
  }
  if (const auto it = m_blocks.find("compute_all_forces_energy"); it != m_blocks.end())
    m_ctx.divide_by_mass = contains_name(it->second, "divide_force_by_type_scalar");
}

bool Runner::condition_value(const std::string& expr) {
  std::string e = expr;
  bool neg = false;
  if (e.rfind("not ", 0) == 0) {
    neg = true;
    e = e.substr(4);
  }
  const bool v = m_ctx.get_bool(e, false);
  return neg ? !v : v;
}

void Runner::run(const std::string& block) { run_named(block, nullptr); }

void Runner::run_named(const std::string& name, const Node* params) {
  if (++m_depth > 64) throw Error("block nesting too deep at '" + name + "'");
  auto fac = OperatorNodeFactory::instance();
  auto it = m_blocks.find(name);
  const bool is_op = fac->has(name);
  if (name == "global") {
    // the deck's `global` map sets global slot values
    if (it != m_blocks.end() && it->second.is_map())
      for (const auto& kv : it->second.map) m_ctx.slots[kv.first] = kv.second;
  } else if (it != m_blocks.end() && !(is_op && (it->second.is_map() && !is_flow_map(it->second)))) {
    const Node& blk = it->second;
    if (blk.is_scalar()) {
      if (blk.scalar != name) run_named(blk.scalar, params);
    } else if (blk.is_seq()) {
      for (const auto& item : blk.seq) run_item(item);
    } else if (is_flow_map(blk)) {
      run_flow(blk);
    } else if (blk.is_map()) {
      for (const auto& kv : blk.map) m_ctx.slots[kv.first] = kv.second;
    }
  } else if (is_op) {
    auto op = fac->make_operator(name);
    Node local;
    if (it != m_blocks.end()) merge_map(local, it->second);  // operator defaults from the deck
    if (params) {
      if (params->is_map()) merge_map(local, *params);
      else local = *params;
    }
    op->set_local(local);
    m_ctx.trace.push_back(name);
    op->execute(m_ctx);
  } else if (params && is_flow_map(*params)) {
    // an inline batch: `name: { rebind: ..., body: [...] }` (e.g. print_dump_file
    // in dump-data.msp:15-19)
    m_ctx.trace.push_back(name);
    run_flow(*params);
  } else {
    throw Error("unknown block or operator '" + name + "'");
  }
  --m_depth;
}

void Runner::run_flow(const Node& blk) {
  const Node* cond = blk.find("condition");
  const Node* body = blk.find("body");
  const Node* reb = blk.find("rebind");
  const bool loop = blk.find("loop") && to_bool(*blk.find("loop"));
  auto body_once = [&]() {
    if (reb)
      for (const auto& kv : reb->map)
        if (m_ctx.slots.count(kv.second.scalar)) m_ctx.slots[kv.first] = m_ctx.slots[kv.second.scalar];
    if (body && body->is_seq())
      for (const auto& item : body->seq) run_item(item);
    if (reb)
      for (const auto& kv : reb->map)
        if (m_ctx.slots.count(kv.first)) {
          m_ctx.slots[kv.second.scalar] = m_ctx.slots[kv.first];
          m_ctx.slots.erase(kv.first);
        }
  };
  if (loop) {
    while (!cond || condition_value(cond->scalar)) body_once();
  } else if (!cond || condition_value(cond->scalar)) {
    body_once();
  }
}

void Runner::run_item(const Node& item) {
  if (item.is_scalar()) {
    run_named(item.scalar, nullptr);
  } else if (item.is_map() && item.map.size() == 1) {
    run_named(item.map[0].first, &item.map[0].second);
  } else {
    throw Error("cannot run item " + dump_yaml(item));
  }
}

}  // namespace xnbhost

// ---------------------------------------------------------------------------
int main(int argc, char** argv) {
  using namespace xnbhost;
  bool dry = false, verbose = false;
  int precision = XNB_PREC_FP64_EXACT;
  std::string deck;
  for (int k = 1; k < argc; ++k) {
    if (!std::strcmp(argv[k], "--dry-run")) dry = true;
    else if (!std::strcmp(argv[k], "--verbose")) verbose = true;
    else if (!std::strcmp(argv[k], "--precision") && k + 1 < argc) {
      const std::string p = argv[++k];
      precision = p == "fp64" ? XNB_PREC_FP64 : p == "mixed" ? XNB_PREC_MIXED : XNB_PREC_FP64_EXACT;
    } else deck = argv[k];
  }
  if (deck.empty()) {
    std::fprintf(stderr, "usage: xnb-exec [--dry-run] [--verbose] [--precision fp64_exact|fp64|mixed] deck.msp\n");
    return 2;
  }
  try {
    register_hot_path_operators();
    Context ctx;
    ctx.dry_run = dry;
    ctx.verbose = verbose;
    ctx.precision = precision;
    const size_t slash = deck.find_last_of('/');
    ctx.slots["deck_dir"] = Node::make_scalar(slash == std::string::npos ? "." : deck.substr(0, slash));
    Runner r(ctx);
    r.load_defaults();
    const Node d = parse_yaml_file(deck);
    r.load_deck(d);
    const Node* sim = d.find("simulation");
    r.run(sim ? sim->scalar : "default_simulation");
    if (dry) {
      for (const auto& t : ctx.trace) std::printf("%s\n", t.c_str());
    }
    std::printf("xnb-exec: done, %ld steps\n", ctx.timestep > 0 ? ctx.timestep - 1 : 0);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "xnb-exec: error: %s\n", e.what());
    return 1;
  }
  return 0;
}
