// Host-side mirror of the reference's operator interface for the particle hot
// path: OperatorNode subclasses registered by name in an OperatorNodeFactory,
// wired through named slots, driven by YAML decks (.msp) -- the shape of
// exaNBody's onika layer (OperatorNode / ADD_SLOT / register_factory,
// e.g. contribs/md/lennard_jones/lennard_jones.cu:171-223), re-provided here in
// a minimal form that calls the GPU through include/xnb_gpu.h.
#pragma once

#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "xnb_dump.h"
#include "xnb_gpu.h"

namespace xnbhost {

// ---------------------------------------------------------------------------
// YAML subset: block maps and sequences by indentation, flow sequences [..],
// flow maps {..}, scalars (plain or quoted), '#' comments. Enough for .msp decks.
struct Node {
  enum Kind { Null, Scalar, Seq, Map } kind = Null;
  std::string scalar;
  std::vector<Node> seq;
  std::vector<std::pair<std::string, Node>> map;  // insertion order kept

  bool is_map() const { return kind == Map; }
  bool is_seq() const { return kind == Seq; }
  bool is_scalar() const { return kind == Scalar; }
  const Node* find(const std::string& k) const;
  Node* find(const std::string& k);
  void set(const std::string& k, const Node& v);
  static Node make_scalar(const std::string& s);
};

Node parse_yaml(const std::string& text);
Node parse_yaml_file(const std::string& path);
std::string dump_yaml(const Node& n, int indent = 0);

// Quantities: "2e-3 ps", "4.1 ang", "0.3729 eV", "58.693 Da" -> internal units
// (angstrom, dalton, picosecond; energies in Da*A^2/ps^2).
double quantity(const Node& n);
double quantity(const std::string& s);
bool to_bool(const Node& n);
long to_long(const Node& n);

// ---------------------------------------------------------------------------
// Simulation state shared by the operators (slot values by name, plus the GPU batch).
struct HostParticles {
  // per interior cell, in the reference grid's linear order
  std::vector<int64_t> cell_counts;
  std::vector<double> rx, ry, rz, vx, vy, vz;
  std::vector<uint64_t> id;
  std::vector<uint8_t> type;  // empty: all type 0
};

struct Context {
  std::map<std::string, Node> slots;  // global slot values (YAML scalars / maps)
  xnb_lj_params params{};
  bool domain_set = false;
  bool domain_expandable = true;  // Domain() starts expandable (core/include/exanb/core/domain.h:104)
  double mass = 1.0;
  bool divide_by_mass = false;
  HostParticles host;
  xnb_batch* batch = nullptr;
  int32_t sys = -1;
  int32_t precision = XNB_PREC_FP64_EXACT;
  bool forces_written = false;  // a force operator of the current force block has written forces
  xnb_snap* snap = nullptr;     // snap_force_generic's potential, built at its first call
  long timestep = 0;
  double physical_time = 0.0;
  bool verbose = false;
  std::vector<std::string> trace;  // executed operator names (dry runs, tests)
  bool dry_run = false;

  ~Context();
  double get_double(const std::string& k, double dflt) const;
  bool get_bool(const std::string& k, bool dflt) const;
  long get_long(const std::string& k, long dflt) const;
  void set_bool(const std::string& k, bool v);
  void set_double(const std::string& k, double v);
};

// ---------------------------------------------------------------------------
enum SlotDir { INPUT, OUTPUT, INPUT_OUTPUT };

struct SlotDecl {
  std::string name;
  SlotDir dir;
  std::string doc;
};

class OperatorNode {
 public:
  virtual ~OperatorNode() = default;
  // local parameters from the deck (`op: { key: value }`) override global slots
  void set_local(const Node& params) { m_local = params; }
  virtual void execute(Context& ctx) = 0;
  virtual std::vector<SlotDecl> slots() const { return {}; }
  const std::string& name() const { return m_name; }
  void set_name(const std::string& n) { m_name = n; }

 protected:
  const Node* local(const std::string& k) const { return m_local.is_map() ? m_local.find(k) : nullptr; }
  double param_double(const Context& ctx, const std::string& k, double dflt) const;
  bool param_bool(const Context& ctx, const std::string& k, bool dflt) const;
  Node m_local;
  std::string m_name;
};

class OperatorNodeFactory {
 public:
  using Creator = std::function<std::unique_ptr<OperatorNode>()>;
  static OperatorNodeFactory* instance();
  void register_factory(const std::string& name, Creator c);
  bool has(const std::string& name) const { return m_creators.count(name) != 0; }
  std::unique_ptr<OperatorNode> make_operator(const std::string& name) const;
  std::vector<std::string> names() const;

 private:
  std::map<std::string, Creator> m_creators;
};

void register_hot_path_operators();

// ---------------------------------------------------------------------------
// Deck runner: blocks are operator names, sequences of items, or maps with
// condition / body / loop / rebind; a deck's top-level keys define or override
// blocks; `simulation` names the block to run.
class Runner {
 public:
  explicit Runner(Context& ctx) : m_ctx(ctx) {}
  void load_defaults();
  void load_deck(const Node& deck);
  void run(const std::string& block);
  void run_item(const Node& item);

 private:
  void run_named(const std::string& name, const Node* params);
  void run_flow(const Node& blk);
  bool condition_value(const std::string& name);
  Context& m_ctx;
  std::map<std::string, Node> m_blocks;
  int m_depth = 0;
};

struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

}  // namespace xnbhost
