// Minimal YAML reader for .msp decks (block maps/sequences by indentation,
// flow [..] and {..}, plain and quoted scalars, comments).
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>

#include "xnb_host.hpp"

namespace xnbhost {

const Node* Node::find(const std::string& k) const {
  for (const auto& kv : map)
    if (kv.first == k) return &kv.second;
  return nullptr;
}

Node* Node::find(const std::string& k) {
  for (auto& kv : map)
    if (kv.first == k) return &kv.second;
  return nullptr;
}

void Node::set(const std::string& k, const Node& v) {
  kind = Map;
  if (Node* n = find(k)) *n = v;
  else map.emplace_back(k, v);
}

Node Node::make_scalar(const std::string& s) {
  Node n;
  n.kind = Scalar;
  n.scalar = s;
  return n;
}

namespace {

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace(static_cast<unsigned char>(s[a]))) ++a;
  while (b > a && std::isspace(static_cast<unsigned char>(s[b - 1]))) --b;
  return s.substr(a, b - a);
}

std::string unquote(const std::string& s) {
  if (s.size() >= 2 && ((s.front() == '"' && s.back() == '"') || (s.front() == '\'' && s.back() == '\'')))
    return s.substr(1, s.size() - 2);
  return s;
}

// remove a trailing comment that is not inside quotes
std::string strip_comment(const std::string& s) {
  bool dq = false, sq = false;
  for (size_t i = 0; i < s.size(); ++i) {
    const char c = s[i];
    if (c == '"' && !sq) dq = !dq;
    else if (c == '\'' && !dq) sq = !sq;
    else if (c == '#' && !dq && !sq && (i == 0 || std::isspace(static_cast<unsigned char>(s[i - 1])))) return s.substr(0, i);
  }
  return s;
}

struct Line {
  int indent;
  std::string text;
  int number;
};

// position of the ':' that separates a key from its value, or npos
size_t key_colon(const std::string& s) {
  int depth = 0;
  bool dq = false, sq = false;
  for (size_t i = 0; i < s.size(); ++i) {
    const char c = s[i];
    if (c == '"' && !sq) dq = !dq;
    else if (c == '\'' && !dq) sq = !sq;
    else if (dq || sq) continue;
    else if (c == '[' || c == '{') ++depth;
    else if (c == ']' || c == '}') --depth;
    else if (c == ':' && depth == 0 && (i + 1 == s.size() || s[i + 1] == ' ')) return i;
  }
  return std::string::npos;
}

struct Flow {
  const std::string& s;
  size_t p = 0;
  void ws() {
    while (p < s.size() && std::isspace(static_cast<unsigned char>(s[p]))) ++p;
  }
  Node value() {
    ws();
    if (p < s.size() && s[p] == '[') {
      ++p;
      Node n;
      n.kind = Node::Seq;
      ws();
      if (p < s.size() && s[p] == ']') { ++p; return n; }
      for (;;) {
        n.seq.push_back(value());
        ws();
        if (p < s.size() && s[p] == ',') { ++p; continue; }
        if (p < s.size() && s[p] == ']') { ++p; break; }
        throw Error("flow sequence: expected ',' or ']' in: " + s);
      }
      return n;
    }
    if (p < s.size() && s[p] == '{') {
      ++p;
      Node n;
      n.kind = Node::Map;
      ws();
      if (p < s.size() && s[p] == '}') { ++p; return n; }
      for (;;) {
        ws();
        const size_t k0 = p;
        while (p < s.size() && s[p] != ':' && s[p] != '}' && s[p] != ',') ++p;
        const std::string key = unquote(trim(s.substr(k0, p - k0)));
        if (p < s.size() && s[p] == ':') {
          ++p;
          n.map.emplace_back(key, value());
        } else {
          n.map.emplace_back(key, Node());
        }
        ws();
        if (p < s.size() && s[p] == ',') { ++p; continue; }
        if (p < s.size() && s[p] == '}') { ++p; break; }
        throw Error("flow map: expected ',' or '}' in: " + s);
      }
      return n;
    }
    // scalar up to , ] }
    bool dq = false, sq = false;
    const size_t a = p;
    while (p < s.size()) {
      const char c = s[p];
      if (c == '"' && !sq) dq = !dq;
      else if (c == '\'' && !dq) sq = !sq;
      else if (!dq && !sq && (c == ',' || c == ']' || c == '}')) break;
      ++p;
    }
    return Node::make_scalar(unquote(trim(s.substr(a, p - a))));
  }
};

Node inline_value(const std::string& v) {
  const std::string t = trim(v);
  if (t.empty()) return Node();
  if (t[0] == '[' || t[0] == '{') {
    Flow f{t};
    return f.value();
  }
  return Node::make_scalar(unquote(t));
}

class Parser {
 public:
  explicit Parser(std::vector<Line> lines) : L(std::move(lines)) {}
  Node block(size_t& i, int indent);

 private:
  Node map_block(size_t& i, int indent);
  Node seq_block(size_t& i, int indent);
  std::vector<Line> L;
};

bool is_dash(const std::string& t) { return t == "-" || (t.size() >= 2 && t[0] == '-' && t[1] == ' '); }

Node Parser::block(size_t& i, int indent) {
  if (i >= L.size() || L[i].indent < indent) return Node();
  if (is_dash(L[i].text)) return seq_block(i, L[i].indent);
  return map_block(i, L[i].indent);
}

Node Parser::seq_block(size_t& i, int indent) {
  Node n;
  n.kind = Node::Seq;
  while (i < L.size() && L[i].indent == indent && is_dash(L[i].text)) {
    const std::string rest = trim(L[i].text.substr(1));
    const int item_indent = indent + 2;
    ++i;
    if (rest.empty()) {
      n.seq.push_back(block(i, item_indent));
      continue;
    }
    const size_t c = key_colon(rest);
    if (rest[0] != '[' && rest[0] != '{' && rest[0] != '"' && c != std::string::npos) {
      // a map item: first pair on the dash line, more pairs indented below
      Node m;
      m.kind = Node::Map;
      const std::string key = unquote(trim(rest.substr(0, c)));
      const std::string val = trim(rest.substr(c + 1));
      if (val.empty()) {
        m.map.emplace_back(key, (i < L.size() && L[i].indent > indent) ? block(i, L[i].indent) : Node());
      } else {
        m.map.emplace_back(key, inline_value(val));
      }
      if (i < L.size() && L[i].indent > indent && !is_dash(L[i].text)) {
        Node more = map_block(i, L[i].indent);
        for (auto& kv : more.map) m.map.push_back(kv);
      }
      n.seq.push_back(m);
    } else {
      n.seq.push_back(inline_value(rest));
    }
  }
  return n;
}

Node Parser::map_block(size_t& i, int indent) {
  Node n;
  n.kind = Node::Map;
  while (i < L.size() && L[i].indent == indent && !is_dash(L[i].text)) {
    const std::string& t = L[i].text;
    const size_t c = key_colon(t);
    if (c == std::string::npos) throw Error("line " + std::to_string(L[i].number) + ": expected 'key: value': " + t);
    const std::string key = unquote(trim(t.substr(0, c)));
    const std::string val = trim(t.substr(c + 1));
    ++i;
    if (!val.empty()) {
      n.set(key, inline_value(val));
    } else if (i < L.size() && (L[i].indent > indent || (L[i].indent == indent && is_dash(L[i].text)))) {
      n.set(key, block(i, L[i].indent));
    } else {
      n.set(key, Node());
    }
  }
  return n;
}

}  // namespace

Node parse_yaml(const std::string& text) {
  std::vector<Line> lines;
  std::istringstream in(text);
  std::string raw;
  int number = 0;
  std::string pending;  // a double-quoted scalar spanning lines
  int pending_indent = 0, pending_number = 0;
  while (std::getline(in, raw)) {
    ++number;
    if (!raw.empty() && raw.back() == '\r') raw.pop_back();
    if (!pending.empty()) {
      pending += " " + trim(raw);
      size_t q = 0;
      for (char ch : pending) q += (ch == '"');
      if (q % 2 == 0) {
        lines.push_back({pending_indent, trim(strip_comment(pending)), pending_number});
        pending.clear();
      }
      continue;
    }
    const std::string s = strip_comment(raw);
    const std::string t = trim(s);
    if (t.empty()) continue;
    int ind = 0;
    while (ind < static_cast<int>(s.size()) && s[ind] == ' ') ++ind;
    size_t q = 0;
    for (char ch : t) q += (ch == '"');
    if (q % 2 == 1) {
      pending = t;
      pending_indent = ind;
      pending_number = number;
      continue;
    }
    lines.push_back({ind, t, number});
  }
  if (lines.empty()) return Node();
  Parser p(lines);
  size_t i = 0;
  Node root = p.block(i, lines[0].indent);
  if (i != lines.size())
    throw Error("line " + std::to_string(lines[i].number) + ": unexpected indentation: " + lines[i].text);
  return root;
}

Node parse_yaml_file(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw Error("cannot open " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return parse_yaml(ss.str());
}

std::string dump_yaml(const Node& n, int indent) {
  const std::string pad(static_cast<size_t>(indent), ' ');
  std::ostringstream o;
  switch (n.kind) {
    case Node::Null: o << "~"; break;
    case Node::Scalar: o << n.scalar; break;
    case Node::Seq:
      o << "[";
      for (size_t k = 0; k < n.seq.size(); ++k) o << (k ? ", " : "") << dump_yaml(n.seq[k], indent);
      o << "]";
      break;
    case Node::Map:
      o << "{";
      for (size_t k = 0; k < n.map.size(); ++k) o << (k ? ", " : "") << n.map[k].first << ": " << dump_yaml(n.map[k].second, indent);
      o << "}";
      break;
  }
  return pad + o.str();
}

// ---------------------------------------------------------------------------
// Units of the reference's internal system: angstrom, dalton, picosecond.
// The electron-volt and dalton values are the ones that reproduce the
// reference's golden data (contribs/microStamp/samples/benchmark_lj_snap/).
double quantity(const std::string& s) {
  const std::string t = trim(s);
  char* end = nullptr;
  const double v = std::strtod(t.c_str(), &end);
  if (end == t.c_str()) throw Error("not a number: " + s);
  const std::string unit = trim(std::string(end));
  if (unit.empty()) return v;
  static const double ev_j = 1.6021892e-19, da_kg = 1.66053904e-27;
  static const double energy_internal_j = da_kg * 1e-20 / 1e-24;
  static const std::map<std::string, double> table = {
      {"ang", 1.0},   {"angstrom", 1.0}, {"nm", 10.0},  {"um", 1e4},     {"m", 1e10},
      {"ps", 1.0},    {"fs", 1e-3},      {"ns", 1e3},   {"s", 1e12},     {"Da", 1.0},
      {"dalton", 1.0}, {"eV", ev_j / energy_internal_j}, {"J", 1.0 / energy_internal_j},
      {"ang/ps", 1.0}, {"K", 1.0}};
  auto it = table.find(unit);
  if (it == table.end()) throw Error("unknown unit '" + unit + "' in: " + s);
  return v * it->second;
}

double quantity(const Node& n) {
  if (!n.is_scalar()) throw Error("expected a quantity, got " + dump_yaml(n));
  return quantity(n.scalar);
}

bool to_bool(const Node& n) {
  if (!n.is_scalar()) throw Error("expected a boolean");
  const std::string s = n.scalar;
  if (s == "true" || s == "True" || s == "1" || s == "yes") return true;
  if (s == "false" || s == "False" || s == "0" || s == "no") return false;
  throw Error("not a boolean: " + s);
}

long to_long(const Node& n) {
  if (!n.is_scalar()) throw Error("expected an integer");
  return std::strtol(n.scalar.c_str(), nullptr, 10);
}

}  // namespace xnbhost
