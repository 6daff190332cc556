// VQL parser and plan builder (see vql.hh).  The grammar
// (src/objects/vql/grammar/vql.g4) is small enough for a hand-written
// recursive-descent parser; the listener semantics follow
// src/objects/vql/query_builder.cpp:199-290 and the plan shape
// Builder::build (:27-92) / Builder::get_ve (:103-147).
#include "vql.hh"

#include <algorithm>
#include <cctype>
#include <cstring>
#include <map>

namespace vsgb {
namespace query {

void Vertex::merge(const Vertex &v) {
  if (filter_type == VertexFilterType::ALL) {
    filter_type = v.filter_type;
    id = v.id;
    tag_lo = v.tag_lo;
    tag_hi = v.tag_hi;
  } else if (v.filter_type != VertexFilterType::ALL) {
    throw Error(VS_ERR_ARG, "vertex " + name + " has two filters");  // assert(0) in the reference
  }
}

namespace {

class Parser {
  const std::string &s;
  size_t i = 0;

 public:
  std::map<VariableName, Vertex> vertices;
  std::vector<Edge> edges;
  std::vector<Variable> returned;
  bool only_count = false;
  std::optional<Edge> last_edge;
  VariableName last_vertex;

  explicit Parser(const std::string &text) : s(text) {}

  [[noreturn]] void bad(const std::string &what) {
    throw Error(VS_ERR_ARG, "VQL: " + what + " at offset " + std::to_string(i));
  }
  void ws() {
    while (i < s.size() && std::isspace((unsigned char)s[i])) i++;
  }
  bool peek(const char *lit) {
    ws();
    return s.compare(i, std::char_traits<char>::length(lit), lit) == 0;
  }
  bool accept(const char *lit) {
    if (!peek(lit)) return false;
    i += std::char_traits<char>::length(lit);
    return true;
  }
  void expect(const char *lit) {
    if (!accept(lit)) bad(std::string("expected '") + lit + "'");
  }
  uint64_t integer() {
    ws();
    size_t b = i;
    while (i < s.size() && std::isdigit((unsigned char)s[i])) i++;
    if (b == i) bad("expected an integer");
    return std::stoull(s.substr(b, i - b));
  }
  bool at_integer() {
    ws();
    return i < s.size() && std::isdigit((unsigned char)s[i]);
  }
  VariableName var() {
    ws();
    size_t b = i;
    if (i < s.size() && (std::isalpha((unsigned char)s[i]) || s[i] == '_')) i++;
    else bad("expected a variable");
    while (i < s.size() && (std::isalnum((unsigned char)s[i]) || s[i] == '_')) i++;
    return s.substr(b, i - b);
  }

  // vertex: '(' VAR vertex_filter? ')'  (exitVertex, query_builder.cpp:199-232)
  void vertex() {
    expect("(");
    Vertex v;
    v.name = var();
    if (accept("{")) {
      if (accept("id:")) {
        v.filter_type = VertexFilterType::ID;
        v.id = integer();
      } else if (accept("tag:")) {
        v.filter_type = VertexFilterType::TAG;
        v.tag_lo = (int64_t)integer();
        expect("-");
        v.tag_hi = (int64_t)integer();
      } else {
        bad("expected 'id:' or 'tag:'");
      }
      expect("}");
    }
    expect(")");
    if (last_edge) {
      last_edge->dst = v.name;
      edges.push_back(*last_edge);
      last_edge.reset();
    }
    last_vertex = v.name;
    auto it = vertices.find(v.name);
    if (it == vertices.end())
      vertices.emplace(v.name, v);
    else
      it->second.merge(v);
  }

  // length: '[' INT? ']' | '[' INT? '..' INT ']'; then an optional 's'
  void length(Edge &e) {
    expect("[");
    if (accept("]")) {  // fixed length without a number: 1 (exitEdge, :255-262)
      e.k_min = e.k_max = 1;
    } else {
      uint64_t a = 1;
      bool have_a = false;
      if (at_integer()) {
        a = integer();
        have_a = true;
      }
      if (accept("..")) {
        if (!have_a) bad("a variable length needs its first bound");  // variable_length: '[' INT? '..' INT ']'
        e.k_min = a;
        e.k_max = integer();
      } else {
        e.k_min = e.k_max = a;
      }
      expect("]");
    }
    ws();
    if (i < s.size() && s[i] == 's') {
      i++;
      e.path_type = ExpandPathType::Shortest;
    }
  }

  // edge (exitEdge, query_builder.cpp:234-278)
  void edge() {
    Edge e;
    e.src = last_vertex;
    if (accept("<-")) {
      e.dir = Direction::Backward;
      if (peek("[")) {
        length(e);
        expect("-");
      }
    } else if (accept("->")) {
      e.dir = Direction::Forward;
    } else if (accept("-")) {
      if (peek("[")) {
        length(e);
        if (accept("->"))
          e.dir = Direction::Forward;
        else if (accept("-"))
          e.dir = Direction::Both;
        else
          bad("expected '->' or '-'");
      } else {
        e.dir = Direction::Both;
      }
    } else {
      bad("expected an edge");
    }
    if (e.k_min > e.k_max) bad("hop range with start above end");
    last_edge = e;
  }

  void pattern() {
    vertex();
    while (peek("-") || peek("<-")) {
      edge();
      vertex();
    }
  }

  // query: 'vmatch' patterns 'return' count_only? var_props ';'
  void query() {
    expect("vmatch");
    pattern();
    while (accept(",")) pattern();
    expect("return");
    if (accept("count of")) only_count = true;  // count_only: 'count of'
    do {
      Variable v;
      v.vname = var();
      if (accept(".")) v.property = var();
      returned.push_back(v);
    } while (accept(","));
    expect(";");
    ws();
    if (i != s.size()) bad("text after ';'");
  }
};

}  // namespace

Builder::Builder(std::string query) : text(std::move(query)) {}

void Builder::parse() {
  Parser p(text);
  p.query();
  vertices.clear();
  for (auto &kv : p.vertices) vertices.push_back(kv.second);  // name order (std::map)
  edges = p.edges;
  return_vertices = p.returned;
  only_count = p.only_count;
}

std::vector<VariableName> Builder::variable_apperance_order() const {
  std::vector<VariableName> o;
  for (auto &v : vertices) o.push_back(v.name);
  return o;
}

SharedBigOperator Builder::get_vertex(const VariableName &name) {
  for (auto &op : vertex_scan)
    if (op->results_schema.columns[0].name == name + ".id") return op;
  throw Error(VS_ERR_ARG, "no vertex " + name);
}

SharedBigOperator *Builder::find_ve(const VariableName &src, const VariableName &dst, TableType t) {
  for (auto &e : ves)
    if (std::get<0>(e) == src && std::get<1>(e) == dst && std::get<2>(e) == t) return &std::get<3>(e);
  return nullptr;
}

// Builder::get_ve (query_builder.cpp:103-147): the expand src -> dst as
// asked, converting (and transposing, for the reverse edge) to ColMain.
std::optional<SharedBigOperator> Builder::get_ve(const VariableName &src, const VariableName &dst,
                                                 std::optional<TableType> type) {
  if (type) {
    if (auto *x = find_ve(src, dst, *type)) return *x;
  } else {
    if (auto *x = find_ve(src, dst, TableType::VarRowMatrix)) return *x;
    if (auto *x = find_ve(src, dst, TableType::ColMainMatrix)) return *x;
  }
  SharedBigOperator ve;
  bool transpose = false;
  if (auto *x = find_ve(src, dst, TableType::VarRowMatrix)) ve = *x;
  if (auto *x = find_ve(dst, src, TableType::VarRowMatrix)) {
    ve = *x;
    transpose = true;
  }
  if (!ve) return std::nullopt;
  if (!type) throw Error(VS_ERR_ARG, "the first two vertices must be joined by an edge in their order");
  auto t = std::make_shared<TableConvert>(*type, transpose);
  t->addLastDependency(ve);
  ves.emplace_back(src, dst, *type, t);
  return t;
}

// Builder::build (query_builder.cpp:27-92)
SharedBigOperator Builder::build(const std::vector<VariableName> &order) {
  vertex_scan.clear();
  ves.clear();
  for (auto &v : vertices) {
    std::vector<VariableFilter> f;
    if (v.filter_type == VertexFilterType::ID)
      throw Error(VS_ERR_UNSUPPORTED, "id filters are not built (assert(0) in the reference's builder)");
    if (v.filter_type == VertexFilterType::TAG) f.push_back({"Person.community", v.tag_lo, v.tag_hi});
    auto scan = std::make_shared<Scan>("Person", std::vector<VariableName>{"id"}, f);
    auto proj = std::make_shared<Projection>(Projection::MapPairs{{"Person.id", v.name + ".id"}});
    proj->addLastDependency(scan);
    vertex_scan.push_back(proj);
  }
  for (auto &e : edges) {
    // vexpand_knows (plan/usual_pattern.hh:94-110)
    auto ve = std::make_shared<VExpand>("Person", "Person", "knows", e.dir, e.k_min, e.k_max, e.path_type,
                                        ExpandStrategy::Dense, e.src + ".id", e.dst + ".id");
    ve->addLastDependency(get_vertex(e.src));
    auto sel = std::make_shared<MatrixTableSelect>(e.dst + ".id");
    sel->addDependency(ve);
    sel->addLastDependency(get_vertex(e.dst));
    if (auto *x = find_ve(e.src, e.dst, TableType::VarRowMatrix))
      *x = sel;
    else
      ves.emplace_back(e.src, e.dst, TableType::VarRowMatrix, sel);
  }
  if (order.size() < 2) return get_vertex(order.at(0));
  auto first = get_ve(order[0], order[1], std::nullopt);
  if (!first) throw Error(VS_ERR_ARG, "no edge between " + order[0] + " and " + order[1]);
  SharedBigOperator last = *first;
  for (size_t i = 2; i < order.size(); i++) {
    const bool oc = i == order.size() - 1 ? only_count : true;
    auto mint = std::make_shared<Mintersect>(order[i] + ".id", "Person", oc);
    mint->addDependency(last);
    for (size_t j = 0; j < i; j++)
      if (auto ve = get_ve(order[i], order[j], TableType::ColMainMatrix)) mint->addDependency(*ve);
    mint->finishAddingDependency();
    last = mint;
  }
  return last;
}

}  // namespace query
}  // namespace vsgb

// Parse only (no graph, no GPU work): a one-line description of the parsed
// query for tests and tools —
//   "V a:TAG:1-1 b:ALL ... | E a>b:F:1-1:any ... | R a.id b ... | count"
// Returns 0, or VS_ERR_ARG with the parse error in buf.
extern "C" int vsops_vql_describe(const char *query, char *buf, size_t cap) {
  using namespace vsgb::query;
  std::string out;
  int rc = 0;
  try {
    Builder b(query ? query : "");
    b.parse();
    out = "V";
    for (auto &v : b.parsed_vertices()) {
      out += " " + v.name + ":";
      if (v.filter_type == VertexFilterType::ALL) out += "ALL";
      if (v.filter_type == VertexFilterType::ID) out += "ID:" + std::to_string(v.id);
      if (v.filter_type == VertexFilterType::TAG)
        out += "TAG:" + std::to_string(v.tag_lo) + "-" + std::to_string(v.tag_hi);
    }
    out += " | E";
    for (auto &e : b.parsed_edges()) {
      const char *d = e.dir == vsgb::Direction::Forward ? "F" : e.dir == vsgb::Direction::Backward ? "B" : "U";
      out += " " + e.src + ">" + e.dst + ":" + d + ":" + std::to_string(e.k_min) + "-" + std::to_string(e.k_max) +
             ":" + (e.path_type == vsgb::ExpandPathType::Shortest ? "shortest" : "any");
    }
    out += " | R";
    for (auto &r : b.returned()) out += " " + r.vname + (r.property ? "." + *r.property : "");
    if (b.only_count) out += " | count";
  } catch (const std::exception &e) {
    out = e.what();
    rc = VS_ERR_ARG;
  }
  if (buf && cap) {
    const size_t n = std::min(cap - 1, out.size());
    std::memcpy(buf, out.data(), n);
    buf[n] = 0;
  }
  return rc;
}
