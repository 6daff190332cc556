// VQL front end: the reference's pattern language (src/objects/vql/grammar/vql.g4)
// parsed by hand and built into the operator plan its query builder makes
// (src/objects/vql/query_builder.cpp:19-147), over this library's operators.
//
//   vmatch (a{tag:1-1})->(b), (b{tag:3-3})<-[2..4]-(c{tag:2-2})-[]s-(a) return a.id, b, c;
//
// Vertices (Person) are scanned with an optional range filter on
// Person.community ("tag:lo-hi"); every edge becomes a VExpand over "knows"
// from its first vertex, restricted to its second vertex's scan
// (MatrixTableSelect); the vertices, in name order, are then intersected one
// after another (Mintersect over ColMain forms of the edges to the vertices
// before them).
#pragma once
#include <optional>
#include <string>
#include <tuple>
#include <vector>

#include "vs_operators.hh"

namespace vsgb {
namespace query {

enum class VertexFilterType { ID, TAG, ALL };

struct Vertex {
  VariableName name;
  VertexFilterType filter_type = VertexFilterType::ALL;
  uint64_t id = 0;
  int64_t tag_lo = 0, tag_hi = 0;
  void merge(const Vertex &v);  // Vertex::merge (query_builder.cpp:185-197)
};

struct Edge {
  VariableName src, dst;
  Direction dir = Direction::Forward;
  ExpandPathType path_type = ExpandPathType::Any;
  size_t k_min = 1, k_max = 1;
};

struct Variable {
  VariableName vname;
  std::optional<VariableName> property;
};

class Builder {
  std::string text;
  std::vector<Vertex> vertices;  // by name, as the reference's std::map orders them
  std::vector<Edge> edges;
  std::vector<Variable> return_vertices;
  std::vector<SharedBigOperator> vertex_scan;
  std::vector<std::tuple<VariableName, VariableName, TableType, SharedBigOperator>> ves;

  SharedBigOperator get_vertex(const VariableName &name);
  std::optional<SharedBigOperator> get_ve(const VariableName &src, const VariableName &dst,
                                          std::optional<TableType> type);
  SharedBigOperator *find_ve(const VariableName &src, const VariableName &dst, TableType t);

 public:
  bool only_count = false;
  explicit Builder(std::string query);
  void parse();  // throws Error(VS_ERR_ARG) with the offset of a syntax error
  std::vector<VariableName> variable_apperance_order() const;
  SharedBigOperator build(const std::vector<VariableName> &join_order);
  const std::vector<Edge> &parsed_edges() const { return edges; }
  const std::vector<Vertex> &parsed_vertices() const { return vertices; }
  const std::vector<Variable> &returned() const { return return_vertices; }
};

}  // namespace query
}  // namespace vsgb
