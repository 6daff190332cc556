// C++ operator and plan interface of VertexSurge's hot path, backed by the
// GB300 C ABI (include/vertexsurge_gb300.h).
//
// This mirrors the reference's operator API so a plan written against it
// ports by changing includes:
//   BigOperator / addDependency / addLastDependency / finishAddingDependency /
//   run / results / results_schema      src/include/operator/physical_operator.hh:77-125
//   VExpand, HashJoin, Mintersect      src/include/operator/big_operators.hh:40-183
//   InlinedData, Count, TableConvert, Projection, MatrixTableSelect
//                                       src/include/operator/big_operators2.hh:13-100
//   TableSchema, ValueSchema            src/include/execution/tuple.hh, tuple.cpp:289-342
//   Graph (CSR upload + schema)         src/include/storage/graph_store.hh
// Tables live in HBM: FlatTable wraps a vs_flat, VarRowMatrixTable and
// ColMainMatrixTable wrap a vs_bitmat (row_map / col_map on the device).
// Errors from the device layer throw vsgb::Error (the reference asserts or
// exits; see vexpand.cpp:88-91, join.cpp:82-85).
#pragma once
#include <array>
#include <cstdint>
#include <filesystem>
#include <map>
#include <memory>
#include <optional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "vertexsurge_gb300.h"

namespace vsgb {

using VID = uint32_t;
using Int64 = int64_t;
using VariableName = std::string;
using TypeName = std::string;

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};
void check(int rc);

enum class Type { VID, Int64 };
enum class TableType { Flat, VarRowMatrix, ColMainMatrix, MultipleVarRowMatrix };
enum class Direction { Forward, Backward, Both, Undecide };
enum class ExpandPathType { Any, Shortest, FindShortest };
enum class ExpandStrategy { Adaptive, CSR, Dense };

struct ValueSchema {
  VariableName name;
  Type type;
  bool operator==(const ValueSchema &o) const { return name == o.name && type == o.type; }
};

struct TableSchema {
  std::vector<ValueSchema> columns;
  std::optional<std::pair<ValueSchema, size_t>> get_schema(const VariableName &n) const;
  static TableSchema join_schema(const TableSchema &a, const TableSchema &b,
                                 std::optional<VariableName> key);
  bool has_duplicate_variable() const;
};

struct VExpandPathParameters {
  ExpandPathType path_type = ExpandPathType::Any;
  static const size_t K_MAX_FIND_SHORTEST = 50;
  bool with_distance = false;
  static VExpandPathParameters Any();
  static VExpandPathParameters Shortest();
  static VExpandPathParameters FindShortest();
  VExpandPathParameters set_with_distance() {
    with_distance = true;
    return *this;
  }
};

class FlatTable;
class MatrixTable;

class Table {
 public:
  TableSchema schema;
  TableType type;
  Table(TableSchema s, TableType t) : schema(std::move(s)), type(t) {}
  virtual ~Table() = default;
  virtual size_t tuple_count() = 0;
  FlatTable *down_to_flat_table();
  MatrixTable *down_to_matrix_table();
};

class FlatTable : public Table {
 public:
  vs_flat *h = nullptr;
  explicit FlatTable(TableSchema s) : Table(std::move(s), TableType::Flat) {}
  FlatTable(TableSchema s, vs_flat *handle) : Table(std::move(s), TableType::Flat), h(handle) {}
  ~FlatTable() override;
  size_t tuple_count() override;
  // host columns (VID columns as uint32, Int64 columns as int64)
  void set_columns(const std::vector<std::vector<uint64_t>> &cols);
  std::vector<uint64_t> column(size_t i) const;  // values widened to 64 bits
};

class MatrixTable : public Table {
 public:
  vs_bitmat *h = nullptr;
  MatrixTable(TableSchema s, TableType t) : Table(std::move(s), t) {}
  ~MatrixTable() override;
  size_t tuple_count() override;
  size_t row_count() const;
  size_t col_count() const;
  void set_matrix(vs_bitmat *m) { h = m; }
  bool get(size_t r, size_t c) const;  // downloads (test helper)
  std::vector<uint64_t> logical_words() const;
};

class VarRowMatrixTable : public MatrixTable {
 public:
  explicit VarRowMatrixTable(TableSchema s) : MatrixTable(std::move(s), TableType::VarRowMatrix) {}
};

// One matrix per distance: VExpand with_distance, Dense (matrix_table.hh:132-149).
// The schema ends with the distance column (Int64 here, Int32 in the reference).
class MultipleMatrixTable : public Table {
 public:
  std::vector<int32_t> dis;
  std::vector<std::shared_ptr<MatrixTable>> mats;
  explicit MultipleMatrixTable(TableSchema s) : Table(std::move(s), TableType::MultipleVarRowMatrix) {}
  void add_mat(std::shared_ptr<MatrixTable> t, int32_t d);
  size_t tuple_count() override;
  // (row value, column value, distance) tuples, layer by layer (bit_matrix_table.cpp:302-340)
  std::shared_ptr<FlatTable> output_to_flat() const;
  // the same with each (row, column) pair once, at its smallest distance
  // (VExpand::merge_to_Flat for Any paths, vexpand.cpp:383-405)
  std::shared_ptr<FlatTable> output_to_flat_first() const;
};
class ColMainMatrixTable : public MatrixTable {
 public:
  explicit ColMainMatrixTable(TableSchema s) : MatrixTable(std::move(s), TableType::ColMainMatrix) {}
};

// Vertex / edge schema and device CSR per edge type ("Src_edge_Dst").
class Graph {
 public:
  struct EdgeType {
    TypeName src, dst, name;
    bool directed;
    vs_graph *g;
  };
  std::map<TypeName, size_t> vertex_count;
  std::map<std::string, EdgeType> edges;
  // vertex properties ("Type.name"), one device column each (1/2/4-byte
  // unsigned values widened to VID, Int64 kept); read from the directory
  std::map<std::string, vs_flat *> properties;
  void add_vertex_property(const std::string &var, const std::vector<uint64_t> &values, Type t);
  std::filesystem::path dir;  // the reference's graph directory (empty: types added by hand)
  Graph() = default;
  // Graph(dir) + load(): schema.json and the CSR DiskArray files the reference
  // writes and reads (storage/graph_store.cpp:46-73)
  explicit Graph(std::filesystem::path d) : dir(std::move(d)) {}
  Graph(const Graph &) = delete;
  Graph &operator=(const Graph &) = delete;
  ~Graph();
  void add_vertex_type(const TypeName &t, size_t count) { vertex_count[t] = count; }
  void add_edge_type(const TypeName &src, const TypeName &edge, const TypeName &dst, bool directed,
                     uint32_t V, uint64_t E, const int64_t *fwd_off, const uint32_t *fwd_dst,
                     const int64_t *rev_off, const uint32_t *rev_src);
  const EdgeType &edge(const TypeName &src, const TypeName &e, const TypeName &dst) const;
  // Graph::load sets the global store (graph_store.cpp:48-73); with a
  // directory it first uploads every self edge type's CSR found there
  void load();

 private:
  void load_dir();
};
// Variable names of an edge type's CSR files (meta/schema.cpp:36-66)
std::string forward_edge_name(const TypeName &src, const TypeName &e, const TypeName &dst, bool directed);
std::string backward_edge_name(const TypeName &src, const TypeName &e, const TypeName &dst, bool directed);

class BigOperator;
using SharedBigOperator = std::shared_ptr<BigOperator>;

class BigOperator {
 protected:
  std::vector<SharedBigOperator> deps;
  std::vector<std::shared_ptr<Table>> dep_results;
  virtual bool before_execution() { return true; }
  virtual void run_internal();

 public:
  static Graph *graph_store;
  static vs_stream_t stream;
  std::shared_ptr<Table> results;
  TableSchema results_schema;
  virtual ~BigOperator() = default;
  void addDependency(SharedBigOperator d);
  void addLastDependency(SharedBigOperator d);
  virtual void finishAddingDependency() {}
  void run();
};

class InlinedData : public BigOperator {
  void run_internal() override {}
};

// An inclusive range filter on a vertex property ("Person.community"),
// VariableFilter with Range (meta/type.hh:250-310, utils/utils.hh:574-586).
struct VariableFilter {
  VariableName property;
  int64_t lo, hi;
};

// Scan(vertex_type, {"id"}, filters) (big_operators.hh:21-38, scan.cpp:14-70):
// the ids of the vertices passing the filter, as "Type.id".  Fetches only
// the id (the plans' use); at most one filter.
class Scan : public BigOperator {
  TypeName vertex_type;
  std::vector<VariableFilter> filters;
  void run_internal() override;

 public:
  Scan(TypeName vertex_type, std::vector<VariableName> fetch_properties, std::vector<VariableFilter> filters = {});
};

class VExpand : public BigOperator {
  TypeName start_type, target_type, edge_type;
  Direction dir;
  size_t k_min, k_max;
  VExpandPathParameters path_params;
  ExpandStrategy strategy;
  VariableName start_variable_name;
  std::optional<VariableName> target_variable_name;
  void run_internal() override;

 public:
  vs_expand_stats stats{};
  VExpand(TypeName src_type, TypeName dst_type, TypeName edge_type, Direction dir, size_t k_min,
          size_t k_max, ExpandPathType path_type, ExpandStrategy strategy,
          VariableName variable_name, std::optional<VariableName> target_variable_name);
  // FindShortest
  VExpand(TypeName src_type, TypeName dst_type, TypeName edge_type, Direction dir,
          VExpandPathParameters path_params, ExpandStrategy strategy, VariableName variable_name,
          VariableName target_variable_name);
  // one edge type with path parameters (with_distance)
  VExpand(TypeName src_type, TypeName dst_type, TypeName edge_type, Direction dir, size_t k_min,
          size_t k_max, VExpandPathParameters path_params, ExpandStrategy strategy,
          VariableName variable_name, std::optional<VariableName> target_variable_name);
  void finishAddingDependency() override;
};

class HashJoin : public BigOperator {
  VariableName key_variable_name;
  bool only_count;
  void run_internal() override;

 public:
  uint64_t max_rows = ~0ull >> 2;
  HashJoin(std::string key_variable_name, bool only_count);
  void finishAddingDependency() override;
};

class Mintersect : public BigOperator {
  VariableName new_vertex_var_name;
  TypeName new_vertex_type;
  bool only_count;
  size_t new_vertex_count = 0;
  void run_internal() override;

 public:
  uint64_t max_rows = ~0ull >> 2;
  Mintersect(VariableName new_vertex_var_name, TypeName new_vertex_type, bool only_count);
  void finishAddingDependency() override;
};

class Count : public BigOperator {
  void run_internal() override;
};

class TableConvert : public BigOperator {
  TableType convert_to;
  bool transpose;
  void run_internal() override;

 public:
  TableConvert(TableType type, bool transpose = false);
  void finishAddingDependency() override;
};

class Projection : public BigOperator {
  std::vector<std::pair<VariableName, VariableName>> projection_map;
  std::vector<size_t> old_variable_idx;
  void run_internal() override;

 public:
  using MapPair = std::pair<VariableName, VariableName>;
  using MapPairs = std::vector<MapPair>;
  explicit Projection(MapPairs m);
  void finishAddingDependency() override;
};

class MatrixTableSelect : public BigOperator {
  VariableName key_name;
  void run_internal() override;

 public:
  explicit MatrixTableSelect(VariableName key_name);
  void finishAddingDependency() override;
};

// MatrixTableFilter (big_operators2.hh:53-61,142-170).  The reference takes a
// host predicate f(row value, column value) and clears the bits where it is
// false, in its input table; here the predicate is the AND of device forms
// (vs_matrix_filter): a bitset over row values, a bitset over column values
// and a pair list (kept or dropped).  The input table is filtered in place and
// becomes the result, as in the reference; a MultipleMatrixTable is filtered
// layer by layer.
struct MatrixFilter {
  std::vector<uint64_t> row_keep;  // bitset over row values (empty: no row condition)
  uint32_t row_values = 0;         // values at or above fail
  std::vector<uint64_t> col_keep;  // bitset over column values (empty: no column condition)
  uint32_t col_values = 0;
  std::vector<std::pair<VID, VID>> pairs;  // (row value, column value)
  int pairs_mode = 0;                      // 1: keep listed pairs only, 2: drop listed pairs
  // the bitset of vertices v with a neighbour u (edge type of g) whose uint8
  // property equals value: tcr1's "signed in to a blocked medium" (tcr1.cpp:46-57)
  static std::vector<uint64_t> any_neighbor(class Graph &g, const std::string &edge_key,
                                            const std::vector<uint8_t> &prop, uint8_t value);
};

class MatrixTableFilter : public BigOperator {
  MatrixFilter f;
  void run_internal() override;

 public:
  explicit MatrixTableFilter(MatrixFilter f);
  void finishAddingDependency() override;
};

// Result consumers (big_operators2.hh, big_operators3.hh).
enum class SortOrder { ASC, DESC };

// (column value, bit count) per column (matrix_column_count.cpp:6-87); the
// count column is Int64 here (Int32 in the reference).
class MatrixColumnCount : public BigOperator {
  VariableName count_name;
  std::optional<SortOrder> ord;
  void run_internal() override;

 public:
  explicit MatrixColumnCount(VariableName count_name, std::optional<SortOrder> ord = std::nullopt);
  void finishAddingDependency() override;
};

// The column values holding any bit (matrix_row_or_sum.cpp:7-54).
class MatrixRowOrSum : public BigOperator {
  void run_internal() override;

 public:
  MatrixRowOrSum() = default;
  void finishAddingDependency() override;
};

// SemiJoin<N> (semi_join.cpp:7-262): N = 1 or 2 key variables (two keys must
// be vertex ids); flat or VarRow inputs.
template <size_t N> class SemiJoin : public BigOperator {
  std::array<VariableName, N> key_variables;
  bool only_count;
  void run_internal() override;

 public:
  SemiJoin(std::array<VariableName, N> key_variables, bool only_count);
  void finishAddingDependency() override;
};

// Count of a Count/only_count result table (single Int64 tuple).
int64_t single_count(Table *t);

}  // namespace vsgb
