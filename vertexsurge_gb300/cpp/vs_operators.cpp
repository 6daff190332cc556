// C++ operator layer over the GB300 C ABI (see vs_operators.hh).
#include "vs_operators.hh"

#include <algorithm>
#include <cstring>

namespace vsgb {

Graph *BigOperator::graph_store = nullptr;
vs_stream_t BigOperator::stream = nullptr;

void check(int rc) {
  if (rc != VS_OK && rc != VS_ERR_CAPACITY) throw Error(rc, vs_last_error());
}

// ---- schemas ----------------------------------------------------------------
std::optional<std::pair<ValueSchema, size_t>> TableSchema::get_schema(const VariableName &n) const {
  for (size_t i = 0; i < columns.size(); i++)
    if (columns[i].name == n) return std::make_pair(columns[i], i);
  return std::nullopt;
}

bool TableSchema::has_duplicate_variable() const {
  for (size_t i = 0; i < columns.size(); i++)
    for (size_t j = i + 1; j < columns.size(); j++)
      if (columns[i].name == columns[j].name) return true;
  return false;
}

// TableSchema::join_schema (tuple.cpp:317-342)
TableSchema TableSchema::join_schema(const TableSchema &a, const TableSchema &b,
                                     std::optional<VariableName> key) {
  TableSchema r;
  if (key) {
    if (!a.get_schema(*key) || !b.get_schema(*key)) throw Error(VS_ERR_ARG, "join key " + *key + " missing");
    r.columns = a.columns;
    for (const auto &c : b.columns)
      if (c.name != *key) r.columns.push_back(c);
  } else {
    r.columns = a.columns;
    r.columns.insert(r.columns.end(), b.columns.begin(), b.columns.end());
  }
  if (r.has_duplicate_variable()) throw Error(VS_ERR_ARG, "duplicate variable in join schema");
  return r;
}

VExpandPathParameters VExpandPathParameters::Any() { return {ExpandPathType::Any, false}; }
VExpandPathParameters VExpandPathParameters::Shortest() { return {ExpandPathType::Shortest, false}; }
VExpandPathParameters VExpandPathParameters::FindShortest() {
  return {ExpandPathType::FindShortest, true};
}

// ---- tables -------------------------------------------------------------------
FlatTable *Table::down_to_flat_table() { return dynamic_cast<FlatTable *>(this); }

void MultipleMatrixTable::add_mat(std::shared_ptr<MatrixTable> t, int32_t d) {
  mats.push_back(std::move(t));
  dis.push_back(d);
}

size_t MultipleMatrixTable::tuple_count() {
  size_t n = 0;
  for (auto &m : mats) n += m->tuple_count();
  return n;
}

std::shared_ptr<FlatTable> MultipleMatrixTable::output_to_flat() const {
  std::vector<const vs_bitmat *> hs;
  for (auto &m : mats) hs.push_back(m->h);
  vs_flat *f = nullptr;
  check(vs_layers_to_flat(hs.data(), dis.data(), (uint32_t)hs.size(), &f, BigOperator::stream));
  return std::make_shared<FlatTable>(schema, f);
}

std::shared_ptr<FlatTable> MultipleMatrixTable::output_to_flat_first() const {
  std::vector<const vs_bitmat *> hs;
  for (auto &m : mats) hs.push_back(m->h);
  vs_flat *f = nullptr;
  check(vs_layers_to_flat_first(hs.data(), dis.data(), (uint32_t)hs.size(), &f, BigOperator::stream));
  return std::make_shared<FlatTable>(schema, f);
}
MatrixTable *Table::down_to_matrix_table() { return dynamic_cast<MatrixTable *>(this); }

static int32_t abi_type(Type t) { return t == Type::Int64 ? VS_T_I64 : VS_T_VID; }

FlatTable::~FlatTable() { vs_flat_free(h); }

size_t FlatTable::tuple_count() {
  if (!h) return 0;
  uint64_t n = 0;
  check(vs_flat_info(h, nullptr, &n, nullptr));
  return n;
}

void FlatTable::set_columns(const std::vector<std::vector<uint64_t>> &cols) {
  if (cols.size() != schema.columns.size()) throw Error(VS_ERR_ARG, "column count differs from schema");
  const size_t n = cols.empty() ? 0 : cols[0].size();
  std::vector<int32_t> types;
  for (const auto &c : schema.columns) types.push_back(abi_type(c.type));
  vs_flat *f = nullptr;
  check(vs_flat_create((uint32_t)types.size(), types.data(), n, &f));
  for (size_t i = 0; i < cols.size(); i++) {
    if (types[i] == VS_T_I64) {
      std::vector<int64_t> v(cols[i].begin(), cols[i].end());
      check(vs_flat_upload(f, (uint32_t)i, v.data(), BigOperator::stream));
    } else {
      std::vector<uint32_t> v(cols[i].begin(), cols[i].end());
      check(vs_flat_upload(f, (uint32_t)i, v.data(), BigOperator::stream));
    }
  }
  vs_flat_free(h);
  h = f;
}

std::vector<uint64_t> FlatTable::column(size_t i) const {
  uint32_t nc = 0;
  uint64_t n = 0;
  int32_t types[16];
  check(vs_flat_info(h, &nc, &n, types));
  std::vector<uint64_t> out(n);
  if (types[i] == VS_T_I64) {
    std::vector<int64_t> v(n);
    check(vs_flat_download(h, (uint32_t)i, v.data(), BigOperator::stream));
    for (size_t k = 0; k < n; k++) out[k] = (uint64_t)v[k];
  } else {
    std::vector<uint32_t> v(n);
    check(vs_flat_download(h, (uint32_t)i, v.data(), BigOperator::stream));
    for (size_t k = 0; k < n; k++) out[k] = v[k];
  }
  return out;
}

MatrixTable::~MatrixTable() { vs_bitmat_free(h); }

size_t MatrixTable::tuple_count() {
  if (!h) return 0;
  uint64_t c = 0;
  check(vs_bitmat_count(h, &c, BigOperator::stream));
  return c;
}

size_t MatrixTable::row_count() const {
  vs_bitmat_info i;
  check(vs_bitmat_get_info(h, &i));
  return i.rows;
}

size_t MatrixTable::col_count() const {
  vs_bitmat_info i;
  check(vs_bitmat_get_info(h, &i));
  return i.cols;
}

std::vector<uint64_t> MatrixTable::logical_words() const {
  vs_bitmat_info i;
  check(vs_bitmat_get_info(h, &i));
  std::vector<uint64_t> w((size_t)i.cols * ((i.rows + 63) / 64));
  check(vs_bitmat_download(h, w.data(), BigOperator::stream));
  return w;
}

bool MatrixTable::get(size_t r, size_t c) const {
  vs_bitmat_info i;
  check(vs_bitmat_get_info(h, &i));
  const auto w = logical_words();
  return (w[c * ((i.rows + 63) / 64) + r / 64] >> (r % 64)) & 1;
}

// ---- graph --------------------------------------------------------------------
Graph::~Graph() {
  for (auto &kv : edges) vs_graph_free(kv.second.g);
  for (auto &kv : properties) vs_flat_free(kv.second);
  if (BigOperator::graph_store == this) BigOperator::graph_store = nullptr;
}

void Graph::add_edge_type(const TypeName &src, const TypeName &edge, const TypeName &dst,
                          bool directed, uint32_t V, uint64_t E, const int64_t *fwd_off,
                          const uint32_t *fwd_dst, const int64_t *rev_off, const uint32_t *rev_src) {
  EdgeType t{src, dst, edge, directed, nullptr};
  check(vs_graph_upload(V, E, fwd_off, fwd_dst, rev_off, rev_src, directed ? 1 : 0,
                        BigOperator::stream, &t.g));
  edges[src + "_" + edge + "_" + dst] = t;
}

void Graph::add_vertex_property(const std::string &var, const std::vector<uint64_t> &values, Type t) {
  const int32_t ty = t == Type::Int64 ? VS_T_I64 : VS_T_VID;
  vs_flat *f = nullptr;
  check(vs_flat_create(1, &ty, values.size(), &f));
  if (t == Type::Int64) {
    check(vs_flat_upload(f, 0, values.data(), BigOperator::stream));
  } else {
    std::vector<uint32_t> v(values.begin(), values.end());
    check(vs_flat_upload(f, 0, v.data(), BigOperator::stream));
  }
  auto it = properties.find(var);
  if (it != properties.end()) vs_flat_free(it->second);
  properties[var] = f;
}

const Graph::EdgeType &Graph::edge(const TypeName &src, const TypeName &e, const TypeName &dst) const {
  auto it = edges.find(src + "_" + e + "_" + dst);
  if (it == edges.end()) throw Error(VS_ERR_ARG, "no edge type " + src + "_" + e + "_" + dst);
  return it->second;
}

void Graph::load() {
  if (!dir.empty()) load_dir();
  BigOperator::graph_store = this;
}

// ---- operator runtime (PhysicalOperator::run, physical_operator.cpp:62-101) ----
void BigOperator::addDependency(SharedBigOperator d) {
  deps.push_back(std::move(d));
  dep_results.push_back(nullptr);
}

void BigOperator::addLastDependency(SharedBigOperator d) {
  addDependency(std::move(d));
  finishAddingDependency();
}

void BigOperator::run_internal() {
  results_schema = dep_results[0]->schema;
  results = dep_results[0];
}

void BigOperator::run() {
  for (size_t i = 0; i < deps.size(); i++) {
    deps[i]->run();
    dep_results[i] = deps[i]->results;
  }
  if (before_execution()) run_internal();
}

static std::vector<uint32_t> flat_vid_column(const std::shared_ptr<Table> &t, const VariableName &n) {
  auto *f = t->down_to_flat_table();
  if (!f) throw Error(VS_ERR_ARG, "variable " + n + " is not in a flat table");
  auto s = f->schema.get_schema(n);
  if (!s) throw Error(VS_ERR_ARG, "variable " + n + " not found");
  auto c = f->column(s->second);
  return std::vector<uint32_t>(c.begin(), c.end());
}

static int abi_dir(Direction d, bool directed) {
  switch (d) {
    case Direction::Forward: return VS_DIR_FORWARD;
    case Direction::Backward: return VS_DIR_BACKWARD;
    case Direction::Both: return VS_DIR_BOTH;
    default:
      if (directed) throw Error(VS_ERR_ARG, "a directed self edge needs a direction");
      return VS_DIR_FORWARD;
  }
}

// ---- Scan ---------------------------------------------------------------------
Scan::Scan(TypeName type, std::vector<VariableName> fetch, std::vector<VariableFilter> f)
    : vertex_type(std::move(type)), filters(std::move(f)) {
  if (fetch.size() != 1 || fetch[0] != "id")
    throw Error(VS_ERR_UNSUPPORTED, "Scan fetches the vertex id only");
  if (filters.size() > 1) throw Error(VS_ERR_UNSUPPORTED, "Scan takes at most one range filter");
  results_schema = TableSchema{{{vertex_type + ".id", Type::VID}}};  // Scan::set_table_schema (scan.cpp:22-29)
}

void Scan::run_internal() {
  if (!graph_store || !graph_store->vertex_count.count(vertex_type))
    throw Error(VS_ERR_ARG, "vertex type " + vertex_type + " is not in the loaded graph");
  const size_t V = graph_store->vertex_count.at(vertex_type);
  const void *vals = nullptr;
  int bytes = 0;
  int64_t lo = 0, hi = 0;
  if (!filters.empty()) {
    auto it = graph_store->properties.find(filters[0].property);
    if (it == graph_store->properties.end()) throw Error(VS_ERR_ARG, "no vertex property " + filters[0].property);
    int32_t ty = 0;
    uint64_t n = 0;
    check(vs_flat_info(it->second, nullptr, &n, &ty));
    if (n != V) throw Error(VS_ERR_ARG, "property " + filters[0].property + " has a value per vertex");
    check(vs_flat_column(it->second, 0, &vals));
    bytes = ty == VS_T_I64 ? 8 : 4;
    lo = filters[0].lo;
    hi = filters[0].hi;
  }
  vs_flat *f = nullptr;
  check(vs_select_ids_in_range(vals, bytes, (uint32_t)V, lo, hi, &f, stream));
  results = std::make_shared<FlatTable>(results_schema, f);
}

// ---- VExpand ------------------------------------------------------------------
VExpand::VExpand(TypeName src_type, TypeName dst_type, TypeName edge_type, Direction dir, size_t k_min,
                 size_t k_max, ExpandPathType path_type, ExpandStrategy strategy,
                 VariableName variable_name, std::optional<VariableName> target_variable_name)
    : start_type(std::move(src_type)), target_type(std::move(dst_type)), edge_type(std::move(edge_type)),
      dir(dir), k_min(k_min), k_max(k_max), path_params{path_type, false}, strategy(strategy),
      start_variable_name(std::move(variable_name)), target_variable_name(std::move(target_variable_name)) {
  if (k_max > 1 && start_type != target_type)  // vexpand.cpp:88-91
    throw Error(VS_ERR_ARG, "k max should be 1 when edge is not self edge");
}

VExpand::VExpand(TypeName src_type, TypeName dst_type, TypeName edge_type, Direction dir, size_t k_min,
                 size_t k_max, VExpandPathParameters path_params, ExpandStrategy strategy,
                 VariableName variable_name, std::optional<VariableName> target_variable_name)
    : VExpand(std::move(src_type), std::move(dst_type), std::move(edge_type), dir, k_min, k_max,
              path_params.path_type, strategy, std::move(variable_name), std::move(target_variable_name)) {
  if (path_params.path_type == ExpandPathType::FindShortest)
    throw Error(VS_ERR_ARG, "FindShortest has its own constructor");
  this->path_params = path_params;
}

VExpand::VExpand(TypeName src_type, TypeName dst_type, TypeName edge_type, Direction dir,
                 VExpandPathParameters path_params, ExpandStrategy strategy, VariableName variable_name,
                 VariableName target_variable_name)
    : VExpand(std::move(src_type), std::move(dst_type), std::move(edge_type), dir, 1,
              VExpandPathParameters::K_MAX_FIND_SHORTEST, path_params.path_type, strategy,
              std::move(variable_name), std::move(target_variable_name)) {
  if (path_params.path_type != ExpandPathType::FindShortest)
    throw Error(VS_ERR_ARG, "this constructor is for FindShortest");
  this->path_params = path_params;
}

// VExpand::finishAddingDependency (vexpand.cpp:103-164)
void VExpand::finishAddingDependency() {
  if (deps.size() != 1) throw Error(VS_ERR_ARG, "VExpand takes one dependency");
  auto sv = deps[0]->results_schema.get_schema(start_variable_name);
  if (!sv) throw Error(VS_ERR_ARG, "start variable " + start_variable_name + " missing");
  ValueSchema target_vs{target_variable_name ? *target_variable_name : target_type + ".id", Type::VID};
  if (path_params.path_type == ExpandPathType::FindShortest) {
    auto tv = deps[0]->results_schema.get_schema(*target_variable_name);
    if (!tv) throw Error(VS_ERR_ARG, "target variable missing");
    results_schema = deps[0]->results_schema;
    results_schema.columns.push_back({"distance", Type::Int64});
    return;
  }
  results_schema = TableSchema{{sv->first, target_vs}};
  if (path_params.with_distance) results_schema.columns.push_back({"distance", Type::Int64});  // vexpand.cpp:120-123
}

void VExpand::run_internal() {
  if (!graph_store) throw Error(VS_ERR_ARG, "no graph loaded");
  const auto &et = graph_store->edge(start_type, edge_type, target_type);
  auto src = flat_vid_column(dep_results[0], start_variable_name);
  vs_expand_params p{};
  p.k_min = (uint32_t)k_min;
  p.k_max = (uint32_t)k_max;
  p.path_type = path_params.path_type == ExpandPathType::Any        ? VS_PATH_ANY
                : path_params.path_type == ExpandPathType::Shortest ? VS_PATH_SHORTEST
                                                                    : VS_PATH_FIND_SHORTEST;
  p.direction = abi_dir(dir, et.directed);
  p.strategy = VS_STRAT_AUTO;
  if (path_params.path_type == ExpandPathType::FindShortest) {
    auto tgt = flat_vid_column(dep_results[0], *target_variable_name);
    std::vector<int32_t> dist(src.size(), -1);
    if (!src.empty())
      check(vs_expand(et.g, src.data(), (uint32_t)src.size(), &p, tgt.data(), dist.data(), nullptr,
                      &stats, stream));
    // results = the dependency's table extended with the distance column
    auto *in = dep_results[0]->down_to_flat_table();
    auto out = std::make_shared<FlatTable>(results_schema);
    std::vector<std::vector<uint64_t>> cols;
    for (size_t i = 0; i < in->schema.columns.size(); i++) cols.push_back(in->column(i));
    std::vector<uint64_t> d(dist.size());
    for (size_t i = 0; i < dist.size(); i++) d[i] = (uint64_t)(int64_t)dist[i];
    cols.push_back(d);
    out->set_columns(cols);
    results = out;
    return;
  }
  if (path_params.with_distance) {
    // copy_to_multi_MT (vexpand.cpp:356-378); the CSR strategy's flat output
    // with distances (merge_to_Flat, :380-446) is the same layers as tuples,
    // each (source, vertex) pair once at its smallest distance for Any (the
    // Shortest layers are disjoint)
    std::vector<vs_bitmat *> layers(k_max - k_min + 1, nullptr);
    uint32_t n = 0;
    check(vs_expand_layers(et.g, src.data(), (uint32_t)src.size(), &p, layers.data(), &n, stream));
    TableSchema mat_schema = results_schema;
    mat_schema.columns.pop_back();
    auto multi = std::make_shared<MultipleMatrixTable>(results_schema);
    for (uint32_t i = 0; i < n; i++) {
      auto t = std::make_shared<VarRowMatrixTable>(mat_schema);
      t->set_matrix(layers[i]);
      multi->add_mat(t, (int32_t)(k_min + i));
    }
    if (strategy == ExpandStrategy::CSR) {
      results = path_params.path_type == ExpandPathType::Any ? multi->output_to_flat_first() : multi->output_to_flat();
    } else {
      results = multi;
    }
    return;
  }
  vs_bitmat *m = nullptr;
  check(vs_expand(et.g, src.data(), (uint32_t)src.size(), &p, nullptr, nullptr, &m, &stats, stream));
  if (strategy == ExpandStrategy::CSR) {
    // the CSR strategy's flat (start, target) output (merge_to_Flat, vexpand.cpp:380-446)
    vs_flat *f = nullptr;
    check(vs_bitmat_to_flat(m, &f, stream));
    vs_bitmat_free(m);
    results = std::make_shared<FlatTable>(results_schema, f);
    return;
  }
  auto t = std::make_shared<VarRowMatrixTable>(results_schema);
  t->set_matrix(m);
  results = t;
}

// ---- HashJoin -------------------------------------------------------------------
HashJoin::HashJoin(std::string key, bool only_count) : key_variable_name(std::move(key)), only_count(only_count) {}

void HashJoin::finishAddingDependency() {
  if (deps.size() != 2) throw Error(VS_ERR_ARG, "HashJoin takes two dependencies");
  if (!only_count)
    results_schema = TableSchema::join_schema(deps[0]->results_schema, deps[1]->results_schema,
                                              key_variable_name);
  else
    results_schema = TableSchema{{{"count", Type::Int64}}};
}

static vs_table_ref table_ref(const std::shared_ptr<Table> &t, const VariableName &key) {
  vs_table_ref r{};
  auto s = t->schema.get_schema(key);
  if (!s) throw Error(VS_ERR_ARG, "key " + key + " not in schema");
  r.key_col = (uint32_t)s->second;
  if (auto *f = t->down_to_flat_table())
    r.flat = f->h;
  else
    r.mat = t->down_to_matrix_table()->h;
  return r;
}

static std::shared_ptr<FlatTable> count_table(int64_t c) {
  auto t = std::make_shared<FlatTable>(TableSchema{{{"count", Type::Int64}}});
  t->set_columns({{(uint64_t)c}});
  return t;
}

void HashJoin::run_internal() {
  auto a = table_ref(dep_results[0], key_variable_name);
  auto b = table_ref(dep_results[1], key_variable_name);
  if (dep_results[0]->schema.get_schema(key_variable_name)->first !=
      dep_results[1]->schema.get_schema(key_variable_name)->first)
    throw Error(VS_ERR_ARG, "key " + key_variable_name + " differs in type");  // join.cpp:36-37
  vs_flat *out = nullptr;
  uint64_t count = 0;
  check(vs_hash_join(a, b, only_count ? 1 : 0, max_rows, only_count ? nullptr : &out, &count, stream));
  results = only_count ? std::static_pointer_cast<Table>(count_table((int64_t)count))
                       : std::static_pointer_cast<Table>(std::make_shared<FlatTable>(results_schema, out));
}

// ---- Mintersect -----------------------------------------------------------------
// The vertex type is resolved against the loaded graph at construction, as
// the reference does (mintersect.cpp:11).
Mintersect::Mintersect(VariableName nv, TypeName t, bool only_count)
    : new_vertex_var_name(std::move(nv)), new_vertex_type(std::move(t)), only_count(only_count) {
  if (!graph_store || !graph_store->vertex_count.count(new_vertex_type))
    throw Error(VS_ERR_ARG, "vertex type " + new_vertex_type + " is not in the loaded graph");
  new_vertex_count = graph_store->vertex_count.at(new_vertex_type);
}

// Mintersect::finishAddingDependency (mintersect.cpp:14-46)
void Mintersect::finishAddingDependency() {
  const auto &base = deps[0]->results_schema;
  std::optional<ValueSchema> ks;
  for (size_t i = 1; i < deps.size(); i++) {
    const auto &s = deps[i]->results_schema;
    if (s.columns.size() != 2) throw Error(VS_ERR_ARG, "a Mintersect dependency has two columns");
    auto t = s.get_schema(new_vertex_var_name);
    if (!t || t->first.type != Type::VID) throw Error(VS_ERR_ARG, "new vertex variable must be a VID");
    if (ks && !(*ks == t->first)) throw Error(VS_ERR_ARG, "new vertex variable differs");
    ks = t->first;
    if (!base.get_schema(s.columns[1 - t->second].name))
      throw Error(VS_ERR_ARG, "dependency variable not in the base");
  }
  if (only_count) {
    results_schema = TableSchema{{{"count", Type::Int64}}};
  } else {
    results_schema = base;
    results_schema.columns.push_back(*ks);
  }
}

void Mintersect::run_internal() {
  vs_table_ref base{};
  if (auto *f = dep_results[0]->down_to_flat_table())
    base.flat = f->h;
  else
    base.mat = dep_results[0]->down_to_matrix_table()->h;
  std::vector<vs_isect_dep> ds;
  for (size_t i = 1; i < dep_results.size(); i++) {
    const auto &s = dep_results[i]->schema;
    const size_t nv = s.get_schema(new_vertex_var_name)->second, u = 1 - nv;
    vs_isect_dep d{};
    d.base_col = (uint32_t)dep_results[0]->schema.get_schema(s.columns[u].name)->second;
    if (auto *f = dep_results[i]->down_to_flat_table()) {
      d.flat = f->h;
      d.u_col = (uint32_t)u;
      d.nv_col = (uint32_t)nv;
    } else {
      if (dep_results[i]->type != TableType::ColMainMatrix || nv != 0)  // mintersect.cpp:57-60
        throw Error(VS_ERR_ARG, "a matrix dependency must be ColMain with the new vertex as rows");
      d.mat = dep_results[i]->down_to_matrix_table()->h;
    }
    ds.push_back(d);
  }
  const uint32_t nvc = (uint32_t)new_vertex_count;
  vs_flat *out = nullptr;
  uint64_t count = 0;
  check(vs_mintersect(base, ds.data(), (uint32_t)ds.size(), nvc, only_count ? 1 : 0, max_rows,
                      only_count ? nullptr : &out, &count, stream));
  results = only_count ? std::static_pointer_cast<Table>(count_table((int64_t)count))
                       : std::static_pointer_cast<Table>(std::make_shared<FlatTable>(results_schema, out));
}

// ---- glue operators (big_operators2.cpp) -----------------------------------------
void Count::run_internal() {
  results_schema = TableSchema{{{"count", Type::Int64}}};
  results = count_table((int64_t)dep_results[0]->tuple_count());
}

// ---- result consumers --------------------------------------------------------
MatrixColumnCount::MatrixColumnCount(VariableName count_name, std::optional<SortOrder> ord)
    : count_name(std::move(count_name)), ord(ord) {}

// MatrixColumnCount::finishAddingDependency (matrix_column_count.cpp:10-17)
void MatrixColumnCount::finishAddingDependency() {
  if (deps.size() != 1 || deps[0]->results_schema.columns.size() != 2 ||
      deps[0]->results_schema.columns[1].type != Type::VID)
    throw Error(VS_ERR_ARG, "MatrixColumnCount takes one two-column matrix whose columns are vertices");
  results_schema = TableSchema{{{count_name, Type::VID}, {"count", Type::Int64}}};
}

void MatrixColumnCount::run_internal() {
  auto *m = dep_results[0]->down_to_matrix_table();
  if (!m) throw Error(VS_ERR_ARG, "MatrixColumnCount needs a matrix input");  // matrix_column_count.cpp:20-21
  vs_flat *f = nullptr;
  check(vs_matrix_column_count(m->h, !ord ? 0 : *ord == SortOrder::ASC ? 1 : 2, &f, stream));
  results = std::make_shared<FlatTable>(results_schema, f);
}

// MatrixRowOrSum::finishAddingDependency (matrix_row_or_sum.cpp:7-12)
void MatrixRowOrSum::finishAddingDependency() {
  if (deps.size() != 1 || deps[0]->results_schema.columns.size() != 2 ||
      deps[0]->results_schema.columns[1].type != Type::VID)
    throw Error(VS_ERR_ARG, "MatrixRowOrSum takes one two-column matrix whose columns are vertices");
  results_schema = TableSchema{{deps[0]->results_schema.columns[1]}};
}

void MatrixRowOrSum::run_internal() {
  auto *m = dep_results[0]->down_to_matrix_table();
  if (!m) throw Error(VS_ERR_ARG, "MatrixRowOrSum needs a matrix input");
  vs_flat *f = nullptr;
  check(vs_matrix_row_or_sum(m->h, &f, stream));
  results = std::make_shared<FlatTable>(results_schema, f);
}

template <size_t N>
SemiJoin<N>::SemiJoin(std::array<VariableName, N> keys, bool only_count)
    : key_variables(std::move(keys)), only_count(only_count) {}

// SemiJoin<N>::finishAddingDependency (semi_join.cpp:22-56): both inputs hold
// every key with the same type; the result keeps the left input's schema.
template <size_t N> void SemiJoin<N>::finishAddingDependency() {
  if (deps.size() != 2) throw Error(VS_ERR_ARG, "SemiJoin takes two dependencies");
  for (const auto &k : key_variables) {
    auto x = deps[0]->results_schema.get_schema(k), y = deps[1]->results_schema.get_schema(k);
    if (!x || !y) throw Error(VS_ERR_ARG, "SemiJoin key " + k + " is missing from an input");
    if (!(x->first == y->first)) throw Error(VS_ERR_ARG, "SemiJoin key " + k + " differs between the inputs");
  }
  results_schema = only_count ? TableSchema{{{"count", Type::Int64}}} : deps[0]->results_schema;
}

template <size_t N> void SemiJoin<N>::run_internal() {
  vs_table_ref ra{}, rb{};
  uint32_t ak[N], bk[N];
  for (size_t i = 0; i < N; i++) {
    ak[i] = (uint32_t)dep_results[0]->schema.get_schema(key_variables[i])->second;
    bk[i] = (uint32_t)dep_results[1]->schema.get_schema(key_variables[i])->second;
  }
  for (auto [r, t] : {std::pair<vs_table_ref *, const std::shared_ptr<Table> *>{&ra, &dep_results[0]},
                      {&rb, &dep_results[1]}}) {
    if (auto *f = (*t)->down_to_flat_table())
      r->flat = f->h;
    else
      r->mat = (*t)->down_to_matrix_table()->h;
  }
  vs_flat *of = nullptr;
  vs_bitmat *om = nullptr;
  uint64_t count = 0;
  check(vs_semi_join(ra, rb, (uint32_t)N, ak, bk, only_count ? 1 : 0, &of, &om, &count, stream));
  if (only_count) {
    results = count_table((int64_t)count);
  } else if (of) {
    results = std::make_shared<FlatTable>(results_schema, of);
  } else {
    auto t = std::make_shared<VarRowMatrixTable>(results_schema);
    t->set_matrix(om);
    results = t;
  }
}

template class SemiJoin<1>;
template class SemiJoin<2>;

TableConvert::TableConvert(TableType type, bool transpose) : convert_to(type), transpose(transpose) {}

void TableConvert::finishAddingDependency() {
  results_schema = deps[0]->results_schema;
  if (transpose) {
    if (results_schema.columns.size() != 2) throw Error(VS_ERR_ARG, "transpose needs two columns");
    std::swap(results_schema.columns[0], results_schema.columns[1]);
  }
}

void TableConvert::run_internal() {
  auto *m = dep_results[0]->down_to_matrix_table();
  if (convert_to == TableType::ColMainMatrix && dep_results[0]->type == TableType::VarRowMatrix) {
    vs_bitmat *r = nullptr;
    check(vs_table_convert(m->h, transpose ? 1 : 0, &r, stream));
    auto t = std::make_shared<ColMainMatrixTable>(results_schema);
    t->set_matrix(r);
    results = t;
  } else if (convert_to == TableType::Flat && m) {
    vs_flat *f = nullptr;
    check(vs_bitmat_to_flat(m->h, &f, stream));
    results = std::make_shared<FlatTable>(results_schema, f);
  } else {
    throw Error(VS_ERR_UNSUPPORTED, "TableConvert combination not supported");  // big_operators2.cpp:80-84
  }
}

Projection::Projection(MapPairs m) : projection_map(std::move(m)) {}

void Projection::finishAddingDependency() {
  results_schema = TableSchema{};
  old_variable_idx.clear();
  for (auto &[a, b] : projection_map) {
    auto s = deps[0]->results_schema.get_schema(a);
    if (!s) throw Error(VS_ERR_ARG, "variable " + a + " not found");
    ValueSchema vs = s->first;
    vs.name = b;
    results_schema.columns.push_back(vs);
    old_variable_idx.push_back(s->second);
  }
}

void Projection::run_internal() {
  if (auto *f = dep_results[0]->down_to_flat_table()) {
    auto t = std::make_shared<FlatTable>(results_schema);
    std::vector<std::vector<uint64_t>> cols;
    for (size_t i : old_variable_idx) cols.push_back(f->column(i));
    t->set_columns(cols);
    results = t;
  } else {
    dep_results[0]->schema = results_schema;  // matrices are renamed in place (big_operators2.cpp:120-130)
    results = dep_results[0];
  }
}

MatrixTableSelect::MatrixTableSelect(VariableName k) : key_name(std::move(k)) {}

void MatrixTableSelect::finishAddingDependency() {
  if (deps.size() != 2) throw Error(VS_ERR_ARG, "MatrixTableSelect takes two dependencies");
  results_schema = deps[0]->results_schema;
  auto k0 = deps[0]->results_schema.get_schema(key_name), k1 = deps[1]->results_schema.get_schema(key_name);
  if (!k0 || !k1 || !(k0->first == k1->first) || k0->second != 1)
    throw Error(VS_ERR_ARG, "select key must be the matrix column variable");
}

void MatrixTableSelect::run_internal() {
  if (dep_results[0]->type != TableType::VarRowMatrix)
    throw Error(VS_ERR_UNSUPPORTED, "MatrixTableSelect on a ColMain matrix");  // big_operators2.cpp:204-208
  auto targets = flat_vid_column(dep_results[1], key_name);
  vs_bitmat *r = nullptr;
  check(vs_matrix_select(dep_results[0]->down_to_matrix_table()->h, targets.data(),
                         (uint32_t)targets.size(), &r, stream));
  auto t = std::make_shared<VarRowMatrixTable>(results_schema);
  t->set_matrix(r);
  results = t;
}

// MatrixTableFilter<F>::finishAddingDependency / run_internal
// (big_operators2.hh:142-170): one dependency, the same schema, the input
// table filtered in place.
MatrixTableFilter::MatrixTableFilter(MatrixFilter f) : f(std::move(f)) {}

void MatrixTableFilter::finishAddingDependency() {
  if (deps.size() != 1) throw Error(VS_ERR_ARG, "MatrixTableFilter takes one dependency");
  results_schema = deps[0]->results_schema;
}

void MatrixTableFilter::run_internal() {
  results = dep_results[0];
  std::vector<uint64_t> keys;
  for (const auto &p : f.pairs) keys.push_back((uint64_t)p.first << 32 | p.second);
  std::sort(keys.begin(), keys.end());
  auto apply = [&](MatrixTable *m) {
    check(vs_matrix_filter(m->h, f.row_keep.empty() ? nullptr : f.row_keep.data(), f.row_values,
                           f.col_keep.empty() ? nullptr : f.col_keep.data(), f.col_values,
                           keys.empty() ? nullptr : keys.data(), keys.size(), f.pairs_mode, stream));
  };
  if (auto *mm = dynamic_cast<MultipleMatrixTable *>(results.get())) {
    for (auto &m : mm->mats) apply(m.get());
    return;
  }
  auto *m = results->down_to_matrix_table();
  if (!m) throw Error(VS_ERR_ARG, "MatrixTableFilter needs a matrix table");  // big_operators2.hh:147
  apply(m);
}

std::vector<uint64_t> MatrixFilter::any_neighbor(Graph &g, const std::string &edge_key,
                                                 const std::vector<uint8_t> &prop, uint8_t value) {
  auto it = g.edges.find(edge_key);
  if (it == g.edges.end()) throw Error(VS_ERR_ARG, "no edge type " + edge_key);
  uint32_t V = 0;
  uint64_t E = 0;
  int directed = 0;
  check(vs_graph_info(it->second.g, &V, &E, &directed));
  std::vector<uint64_t> mask(((size_t)V + 63) / 64);
  check(vs_vertex_mask_any_neighbor(it->second.g, VS_DIR_FORWARD, prop.data(), (uint32_t)prop.size(), value,
                                    mask.data(), BigOperator::stream));
  return mask;
}

int64_t single_count(Table *t) {
  auto *f = t->down_to_flat_table();
  if (!f || f->tuple_count() != 1) throw Error(VS_ERR_ARG, "not a count table");
  return (int64_t)f->column(0)[0];
}

}  // namespace vsgb
