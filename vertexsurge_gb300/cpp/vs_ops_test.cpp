// Operator-level tests through the C++ operator API on the GPU, restating the
// reference's own unit tests:
//   HashJoin{FlatFlat,FlatMat,MatFlat,MatMat}[CountOnly] == 18   (join.cpp:451-920)
//   Mintersect{FlatFlatFlat,FlatMatMat} == 3                     (mintersect.cpp:347-511)
//   TableConvertVRtoCM / _T exactness                            (big_operators2.cpp:215-296)
// and plan shapes of the query drivers (e1-self-ring, p3-tri3-1, p4-exp4-1,
// tcr1's expand + MatrixTableFilter) on a small generated graph, checked
// against host-side breadth-first search.
// Exit status 0 = every test passed.
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <map>
#include <queue>
#include <random>
#include <set>
#include <vector>

#include "../cpp/vql.hh"
#include "../cpp/vs_operators.hh"

using namespace vsgb;
using std::make_shared;
using std::shared_ptr;
using std::vector;

static int g_fail = 0, g_pass = 0;
#define EXPECT_EQ(a, b)                                                                    \
  do {                                                                                     \
    auto _a = (a);                                                                         \
    auto _b = (b);                                                                         \
    if (!(_a == _b)) {                                                                     \
      std::fprintf(stderr, "  %s:%d: %s != %s (%lld vs %lld)\n", __FILE__, __LINE__, #a, #b, \
                   (long long)_a, (long long)_b);                                          \
      ok = false;                                                                          \
    }                                                                                      \
  } while (0)

static void run_test(const char *name, const std::function<bool()> &f) {
  bool ok = false;
  try {
    ok = f();
  } catch (const std::exception &e) {
    std::fprintf(stderr, "  exception: %s\n", e.what());
    ok = false;
  }
  std::printf("[%s] %s\n", ok ? "PASS" : "FAIL", name);
  (ok ? g_pass : g_fail)++;
}

static const vector<uint64_t> A8 = {1, 2, 3, 4, 5, 6, 7, 8};
static const vector<uint64_t> K8 = {1, 1, 1, 2, 2, 3, 3, 4};

static shared_ptr<BigOperator> inlined_flat(TableSchema s, vector<vector<uint64_t>> cols) {
  auto d = make_shared<InlinedData>();
  d->results_schema = s;
  auto t = make_shared<FlatTable>(s);
  t->set_columns(cols);
  d->results = t;
  return d;
}

// ColMain (rows x cols): set(row_vals[i], k_map[keys[i]]), col_map = distinct keys
// (extra columns get keys that match nothing).
static shared_ptr<BigOperator> inlined_colmain(TableSchema s, size_t rows, size_t cols,
                                               const vector<uint64_t> &row_vals,
                                               const vector<uint64_t> &keys) {
  std::map<uint64_t, size_t> k_map;
  vector<uint32_t> k_mapv;
  for (auto k : keys)
    if (!k_map.count(k)) {
      k_map[k] = k_map.size();
      k_mapv.push_back((uint32_t)k);
    }
  for (size_t i = k_mapv.size(); i < cols; i++) k_mapv.push_back(1000 + (uint32_t)i);
  const size_t wpc = (rows + 63) / 64;
  vector<uint64_t> w(wpc * cols, 0);
  for (size_t i = 0; i < row_vals.size(); i++) {
    size_t r = row_vals[i], c = k_map[keys[i]];
    w[c * wpc + r / 64] |= 1ull << (r % 64);
  }
  vs_bitmat *m = nullptr;
  check(vs_bitmat_create((uint32_t)rows, (uint32_t)cols, VS_KIND_COLMAIN, nullptr, &m));
  check(vs_bitmat_upload(m, w.data(), nullptr));
  check(vs_bitmat_set_maps(m, nullptr, k_mapv.data(), nullptr));
  auto d = make_shared<InlinedData>();
  d->results_schema = s;
  auto t = make_shared<ColMainMatrixTable>(s);
  t->set_matrix(m);
  d->results = t;
  return d;
}

static bool join_case(bool a_mat, bool b_mat, size_t ncols_b, bool only_count, Type key_type) {
  bool ok = true;
  auto op = make_shared<HashJoin>("k", only_count);
  if (a_mat)
    op->addDependency(inlined_colmain({{{"a", Type::VID}, {"k", Type::VID}}}, 10, 4, A8, K8));
  else
    op->addDependency(inlined_flat({{{"a", Type::VID}, {"k", key_type}}}, {A8, K8}));
  if (b_mat)
    op->addDependency(inlined_colmain({{{"b", Type::VID}, {"k", Type::VID}}}, 10, ncols_b, A8, K8));
  else
    op->addDependency(inlined_flat({{{"b", Type::VID}, {"k", key_type}}}, {A8, K8}));
  op->finishAddingDependency();
  op->run();
  if (only_count) {
    EXPECT_EQ(op->results->tuple_count(), (size_t)1);
    EXPECT_EQ(single_count(op->results.get()), (int64_t)18);
  } else {
    EXPECT_EQ(op->results->tuple_count(), (size_t)18);
    EXPECT_EQ(op->results_schema.columns.size(), (size_t)3);
    // every tuple joins equal keys: (a, k, b) with K8[a-1] == k == K8[b-1]
    auto *f = op->results->down_to_flat_table();
    auto ca = f->column(0), ck = f->column(1), cb = f->column(2);
    std::multiset<std::tuple<uint64_t, uint64_t, uint64_t>> got, exp;
    for (size_t i = 0; i < ca.size(); i++) got.insert({ca[i], ck[i], cb[i]});
    for (size_t i = 0; i < 8; i++)
      for (size_t j = 0; j < 8; j++)
        if (K8[i] == K8[j]) exp.insert({A8[i], K8[i], A8[j]});
    EXPECT_EQ(got == exp, true);
  }
  return ok;
}

static bool mintersect_case(bool mats, bool only_count) {
  bool ok = true;
  auto op = make_shared<Mintersect>("c", "Person", only_count);
  op->addDependency(inlined_flat({{{"a", Type::VID}, {"b", Type::VID}}}, {A8, K8}));
  if (!mats) {
    op->addDependency(inlined_flat({{{"a", Type::VID}, {"c", Type::VID}}}, {A8, K8}));
    op->addDependency(inlined_flat({{{"b", Type::VID}, {"c", Type::VID}}}, {A8, K8}));
  } else {
    op->addDependency(inlined_colmain({{{"c", Type::VID}, {"a", Type::VID}}}, 10, 10, K8, A8));
    op->addDependency(inlined_colmain({{{"c", Type::VID}, {"b", Type::VID}}}, 10, 10, K8, A8));
  }
  op->finishAddingDependency();
  op->run();
  if (only_count)
    EXPECT_EQ(single_count(op->results.get()), (int64_t)3);
  else
    EXPECT_EQ(op->results->tuple_count(), (size_t)3);
  return ok;
}

static bool table_convert_case(bool transpose) {
  bool ok = true;
  std::mt19937 gen(123);
  const size_t rows = 1000, cols = 10000, wpc = (rows + 63) / 64;
  vector<uint64_t> w(wpc * cols);
  for (auto &x : w) x = ((uint64_t)gen() << 32) | gen();
  for (size_t c = 0; c < cols; c++) w[c * wpc + wpc - 1] &= (1ull << (rows % 64)) - 1;
  vs_bitmat *m = nullptr;
  check(vs_bitmat_create(rows, cols, VS_KIND_VARROW, nullptr, &m));
  check(vs_bitmat_upload(m, w.data(), nullptr));
  auto d = make_shared<InlinedData>();
  d->results_schema = {{{"b", Type::VID}, {"k", Type::VID}}};
  auto t = make_shared<VarRowMatrixTable>(d->results_schema);
  t->set_matrix(m);
  d->results = t;
  auto op = make_shared<TableConvert>(TableType::ColMainMatrix, transpose);
  op->addLastDependency(d);
  op->run();
  auto *r = op->results->down_to_matrix_table();
  auto rw = r->logical_words();
  const size_t rwpc = ((transpose ? cols : rows) + 63) / 64;
  size_t bad = 0;
  for (size_t i = 0; i < rows; i++)
    for (size_t j = 0; j < cols; j++) {
      bool a = (w[j * wpc + i / 64] >> (i % 64)) & 1;
      bool b = transpose ? (rw[i * rwpc + j / 64] >> (j % 64)) & 1 : (rw[j * rwpc + i / 64] >> (i % 64)) & 1;
      bad += a != b;
    }
  EXPECT_EQ(bad, (size_t)0);
  EXPECT_EQ(op->results_schema.columns[0].name == std::string(transpose ? "k" : "b"), true);
  return ok;
}

// A small undirected graph (R-MAT style, generated here) and host BFS.
struct HostGraph {
  uint32_t V;
  vector<int64_t> off;
  vector<uint32_t> adj;
};

static HostGraph small_graph() {
  std::mt19937_64 gen(7);
  const uint32_t V = 1500;
  std::set<std::pair<uint32_t, uint32_t>> es;
  for (int i = 0; i < 6000; i++) {
    uint32_t u = gen() % V, v = (uint32_t)((gen() % V) * (gen() % 3 == 0 ? 1 : 0) + (gen() % 40));
    v %= V;
    if (u == v) continue;
    es.insert({u, v});
    es.insert({v, u});
  }
  HostGraph g{V, vector<int64_t>(V + 1, 0), {}};
  for (auto [u, v] : es) g.off[u + 1]++;
  for (uint32_t i = 0; i < V; i++) g.off[i + 1] += g.off[i];
  for (auto [u, v] : es) g.adj.push_back(v);
  return g;
}

static vector<int> bfs(const HostGraph &g, uint32_t s) {
  vector<int> d(g.V, -1);
  std::queue<uint32_t> q;
  d[s] = 0;
  q.push(s);
  while (!q.empty()) {
    uint32_t u = q.front();
    q.pop();
    for (int64_t j = g.off[u]; j < g.off[u + 1]; j++)
      if (d[g.adj[j]] < 0) {
        d[g.adj[j]] = d[u] + 1;
        q.push(g.adj[j]);
      }
  }
  return d;
}

static shared_ptr<BigOperator> ids(const std::string &name, const vector<uint64_t> &v) {
  return inlined_flat({{{name, Type::VID}}}, {v});
}

static bool plans_case(const HostGraph &hg) {
  bool ok = true;
  vector<uint64_t> sa, sb, sc;
  for (uint64_t i = 0; i < 120; i++) sa.push_back((i * 37) % hg.V);
  for (uint64_t i = 0; i < 90; i++) sb.push_back((i * 53 + 5) % hg.V);
  for (uint64_t i = 0; i < 100; i++) sc.push_back((i * 71 + 11) % hg.V);
  auto A = ids("a.id", sa), B = ids("b.id", sb), Cn = ids("c.id", sc);
  auto vexp = [&](shared_ptr<BigOperator> s, shared_ptr<BigOperator> t, std::string sn, std::string tn, size_t k0,
                  size_t k1) {
    auto ve = make_shared<VExpand>("Person", "Person", "knows", Direction::Both, k0, k1, ExpandPathType::Shortest,
                                   ExpandStrategy::Dense, sn, tn);
    ve->addLastDependency(s);
    auto sel = make_shared<MatrixTableSelect>(tn);
    sel->addDependency(ve);
    sel->addLastDependency(t);
    return sel;
  };
  vector<vector<int>> da, db;
  for (auto s : sa) da.push_back(bfs(hg, (uint32_t)s));
  for (auto s : sb) db.push_back(bfs(hg, (uint32_t)s));
  auto within = [](int d, int k0, int k1) { return d >= k0 && d <= k1; };
  // e1-self-ring: Count(Select(VExpand(a, [0,3]), targets = a))
  {
    auto B2 = ids("b.id", sa);
    auto cnt = make_shared<Count>();
    cnt->addLastDependency(vexp(A, B2, "a.id", "b.id", 0, 3));
    cnt->run();
    int64_t exp = 0;
    for (size_t i = 0; i < sa.size(); i++)
      for (size_t j = 0; j < sa.size(); j++) exp += within(da[i][sa[j]], 0, 3);
    EXPECT_EQ(single_count(cnt->results.get()), exp);
  }
  // p3-tri3-1: Mintersect(p12, T(p13), T(p23)) with hops [1,2]
  {
    auto p12 = vexp(A, B, "a.id", "b.id", 1, 2), p13 = vexp(A, Cn, "a.id", "c.id", 1, 2),
         p23 = vexp(B, Cn, "b.id", "c.id", 1, 2);
    auto t13 = make_shared<TableConvert>(TableType::ColMainMatrix, true);
    t13->addLastDependency(p13);
    auto t23 = make_shared<TableConvert>(TableType::ColMainMatrix, true);
    t23->addLastDependency(p23);
    auto mi = make_shared<Mintersect>("c.id", "Person", true);
    mi->addDependency(p12);
    mi->addDependency(t13);
    mi->addLastDependency(t23);
    mi->run();
    int64_t exp = 0;
    for (size_t i = 0; i < sa.size(); i++)
      for (size_t j = 0; j < sb.size(); j++) {
        if (!within(da[i][sb[j]], 1, 2)) continue;
        for (size_t k = 0; k < sc.size(); k++) exp += within(da[i][sc[k]], 1, 2) && within(db[j][sc[k]], 1, 2);
      }
    EXPECT_EQ(single_count(mi->results.get()), exp);
  }
  // p4-exp4-1 first join: HashJoin("b.id") over ColMain(p12) and ColMain^T(p23)
  {
    auto p12 = vexp(A, B, "a.id", "b.id", 1, 2), p23 = vexp(B, Cn, "b.id", "c.id", 1, 2);
    auto c12 = make_shared<TableConvert>(TableType::ColMainMatrix, false);
    c12->addLastDependency(p12);
    auto c23 = make_shared<TableConvert>(TableType::ColMainMatrix, true);
    c23->addLastDependency(p23);
    for (bool oc : {true, false}) {
      auto j = make_shared<HashJoin>("b.id", oc);
      j->addDependency(c12);
      j->addLastDependency(c23);
      j->run();
      int64_t exp = 0;
      for (size_t i = 0; i < sa.size(); i++)
        for (size_t jj = 0; jj < sb.size(); jj++) {
          if (!within(da[i][sb[jj]], 1, 2)) continue;
          for (size_t k = 0; k < sc.size(); k++) exp += within(db[jj][sc[k]], 1, 2);
        }
      if (oc)
        EXPECT_EQ(single_count(j->results.get()), exp);
      else
        EXPECT_EQ((int64_t)j->results->tuple_count(), exp);
    }
  }
  // p3-tri3-2: HashJoin("b.id") of ColMain(p12) and ColMain^T(p23), then
  // SemiJoin<2>({"a.id", "c.id"}) with p13: the triangles again
  {
    auto p12 = vexp(A, B, "a.id", "b.id", 1, 2), p13 = vexp(A, Cn, "a.id", "c.id", 1, 2),
         p23 = vexp(B, Cn, "b.id", "c.id", 1, 2);
    auto c12 = make_shared<TableConvert>(TableType::ColMainMatrix, false);
    c12->addLastDependency(p12);
    auto c32 = make_shared<TableConvert>(TableType::ColMainMatrix, true);
    c32->addLastDependency(p23);
    auto p123 = make_shared<HashJoin>("b.id", false);
    p123->addDependency(c12);
    p123->addLastDependency(c32);
    int64_t exp = 0;
    for (size_t i = 0; i < sa.size(); i++)
      for (size_t j = 0; j < sb.size(); j++) {
        if (!within(da[i][sb[j]], 1, 2)) continue;
        for (size_t k = 0; k < sc.size(); k++) exp += within(da[i][sc[k]], 1, 2) && within(db[j][sc[k]], 1, 2);
      }
    for (bool oc : {true, false}) {
      auto t123 = make_shared<SemiJoin<2>>(std::array<VariableName, 2>{"a.id", "c.id"}, oc);
      t123->addDependency(p123);
      t123->addLastDependency(p13);
      t123->run();
      if (oc)
        EXPECT_EQ(single_count(t123->results.get()), exp);
      else
        EXPECT_EQ((int64_t)t123->results->tuple_count(), exp);
    }
  }
  // MatrixColumnCount and MatrixRowOrSum over p12: per b, the a's within [1,2]
  {
    auto p12 = vexp(A, B, "a.id", "b.id", 1, 2);
    auto mcc = make_shared<MatrixColumnCount>("b.id", SortOrder::DESC);
    mcc->addLastDependency(p12);
    mcc->run();
    auto ids = mcc->results->down_to_flat_table()->column(0), cnt = mcc->results->down_to_flat_table()->column(1);
    EXPECT_EQ(ids.size(), sb.size());
    bool sorted = true, right = true;
    for (size_t i = 0; i < ids.size(); i++) {
      if (i && cnt[i] > cnt[i - 1]) sorted = false;
      int64_t e = 0;
      for (size_t a = 0; a < sa.size(); a++) e += within(da[a][ids[i]], 1, 2);
      if ((int64_t)cnt[i] != e) right = false;
    }
    EXPECT_EQ(sorted, true);
    EXPECT_EQ(right, true);
    auto ros = make_shared<MatrixRowOrSum>();
    ros->addLastDependency(p12);
    ros->run();
    size_t nz = 0;
    for (size_t i = 0; i < ids.size(); i++) nz += cnt[i] != 0;
    EXPECT_EQ(ros->results->tuple_count(), nz);
  }
  // VExpand with_distance (Dense): one matrix per distance; as tuples, every
  // (a, v) at distance 1..3 once with that distance
  {
    auto ve = make_shared<VExpand>("Person", "Person", "knows", Direction::Both, 1, 3,
                                   VExpandPathParameters::Shortest().set_with_distance(), ExpandStrategy::Dense,
                                   "a.id", std::optional<VariableName>("b.id"));
    ve->addLastDependency(A);
    ve->run();
    auto *multi = dynamic_cast<MultipleMatrixTable *>(ve->results.get());
    EXPECT_EQ(multi != nullptr, true);
    int64_t exp = 0;
    for (size_t i = 0; i < sa.size(); i++)
      for (size_t v = 0; v < hg.V; v++) exp += within(da[i][v], 1, 3);
    EXPECT_EQ((int64_t)multi->tuple_count(), exp);
    auto flat = multi->output_to_flat();
    auto r = flat->column(0), c = flat->column(1), d = flat->column(2);
    std::map<uint64_t, size_t> row_of;
    for (size_t i = 0; i < sa.size(); i++) row_of.emplace(sa[i], i);
    size_t bad = 0;
    for (size_t t = 0; t < r.size(); t++) bad += (int64_t)d[t] != (int64_t)da[row_of.at(r[t])][c[t]];
    EXPECT_EQ((int64_t)r.size(), exp);
    EXPECT_EQ(bad, (size_t)0);
  }
  // VExpand with_distance, CSR strategy, Any: each (a, v) pair once, at the
  // smallest walk length in 1..3 (merge_to_Flat, vexpand.cpp:383-405): as many
  // tuples as the Any [1,3] union has bits, each distance in [max(1, BFS distance), 3]
  {
    auto ve = make_shared<VExpand>("Person", "Person", "knows", Direction::Both, 1, 3,
                                   VExpandPathParameters::Any().set_with_distance(), ExpandStrategy::CSR,
                                   "a.id", std::optional<VariableName>("b.id"));
    ve->addLastDependency(A);
    ve->run();
    auto u = make_shared<VExpand>("Person", "Person", "knows", Direction::Both, 1, 3, ExpandPathType::Any,
                                  ExpandStrategy::Dense, "a.id", std::optional<VariableName>("b.id"));
    u->addLastDependency(A);
    u->run();
    auto *flat = ve->results->down_to_flat_table();
    EXPECT_EQ(flat != nullptr, true);
    EXPECT_EQ(ve->results->tuple_count(), u->results->tuple_count());
    auto r = flat->column(0), c = flat->column(1), d = flat->column(2);
    std::map<uint64_t, size_t> row_of;
    for (size_t i = 0; i < sa.size(); i++) row_of.emplace(sa[i], i);
    size_t bad = 0;
    std::set<std::pair<uint64_t, uint64_t>> pairs;
    for (size_t t = 0; t < r.size(); t++) {
      const int64_t dd = (int64_t)d[t], bfs = da[row_of.at(r[t])][c[t]];
      bad += dd < 1 || dd > 3 || bfs < 0 || dd < bfs;
      pairs.emplace(r[t], c[t]);
    }
    EXPECT_EQ(bad, (size_t)0);
    EXPECT_EQ(pairs.size(), r.size());
  }
  // FindShortest over (start, target) pairs
  {
    vector<uint64_t> tg;
    for (size_t i = 0; i < sa.size(); i++) tg.push_back(sb[i % sb.size()]);
    auto data = inlined_flat({{{"a.id", Type::VID}, {"b.id", Type::VID}}}, {sa, tg});
    auto fs = make_shared<VExpand>("Person", "Person", "knows", Direction::Both, VExpandPathParameters::FindShortest(),
                                   ExpandStrategy::Dense, "a.id", "b.id");
    fs->addLastDependency(data);
    fs->run();
    auto dist = fs->results->down_to_flat_table()->column(2);
    size_t bad = 0;
    for (size_t i = 0; i < sa.size(); i++) bad += (int64_t)dist[i] != (int64_t)da[i][tg[i]];
    EXPECT_EQ(bad, (size_t)0);
  }
  return ok;
}

// tcr1 plan shape (ldbc-finbench/tcr1.cpp:41-60): VExpand(Shortest, with
// distances, [1,3]) then MatrixTableFilter keeping the persons signed in to a
// blocked medium (a signIn edge type to mediums numbered after the persons)
static bool filter_case(Graph &g, const HostGraph &hg) {
  bool ok = true;
  const uint32_t nm = 400, VT = hg.V + nm;
  std::mt19937_64 gen(11);
  vector<std::set<uint32_t>> out(VT);
  for (uint32_t i = 0; i < 3 * hg.V; i++) out[gen() % hg.V].insert(hg.V + (uint32_t)(gen() % nm));
  vector<int64_t> off(VT + 1, 0), roff(VT + 1, 0);
  vector<uint32_t> adj, radj;
  vector<vector<uint32_t>> in(VT);
  for (uint32_t u = 0; u < VT; u++) {
    for (uint32_t v : out[u]) {
      adj.push_back(v);
      in[v].push_back(u);
    }
    off[u + 1] = (int64_t)adj.size();
  }
  for (uint32_t v = 0; v < VT; v++) {
    for (uint32_t u : in[v]) radj.push_back(u);
    roff[v + 1] = (int64_t)radj.size();
  }
  g.add_edge_type("Person", "signIn", "Medium", true, VT, adj.size(), off.data(), adj.data(), roff.data(),
                  radj.data());
  vector<uint8_t> blocked(VT, 0);
  for (uint32_t m = hg.V; m < VT; m++) blocked[m] = gen() % 10 == 0;
  MatrixFilter f;
  f.col_keep = MatrixFilter::any_neighbor(g, "Person_signIn_Medium", blocked, 1);
  f.col_values = hg.V;
  auto keeps = [&](uint32_t v) {
    for (uint32_t m : out[v])
      if (blocked[m]) return true;
    return false;
  };
  size_t bad_mask = 0;
  for (uint32_t v = 0; v < hg.V; v++) bad_mask += ((f.col_keep[v >> 6] >> (v & 63)) & 1) != (uint64_t)keeps(v);
  EXPECT_EQ(bad_mask, (size_t)0);
  vector<uint64_t> sa;
  for (uint64_t i = 0; i < 100; i++) sa.push_back((i * 29 + 3) % hg.V);
  auto ve = make_shared<VExpand>("Person", "Person", "knows", Direction::Both, 1, 3,
                                 VExpandPathParameters::Shortest().set_with_distance(), ExpandStrategy::Dense, "a.id",
                                 std::optional<VariableName>("b.id"));
  ve->addLastDependency(ids("a.id", sa));
  auto flt = make_shared<MatrixTableFilter>(f);
  flt->addLastDependency(ve);
  flt->run();
  auto *multi = dynamic_cast<MultipleMatrixTable *>(flt->results.get());
  EXPECT_EQ(multi != nullptr, true);
  int64_t exp = 0;
  for (auto s : sa) {
    auto d = bfs(hg, (uint32_t)s);
    for (uint32_t v = 0; v < hg.V; v++) exp += d[v] >= 1 && d[v] <= 3 && keeps(v);
  }
  EXPECT_EQ((int64_t)multi->tuple_count(), exp);
  return ok;
}

// Reads a graph directory in the reference's layout through Graph(dir).load()
// and prints Count(VExpand(sources i*7 mod V for i < 100, Forward, Shortest,
// [1,3])) over its first self edge type.
static int graph_dir_count(const char *dir) {
  Graph g{std::filesystem::path(dir)};
  g.load();
  if (g.edges.empty()) throw Error(VS_ERR_ARG, "no self edge type in the graph directory");
  const Graph::EdgeType &et = g.edges.begin()->second;
  const uint64_t V = g.vertex_count.at(et.src);
  vector<uint64_t> s;
  for (uint64_t i = 0; i < std::min<uint64_t>(V, 100); i++) s.push_back((i * 7) % V);
  auto ve = make_shared<VExpand>(et.src, et.dst, et.name, Direction::Forward, 1, 3, ExpandPathType::Shortest,
                                 ExpandStrategy::Dense, "a.id", "b.id");
  ve->addLastDependency(ids("a.id", s));
  auto cnt = make_shared<Count>();
  cnt->addLastDependency(ve);
  cnt->run();
  std::printf("count %lld\n", (long long)single_count(cnt->results.get()));
  return 0;
}

// Runs a VQL query over a graph directory: prints "count N" (count of) or
// "rows N" and the rows as "r: v0 v1 ...".
static int vql_run(const char *dir, const char *text) {
  Graph g{std::filesystem::path(dir)};
  g.load();
  query::Builder b(text);
  b.parse();
  auto root = b.build(b.variable_apperance_order());
  root->run();
  if (b.only_count) {  // a two-vertex query ends at its expand: count its pairs
    auto *ft = root->results->down_to_flat_table();
    const bool count_table = ft && ft->schema.columns.size() == 1 && ft->schema.columns[0].name == "count";
    std::printf("count %lld\n", count_table ? (long long)single_count(root->results.get())
                                            : (long long)root->results->tuple_count());
    return 0;
  }
  auto *f = root->results->down_to_flat_table();
  std::vector<std::vector<uint64_t>> cols;
  if (f) {
    for (size_t c = 0; c < f->schema.columns.size(); c++) cols.push_back(f->column(c));
  } else {  // a matrix: its (row value, column value) pairs
    vs_flat *fl = nullptr;
    check(vs_bitmat_to_flat(root->results->down_to_matrix_table()->h, &fl, nullptr));
    FlatTable t(TableSchema{{{"r", Type::VID}, {"c", Type::VID}}}, fl);
    cols = {t.column(0), t.column(1)};
  }
  const size_t n = cols.empty() ? 0 : cols[0].size();
  std::printf("rows %zu\n", n);
  for (size_t r = 0; r < n; r++) {
    std::printf("r:");
    for (auto &c : cols) std::printf(" %llu", (unsigned long long)c[r]);
    std::printf("\n");
  }
  return 0;
}

int main(int argc, char **argv) {
  check(vs_init(0));
  if (argc >= 3 && std::string(argv[1]) == "--graph-dir") return graph_dir_count(argv[2]);
  if (argc >= 4 && std::string(argv[1]) == "--vql") return vql_run(argv[2], argv[3]);
  // like the reference's tests, load a graph first: operators resolve vertex types against it
  HostGraph hg = small_graph();
  Graph g;
  g.add_vertex_type("Person", hg.V);
  g.add_edge_type("Person", "knows", "Person", false, hg.V, hg.adj.size(), hg.off.data(), hg.adj.data(),
                  hg.off.data(), hg.adj.data());
  g.load();
  for (bool oc : {false, true}) {
    std::string s = oc ? "CountOnly" : "";
    run_test(("HashJoinFlatFlat" + s).c_str(), [=] { return join_case(false, false, 0, oc, Type::Int64); });
    run_test(("HashJoinFlatMat" + s).c_str(), [=] { return join_case(false, true, 4, oc, Type::VID); });
    run_test(("HashJoinMatFlat" + s).c_str(), [=] { return join_case(false, true, 10, oc, Type::VID); });
    run_test(("HashJoinMatMat" + s).c_str(), [=] { return join_case(true, true, 4, oc, Type::VID); });
    run_test(("MintersectFlatFlatFlat" + s).c_str(), [=] { return mintersect_case(false, oc); });
    run_test(("MintersectFlatMatMat" + s).c_str(), [=] { return mintersect_case(true, oc); });
  }
  run_test("TableConvertVRtoCM", [] { return table_convert_case(false); });
  run_test("TableConvertVRtoCM_T", [] { return table_convert_case(true); });
  run_test("PlanShapes(e1,p3-tri3-1,p3-tri3-2,p4-exp4-1,consumers,FindShortest)", [&] { return plans_case(hg); });
  run_test("MatrixTableFilter(tcr1)", [&] { return filter_case(g, hg); });
  std::printf("%d passed, %d failed\n", g_pass, g_fail);
  return g_fail ? 1 : 0;
}
