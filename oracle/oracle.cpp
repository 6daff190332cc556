// ORACLE — test infrastructure only (see oracle.h for scope and citations).
//
// CPU restatement of VertexSurge's operators following the reference's scalar
// branches.  Every function names the reference lines it restates.
#include "oracle.h"

#include <omp.h>

#include <algorithm>
#include <array>
#include <bit>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <set>
#include <unordered_map>
#include <vector>

namespace {

int g_threads = 0;

inline int nthreads() { return g_threads > 0 ? g_threads : omp_get_max_threads(); }

inline size_t align_to(size_t x, size_t a) { return (x + a - 1) / a * a; }

// ---------------------------------------------------------------------------
// DenseVarStackMatrix restated (bitmap.hh:329-425, set_derived bitmap.cpp:910-920).
// Rows are grouped into stacks of R rows; a stack stores, for every column,
// R/64 consecutive words (column-major inside the stack).
struct StackMatrix {
  static constexpr size_t V_ALIGN = 8;  // 512-bit alignment of the reference
  size_t row_count, col_count, R, v_per_stack_col, v_per_stack, stack_count, total;
  std::vector<uint64_t> bits;

  StackMatrix(size_t rows, size_t cols, size_t stack_rows)
      : row_count(rows), col_count(cols), R(stack_rows) {
    v_per_stack_col = R / 64;
    v_per_stack = align_to(v_per_stack_col * col_count, V_ALIGN);
    stack_count = align_to(row_count, R) / R;
    total = align_to(v_per_stack * stack_count, V_ALIGN);
    bits.assign(total, 0);
  }
  // get_v_idx, bitmap.hh:350-353
  inline size_t vidx(size_t r, size_t c) const {
    return (r / R) * v_per_stack + c * v_per_stack_col + (r % R) / 64;
  }
  inline bool get(size_t r, size_t c) const { return (bits[vidx(r, c)] >> (r % 64)) & 1; }
  inline void set(size_t r, size_t c, bool to) {
    if (to)
      bits[vidx(r, c)] |= 1ULL << (r % 64);
    else
      bits[vidx(r, c)] &= ~(1ULL << (r % 64));
  }
  // or_stack_col_from scalar branch, bitmap.cpp:1206-1213
  inline void or_stack_col_from(size_t si, size_t c, const StackMatrix &o, size_t oc) {
    size_t r = si * R;
    uint64_t *p = &bits[vidx(r, c)];
    const uint64_t *q = &o.bits[o.vidx(r, oc)];
    for (size_t i = 0; i < v_per_stack_col; i++) p[i] = p[i] | q[i];
  }
  // dedup_and_update_visit_and_count scalar branch, bitmap.cpp:1078-1095
  static size_t dedup_and_update_visit_and_count(StackMatrix &vis, StackMatrix &out) {
    size_t re = 0;
    uint64_t *v = vis.bits.data(), *o = out.bits.data();
    const size_t n = vis.total;
#pragma omp parallel for reduction(+ : re) num_threads(nthreads()) schedule(static)
    for (size_t i = 0; i < n; i++) {
      uint64_t x = v[i] & o[i];
      o[i] = o[i] ^ x;
      v[i] = v[i] | o[i];
      re += std::popcount(v[i]);
    }
    return re;
  }
  // operator|= scalar branch, bitmap.cpp:995-1001
  void or_from(const StackMatrix &o) {
    uint64_t *v = bits.data();
    const uint64_t *q = o.bits.data();
#pragma omp parallel for num_threads(nthreads()) schedule(static)
    for (size_t i = 0; i < total; i++) v[i] = v[i] | q[i];
  }
  // count scalar branch, bitmap.cpp:1113-1124
  size_t count() const {
    size_t re = 0;
    const uint64_t *p = bits.data();
#pragma omp parallel for reduction(+ : re) num_threads(nthreads()) schedule(static)
    for (size_t i = 0; i < total; i++) re += std::popcount(p[i]);
    return re;
  }
  bool col_nonzero(size_t si, size_t c) const {
    const uint64_t *q = &bits[vidx(si * R, c)];
    for (size_t i = 0; i < v_per_stack_col; i++)
      if (q[i]) return true;
    return false;
  }
  void to_logical(uint64_t *out) const {
    const size_t wpc = (row_count + 63) / 64;
#pragma omp parallel for num_threads(nthreads()) schedule(static)
    for (size_t c = 0; c < col_count; c++)
      for (size_t w = 0; w < wpc; w++) out[c * wpc + w] = bits[vidx(w * 64, c)];
  }
  void from_logical(const uint64_t *in) {
    const size_t wpc = (row_count + 63) / 64;
    for (size_t c = 0; c < col_count; c++)
      for (size_t w = 0; w < wpc; w++) bits[vidx(w * 64, c)] = in[c * wpc + w];
  }
};

// DenseColMainMatrix restated (bitmap.hh:262-326, bitmap.cpp:580-609): every
// column holds v_per_col words, v_per_col aligned to 8 words.
struct ColMain {
  size_t row_count, col_count, v_per_col;
  std::vector<uint64_t> bits;
  ColMain(size_t rows, size_t cols) : row_count(rows), col_count(cols) {
    v_per_col = align_to(align_to(rows, 64) / 64, 8);
    bits.assign(v_per_col * cols, 0);
  }
  inline bool get(size_t r, size_t c) const { return (bits[c * v_per_col + r / 64] >> (r % 64)) & 1; }
  inline void set(size_t r, size_t c, bool to) {
    if (to)
      bits[c * v_per_col + r / 64] |= 1ULL << (r % 64);
    else
      bits[c * v_per_col + r / 64] &= ~(1ULL << (r % 64));
  }
  uint64_t *col(size_t c) { return &bits[c * v_per_col]; }
  const uint64_t *col(size_t c) const { return &bits[c * v_per_col]; }
  // set_col_to scalar branch, bitmap.cpp:829-841
  void set_col_to(size_t c, bool to) {
    uint64_t *p = col(c);
    for (size_t i = 0; i < v_per_col; i++) p[i] = to ? ~0ULL : 0ULL;
  }
  // and_col_from scalar branch, bitmap.cpp:874-879
  void and_col_from(size_t c, const ColMain &o, size_t oc) {
    uint64_t *p = col(c);
    const uint64_t *q = o.col(oc);
    for (size_t i = 0; i < v_per_col; i++) p[i] = p[i] & q[i];
  }
  // count_bits_in_col scalar branch, bitmap.cpp:655-666
  size_t count_bits_in_col(size_t c) const {
    size_t re = 0;
    const uint64_t *p = col(c);
    for (size_t i = 0; i < v_per_col; i++) re += std::popcount(p[i]);
    return re;
  }
  void from_logical(const uint64_t *in) {
    const size_t wpc = (row_count + 63) / 64;
    for (size_t c = 0; c < col_count; c++)
      for (size_t w = 0; w < wpc; w++) bits[c * v_per_col + w] = in[c * wpc + w];
  }
};

// ---------------------------------------------------------------------------
// Edge sets of one expand step: the lists of "base" vertices u whose column is
// OR-ed into target column v (out[v] |= base[u]).  Direction rules follow
// EdgeSchema::check_src_or_dst_for_edge_ref (schema.cpp:261-302): directed
// Forward uses src->dst, Backward uses dst->src, Both uses both; undirected
// edge types are stored both ways and use the src->dst list.
struct InLists {
  const int64_t *off[2];
  const uint32_t *adj[2];
  int n = 0;
};

InLists in_lists(const int64_t *fwd_off, const uint32_t *fwd_dst, const int64_t *rev_off,
                 const uint32_t *rev_src, int directed, int dir) {
  InLists L;
  bool use_fwd = !directed || dir == OR_FORWARD || dir == OR_BOTH;
  bool use_bwd = directed && (dir == OR_BACKWARD || dir == OR_BOTH);
  // out[v] |= base[u] for u->v means v's in-list (reverse CSR)
  if (use_fwd) {
    L.off[L.n] = rev_off;
    L.adj[L.n] = rev_src;
    L.n++;
  }
  // moving against u->v: out[u] |= base[v], i.e. u's out-list
  if (use_bwd) {
    L.off[L.n] = fwd_off;
    L.adj[L.n] = fwd_dst;
    L.n++;
  }
  return L;
}

// One dense hop over the CSR in-lists: edges are owned by their target
// column, and every stack of a target is finished before the next target.
// Same OR set as the reference's dense hop (expand.cpp:210-344); the
// reference's own loop order is expand_blocks below.
void expand_dense(const InLists &L, uint32_t V, const StackMatrix &base, StackMatrix &out) {
#pragma omp parallel for num_threads(nthreads()) schedule(dynamic, 256)
  for (size_t v = 0; v < V; v++) {
    for (size_t si = 0; si < base.stack_count; si++) {
      for (int l = 0; l < L.n; l++) {
        for (int64_t j = L.off[l][v]; j < L.off[l][v + 1]; j++) {
          out.or_stack_col_from(si, v, base, L.adj[l][j]);
        }
      }
    }
  }
}

uint64_t active_edges(const InLists &L, uint32_t V, const StackMatrix &base) {
  uint64_t n = 0;
#pragma omp parallel for reduction(+ : n) num_threads(nthreads()) schedule(dynamic, 256)
  for (size_t v = 0; v < V; v++) {
    for (int l = 0; l < L.n; l++) {
      for (int64_t j = L.off[l][v]; j < L.off[l][v + 1]; j++) {
        uint32_t u = L.adj[l][j];
        bool nz = false;
        for (size_t si = 0; si < base.stack_count && !nz; si++) nz = base.col_nonzero(si, u);
        n += nz;
      }
    }
  }
  return n;
}

// ---------------------------------------------------------------------------
// The reference's BlockHilbert edge layout and hop.
//
// Layout (graph_loader.hh:239-276): the (u, v) pairs of the expand direction
// (VIDPair: base column u is OR-ed into column v), sorted by target, cut into
// blocks by partition_by_dst (graph_loader.hh:110-138: block i ends at the
// first target change at or after pos + (n - pos) / (count - i)), and each
// block sorted by the curve index XYToIndex(n, src, dst, RA) of the edge's
// (source, target) with n the power of two at least V (sort_edge_in_peano2,
// graph_concepts.hh:164-174; curve utils/peano.hh:20-89).  Blocks are cut on
// the written column v, so no two blocks write the same column.
struct VPair {
  uint32_t u, v;
};

struct FlatBlocks {
  uint32_t V = 0;
  std::vector<VPair> pairs;
  std::vector<uint64_t> off;  // block b holds pairs [off[b], off[b + 1])
  size_t count() const { return off.empty() ? 0 : off.size() - 1; }
};

// XYToIndex(n, x, y, RA), utils/peano.hh:72-89, one level per iteration.
// States RA, RD, CA, CD; kPos[state][quadrant] is the quadrant's place in
// the state's visiting order (order(), peano.hh:27-39), kSub[state][place]
// the state of that sub-square (subPeanoDirection(), peano.hh:41-53).
inline uint64_t curve_index(uint64_t n, uint64_t x, uint64_t y) {
  static const uint8_t kPos[4][4] = {{0, 1, 3, 2}, {2, 3, 1, 0}, {0, 3, 1, 2}, {2, 1, 3, 0}};
  static const uint8_t kSub[4][4] = {{2, 0, 0, 3}, {3, 1, 1, 2}, {0, 2, 2, 1}, {1, 3, 3, 0}};
  uint64_t idx = 0;
  int st = 0;
  for (uint64_t half = n / 2; half >= 1; half /= 2) {
    const int q = (x >= half ? 2 : 0) + (y >= half ? 1 : 0);
    const int p = kPos[st][q];
    idx = idx * 4 + (uint64_t)p;
    st = kSub[st][p];
    if (x >= half) x -= half;
    if (y >= half) y -= half;
  }
  return idx;
}

FlatBlocks *make_flat_blocks(const InLists &L, uint32_t V, bool fwd_first, uint32_t n_blocks) {
  auto *B = new FlatBlocks;
  B->V = V;
  // pairs grouped by target v in ascending order: the in-lists in CSR order
  std::vector<uint64_t> start(V + 1, 0);
  for (size_t v = 0; v < V; v++) {
    uint64_t d = 0;
    for (int l = 0; l < L.n; l++) d += (uint64_t)(L.off[l][v + 1] - L.off[l][v]);
    start[v + 1] = start[v] + d;
  }
  const uint64_t n = start[V];
  B->pairs.resize(n);
#pragma omp parallel for num_threads(nthreads()) schedule(dynamic, 1024)
  for (size_t v = 0; v < V; v++) {
    uint64_t k = start[v];
    for (int l = 0; l < L.n; l++)
      for (int64_t j = L.off[l][v]; j < L.off[l][v + 1]; j++) B->pairs[k++] = VPair{L.adj[l][j], (uint32_t)v};
  }
  // partition_by_dst over the target-grouped pairs
  const uint32_t cnt = n_blocks ? n_blocks : 1;
  B->off.assign(cnt + 1, n);
  B->off[0] = 0;
  uint64_t pos = 0;
  for (uint32_t i = 0; i < cnt; i++) {
    B->off[i] = pos;
    if (pos >= n) continue;
    const uint64_t expected = pos + (n - pos) / (cnt - i);
    uint64_t e = pos + 1;
    while (e < n && !(e >= expected && B->pairs[e].v != B->pairs[e - 1].v)) e++;
    pos = e;
  }
  B->off[cnt] = n;
  // curve order inside every block, over the edge's (source, target): the
  // pair (u, v) of a forward list is the edge (u, v), of a backward list the
  // edge (v, u)
  uint64_t side = 1;
  while (side < V) side <<= 1;
#pragma omp parallel for num_threads(nthreads()) schedule(dynamic, 1)
  for (size_t b = 0; b < cnt; b++) {
    const uint64_t lo = B->off[b], hi = B->off[b + 1];
    std::vector<std::pair<uint64_t, VPair>> kp(hi - lo);
    for (uint64_t i = lo; i < hi; i++) {
      const VPair e = B->pairs[i];
      const uint64_t key = fwd_first ? curve_index(side, e.u, e.v) : curve_index(side, e.v, e.u);
      kp[i - lo] = {key, e};
    }
    std::sort(kp.begin(), kp.end(), [](const auto &a, const auto &c) { return a.first < c.first; });
    for (uint64_t i = lo; i < hi; i++) B->pairs[i] = kp[i - lo].second;
  }
  return B;
}

// DenseVarStackMatrix::prefetch_cols (bitmap.cpp:1173-1185): every 64-byte
// line of the written and the read column of each pair.
inline void prefetch_cols(size_t si, const StackMatrix &out, const StackMatrix &base, const VPair *e,
                          size_t m) {
  const size_t r = si * out.R;
  const size_t lines = (out.v_per_stack_col + 7) / 8;
  for (size_t i = 0; i < m; i++) {
    const uint64_t *p = &out.bits[out.vidx(r, e[i].v)];
    const uint64_t *q = &base.bits[base.vidx(r, e[i].u)];
    for (size_t k = 0; k < lines; k++) {
      __builtin_prefetch(p + 8 * k, 1);
      __builtin_prefetch(q + 8 * k, 0);
    }
  }
}

// The BlockHilbert hop (expand.cpp:263-311 with WITH_PREFETCH and
// BLOCK_PREFETCH, common.hh:52-63): blocks in parallel (guided); inside a
// block every stack in turn; the pairs in runs of BLOCK_PREFETCH_COUNT = 20,
// the run's columns prefetched, then OR-ed (prefetch_or_stack_cols_from,
// bitmap.cpp:1187-1194).
constexpr size_t kBlockPrefetchCount = 20;

void expand_blocks(const FlatBlocks &B, const StackMatrix &base, StackMatrix &out) {
#pragma omp parallel for num_threads(nthreads()) schedule(guided)
  for (size_t b = 0; b < B.count(); b++) {
    const VPair *e = B.pairs.data() + B.off[b];
    const size_t n = B.off[b + 1] - B.off[b];
    for (size_t si = 0; si < base.stack_count; si++) {
      for (size_t i = 0; i < n; i += kBlockPrefetchCount) {
        const size_t m = std::min(n - i, kBlockPrefetchCount);
        prefetch_cols(si, out, base, e + i, m);
        for (size_t j = 0; j < m; j++) out.or_stack_col_from(si, e[i + j].v, base, e[i + j].u);
      }
    }
  }
}

uint64_t active_pairs(const FlatBlocks &B, const StackMatrix &base) {
  uint64_t n = 0;
  const size_t np = B.pairs.size();
#pragma omp parallel for reduction(+ : n) num_threads(nthreads()) schedule(static)
  for (size_t i = 0; i < np; i++) {
    bool nz = false;
    for (size_t si = 0; si < base.stack_count && !nz; si++) nz = base.col_nonzero(si, B.pairs[i].u);
    n += nz;
  }
  return n;
}

// VExpand with ExpandStrategy::Dense over DenseVarStackMatrix, for either hop
// form (hop(base, out) ORs every edge; active(base) counts the edges whose
// base column is non-zero):
//   ExpandStatus init        expand_impl.hh:135-169 (stack size), :252-277 (layer 0 + visit)
//   hop loop                  PhysicalOperator::run (physical_operator.cpp:62-101) with
//                             VExpand::after_child (vexpand.cpp:222-284)
//   one hop + dedup           expand.cpp:263-344
//   result                    VExpand::merge_to_MT (vexpand.cpp:298-354)
template <class Hop, class Active>
int vexpand_run(uint32_t V, Hop hop, Active active, const uint32_t *sources, uint32_t S, uint32_t k_min,
                uint32_t k_max, int path_type, uint32_t stack_row_count, const uint32_t *targets,
                int32_t *dist, uint64_t *out_words, uint64_t *hop_stats) {
  if (V == 0 || (S > 0 && !sources) || k_min > k_max || k_max > 64) return 1;
  if (path_type < OR_ANY || path_type > OR_FIND_SHORTEST) return 1;
  if (path_type == OR_FIND_SHORTEST && (!targets || !dist)) return 1;
  for (uint32_t i = 0; i < S; i++)
    if (sources[i] >= V || (targets && targets[i] >= V)) return 1;
  const size_t R = stack_row_count ? stack_row_count : 1024;  // decide_k0, expand.cpp:416-417
  if (R % 512 != 0) return 1;
  if (S == 0) return 0;  // VExpand::before_execution returns false: empty result
  const bool dedup = path_type != OR_ANY;

  std::vector<std::unique_ptr<StackMatrix>> layers;
  auto layer = [&](size_t i) -> StackMatrix & {
    while (layers.size() <= i) layers.emplace_back(new StackMatrix(S, V, R));
    return *layers[i];
  };
  std::unique_ptr<StackMatrix> visit;
  if (dedup) visit.reset(new StackMatrix(S, V, R));
  // init_first_m_layer (expand_impl.hh:252-277)
  for (size_t i = 0; i < S; i++) {
    layer(0).set(i, sources[i], true);
    if (dedup) visit->set(i, sources[i], true);
  }
  size_t visit_count = S;
  size_t last_visit_count = visit_count;
  size_t found = 0;
  if (path_type == OR_FIND_SHORTEST) {  // VExpand::before_execution, vexpand.cpp:179-195
    for (size_t r = 0; r < S; r++) {
      dist[r] = -1;
      if (sources[r] == targets[r]) {
        dist[r] = 0;
        found++;
      }
    }
  }
  layer(std::max<size_t>(3, k_max) - 1);  // init_multiple_m_layer, vexpand.cpp:213-214
  size_t k_actual_max = 0;
  for (size_t i = 0; i < k_max; i++) {
    StackMatrix &base = layer(i);
    StackMatrix &out = layer(i + 1);
    if (hop_stats) hop_stats[2 * 64 + i + 1] = active(base);
    hop(base, out);
    if (dedup) visit_count = StackMatrix::dedup_and_update_visit_and_count(*visit, out);
    if (hop_stats) {
      hop_stats[0 * 64 + i + 1] = visit_count;
      hop_stats[1 * 64 + i + 1] = out.count();
    }
    k_actual_max = i + 1;  // after_child
    bool cont = true;
    if (path_type == OR_SHORTEST) {
      if (last_visit_count == visit_count) cont = false;
      last_visit_count = visit_count;
    } else if (path_type == OR_FIND_SHORTEST) {
      const int32_t d = (int32_t)(i + 1);
      for (size_t r = 0; r < S; r++) {
        if (dist[r] == -1 && out.get(r, targets[r])) {
          dist[r] = d;
          found++;
        }
      }
      if (found == S)
        cont = false;
      else if (last_visit_count == visit_count)
        cont = false;
      last_visit_count = visit_count;
    }
    if (!cont) break;
  }
  if (hop_stats) hop_stats[3 * 64] = k_actual_max;
  if (path_type == OR_FIND_SHORTEST || !out_words) return 0;
  // merge_to_MT
  if (path_type == OR_SHORTEST && k_min == 0) {
    visit->to_logical(out_words);
    return 0;
  }
  StackMatrix merged(S, V, R);
  for (size_t i = k_min; i <= k_actual_max; i++) merged.or_from(layer(i));
  merged.to_logical(out_words);
  return 0;
}

}  // namespace

extern "C" {

void oracle_set_threads(int n) { g_threads = n; }
int oracle_get_threads(void) { return nthreads(); }

int oracle_vexpand(uint32_t V, const int64_t *fwd_off, const uint32_t *fwd_dst,
                   const int64_t *rev_off, const uint32_t *rev_src, int directed,
                   const uint32_t *sources, uint32_t S, uint32_t k_min, uint32_t k_max,
                   int path_type, int dir, uint32_t stack_row_count, const uint32_t *targets,
                   int32_t *dist, uint64_t *out_words, uint64_t *hop_stats) {
  if (dir < 0 || dir > 2) return 1;
  InLists L = in_lists(fwd_off, fwd_dst, rev_off, rev_src, directed, dir);
  return vexpand_run(
      V, [&](const StackMatrix &base, StackMatrix &out) { expand_dense(L, V, base, out); },
      [&](const StackMatrix &base) { return active_edges(L, V, base); }, sources, S, k_min, k_max,
      path_type, stack_row_count, targets, dist, out_words, hop_stats);
}

void *oracle_flat_blocks(uint32_t V, const int64_t *fwd_off, const uint32_t *fwd_dst,
                         const int64_t *rev_off, const uint32_t *rev_src, int directed, int dir,
                         uint32_t n_blocks) {
  if (V == 0 || dir < 0 || dir > 2 || n_blocks == 0) return nullptr;
  InLists L = in_lists(fwd_off, fwd_dst, rev_off, rev_src, directed, dir);
  // a forward (or undirected) list holds the edges u -> v; a backward one v -> u
  const bool fwd_first = !directed || dir != OR_BACKWARD;
  return make_flat_blocks(L, V, fwd_first, n_blocks);
}

void oracle_flat_blocks_free(void *h) { delete static_cast<FlatBlocks *>(h); }

uint64_t oracle_flat_blocks_export(const void *h, uint64_t *off, uint32_t *pairs) {
  const auto *B = static_cast<const FlatBlocks *>(h);
  if (off)
    for (size_t b = 0; b <= B->count(); b++) off[b] = B->off[b];
  if (pairs)
    for (size_t i = 0; i < B->pairs.size(); i++) {
      pairs[2 * i] = B->pairs[i].u;
      pairs[2 * i + 1] = B->pairs[i].v;
    }
  return B->pairs.size();
}

int oracle_vexpand_blocks(const void *h, const uint32_t *sources, uint32_t S, uint32_t k_min,
                          uint32_t k_max, int path_type, uint32_t stack_row_count,
                          const uint32_t *targets, int32_t *dist, uint64_t *out_words,
                          uint64_t *hop_stats) {
  if (!h) return 1;
  const auto &B = *static_cast<const FlatBlocks *>(h);
  return vexpand_run(
      B.V, [&](const StackMatrix &base, StackMatrix &out) { expand_blocks(B, base, out); },
      [&](const StackMatrix &base) { return active_pairs(B, base); }, sources, S, k_min, k_max,
      path_type, stack_row_count, targets, dist, out_words, hop_stats);
}

uint64_t oracle_matrix_count(uint32_t rows, uint32_t cols, const uint64_t *words,
                             uint32_t stack_row_count) {
  StackMatrix m(rows, cols, stack_row_count ? stack_row_count : 1024);
  m.from_logical(words);
  return m.count();
}

// MatrixTableSelect::run_internal, VarRowMatrix branch (big_operators2.cpp:152-213)
int oracle_matrix_select(uint32_t rows, uint32_t cols, const uint64_t *words,
                         uint32_t stack_row_count, const uint32_t *targets, uint32_t T,
                         uint64_t *out_words) {
  const size_t R = stack_row_count ? stack_row_count : 1024;
  for (uint32_t i = 0; i < T; i++)
    if (targets[i] >= cols) return 1;
  StackMatrix old(rows, cols, R);
  old.from_logical(words);
  StackMatrix nm(rows, T, R);
#pragma omp parallel for num_threads(nthreads())
  for (size_t ci = 0; ci < T; ci++)
    for (size_t si = 0; si < nm.stack_count; si++) nm.or_stack_col_from(si, ci, old, targets[ci]);
  nm.to_logical(out_words);
  return 0;
}

// TableConvert::run_internal, VarRow -> ColMain (big_operators2.cpp:28-61)
int oracle_table_convert(uint32_t rows, uint32_t cols, const uint64_t *words,
                         uint32_t stack_row_count, int transpose, uint64_t *out_words) {
  StackMatrix src(rows, cols, stack_row_count ? stack_row_count : 1024);
  src.from_logical(words);
  if (transpose) {
    ColMain dst(cols, rows);
#pragma omp parallel for num_threads(nthreads())
    for (size_t r = 0; r < rows; r++)
      for (size_t c = 0; c < cols; c++) dst.set(c, r, src.get(r, c));
    const size_t wpc = ((size_t)cols + 63) / 64;
    for (size_t c = 0; c < rows; c++)
      for (size_t w = 0; w < wpc; w++) out_words[c * wpc + w] = dst.bits[c * dst.v_per_col + w];
  } else {
    // copy_from_variable_row_mat has no scalar path (bitmap.cpp:896-899); its
    // SIMD path copies each stack column verbatim, i.e. an identical logical matrix.
    ColMain dst(rows, cols);
    const size_t wpc = ((size_t)rows + 63) / 64;
    for (size_t c = 0; c < cols; c++)
      for (size_t w = 0; w < wpc; w++) dst.bits[c * dst.v_per_col + w] = src.bits[src.vidx(w * 64, c)];
    for (size_t c = 0; c < cols; c++)
      for (size_t w = 0; w < wpc; w++) out_words[c * wpc + w] = dst.bits[c * dst.v_per_col + w];
  }
  return 0;
}

// VarRowMatrixTable::Iterator::next (bit_matrix_table.cpp:133-188) over every
// stack; BitmapIterator::next (bitmap.hh:108-123) is the ctz loop.
uint64_t oracle_matrix_iterate(uint32_t rows, uint32_t cols, const uint64_t *words,
                               uint32_t stack_row_count, const uint32_t *row_map,
                               const uint32_t *col_map, uint32_t *out_r, uint32_t *out_c) {
  StackMatrix m(rows, cols, stack_row_count ? stack_row_count : 1024);
  m.from_logical(words);
  uint64_t n = 0;
  for (size_t si = 0; si < m.stack_count; si++) {
    const uint64_t *start = &m.bits[m.vidx(si * m.R, 0)];
    const size_t nw = m.v_per_stack_col * cols;
    for (size_t wi = 0; wi < nw; wi++) {
      uint64_t d = start[wi];
      while (d) {
        size_t bitpos = wi * 64 + std::countr_zero(d);
        d &= d - 1;
        uint32_t r = (uint32_t)(bitpos % m.R + si * m.R);
        uint32_t c = (uint32_t)(wi / m.v_per_stack_col);
        if (row_map) r = row_map[r];
        if (col_map) c = col_map[c];
        if (out_r) {
          out_r[n] = r;
          out_c[n] = c;
        }
        n++;
      }
    }
  }
  return n;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Tables for HashJoin and Mintersect.
namespace {

struct Schema {
  std::vector<int32_t> var, type;
  int index(int32_t v) const {
    for (size_t i = 0; i < var.size(); i++)
      if (var[i] == v) return (int)i;
    return -1;
  }
};

// TableSchema::join_schema (tuple.cpp:317-342)
Schema join_schema(const Schema &a, const Schema &b, int32_t key) {
  Schema r = a;
  for (size_t i = 0; i < b.var.size(); i++)
    if (b.var[i] != key) {
      r.var.push_back(b.var[i]);
      r.type.push_back(b.type[i]);
    }
  return r;
}

// TableSchema::map_to (tuple.cpp:289-300)
std::vector<int> map_to(const Schema &from, const Schema &to) {
  std::vector<int> m;
  for (auto v : from.var) m.push_back(to.index(v));
  return m;
}

Schema schema_of(const or_table *t) {
  Schema s;
  for (uint32_t i = 0; i < t->ncols; i++) {
    s.var.push_back(t->var[i]);
    s.type.push_back(t->kind == OR_FLAT ? t->type[i] : OR_T_VID);
  }
  return s;
}

inline uint64_t flat_get(const or_table *t, uint64_t row, uint32_t col) {
  if (t->type[col] == OR_T_I64) return (uint64_t)((const int64_t *)t->cols[col])[row];
  return ((const uint32_t *)t->cols[col])[row];
}

uint64_t tuple_count(const or_table *t) {
  if (t->kind == OR_FLAT) return t->nrows;
  const size_t wpc = ((size_t)t->mrows + 63) / 64;
  uint64_t n = 0;
  for (size_t i = 0; i < wpc * t->mcols; i++) n += std::popcount(t->words[i]);
  return n;
}

struct ColMainView {
  const or_table *t;
  ColMain m;
  std::unordered_map<uint32_t, uint32_t> col_hash, row_hash;
  explicit ColMainView(const or_table *tt) : t(tt), m(tt->mrows, tt->mcols) {
    m.from_logical(tt->words);
    if (tt->col_map)
      for (uint32_t i = 0; i < tt->mcols; i++) col_hash.emplace(tt->col_map[i], i);
    if (tt->row_map)
      for (uint32_t i = 0; i < tt->mrows; i++) row_hash.emplace(tt->row_map[i], i);
  }
  uint32_t col_value(size_t c) const { return t->col_map ? t->col_map[c] : (uint32_t)c; }
  uint32_t row_value(size_t r) const { return t->row_map ? t->row_map[r] : (uint32_t)r; }
  // MatrixTable::find_col_idx (bit_matrix_table.cpp:53-61)
  bool find_col_idx(uint32_t v, size_t *out) const {
    if (!t->col_map) {
      if (v < t->mcols) {
        *out = v;
        return true;
      }
      return false;
    }
    auto it = col_hash.find(v);
    if (it == col_hash.end()) return false;
    *out = it->second;
    return true;
  }
  // ColMainMatrixTable::Iterator over one column (bit_matrix_table.cpp:242-289)
  template <typename F> void for_rows(size_t c, F f) const {
    const uint64_t *p = m.col(c);
    for (size_t w = 0; w < m.v_per_col; w++) {
      uint64_t d = p[w];
      while (d) {
        size_t r = w * 64 + std::countr_zero(d);
        d &= d - 1;
        f(row_value(r));
      }
    }
  }
};

struct ResultBuilder {
  Schema s;
  std::vector<std::vector<uint64_t>> cols;
  explicit ResultBuilder(const Schema &sc) : s(sc), cols(sc.var.size()) {}
  void finish(or_result *out) {
    out->ncols = (uint32_t)s.var.size();
    out->nrows = cols.empty() ? 0 : cols[0].size();
    for (size_t i = 0; i < s.var.size(); i++) {
      out->var[i] = s.var[i];
      out->type[i] = s.type[i];
      if (s.type[i] == OR_T_I64) {
        int64_t *p = (int64_t *)std::malloc(sizeof(int64_t) * (out->nrows + 1));
        for (uint64_t r = 0; r < out->nrows; r++) p[r] = (int64_t)cols[i][r];
        out->cols[i] = p;
      } else {
        uint32_t *p = (uint32_t *)std::malloc(sizeof(uint32_t) * (out->nrows + 1));
        for (uint64_t r = 0; r < out->nrows; r++) p[r] = (uint32_t)cols[i][r];
        out->cols[i] = p;
      }
    }
  }
};

}  // namespace

extern "C" {

void oracle_free_result(or_result *r) {
  if (!r) return;
  for (uint32_t i = 0; i < r->ncols && i < 16; i++) std::free(r->cols[i]);
  std::memset(r, 0, sizeof(*r));
}

// HashJoin::build + HashJoin::probe (join.cpp:26-444).  The reference's hash
// maps are tbb::concurrent_hash_map keyed by XXH64 of a TupleValue; the hash
// function is unobservable, so std::unordered_map stands in.
int oracle_hash_join(const or_table *a, const or_table *b, int32_t key_var, int only_count,
                     or_result *out) {
  std::memset(out, 0, sizeof(*out));
  if (a->kind == OR_VARROW || b->kind == OR_VARROW) return 1;  // not supported (join.cpp:73-77)
  Schema sa = schema_of(a), sb = schema_of(b);
  int ka = sa.index(key_var), kb = sb.index(key_var);
  if (ka < 0 || kb < 0 || sa.type[ka] != sb.type[kb]) return 1;
  Schema rs = only_count ? Schema{{-1}, {OR_T_I64}} : join_schema(sa, sb, key_var);
  if (rs.var.size() > 16) return 1;

  const or_table *build = a, *probe = b;
  auto col_count = [](const or_table *t) -> uint64_t { return t->mcols; };
  // build-side choice, join.cpp:39-72
  if (build->kind == OR_FLAT && probe->kind == OR_FLAT) {
    if (build->nrows < probe->nrows) std::swap(build, probe);
  } else if (build->kind == OR_FLAT && probe->kind == OR_COLMAIN) {
    if (build->nrows < col_count(probe)) std::swap(build, probe);
  } else if (build->kind == OR_COLMAIN && probe->kind == OR_FLAT) {
    if (col_count(build) < probe->nrows) std::swap(build, probe);
  } else {
    if (col_count(build) < col_count(probe)) std::swap(build, probe);
  }
  Schema bs = schema_of(build), ps = schema_of(probe);
  const int bk = bs.index(key_var), pk = ps.index(key_var);
  if ((build->kind == OR_COLMAIN && bk != 1) || (probe->kind == OR_COLMAIN && pk != 1)) return 1;

  std::unordered_map<uint64_t, std::vector<uint64_t>> flat_map;  // key -> build rows
  std::unordered_map<uint64_t, uint64_t> count_map;              // key -> multiplicity
  std::unique_ptr<ColMainView> bview, pview;
  if (build->kind == OR_COLMAIN) bview.reset(new ColMainView(build));
  if (probe->kind == OR_COLMAIN) pview.reset(new ColMainView(probe));

  // build (join.cpp:86-155)
  if (build->kind == OR_FLAT) {
    for (uint64_t i = 0; i < build->nrows; i++) {
      uint64_t k = flat_get(build, i, bk);
      if (only_count)
        count_map[k]++;
      else
        flat_map[k].push_back(i);
    }
  } else if (only_count) {
    for (size_t c = 0; c < build->mcols; c++)
      count_map.emplace(bview->col_value(c), bview->m.count_bits_in_col(c));  // insert keeps the first
  }

  ResultBuilder res(rs);
  int64_t total = 0;
  auto push_row = [&](std::vector<uint64_t> &vals) {
    for (size_t i = 0; i < vals.size(); i++) res.cols[i].push_back(vals[i]);
  };
  const std::vector<int> pmap = map_to(ps, rs), bmap = map_to(bs, rs);

  if (probe->kind == OR_FLAT) {
    if (only_count) {  // join.cpp:266-278
      for (uint64_t i = 0; i < probe->nrows; i++) {
        auto it = count_map.find(flat_get(probe, i, pk));
        if (it != count_map.end()) total += (int64_t)it->second;
      }
    } else if (build->kind == OR_FLAT) {  // join.cpp:183-225
      std::vector<uint64_t> vals(rs.var.size());
      for (uint64_t pi = 0; pi < probe->nrows; pi++) {
        auto it = flat_map.find(flat_get(probe, pi, pk));
        if (it == flat_map.end()) continue;
        for (uint64_t bi : it->second) {
          for (size_t c = 0; c < pmap.size(); c++)
            if (pmap[c] >= 0 && (int)c != pk) vals[pmap[c]] = flat_get(probe, pi, c);
          for (size_t c = 0; c < bmap.size(); c++)
            if (bmap[c] >= 0) vals[bmap[c]] = flat_get(build, bi, c);
          push_row(vals);
        }
      }
    } else {  // Flat probe x ColMain build, join.cpp:226-262
      std::vector<uint64_t> vals(rs.var.size());
      const int payload = bmap[0];
      for (uint64_t i = 0; i < probe->nrows; i++) {
        uint32_t vid = (uint32_t)flat_get(probe, i, pk);
        size_t col;
        // the reference dereferences a failed lookup (join.cpp:241-244); a
        // missing key contributes no tuple here
        if (!bview->find_col_idx(vid, &col)) continue;
        bview->for_rows(col, [&](uint32_t r) {
          for (size_t c = 0; c < pmap.size(); c++)
            if (pmap[c] >= 0) vals[pmap[c]] = flat_get(probe, i, c);
          vals[payload] = r;
          push_row(vals);
        });
      }
    }
  } else {  // probe is ColMain
    if (only_count) {  // join.cpp:406-430
      for (size_t c = 0; c < probe->mcols; c++) {
        auto it = count_map.find(pview->col_value(c));
        if (it != count_map.end()) total += (int64_t)(it->second * pview->m.count_bits_in_col(c));
      }
    } else if (build->kind == OR_FLAT) {  // join.cpp:281-331
      std::vector<uint64_t> vals(rs.var.size());
      for (size_t c = 0; c < probe->mcols; c++) {
        auto it = flat_map.find(pview->col_value(c));
        if (it == flat_map.end()) continue;
        pview->for_rows(c, [&](uint32_t prow) {
          for (uint64_t bri : it->second) {
            vals[pmap[0]] = prow;
            for (size_t bc = 0; bc < bmap.size(); bc++)
              if (bmap[bc] >= 0) vals[bmap[bc]] = flat_get(build, bri, bc);
            push_row(vals);
          }
        });
      }
    } else {  // ColMain x ColMain, join.cpp:333-401
      std::vector<uint64_t> vals(rs.var.size());
      const int payload = bmap[0];
      for (size_t c = 0; c < probe->mcols; c++) {
        uint32_t key = pview->col_value(c);
        size_t bcol;
        if (!bview->find_col_idx(key, &bcol)) continue;
        std::vector<uint32_t> brows;
        bview->for_rows(bcol, [&](uint32_t r) { brows.push_back(r); });
        pview->for_rows(c, [&](uint32_t pr) {
          for (uint32_t br : brows) {
            vals[pmap[0]] = pr;
            vals[pmap[1]] = key;
            vals[payload] = br;
            push_row(vals);
          }
        });
      }
    }
  }
  if (only_count) {
    out->ncols = 1;
    out->nrows = 1;
    out->var[0] = -1;
    out->type[0] = OR_T_I64;
    int64_t *p = (int64_t *)std::malloc(sizeof(int64_t));
    *p = total;
    out->cols[0] = p;
    out->count = total;
    return 0;
  }
  res.finish(out);
  out->count = (int64_t)out->nrows;
  return 0;
}

// Mintersect::finishAddingDependency + run_internal (mintersect.cpp:14-345).
int oracle_mintersect(const or_table *base, const or_table *deps, uint32_t ndeps,
                      int32_t new_var, uint32_t new_type_vertex_count, int only_count,
                      or_result *out) {
  std::memset(out, 0, sizeof(*out));
  if (ndeps == 0 || base->kind == OR_COLMAIN) return 1;
  Schema bsch = schema_of(base);
  std::vector<int> var_base_idx(ndeps), edges_u_idx(ndeps), edges_nv_idx(ndeps);
  for (uint32_t i = 0; i < ndeps; i++) {
    const or_table *d = &deps[i];
    if (d->ncols != 2 || d->kind == OR_VARROW) return 1;
    Schema ds = schema_of(d);
    int nv = ds.index(new_var);
    if (nv < 0 || ds.type[nv] != OR_T_VID) return 1;
    edges_nv_idx[i] = nv;
    edges_u_idx[i] = 1 - nv;
    var_base_idx[i] = bsch.index(ds.var[1 - nv]);
    if (var_base_idx[i] < 0) return 1;
    // a ColMain dependency has the new vertex as its row variable (mintersect.cpp:59)
    if (d->kind == OR_COLMAIN && nv != 0) return 1;
  }
  Schema rs;
  if (only_count) {
    rs = Schema{{-1}, {OR_T_I64}};
  } else {
    rs = bsch;
    rs.var.push_back(new_var);
    rs.type.push_back(OR_T_VID);
  }
  // cache rows: the ColMain row count when every dependency is a matrix
  size_t ncm = 0, cm_rows = 0;
  std::vector<std::unique_ptr<ColMainView>> views(ndeps);
  const uint32_t *target_row_map = nullptr;
  for (uint32_t i = 0; i < ndeps; i++) {
    if (deps[i].kind == OR_COLMAIN) {
      views[i].reset(new ColMainView(&deps[i]));
      if (ncm && cm_rows != deps[i].mrows) return 1;
      cm_rows = deps[i].mrows;
      if (!ncm) target_row_map = deps[i].row_map;
      ncm++;
    }
  }
  const size_t cache_rows = (ncm == ndeps) ? cm_rows : new_type_vertex_count;

  // base tuples: Flat rows or the (row, col) pairs of a VarRow matrix
  std::vector<std::vector<uint64_t>> base_rows;
  if (base->kind == OR_FLAT) {
    base_rows.resize(base->nrows);
    for (uint64_t i = 0; i < base->nrows; i++)
      for (uint32_t c = 0; c < base->ncols; c++) base_rows[i].push_back(flat_get(base, i, c));
  } else {
    uint64_t n = oracle_matrix_iterate(base->mrows, base->mcols, base->words, 1024, nullptr,
                                       nullptr, nullptr, nullptr);
    std::vector<uint32_t> r(n), c(n);
    oracle_matrix_iterate(base->mrows, base->mcols, base->words, 1024, base->row_map,
                          base->col_map, r.data(), c.data());
    base_rows.resize(n);
    for (uint64_t i = 0; i < n; i++) base_rows[i] = {r[i], c[i]};
  }

  ResultBuilder res(rs);
  int64_t total = 0;
  const size_t nbase = base_rows.size();
  const int nt = nthreads();
  std::vector<std::vector<std::vector<uint64_t>>> per_thread(nt);
#pragma omp parallel num_threads(nt) reduction(+ : total)
  {
    const int t = omp_get_thread_num();
    ColMain ir(cache_rows, 2);  // col 0 = result, col 1 = flat scratch
#pragma omp for schedule(dynamic, 64)
    for (size_t bi = 0; bi < nbase; bi++) {
      ir.set_col_to(0, true);
      for (uint32_t di = 0; di < ndeps; di++) {
        uint32_t bvid = (uint32_t)base_rows[bi][var_base_idx[di]];
        const or_table *d = &deps[di];
        if (d->kind == OR_COLMAIN) {
          size_t col;
          if (views[di]->find_col_idx(bvid, &col))
            ir.and_col_from(0, views[di]->m, col);
          else
            ir.set_col_to(0, false);
        } else {
          // linear scan of the flat dependency (mintersect.cpp:149-165);
          // the dependency's own u column is used for both base kinds
          ir.set_col_to(1, false);
          for (uint64_t i = 0; i < d->nrows; i++) {
            if ((uint32_t)flat_get(d, i, edges_u_idx[di]) != bvid) continue;
            uint64_t payload = flat_get(d, i, edges_nv_idx[di]);
            if (payload < cache_rows) ir.set(payload, 1, true);
          }
          ir.and_col_from(0, ir, 1);
        }
      }
      size_t num = ir.count_bits_in_col(0);
      total += (int64_t)num;
      if (num == 0 || only_count) continue;
      const uint64_t *p = ir.col(0);
      for (size_t w = 0; w < ir.v_per_col; w++) {
        uint64_t dd = p[w];
        while (dd) {
          uint32_t x = (uint32_t)(w * 64 + std::countr_zero(dd));
          dd &= dd - 1;
          if (target_row_map) x = target_row_map[x];
          std::vector<uint64_t> row = base_rows[bi];
          row.push_back(x);
          per_thread[t].push_back(std::move(row));
        }
      }
    }
  }
  if (only_count) {
    out->ncols = 1;
    out->nrows = 1;
    out->var[0] = -1;
    out->type[0] = OR_T_I64;
    int64_t *p = (int64_t *)std::malloc(sizeof(int64_t));
    *p = total;
    out->cols[0] = p;
    out->count = total;
    return 0;
  }
  for (auto &v : per_thread)
    for (auto &row : v)
      for (size_t i = 0; i < row.size(); i++) res.cols[i].push_back(row[i]);
  res.finish(out);
  out->count = (int64_t)out->nrows;
  return 0;
}

// ---- result consumers --------------------------------------------------------
namespace {
inline uint32_t mat_col_value(const or_table *m, size_t c) { return m->col_map ? m->col_map[c] : (uint32_t)c; }
inline uint32_t mat_row_value(const or_table *m, size_t r) { return m->row_map ? m->row_map[r] : (uint32_t)r; }
inline size_t mat_wpc(const or_table *m) { return ((size_t)m->mrows + 63) / 64; }
}  // namespace

// MatrixColumnCount::run_internal (matrix_column_count.cpp:19-87):
// count_bits_in_col per column; with an order, the (count, col) pairs sorted
// with std::less / std::greater.
int oracle_matrix_column_count(const or_table *m, int ord, uint32_t *out_col, int64_t *out_count) {
  if (m->kind != OR_VARROW && m->kind != OR_COLMAIN) return 1;
  const size_t wpc = mat_wpc(m);
  std::vector<std::pair<int64_t, uint32_t>> pairs(m->mcols);
#pragma omp parallel for num_threads(nthreads())
  for (size_t c = 0; c < m->mcols; c++) {
    int64_t n = 0;
    for (size_t w = 0; w < wpc; w++) n += std::popcount(m->words[c * wpc + w]);
    pairs[c] = {n, mat_col_value(m, c)};
  }
  if (ord == 1) std::sort(pairs.begin(), pairs.end(), std::less<std::pair<int64_t, uint32_t>>());
  if (ord == 2) std::sort(pairs.begin(), pairs.end(), std::greater<std::pair<int64_t, uint32_t>>());
  for (size_t i = 0; i < pairs.size(); i++) {
    out_col[i] = pairs[i].second;
    out_count[i] = pairs[i].first;
  }
  return 0;
}

// MatrixRowOrSum::run_internal (matrix_row_or_sum.cpp:14-54): has_bits_in_col.
uint64_t oracle_matrix_row_or_sum(const or_table *m, uint32_t *out_col) {
  const size_t wpc = mat_wpc(m);
  uint64_t n = 0;
  for (size_t c = 0; c < m->mcols; c++) {
    bool any = false;
    for (size_t w = 0; w < wpc && !any; w++) any = m->words[c * wpc + w] != 0;
    if (!any) continue;
    if (out_col) out_col[n] = mat_col_value(m, c);
    n++;
  }
  return n;
}

// MatrixTableFilter<F>::run_internal (big_operators2.hh:142-170): the matrix
// table's iterators visit every set bit, map the row through row_map and the
// column through col_map, and clear the bit when f(r, c) is false
// (matrix_table.hh:153-200).  f is the AND of the device forms.
uint64_t oracle_matrix_filter(const or_table *m, const uint64_t *row_keep, uint32_t row_values,
                              const uint64_t *col_keep, uint32_t col_values, const uint64_t *pairs,
                              uint64_t npairs, int pairs_mode) {
  auto in_bits = [](const uint64_t *bits, uint32_t n, uint32_t v) {
    return v < n && ((bits[v >> 6] >> (v & 63)) & 1ull);
  };
  auto f = [&](uint32_t r, uint32_t c) {
    if (row_keep && !in_bits(row_keep, row_values, r)) return false;
    if (col_keep && !in_bits(col_keep, col_values, c)) return false;
    if (pairs_mode) {
      const bool listed = std::binary_search(pairs, pairs + npairs, ((uint64_t)r << 32) | c);
      if (listed != (pairs_mode == 1)) return false;
    }
    return true;
  };
  const size_t wpc = mat_wpc(m);
  uint64_t cleared = 0;
  for (size_t c = 0; c < m->mcols; c++)
    for (size_t w = 0; w < wpc; w++) {
      uint64_t x = m->words[c * wpc + w];
      while (x) {
        const unsigned b = (unsigned)std::countr_zero(x);
        x &= x - 1;
        const size_t r = w * 64 + b;
        if (!f(mat_row_value(m, r), mat_col_value(m, c))) {
          const_cast<uint64_t *>(m->words)[c * wpc + w] &= ~(1ull << b);
          cleared++;
        }
      }
    }
  return cleared;
}

// VertexNeighborFetcher + VertexPropertyFetcher as tcr1.cpp:46-57 uses them.
void oracle_vertex_mask_any_neighbor(const int64_t *off, const uint32_t *adj, uint32_t V, const uint8_t *prop,
                                     uint8_t value, uint64_t *mask) {
  for (size_t i = 0; i < ((size_t)V + 63) / 64; i++) mask[i] = 0;
  for (uint32_t v = 0; v < V; v++)
    for (int64_t j = off[v]; j < off[v + 1]; j++)
      if (prop[adj[j]] == value) {
        mask[v >> 6] |= 1ull << (v & 63);
        break;
      }
}

// SemiJoin<N>::build / probe_once / probe (semi_join.cpp:58-262).  Key
// tuples are compared by value (TupleValue equality); std::set stands in for
// the reference's concurrent set.
int oracle_semi_join(const or_table *a, const or_table *b, const int32_t *key_vars, uint32_t N,
                     int only_count, or_result *out, uint64_t *out_words) {
  std::memset(out, 0, sizeof(*out));
  if (N == 0 || N > 4) return 1;
  if (a->kind == OR_COLMAIN || b->kind == OR_COLMAIN) return 1;  // assert(0) in the reference
  Schema sa = schema_of(a), sb = schema_of(b);
  int ai[4], bi[4];
  for (uint32_t k = 0; k < N; k++) {
    ai[k] = sa.index(key_vars[k]);
    bi[k] = sb.index(key_vars[k]);
    if (ai[k] < 0 || bi[k] < 0 || sa.type[ai[k]] != sb.type[bi[k]]) return 1;
  }
  using Tup = std::array<uint64_t, 4>;
  std::set<Tup> bset;
  const size_t bwpc = b->kind == OR_FLAT ? 0 : mat_wpc(b);
  std::unordered_map<uint32_t, size_t> brow, bcol;  // VarRow b with N == 2: direct bit lookups
  if (b->kind == OR_FLAT) {
    for (uint64_t i = 0; i < b->nrows; i++) {
      Tup t{};
      for (uint32_t k = 0; k < N; k++) t[k] = flat_get(b, i, (uint32_t)bi[k]);
      bset.insert(t);
    }
  } else if (N == 2) {
    for (size_t r = 0; r < b->mrows; r++) brow.emplace(mat_row_value(b, r), r);
    for (size_t c = 0; c < b->mcols; c++) bcol.emplace(mat_col_value(b, c), c);
  } else {
    for (size_t c = 0; c < b->mcols; c++)
      for (size_t w = 0; w < bwpc; w++) {
        uint64_t d = b->words[c * bwpc + w];
        while (d) {
          const size_t r = w * 64 + std::countr_zero(d);
          d &= d - 1;
          Tup t{};
          for (uint32_t k = 0; k < N; k++) t[k] = bi[k] == 0 ? mat_row_value(b, r) : mat_col_value(b, c);
          bset.insert(t);
        }
      }
  }
  auto member = [&](const Tup &t) -> bool {
    if (b->kind == OR_FLAT || N != 2) return bset.count(t) != 0;
    uint64_t r = t[0], c = t[1];
    if (bi[0] == 1 && bi[1] == 0) std::swap(r, c);
    auto ir = brow.find((uint32_t)r), ic = bcol.find((uint32_t)c);
    if (ir == brow.end() || ic == bcol.end()) return false;
    return (b->words[ic->second * bwpc + ir->second / 64] >> (ir->second % 64)) & 1;
  };
  int64_t count = 0;
  if (a->kind == OR_FLAT) {
    ResultBuilder res(sa);
    for (uint64_t i = 0; i < a->nrows; i++) {
      Tup t{};
      for (uint32_t k = 0; k < N; k++) t[k] = flat_get(a, i, (uint32_t)ai[k]);
      if (!member(t)) continue;
      count++;
      if (!only_count)
        for (uint32_t c = 0; c < a->ncols; c++) res.cols[c].push_back(flat_get(a, i, c));
    }
    if (!only_count) res.finish(out);
  } else {
    const size_t wpc = mat_wpc(a);
    for (size_t c = 0; c < a->mcols; c++)
      for (size_t w = 0; w < wpc; w++) {
        uint64_t d = a->words[c * wpc + w], keep = 0;
        uint64_t dd = d;
        while (dd) {
          const size_t r = w * 64 + std::countr_zero(dd);
          const uint64_t bit = dd & (~dd + 1);
          dd &= dd - 1;
          Tup t{};
          for (uint32_t k = 0; k < N; k++) t[k] = ai[k] == 0 ? mat_row_value(a, r) : mat_col_value(a, c);
          if (member(t)) {
            keep |= bit;
            count++;
          }
        }
        if (!only_count && out_words) out_words[c * wpc + w] = keep;
      }
  }
  out->count = count;
  return 0;
}

}  // extern "C"
