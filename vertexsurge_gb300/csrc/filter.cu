// MatrixTableFilter (src/include/operator/big_operators2.hh:53-61,142-170,
// over VarRowMatrixTable::filter and ColMainMatrixTable::filter,
// src/include/execution/matrix_table.hh:153-200) re-designed for sm_103a.
//
// The reference walks every set bit with an iterator, maps its row and
// column through row_map / col_map and clears it when a host predicate
// f(row value, column value) is false.  A host predicate cannot run here, so
// the predicate comes in three device forms that compose by AND:
//   * a bitset over row values      (keep rows whose value's bit is set)
//   * a bitset over column values   (keep columns whose value's bit is set)
//   * a sorted list of (row value << 32 | column value) keys, either the only
//     pairs kept or the pairs dropped.
// The two bitsets cost no per-bit work: the row bitset becomes one word mask
// per matrix word position (the same for every column, the matrix being
// column-major with the rows of a column in consecutive words) and a dropped
// column is zeroed whole, so a filter is one read and at most one write of
// the matrix.  Only the pair list visits bits, each with a binary search.
// The tcr1 driver's predicate ("the other account signed in to a blocked
// medium", ldbc-finbench/tcr1.cpp:46-57) is a column bitset, built on the
// device by vs_vertex_mask_any_neighbor from the signIn lists of a graph.
#include <algorithm>

#include "dev_util.cuh"
#include "vs_internal.cuh"

namespace vs {
namespace fl {

int grid_for(uint64_t n, int per_block = 256) {
  return (int)std::max<uint64_t>(1, std::min<uint64_t>((n + per_block - 1) / per_block,
                                                       (uint64_t)sm_count() * 16));
}

__device__ __forceinline__ bool value_bit(const uint64_t *__restrict__ bits, uint32_t nvalues, uint32_t v) {
  return v < nvalues && ((__ldg(bits + (v >> 6)) >> (v & 63)) & 1ull);
}

// Word masks of the row bitset: word q keeps row 64q + b when the value of
// that row (row_map or the index) has its bit set; rows past the matrix are 0.
__global__ void k_row_words(const uint64_t *__restrict__ keep, uint32_t nvalues, const uint32_t *__restrict__ row_map,
                            uint32_t rows, uint32_t wpc, uint64_t *__restrict__ out) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < wpc; q += gridDim.x * blockDim.x) {
    uint64_t w = 0;
    for (uint32_t b = 0; b < 64; b++) {
      const uint32_t r = q * 64 + b;
      if (r >= rows) break;
      const uint32_t v = row_map ? __ldg(row_map + r) : r;
      if (value_bit(keep, nvalues, v)) w |= 1ull << b;
    }
    out[q] = w;
  }
}

// Membership of k in a sorted key list (binary search).
__device__ __forceinline__ bool has_key(const uint64_t *__restrict__ keys, uint64_t n, uint64_t k) {
  uint64_t lo = 0, hi = n;
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    const uint64_t x = __ldg(keys + mid);
    if (x < k) lo = mid + 1; else hi = mid;
  }
  return lo < n && __ldg(keys + lo) == k;
}

struct FilterArgs {
  uint64_t *w;
  uint32_t rows, cols, wpc;
  const uint32_t *row_map, *col_map, *colnz;
  const uint64_t *row_words;  // per word position (NULL: no row condition)
  const uint64_t *col_keep;   // bitset over column values (NULL: no column condition)
  uint32_t col_values;
  const uint64_t *pairs;      // sorted (row value << 32 | column value) keys (NULL: none)
  uint64_t npairs;
  int pairs_mode;             // 1: keep listed pairs only, 2: drop listed pairs
};

// A warp per column, lanes over its words; a word is stored only if it changes.
__global__ void __launch_bounds__(256) k_filter(FilterArgs a) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  for (uint64_t c = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < a.cols; c += warps) {
    if (a.colnz && !__ldg(a.colnz + c)) continue;  // a zero column stays zero
    const uint32_t cv = a.col_map ? __ldg(a.col_map + c) : (uint32_t)c;
    const bool col_ok = !a.col_keep || value_bit(a.col_keep, a.col_values, cv);
    uint64_t *col = a.w + c * a.wpc;
    for (uint32_t q = lane; q < a.wpc; q += 32) {
      const uint64_t x0 = col[q];
      if (!x0) continue;
      uint64_t x = col_ok ? x0 : 0ull;
      if (x && a.row_words) x &= __ldg(a.row_words + q);
      if (x && a.pairs) {
        uint64_t bits = x;
        while (bits) {
          const uint32_t b = __ffsll((long long)bits) - 1;
          bits &= bits - 1;
          const uint32_t r = q * 64 + b;
          const uint32_t rv = a.row_map ? __ldg(a.row_map + r) : r;
          const bool listed = has_key(a.pairs, a.npairs, ((uint64_t)rv << 32) | cv);
          if (listed != (a.pairs_mode == 1)) x &= ~(1ull << b);
        }
      }
      if (x != x0) col[q] = x;
    }
  }
}

// bit i of flag: keys[i] > keys[i + 1] (the list is not sorted ascending)
__global__ void k_unsorted(const uint64_t *__restrict__ keys, uint64_t n, int *flag) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i + 1 < n; i += (uint64_t)gridDim.x * blockDim.x)
    if (__ldg(keys + i) > __ldg(keys + i + 1)) *flag = 1;
}

// mask bit v = some neighbour u of v has prop[u] == value; a warp covers 32
// consecutive vertices, one per lane, and writes their 32-bit mask word.
__global__ void k_any_neighbor(const int64_t *__restrict__ off, const uint32_t *__restrict__ adj, uint32_t V,
                               const uint8_t *__restrict__ prop, uint32_t nprop, uint8_t value,
                               uint32_t *__restrict__ mask32, int *bad) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t base = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~31ull; base < V; base += step) {
    const uint64_t v = base + lane;
    bool hit = false;
    if (v < V) {
      const int64_t b = __ldg(off + v), e = __ldg(off + v + 1);
      for (int64_t j = b; j < e && !hit; j++) {
        const uint32_t u = __ldg(adj + j);
        if (u >= nprop) {
          *bad = 1;  // a neighbour id outside the property column
          break;
        }
        hit = __ldg(prop + u) == value;
      }
    }
    const unsigned m = __ballot_sync(FULLMASK, hit);
    if (lane == 0) mask32[base >> 5] = m;
  }
}

bool is_device(const void *p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

}  // namespace fl
}  // namespace vs

using namespace vs;
using namespace vs::fl;

extern "C" {

int vs_matrix_filter(vs_bitmat *m, const uint64_t *row_keep, uint32_t row_values, const uint64_t *col_keep,
                     uint32_t col_values, const uint64_t *pairs, uint64_t npairs, int pairs_mode,
                     vs_stream_t stream) {
  if (!m) return fail(VS_ERR_ARG, "vs_matrix_filter: null matrix");
  if (m->kind != VS_KIND_VARROW && m->kind != VS_KIND_COLMAIN)
    return fail(VS_ERR_ARG, "MatrixTableFilter takes a VarRow or ColMain matrix");  // big_operators2.hh:147
  if (pairs_mode < 0 || pairs_mode > 2) return fail(VS_ERR_ARG, "vs_matrix_filter: pair mode must be 0, 1 or 2");
  if (pairs_mode && npairs && !pairs) return fail(VS_ERR_ARG, "vs_matrix_filter: null pair list");
  if (!pairs_mode) npairs = 0;
  cudaStream_t st = S(stream);
  // predicate arrays in host memory are copied in (and the call syncs before returning)
  const uint64_t *src[3] = {row_keep, col_keep, npairs ? pairs : nullptr};
  const uint64_t len[3] = {((uint64_t)row_values + 63) / 64, ((uint64_t)col_values + 63) / 64, npairs};
  const uint64_t *dev[3] = {nullptr, nullptr, nullptr};
  uint64_t *owned[3] = {nullptr, nullptr, nullptr};
  bool copied = false;
  int rc = VS_OK;
  for (int i = 0; i < 3 && rc == VS_OK; i++) {
    if (!src[i]) continue;
    if (is_device(src[i]) || len[i] == 0) {
      dev[i] = src[i];
      continue;
    }
    if ((rc = dalloc_n(&owned[i], len[i], st)) != VS_OK) break;
    const cudaError_t e = cudaMemcpyAsync(owned[i], src[i], len[i] * 8, cudaMemcpyDefault, st);
    if (e != cudaSuccess) rc = cuda_fail(e, "vs_matrix_filter", __FILE__, __LINE__);
    dev[i] = owned[i];
    copied = true;
  }
  uint64_t *row_words = nullptr;
  int *d_flag = nullptr;
  if (rc == VS_OK && npairs > 1 && (rc = dalloc_n(&d_flag, 1, st)) == VS_OK) {
    // the pair list must be sorted ascending (binary search)
    int h_flag = 0;
    cudaError_t e = cudaMemsetAsync(d_flag, 0, sizeof(int), st);
    if (e == cudaSuccess) {
      k_unsorted<<<grid_for(npairs), 256, 0, st>>>(dev[2], npairs, d_flag);
      vs::note_launch();
      e = cudaMemcpyAsync(&h_flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
      rc = cuda_fail(e, "vs_matrix_filter", __FILE__, __LINE__);
    else if (h_flag)
      rc = fail(VS_ERR_ARG, "vs_matrix_filter: the pair list is not sorted ascending");
  }
  if (rc == VS_OK && m->cols && m->rows) {
    if (pairs_mode == 1 && npairs == 0) {  // keep only listed pairs, none listed: every bit goes
      const cudaError_t e = cudaMemsetAsync(m->words, 0, (size_t)m->cols * m->wpc * 8, st);
      if (e != cudaSuccess) rc = cuda_fail(e, "vs_matrix_filter", __FILE__, __LINE__);
    } else {
      if (dev[0] && (rc = dalloc_n(&row_words, m->wpc, st)) == VS_OK) {
        k_row_words<<<grid_for(m->wpc), 256, 0, st>>>(dev[0], row_values, m->row_map, m->rows, m->wpc, row_words);
        vs::note_launch();
      }
      if (rc == VS_OK) {
        FilterArgs a{};
        a.w = m->words;
        a.rows = m->rows;
        a.cols = m->cols;
        a.wpc = m->wpc;
        a.row_map = m->row_map;
        a.col_map = m->col_map;
        a.colnz = m->colnz;
        a.row_words = row_words;
        a.col_keep = dev[1];
        a.col_values = col_values;
        a.pairs = npairs ? dev[2] : nullptr;
        a.npairs = npairs;
        a.pairs_mode = pairs_mode;
        k_filter<<<grid_for((uint64_t)m->cols * 32), 256, 0, st>>>(a);
        vs::note_launch();
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = cuda_fail(e, "vs_matrix_filter", __FILE__, __LINE__);
      }
    }
    m->st = st;
  }
  if (copied && rc == VS_OK) {  // host arrays were read by the copies above
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_fail(e, "vs_matrix_filter", __FILE__, __LINE__);
  }
  for (uint64_t *o : owned)
    if (o) dfree(o, st);
  if (row_words) dfree(row_words, st);
  if (d_flag) dfree(d_flag, st);
  return rc;
}

int vs_vertex_mask_any_neighbor(const vs_graph *g, int direction, const uint8_t *prop, uint32_t nprop,
                                uint8_t value, uint64_t *mask, vs_stream_t stream) {
  if (!g || !prop || !mask) return fail(VS_ERR_ARG, "vs_vertex_mask_any_neighbor: null argument");
  if (direction != VS_DIR_FORWARD && direction != VS_DIR_BACKWARD)
    return fail(VS_ERR_ARG, "vs_vertex_mask_any_neighbor: direction must be forward or backward");
  cudaStream_t st = S(stream);
  const uint32_t V = g->V;
  const uint64_t words = ((uint64_t)V + 63) / 64;
  const bool fwd = direction == VS_DIR_FORWARD || !g->directed;
  const int64_t *off = fwd ? g->fwd_off : g->rev_off;
  const uint32_t *adj = fwd ? g->fwd_dst : g->rev_src;
  const bool prop_dev = is_device(prop), mask_dev = is_device(mask);
  uint8_t *d_prop = nullptr;
  uint64_t *d_mask = nullptr;
  int *d_bad = nullptr;
  int h_bad = 0, rc = VS_OK;
  if (!prop_dev && nprop) rc = dalloc_n(&d_prop, nprop, st);
  if (rc == VS_OK && !mask_dev) rc = dalloc_n(&d_mask, words, st);
  if (rc == VS_OK) rc = dalloc_n(&d_bad, 1, st);
  cudaError_t e = cudaSuccess;
  if (rc == VS_OK) {
    const uint8_t *pp = prop_dev ? prop : d_prop;
    uint64_t *mm = mask_dev ? mask : d_mask;
    if (!prop_dev && nprop) e = cudaMemcpyAsync(d_prop, prop, nprop, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(mm, 0, words * 8, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_bad, 0, sizeof(int), st);
    if (e == cudaSuccess && V) {
      k_any_neighbor<<<grid_for(V), 256, 0, st>>>(off, adj, V, pp, nprop, value, reinterpret_cast<uint32_t *>(mm),
                                                   d_bad);
      vs::note_launch();
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && !mask_dev) e = cudaMemcpyAsync(mask, d_mask, words * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_fail(e, "vs_vertex_mask_any_neighbor", __FILE__, __LINE__);
  }
  if (d_prop) dfree(d_prop, st);
  if (d_mask) dfree(d_mask, st);
  if (d_bad) dfree(d_bad, st);
  if (rc == VS_OK && h_bad)
    rc = fail(VS_ERR_ARG, "vs_vertex_mask_any_neighbor: a neighbour id is >= the property count %u", nprop);
  return rc;
}

}  // extern "C"
