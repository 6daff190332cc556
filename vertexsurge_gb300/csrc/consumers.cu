// Result consumers of an expand: MatrixColumnCount, MatrixRowOrSum and
// SemiJoin<N> (src/objects/operator/matrix_column_count.cpp:6-87,
// matrix_row_or_sum.cpp:7-54, semi_join.cpp:7-262) re-designed for sm_103a.
//
// Column counts: G = min(32, pow2 >= words per column) lanes per column
// popcount its words.  The ordered form sorts the 64-bit keys
// (count << 32 | column value) — bit-complemented for descending order, which
// reproduces std::greater on the (count, value) pair — with a stable LSD radix
// sort over the key bytes that vary (8 bits per pass: per-block digit
// histograms, one exclusive scan in digit-major order, then a scatter whose
// rank within a block is built warp by warp with __match_any_sync).
//
// SemiJoin: the right input becomes a 64-bit key set (one key column, or two
// vertex-id key columns packed high/low) in an open-addressing table; a
// right-hand VarRow matrix with two keys is probed in place instead (its row
// and column values located through hash tables of its maps, then one bit
// load).  A flat left input is filtered row by row (scan + gather); a VarRow
// left input keeps the bits whose (row value, column value) key is a member,
// word by word, into a new matrix of the same shape and maps.
#include <algorithm>
#include <cstring>

#include "dev_util.cuh"
#include "hash.cuh"
#include "vs_internal.cuh"

namespace vs {
namespace cs {

int grid_for(uint64_t n, int per_block = 256) {
  return (int)std::max<uint64_t>(1, std::min<uint64_t>((n + per_block - 1) / per_block,
                                                       (uint64_t)sm_count() * 16));
}

struct Scratch {
  cudaStream_t st;
  void *p[32] = {};
  int n = 0;
  template <typename T> int get(T **out, size_t count) {
    int rc = dalloc_n(out, count ? count : 1, st);
    if (rc == VS_OK) p[n++] = *out;
    return rc;
  }
  ~Scratch() {
    for (int i = 0; i < n; i++) dfree(p[i], st);
  }
};

// ---- column popcounts --------------------------------------------------------
__global__ void k_col_counts(const uint64_t *__restrict__ w, uint32_t wpc, uint32_t cols, uint32_t G,
                             const uint32_t *__restrict__ colnz, uint32_t *__restrict__ cnt) {
  const uint32_t lane = threadIdx.x & 31, gl = lane % G, gpw = 32 / G;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const uint64_t warps = (uint64_t)gridDim.x * blockDim.x / 32;
  // warp-uniform loop: every lane reaches the group shuffles
  for (uint64_t base = warp * gpw; base < cols; base += warps * gpw) {
    const uint64_t c = base + lane / G;
    uint32_t s = 0;
    if (c < cols && (!colnz || colnz[c]))
      for (uint32_t q = gl; q < wpc; q += G) s += __popcll(__ldg(w + c * wpc + q));
    for (uint32_t o = G >> 1; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, G);
    if (gl == 0 && c < cols) cnt[c] = s;
  }
}

__global__ void k_cc_keys(const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ col_map, uint32_t cols,
                          int desc, unsigned long long *__restrict__ keys) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += gridDim.x * blockDim.x) {
    const unsigned long long k = ((unsigned long long)cnt[c] << 32) | (col_map ? col_map[c] : c);
    keys[c] = desc ? ~k : k;
  }
}

__global__ void k_cc_emit(const unsigned long long *__restrict__ keys, const uint32_t *__restrict__ cnt,
                          const uint32_t *__restrict__ col_map, uint32_t cols, int sorted, int desc,
                          uint32_t *__restrict__ out_col, long long *__restrict__ out_cnt) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += gridDim.x * blockDim.x) {
    if (sorted) {
      const unsigned long long k = desc ? ~keys[c] : keys[c];
      out_col[c] = (uint32_t)k;
      out_cnt[c] = (long long)(k >> 32);
    } else {
      out_col[c] = col_map ? col_map[c] : c;
      out_cnt[c] = cnt[c];
    }
  }
}

// ---- stable LSD radix sort of 64-bit keys ------------------------------------
constexpr int RS_THREADS = 256, RS_TILE = 4096;  // keys per block per pass

__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const unsigned long long *__restrict__ in, uint64_t n,
                                                        int shift, uint32_t nblk,
                                                        unsigned long long *__restrict__ hist) {
  __shared__ unsigned h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t b0 = (uint64_t)blockIdx.x * RS_TILE, b1 = b0 + RS_TILE < n ? b0 + RS_TILE : n;
  for (uint64_t i = b0 + threadIdx.x; i < b1; i += RS_THREADS) atomicAdd(&h[(in[i] >> shift) & 255u], 1u);
  __syncthreads();
  hist[(uint64_t)threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];  // digit-major
}

__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const unsigned long long *__restrict__ in, uint64_t n,
                                                           int shift, uint32_t nblk,
                                                           const unsigned long long *__restrict__ off,
                                                           unsigned long long *__restrict__ out) {
  __shared__ unsigned long long base[256];  // next free slot per digit for this block
  __shared__ unsigned wcnt[RS_THREADS / 32][256];
  const int wid = threadIdx.x >> 5;
  base[threadIdx.x] = off[(uint64_t)threadIdx.x * nblk + blockIdx.x];
  const uint64_t b0 = (uint64_t)blockIdx.x * RS_TILE, b1 = b0 + RS_TILE < n ? b0 + RS_TILE : n;
  for (uint64_t s = b0; s < b1; s += RS_THREADS) {
    for (int w = 0; w < RS_THREADS / 32; w++) wcnt[w][threadIdx.x] = 0;
    __syncthreads();
    const uint64_t i = s + threadIdx.x;
    const bool valid = i < b1;
    const unsigned long long k = valid ? in[i] : 0ull;
    const unsigned d = valid ? (unsigned)((k >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const unsigned rank = __popc(peers & lanemask_lt());
    if (valid && rank == 0) wcnt[wid][d] = __popc(peers);
    __syncthreads();
    {  // per digit: exclusive prefix over the warps, then advance the block base
      const unsigned t = threadIdx.x;
      unsigned acc = 0;
      for (int w = 0; w < RS_THREADS / 32; w++) {
        const unsigned x = wcnt[w][t];
        wcnt[w][t] = acc;
        acc += x;
      }
      __syncthreads();
      if (valid) out[base[d] + wcnt[wid][d] + rank] = k;
      __syncthreads();
      base[t] += acc;
    }
    __syncthreads();
  }
}

// Sorts keys[0..n) by bits [lo_bit, hi_bit); returns the buffer holding the result.
int radix_sort_u64(Scratch &sc, unsigned long long *keys, uint64_t n, int lo_bit, int hi_bit,
                   unsigned long long **result) {
  *result = keys;
  if (n < 2) return VS_OK;
  const uint32_t nblk = (uint32_t)((n + RS_TILE - 1) / RS_TILE);
  unsigned long long *tmp, *hist, *off;
  VS_TRY(sc.get(&tmp, n));
  VS_TRY(sc.get(&hist, (size_t)256 * nblk));
  VS_TRY(sc.get(&off, (size_t)256 * nblk + 1));
  unsigned long long *src = keys, *dst = tmp;
  for (int shift = lo_bit; shift < hi_bit; shift += 8) {
    { k_rs_hist<<<nblk, RS_THREADS, 0, sc.st>>>(src, n, shift, nblk, hist); vs::note_launch(); }
    VS_TRY(exclusive_scan_u64(hist, off, (size_t)256 * nblk, sc.st));
    { k_rs_scatter<<<nblk, RS_THREADS, 0, sc.st>>>(src, n, shift, nblk, off, dst); vs::note_launch(); }
    std::swap(src, dst);
  }
  VS_CK(cudaGetLastError());
  *result = src;
  return VS_OK;
}

// ---- row-or-sum compaction ------------------------------------------------------
__global__ void k_nz_flags(const uint32_t *__restrict__ cnt, uint32_t cols, unsigned long long *__restrict__ f) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += gridDim.x * blockDim.x)
    f[c] = cnt[c] != 0;
}

__global__ void k_compact_cols(const uint32_t *__restrict__ cnt, const unsigned long long *__restrict__ pos,
                               const uint32_t *__restrict__ col_map, uint32_t cols, uint32_t *__restrict__ out) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += gridDim.x * blockDim.x)
    if (cnt[c]) out[pos[c]] = col_map ? col_map[c] : c;
}

int column_counts(const vs_bitmat *m, Scratch &sc, uint32_t **cnt) {
  VS_TRY(sc.get(cnt, m->cols));
  uint32_t G = 1;
  while (G < 32 && G < m->wpc) G <<= 1;
  if (m->cols)
    { k_col_counts<<<grid_for((uint64_t)m->cols * G), 256, 0, sc.st>>>(m->words, m->wpc, m->cols, G, m->colnz,
                                                                      *cnt); vs::note_launch(); }
  VS_CK(cudaGetLastError());
  return VS_OK;
}

// ---- SemiJoin ---------------------------------------------------------------------
struct KeySide {           // how one input yields its key of a row / bit
  int kind;                // 0 flat, 1 matrix
  const void *col[2];      // flat: key columns
  int type[2];             // flat: VS_T_*
  int mcol[2];             // matrix: 0 = row value, 1 = column value
  uint32_t n;              // number of key columns
};

__device__ __forceinline__ unsigned long long flat_val(const void *col, int type, uint64_t i) {
  return type == VS_T_I64 ? (unsigned long long)((const long long *)col)[i] : ((const uint32_t *)col)[i];
}

__device__ __forceinline__ unsigned long long pack_key(const KeySide &s, unsigned long long v0,
                                                       unsigned long long v1) {
  return s.n == 1 ? v0 : ((v0 << 32) | (v1 & 0xffffffffull));
}

struct MatProbe {          // right-hand VarRow with two keys: direct bit lookups
  const uint64_t *words;
  uint32_t wpc, rows, cols;
  int has_rmap, has_cmap;
  HashTable rmap, cmap;    // value -> index (val)
  int swap;                // keys arrive as (col value, row value)
};

struct Probe {
  int direct;              // MatProbe instead of the key set
  HashTable set;
  MatProbe mp;
};

__device__ __forceinline__ bool member(const Probe &p, unsigned long long key) {
  if (!p.direct) return ht_find(p.set, key) != ~0ull;
  uint32_t r = (uint32_t)(key >> 32), c = (uint32_t)key;
  if (p.mp.swap) {
    const uint32_t t = r;
    r = c;
    c = t;
  }
  uint32_t ri = r, ci = c;
  if (p.mp.has_rmap) {
    const uint64_t s = ht_find(p.mp.rmap, r);
    if (s == ~0ull) return false;
    ri = p.mp.rmap.val[s];
  } else if (r >= p.mp.rows) {
    return false;
  }
  if (p.mp.has_cmap) {
    const uint64_t s = ht_find(p.mp.cmap, c);
    if (s == ~0ull) return false;
    ci = p.mp.cmap.val[s];
  } else if (c >= p.mp.cols) {
    return false;
  }
  return (p.mp.words[(size_t)ci * p.mp.wpc + (ri >> 6)] >> (ri & 63)) & 1ull;
}

__global__ void k_build_map(HashTable t, const uint32_t *vals, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint64_t s = ht_insert(t, vals[i]);
    atomicMin(&t.val[s], i);
  }
}

__global__ void k_set_from_flat(HashTable t, KeySide s, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    ht_insert(t, pack_key(s, flat_val(s.col[0], s.type[0], i), s.n > 1 ? flat_val(s.col[1], s.type[1], i) : 0));
}

// one key column of a matrix: the values of its columns with bits, or of its rows with bits
__global__ void k_set_from_cols(HashTable t, const uint32_t *__restrict__ cnt, const uint32_t *col_map,
                                uint32_t cols) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += gridDim.x * blockDim.x)
    if (cnt[c]) ht_insert(t, col_map ? col_map[c] : c);
}

__global__ void k_rows_any(const uint64_t *__restrict__ w, uint32_t wpc, uint32_t cols,
                           unsigned long long *__restrict__ any) {
  for (uint32_t q = blockIdx.y * blockDim.x + threadIdx.x; q < wpc; q += gridDim.y * blockDim.x) {
    unsigned long long acc = 0;
    for (uint32_t c = blockIdx.x; c < cols; c += gridDim.x) acc |= w[(size_t)c * wpc + q];
    if (acc) atomicOr(any + q, acc);
  }
}

__global__ void k_set_from_rows(HashTable t, const unsigned long long *__restrict__ any, uint32_t rows,
                                const uint32_t *row_map) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x)
    if ((any[r >> 6] >> (r & 63)) & 1ull) ht_insert(t, row_map ? row_map[r] : r);
}

__global__ void k_probe_flat(Probe p, KeySide s, uint64_t n, unsigned long long *__restrict__ keep,
                             unsigned long long *total) {
  unsigned long long cnt = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const bool k = member(p, pack_key(s, flat_val(s.col[0], s.type[0], i),
                                      s.n > 1 ? flat_val(s.col[1], s.type[1], i) : 0));
    if (keep) keep[i] = k;
    cnt += k;
  }
  block_add(cnt, total);
}

__global__ void k_gather_rows(const unsigned long long *__restrict__ keep, const unsigned long long *__restrict__ pos,
                              uint64_t n, const void *src, void *dst, int type) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    if (keep[i]) {
      if (type == VS_T_I64)
        ((long long *)dst)[pos[i]] = ((const long long *)src)[i];
      else
        ((uint32_t *)dst)[pos[i]] = ((const uint32_t *)src)[i];
    }
}

// VarRow left input: word (c, q) of a; its bits' keys are (row value, column value) per mcol
__global__ void k_probe_mat(Probe p, KeySide s, const uint64_t *__restrict__ w, uint32_t wpc, uint32_t rows,
                            uint32_t cols, const uint32_t *row_map, const uint32_t *col_map,
                            const uint32_t *colnz, uint64_t *out, unsigned long long *total) {
  unsigned long long cnt = 0;
  const uint64_t nw = (uint64_t)wpc * cols;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t c = (uint32_t)(i / wpc), q = (uint32_t)(i % wpc);
    uint64_t x = (colnz && !colnz[c]) ? 0ull : w[i], kept = 0;
    const uint32_t cv = col_map ? col_map[c] : c;
    while (x) {
      const int b = __ffsll((long long)x) - 1;
      x &= x - 1;
      const uint32_t r = q * 64 + b;
      if (r >= rows) break;
      const uint32_t rv = row_map ? row_map[r] : r;
      const unsigned long long v0 = s.mcol[0] == 0 ? rv : cv;
      const unsigned long long v1 = s.mcol[1] == 0 ? rv : cv;
      if (member(p, pack_key(s, v0, v1))) kept |= 1ull << b;
    }
    cnt += __popcll(kept);
    if (out) out[i] = kept;
  }
  block_add(cnt, total);
}

int key_side(const vs_table_ref &t, uint32_t n, const uint32_t *cols, KeySide *s) {
  *s = KeySide{};
  s->n = n;
  if (t.flat) {
    s->kind = 0;
    for (uint32_t k = 0; k < n; k++) {
      if (cols[k] >= t.flat->ncols) return fail(VS_ERR_ARG, "semi join key column %u out of range", cols[k]);
      s->col[k] = t.flat->cols[cols[k]];
      s->type[k] = t.flat->types[cols[k]];
    }
  } else {
    if (t.mat->kind != VS_KIND_VARROW)
      return fail(VS_ERR_UNSUPPORTED, "SemiJoin takes flat or VarRow inputs (semi_join.cpp:109-112)");
    s->kind = 1;
    for (uint32_t k = 0; k < n; k++) {
      if (cols[k] > 1) return fail(VS_ERR_ARG, "a matrix key column is 0 (row) or 1 (column)");
      s->mcol[k] = (int)cols[k];
      s->type[k] = VS_T_VID;
    }
  }
  if (n == 2 && (s->type[0] != VS_T_VID || s->type[1] != VS_T_VID))
    return fail(VS_ERR_UNSUPPORTED, "two-column semi join keys must be vertex ids");
  return VS_OK;
}

int hash_alloc(Scratch &sc, uint64_t n, HashTable *t) {
  *t = HashTable{};
  t->cap = ht_capacity(std::max<uint64_t>(n, 1));
  VS_TRY(sc.get(&t->keys, t->cap + 1));
  VS_TRY(sc.get(&t->val, t->cap + 1));
  VS_CK(cudaMemsetAsync(t->keys, 0xff, 8 * (t->cap + 1), sc.st));
  VS_CK(cudaMemsetAsync(t->val, 0xff, 4 * (t->cap + 1), sc.st));
  return VS_OK;
}

// ---- vertex selection by a property range (the Scan filter of the plans) -----
__global__ void k_range_flags(const void *__restrict__ vals, int bytes, uint32_t n, long long lo, long long hi,
                              unsigned long long *__restrict__ f) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    long long v = 0;
    if (vals) {
      if (bytes == 1)
        v = ((const uint8_t *)vals)[i];
      else if (bytes == 2)
        v = ((const uint16_t *)vals)[i];
      else if (bytes == 4)
        v = ((const uint32_t *)vals)[i];
      else
        v = ((const long long *)vals)[i];
    }
    f[i] = !vals || (v >= lo && v <= hi);
  }
}

__global__ void k_compact_ids(const unsigned long long *__restrict__ f, const unsigned long long *__restrict__ pos,
                              uint32_t n, uint32_t *__restrict__ out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (f[i]) out[pos[i]] = i;
}

}  // namespace cs
}  // namespace vs

using namespace vs;
using namespace vs::cs;

extern "C" {

int vs_matrix_column_count(const vs_bitmat *m, int order, vs_flat **out, vs_stream_t stream) {
  if (!m || !out) return fail(VS_ERR_ARG, "vs_matrix_column_count: null argument");
  if (order < 0 || order > 2) return fail(VS_ERR_ARG, "order is 0 (none), 1 (ascending) or 2 (descending)");
  cudaStream_t st = S(stream);
  Scratch sc{st};
  uint32_t *cnt = nullptr;
  VS_TRY(column_counts(m, sc, &cnt));
  const int32_t types[2] = {VS_T_VID, VS_T_I64};
  vs_flat *f = nullptr;
  VS_TRY(flat_alloc(2, types, m->cols, st, &f));
  unsigned long long *keys = nullptr, *sorted = nullptr;
  const int desc = order == 2;
  if (order && m->cols) {
    VS_TRY(sc.get(&keys, m->cols));
    { k_cc_keys<<<grid_for(m->cols), 256, 0, st>>>(cnt, m->col_map, m->cols, desc, keys); vs::note_launch(); }
    // the bytes that can differ: the 32-bit column value, then the count (at most rows)
    int cbits = 0;
    while (cbits < 32 && (1ull << cbits) <= m->rows) cbits++;
    const int hi = 32 + ((cbits + 7) / 8) * 8;
    int rc = radix_sort_u64(sc, keys, m->cols, 0, hi, &sorted);
    if (rc != VS_OK) {
      vs_flat_free(f);
      return rc;
    }
  }
  if (m->cols)
    { k_cc_emit<<<grid_for(m->cols), 256, 0, st>>>(sorted, cnt, m->col_map, m->cols, order != 0, desc,
                                                  (uint32_t *)f->cols[0], (long long *)f->cols[1]); vs::note_launch(); }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    vs_flat_free(f);
    return cuda_fail(e, "vs_matrix_column_count", __FILE__, __LINE__);
  }
  *out = f;
  return VS_OK;
}

int vs_matrix_row_or_sum(const vs_bitmat *m, vs_flat **out, vs_stream_t stream) {
  if (!m || !out) return fail(VS_ERR_ARG, "vs_matrix_row_or_sum: null argument");
  cudaStream_t st = S(stream);
  Scratch sc{st};
  uint32_t *cnt = nullptr;
  VS_TRY(column_counts(m, sc, &cnt));
  unsigned long long *flags, *pos;
  VS_TRY(sc.get(&flags, m->cols));
  VS_TRY(sc.get(&pos, (size_t)m->cols + 1));
  unsigned long long n = 0;
  if (m->cols) {
    { k_nz_flags<<<grid_for(m->cols), 256, 0, st>>>(cnt, m->cols, flags); vs::note_launch(); }
    VS_TRY(exclusive_scan_u64(flags, pos, m->cols, st));
    unsigned long long last[2];
    VS_CK(cudaMemcpyAsync(&last[0], pos + m->cols - 1, 8, cudaMemcpyDeviceToHost, st));
    VS_CK(cudaMemcpyAsync(&last[1], flags + m->cols - 1, 8, cudaMemcpyDeviceToHost, st));
    VS_CK(cudaStreamSynchronize(st));
    n = last[0] + last[1];
  }
  const int32_t types[1] = {VS_T_VID};
  vs_flat *f = nullptr;
  VS_TRY(flat_alloc(1, types, n, st, &f));
  if (n) { k_compact_cols<<<grid_for(m->cols), 256, 0, st>>>(cnt, pos, m->col_map, m->cols, (uint32_t *)f->cols[0]); vs::note_launch(); }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    vs_flat_free(f);
    return cuda_fail(e, "vs_matrix_row_or_sum", __FILE__, __LINE__);
  }
  *out = f;
  return VS_OK;
}

int vs_select_ids_in_range(const void *values, int value_bytes, uint32_t n, int64_t lo, int64_t hi, vs_flat **out,
                           vs_stream_t stream) {
  if (!out) return fail(VS_ERR_ARG, "vs_select_ids_in_range: null output");
  if (values && value_bytes != 1 && value_bytes != 2 && value_bytes != 4 && value_bytes != 8)
    return fail(VS_ERR_ARG, "property values are 1, 2, 4 or 8 bytes wide");
  if (values) {
    cudaPointerAttributes at{};
    VS_CK(cudaPointerGetAttributes(&at, values));
    if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
      return fail(VS_ERR_ARG, "vs_select_ids_in_range: values must be device memory");
  }
  cudaStream_t st = S(stream);
  Scratch sc{st};
  unsigned long long *flags, *pos;
  VS_TRY(sc.get(&flags, n));
  VS_TRY(sc.get(&pos, (size_t)n + 1));
  unsigned long long cnt = 0;
  if (n) {
    { k_range_flags<<<grid_for(n), 256, 0, st>>>(values, value_bytes, n, lo, hi, flags); vs::note_launch(); }
    VS_TRY(exclusive_scan_u64(flags, pos, n, st));
    unsigned long long last[2];
    VS_CK(cudaMemcpyAsync(&last[0], pos + n - 1, 8, cudaMemcpyDeviceToHost, st));
    VS_CK(cudaMemcpyAsync(&last[1], flags + n - 1, 8, cudaMemcpyDeviceToHost, st));
    VS_CK(cudaStreamSynchronize(st));
    cnt = last[0] + last[1];
  }
  const int32_t types[1] = {VS_T_VID};
  vs_flat *f = nullptr;
  VS_TRY(flat_alloc(1, types, cnt, st, &f));
  if (cnt) { k_compact_ids<<<grid_for(n), 256, 0, st>>>(flags, pos, n, (uint32_t *)f->cols[0]); vs::note_launch(); }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    vs_flat_free(f);
    return cuda_fail(e, "vs_select_ids_in_range", __FILE__, __LINE__);
  }
  *out = f;
  return VS_OK;
}

int vs_semi_join(vs_table_ref a, vs_table_ref b, uint32_t nkeys, const uint32_t *a_key_cols,
                 const uint32_t *b_key_cols, int only_count, vs_flat **out_flat, vs_bitmat **out_mat,
                 uint64_t *count, vs_stream_t stream) {
  if (!count || !a_key_cols || !b_key_cols) return fail(VS_ERR_ARG, "vs_semi_join: null argument");
  if (!a.flat == !a.mat || !b.flat == !b.mat) return fail(VS_ERR_ARG, "each input is a flat table or a matrix");
  if (nkeys < 1 || nkeys > 2)
    return fail(VS_ERR_UNSUPPORTED, "SemiJoin with %u key columns: 1 or 2 are supported", nkeys);
  if (!only_count && ((a.flat && !out_flat) || (a.mat && !out_mat)))
    return fail(VS_ERR_ARG, "vs_semi_join: null output");
  KeySide sa, sb;
  VS_TRY(key_side(a, nkeys, a_key_cols, &sa));
  VS_TRY(key_side(b, nkeys, b_key_cols, &sb));
  for (uint32_t k = 0; k < nkeys; k++)
    if (sa.type[k] != sb.type[k]) return fail(VS_ERR_ARG, "key column %u differs in type between the inputs", k);
  cudaStream_t st = S(stream);
  Scratch sc{st};
  Probe p{};
  // build: the right input's key set (or its matrix for two keys)
  if (b.mat && nkeys == 2) {
    const vs_bitmat *m = b.mat;
    p.direct = 1;
    p.mp.words = m->words;
    p.mp.wpc = m->wpc;
    p.mp.rows = m->rows;
    p.mp.cols = m->cols;
    p.mp.swap = sb.mcol[0] == 1 && sb.mcol[1] == 0;
    if (sb.mcol[0] == sb.mcol[1]) return fail(VS_ERR_ARG, "the two matrix keys must be its row and column");
    p.mp.has_rmap = m->row_map != nullptr;
    p.mp.has_cmap = m->col_map != nullptr;
    if (m->row_map) {
      VS_TRY(hash_alloc(sc, m->rows, &p.mp.rmap));
      if (m->rows) { k_build_map<<<grid_for(m->rows), 256, 0, st>>>(p.mp.rmap, m->row_map, m->rows); vs::note_launch(); }
    }
    if (m->col_map) {
      VS_TRY(hash_alloc(sc, m->cols, &p.mp.cmap));
      if (m->cols) { k_build_map<<<grid_for(m->cols), 256, 0, st>>>(p.mp.cmap, m->col_map, m->cols); vs::note_launch(); }
    }
  } else if (b.mat) {
    const vs_bitmat *m = b.mat;
    if (sb.mcol[0] == 1) {
      uint32_t *cnt = nullptr;
      VS_TRY(column_counts(m, sc, &cnt));
      VS_TRY(hash_alloc(sc, m->cols, &p.set));
      if (m->cols) { k_set_from_cols<<<grid_for(m->cols), 256, 0, st>>>(p.set, cnt, m->col_map, m->cols); vs::note_launch(); }
    } else {
      unsigned long long *any = nullptr;
      VS_TRY(sc.get(&any, m->wpc));
      VS_CK(cudaMemsetAsync(any, 0, 8ull * std::max(1u, m->wpc), st));
      if (m->cols && m->wpc) {
        dim3 grid(std::min<uint32_t>(m->cols, 1024), std::min<uint32_t>((m->wpc + 255) / 256, 64));
        k_rows_any<<<grid, 256, 0, st>>>(m->words, m->wpc, m->cols, any);
        vs::note_launch();
      }
      VS_TRY(hash_alloc(sc, m->rows, &p.set));
      if (m->rows) { k_set_from_rows<<<grid_for(m->rows), 256, 0, st>>>(p.set, any, m->rows, m->row_map); vs::note_launch(); }
    }
  } else {
    VS_TRY(hash_alloc(sc, b.flat->nrows, &p.set));
    if (b.flat->nrows) { k_set_from_flat<<<grid_for(b.flat->nrows), 256, 0, st>>>(p.set, sb, b.flat->nrows); vs::note_launch(); }
  }
  unsigned long long *total = nullptr;
  VS_TRY(sc.get(&total, 1));
  VS_CK(cudaMemsetAsync(total, 0, 8, st));
  vs_flat *f = nullptr;
  vs_bitmat *om = nullptr;
  if (a.flat) {
    const vs_flat *t = a.flat;
    unsigned long long *keep = nullptr, *pos = nullptr;
    if (!only_count) {
      VS_TRY(sc.get(&keep, t->nrows));
      VS_TRY(sc.get(&pos, t->nrows + 1));
    }
    if (t->nrows) { k_probe_flat<<<grid_for(t->nrows), 256, 0, st>>>(p, sa, t->nrows, keep, total); vs::note_launch(); }
    unsigned long long n = 0;
    VS_CK(cudaMemcpyAsync(&n, total, 8, cudaMemcpyDeviceToHost, st));
    VS_CK(cudaStreamSynchronize(st));
    *count = n;
    if (only_count) return VS_OK;
    VS_TRY(flat_alloc(t->ncols, t->types, n, st, &f));
    if (n) {
      int rc = exclusive_scan_u64(keep, pos, t->nrows, st);
      if (rc != VS_OK) {
        vs_flat_free(f);
        return rc;
      }
      for (uint32_t c = 0; c < t->ncols; c++)
        { k_gather_rows<<<grid_for(t->nrows), 256, 0, st>>>(keep, pos, t->nrows, t->cols[c], f->cols[c], t->types[c]); vs::note_launch(); }
    }
  } else {
    const vs_bitmat *m = a.mat;
    if (!only_count) {
      VS_TRY(bitmat_alloc(m->rows, m->cols, m->kind, st, &om));
      int rc = vs_bitmat_set_maps(om, m->row_map, m->col_map, stream);
      if (rc != VS_OK) {
        vs_bitmat_free(om);
        return rc;
      }
    }
    const uint64_t nw = (uint64_t)m->wpc * m->cols;
    if (nw)
      { k_probe_mat<<<grid_for(nw), 256, 0, st>>>(p, sa, m->words, m->wpc, m->rows, m->cols, m->row_map, m->col_map,
                                                 m->colnz, om ? om->words : nullptr, total); vs::note_launch(); }
    unsigned long long n = 0;
    cudaError_t e = cudaMemcpyAsync(&n, total, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      if (om) vs_bitmat_free(om);
      return cuda_fail(e, "vs_semi_join", __FILE__, __LINE__);
    }
    *count = n;
  }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    if (f) vs_flat_free(f);
    if (om) vs_bitmat_free(om);
    return cuda_fail(e, "vs_semi_join", __FILE__, __LINE__);
  }
  if (out_flat) *out_flat = f;
  if (out_mat) *out_mat = om;
  return VS_OK;
}

}  // extern "C"
