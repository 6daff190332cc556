// Vertex-id hash join: HashJoin::build / HashJoin::probe
// (src/objects/operator/join.cpp:26-449) re-designed for sm_103a.
//
// Flat x Flat: an open-addressing table in HBM (64-bit keys, linear probing,
// load factor <= 1/2) is built over the smaller side; duplicate keys inside a
// warp are merged with __match_any_sync before one atomic per distinct key, so
// Zipf-skewed keys do not serialise on one slot.  Build rows are grouped by
// key (prefix sum over slot counts + scatter); the probe counts matches per
// probe row, a prefix sum places every probe row's output, and the emit pass
// assigns output rows to threads evenly (a thread binary-searches its probe
// row inside its block's range), so hot keys do not leave one thread writing
// millions of rows.
//
// Matrix operands are relations of (row value, column value) pairs with the
// column variable as key.  Count-only joins never materialise them:
// Flat x Mat sums multiplicity(key) * popcount(column) and Mat x Mat sums
// popcount(a column) * popcount(b column) per shared key, streaming each
// matrix once.  Materialising joins with a matrix operand expand its set
// bits to pairs (TableConvert(Flat)) and run the flat join.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "dev_util.cuh"
#include "hash.cuh"
#include "vs_internal.cuh"

namespace vs {
namespace jn {

constexpr unsigned FULL = 0xffffffffu;
constexpr unsigned long long EMPTY = HT_EMPTY;
using Table = HashTable;

__device__ __forceinline__ unsigned long long load_key(const void *col, int type, uint64_t i) {
  return type == VS_T_I64 ? (unsigned long long)((const long long *)col)[i]
                          : (unsigned long long)((const uint32_t *)col)[i];
}

// Build: count rows per key.  Lanes holding the same key elect one leader
// that adds the group's size (skewed keys cost one atomic per warp).
__global__ void k_build(Table t, const void *keycol, int ktype, uint64_t n, uint32_t *slot_of) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
    const uint64_t i = i0 + threadIdx.x;
    const bool valid = i < n;
    const unsigned long long k = valid ? load_key(keycol, ktype, i) : EMPTY - 1;
    const unsigned active = __ballot_sync(FULL, valid);
    const unsigned peers = __match_any_sync(FULL, k) & active;
    if (valid) {
      const int leader = __ffs(peers) - 1;
      uint64_t slot = 0;
      if ((int)(threadIdx.x & 31) == leader) {
        slot = ht_insert(t, k);
        atomicAdd(&t.cnt[slot], (unsigned long long)__popc(peers));
      }
      slot = __shfl_sync(peers, slot, leader);
      if (slot_of) slot_of[i] = (uint32_t)slot;
    }
  }
}

// Count-only build: each block first counts its rows' keys in a table of
// its own in shared memory and adds every key's block count to the global
// table once, so a hot key costs one global atomic per block instead of one
// per warp (a Zipf-skewed key column sends most warps to the same slot).
// Keys that find no shared slot within a few probes go to the global table
// directly.
constexpr int LOC_SLOTS = 4096;
__global__ void __launch_bounds__(256) k_build_count(Table t, const void *keycol, int ktype, uint64_t n) {
  __shared__ unsigned long long s_key[LOC_SLOTS];
  __shared__ uint32_t s_cnt[LOC_SLOTS];
  for (int i = threadIdx.x; i < LOC_SLOTS; i += blockDim.x) {
    s_key[i] = EMPTY;
    s_cnt[i] = 0;
  }
  __syncthreads();
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const unsigned long long k = load_key(keycol, ktype, i);
    bool done = false;
    if (k != EMPTY) {  // the all-ones key goes straight to its reserved global slot
      uint32_t h = (uint32_t)ht_hash(k) & (LOC_SLOTS - 1);
      for (int probe = 0; probe < 8 && !done; probe++) {
        unsigned long long old = s_key[h];
        if (old == EMPTY) old = atomicCAS(&s_key[h], EMPTY, k);
        if (old == EMPTY || old == k) {
          atomicAdd(&s_cnt[h], 1u);
          done = true;
        }
        h = (h + 1) & (LOC_SLOTS - 1);
      }
    }
    if (!done) {
      const uint64_t slot = ht_insert(t, k);
      atomicAdd(&t.cnt[slot], 1ull);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < LOC_SLOTS; i += blockDim.x)
    if (s_cnt[i]) {
      const uint64_t slot = ht_insert(t, s_key[i]);
      atomicAdd(&t.cnt[slot], (unsigned long long)s_cnt[i]);
    }
}

// Build over matrix columns: key = col_map[c] (or c) -> first column index.
__global__ void k_build_cols(Table t, const uint32_t *col_map, uint32_t cols) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += gridDim.x * blockDim.x) {
    const unsigned long long k = col_map ? col_map[c] : c;
    const uint64_t s = ht_insert(t, k);
    atomicMin(&t.val[s], c);
    atomicAdd(&t.cnt[s], 1ull);
  }
}

__global__ void k_scatter(Table t, const uint32_t *slot_of, uint64_t n, uint32_t *rows_by_key) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t s = slot_of[i];
    rows_by_key[t.off[s] + atomicAdd(&t.cur[s], 1ull)] = (uint32_t)i;
  }
}

// Probe: matches per probe row (and the slot), total into *total.
__global__ void k_probe(Table t, const void *keycol, int ktype, uint64_t n,
                        unsigned long long *pcnt, uint32_t *pslot, unsigned long long *total) {
  unsigned long long s = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t slot = ht_find(t, load_key(keycol, ktype, i));
    const unsigned long long c = slot == ~0ull ? 0ull : t.cnt[slot];
    s += c;
    if (pcnt) {
      pcnt[i] = c;
      pslot[i] = (uint32_t)(slot == ~0ull ? 0 : slot);
    }
  }
  block_add(s, total);
}

// Flat x Mat count: sum over matrix columns of multiplicity(key) * popcount.
__global__ void k_count_mat(Table t, const uint64_t *__restrict__ w, uint32_t cols, uint32_t wpc,
                            const uint32_t *col_map, unsigned long long *total) {
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  unsigned long long s = 0;
  for (uint32_t c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < cols; c += warps) {
    unsigned long long m = 0;
    if (lane == 0) {
      const uint64_t slot = ht_find(t, col_map ? col_map[c] : c);
      m = slot == ~0ull ? 0ull : t.cnt[slot];
    }
    m = __shfl_sync(FULL, m, 0);
    if (!m) continue;
    unsigned long long pc = 0;
    for (uint32_t q = lane; q < wpc; q += 32) pc += __popcll(w[(size_t)c * wpc + q]);
    pc = warp_sum(pc);
    if (lane == 0) s += m * pc;
  }
  block_add(s, total);
}

// Mat x Mat count: for every column of b, the column of a with the same key.
__global__ void k_count_mat_mat(Table ta, const uint64_t *__restrict__ wa, uint32_t cols_a,
                                uint32_t wpc_a, const uint64_t *__restrict__ wb, uint32_t cols_b,
                                uint32_t wpc_b, const uint32_t *col_map_b, int direct,
                                unsigned long long *total) {
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  unsigned long long s = 0;
  for (uint32_t c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < cols_b; c += warps) {
    uint32_t ca = 0xffffffffu;
    if (direct) {
      ca = c < cols_a ? c : 0xffffffffu;
    } else if (lane == 0) {
      const uint64_t slot = ht_find(ta, col_map_b ? col_map_b[c] : c);
      ca = slot == ~0ull ? 0xffffffffu : ta.val[slot];
    }
    ca = __shfl_sync(FULL, ca, 0);
    if (ca == 0xffffffffu) continue;
    unsigned long long pa = 0, pb = 0;
    for (uint32_t q = lane; q < wpc_a; q += 32) pa += __popcll(wa[(size_t)ca * wpc_a + q]);
    for (uint32_t q = lane; q < wpc_b; q += 32) pb += __popcll(wb[(size_t)c * wpc_b + q]);
    pa = warp_sum(pa);
    pb = warp_sum(pb);
    if (lane == 0) s += pa * pb;
  }
  block_add(s, total);
}

// Mat x Mat count when neither operand has a column map (key = column index):
// a warp takes 32 columns, keeps those that may be non-zero in both, and
// popcounts each pair of columns with 16-byte loads and one warp reduction.
__global__ void __launch_bounds__(256) k_count_direct(const uint4 *__restrict__ wa, uint32_t qa,
                                                      const uint4 *__restrict__ wb, uint32_t qb, uint32_t cols,
                                                      const uint32_t *__restrict__ nza,
                                                      const uint32_t *__restrict__ nzb,
                                                      unsigned long long *total) {
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  unsigned long long s = 0;
  for (uint32_t c0 = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; c0 < cols; c0 += warps * 32) {
    const uint32_t cl = c0 + lane;
    unsigned m = __ballot_sync(FULL, cl < cols && (!nza || nza[cl]) && (!nzb || nzb[cl]));
    while (m) {
      const uint32_t c = c0 + __ffs(m) - 1;
      m &= m - 1;
      unsigned pa = 0, pb = 0;
      for (uint32_t q = lane; q < qa; q += 32) {
        const uint4 x = __ldg(wa + (size_t)c * qa + q);
        pa += __popc(x.x) + __popc(x.y) + __popc(x.z) + __popc(x.w);
      }
      for (uint32_t q = lane; q < qb; q += 32) {
        const uint4 x = __ldg(wb + (size_t)c * qb + q);
        pb += __popc(x.x) + __popc(x.y) + __popc(x.z) + __popc(x.w);
      }
      pa = __reduce_add_sync(FULL, pa);
      pb = __reduce_add_sync(FULL, pb);
      s += (unsigned long long)pa * pb;
    }
  }
  if (lane != 0) s = 0;
  block_add(s, total);
}

struct OutCol {
  void *dst;
  const void *src;
  int type;
  int side;  // 0 = probe row, 1 = build row
};

struct EmitArgs {
  OutCol col[16];
  int ncols;
  const unsigned long long *poff;  // n_probe + 1
  const uint32_t *pslot;
  const uint32_t *rows_by_key;
  Table t;
  uint64_t n_probe, out_rows;
};

// Output rows [blk*R, blk*R + R) of every block; thread -> probe row by a
// binary search of poff inside the block's probe range.
constexpr int EMIT_ROWS = 2048;

__global__ void __launch_bounds__(256) k_emit(EmitArgs a) {
  __shared__ uint64_t p_lo, p_hi;
  const uint64_t o0 = (uint64_t)blockIdx.x * EMIT_ROWS;
  if (o0 >= a.out_rows) return;
  const uint64_t o1 = min(o0 + EMIT_ROWS, a.out_rows);
  if (threadIdx.x == 0) {
    // largest p with poff[p] <= o0, and with poff[p] <= o1 - 1
    uint64_t lo = 0, hi = a.n_probe;
    while (hi - lo > 1) {
      uint64_t mid = (lo + hi) / 2;
      if (a.poff[mid] <= o0) lo = mid; else hi = mid;
    }
    p_lo = lo;
    uint64_t lo2 = lo, hi2 = a.n_probe;
    while (hi2 - lo2 > 1) {
      uint64_t mid = (lo2 + hi2) / 2;
      if (a.poff[mid] <= o1 - 1) lo2 = mid; else hi2 = mid;
    }
    p_hi = lo2;
  }
  __syncthreads();
  for (uint64_t o = o0 + threadIdx.x; o < o1; o += blockDim.x) {
    uint64_t lo = p_lo, hi = p_hi + 1;
    while (hi - lo > 1) {
      uint64_t mid = (lo + hi) / 2;
      if (a.poff[mid] <= o) lo = mid; else hi = mid;
    }
    const uint64_t p = lo;
    const uint64_t j = o - a.poff[p];
    const uint32_t s = a.pslot[p];
    const uint64_t b = a.rows_by_key[a.t.off[s] + j];
    for (int c = 0; c < a.ncols; c++) {
      const OutCol &oc = a.col[c];
      const uint64_t r = oc.side ? b : p;
      if (oc.type == VS_T_I64)
        ((long long *)oc.dst)[o] = ((const long long *)oc.src)[r];
      else
        ((uint32_t *)oc.dst)[o] = ((const uint32_t *)oc.src)[r];
    }
  }
}

struct Scratch {
  cudaStream_t st;
  void *p[12] = {};
  int n = 0;
  template <typename T> int get(T **out, size_t count) {
    int rc = dalloc_n(out, count, st);
    if (rc == VS_OK) p[n++] = *out;
    return rc;
  }
  ~Scratch() {
    for (int i = 0; i < n; i++) dfree(p[i], st);
  }
};

int table_alloc(Scratch &sc, uint64_t n_keys, bool with_val, bool with_off, Table *t) {
  t->cap = ht_capacity(std::max<uint64_t>(n_keys, 1));
  VS_TRY(sc.get(&t->keys, t->cap + 1));
  VS_TRY(sc.get(&t->cnt, t->cap + 1));
  VS_CK(cudaMemsetAsync(t->keys, 0xff, 8 * (t->cap + 1), sc.st));
  VS_CK(cudaMemsetAsync(t->cnt, 0, 8 * (t->cap + 1), sc.st));
  t->val = nullptr;
  t->off = t->cur = nullptr;
  if (with_val) {
    VS_TRY(sc.get(&t->val, t->cap + 1));
    VS_CK(cudaMemsetAsync(t->val, 0xff, 4 * (t->cap + 1), sc.st));
  }
  if (with_off) {
    VS_TRY(sc.get(&t->off, t->cap + 2));
    VS_TRY(sc.get(&t->cur, t->cap + 1));
    VS_CK(cudaMemsetAsync(t->cur, 0, 8 * (t->cap + 1), sc.st));
  }
  return VS_OK;
}

int grid_for(uint64_t n, int per_block = 256) {
  return (int)std::max<uint64_t>(1, std::min<uint64_t>((n + per_block - 1) / per_block,
                                                       (uint64_t)sm_count() * 16));
}

int read_total(unsigned long long *d, uint64_t *h, cudaStream_t st) {
  unsigned long long x = 0;
  VS_CK(cudaMemcpyAsync(&x, d, sizeof(x), cudaMemcpyDeviceToHost, st));
  VS_CK(cudaStreamSynchronize(st));
  *h = x;
  return VS_OK;
}

// A flat operand: columns + key column.
struct FlatSide {
  const vs_flat *f;
  uint32_t key;
};

// Flat x Flat join.  a = deps[0], b = deps[1]; result = a cols + b non-key cols.
int join_flat_flat(FlatSide a, FlatSide b, bool only_count, uint64_t max_rows, vs_flat **out,
                   uint64_t *count, cudaStream_t st) {
  if (a.f->types[a.key] != b.f->types[b.key])
    return fail(VS_ERR_ARG, "join key types differ (%d vs %d)", a.f->types[a.key], b.f->types[b.key]);
  // GPU build side: the smaller table (the reference builds on the larger,
  // join.cpp:39-43; the side only changes the output order)
  const bool build_a = a.f->nrows < b.f->nrows;
  const FlatSide &bd = build_a ? a : b, &pr = build_a ? b : a;
  Scratch sc{st};
  Table t;
  VS_TRY(table_alloc(sc, bd.f->nrows, false, !only_count, &t));
  uint32_t *slot_of = nullptr;
  if (!only_count) VS_TRY(sc.get(&slot_of, bd.f->nrows));
  if (bd.f->nrows && only_count)
    { k_build_count<<<std::min(grid_for(bd.f->nrows), 4 * sm_count()), 256, 0, st>>>(
          t, bd.f->cols[bd.key], bd.f->types[bd.key], bd.f->nrows); vs::note_launch(); }
  else if (bd.f->nrows)
    { k_build<<<grid_for(bd.f->nrows), 256, 0, st>>>(t, bd.f->cols[bd.key], bd.f->types[bd.key],
                                                   bd.f->nrows, slot_of); vs::note_launch(); }
  unsigned long long *d_total;
  VS_TRY(sc.get(&d_total, 1));
  VS_CK(cudaMemsetAsync(d_total, 0, 8, st));
  if (only_count) {
    if (pr.f->nrows)
      { k_probe<<<grid_for(pr.f->nrows), 256, 0, st>>>(t, pr.f->cols[pr.key], pr.f->types[pr.key],
                                                     pr.f->nrows, nullptr, nullptr, d_total); vs::note_launch(); }
    VS_CK(cudaGetLastError());
    return read_total(d_total, count, st);
  }
  // group build rows by key
  VS_TRY(exclusive_scan_u64(t.cnt, t.off, t.cap + 1, st));
  uint32_t *rows_by_key;
  VS_TRY(sc.get(&rows_by_key, bd.f->nrows));
  if (bd.f->nrows) { k_scatter<<<grid_for(bd.f->nrows), 256, 0, st>>>(t, slot_of, bd.f->nrows, rows_by_key); vs::note_launch(); }
  unsigned long long *pcnt, *poff;
  uint32_t *pslot;
  VS_TRY(sc.get(&pcnt, pr.f->nrows));
  VS_TRY(sc.get(&poff, pr.f->nrows + 1));
  VS_TRY(sc.get(&pslot, pr.f->nrows));
  if (pr.f->nrows)
    { k_probe<<<grid_for(pr.f->nrows), 256, 0, st>>>(t, pr.f->cols[pr.key], pr.f->types[pr.key],
                                                   pr.f->nrows, pcnt, pslot, d_total); vs::note_launch(); }
  VS_TRY(exclusive_scan_u64(pcnt, poff, pr.f->nrows, st));
  uint64_t total = 0;
  VS_TRY(read_total(d_total, &total, st));
  *count = total;
  const uint64_t rows = std::min<uint64_t>(total, max_rows);
  // result schema: a's columns, then b's non-key columns
  int32_t types[16];
  EmitArgs ea{};
  int nc = 0;
  for (uint32_t i = 0; i < a.f->ncols; i++) {
    types[nc] = a.f->types[i];
    ea.col[nc].src = a.f->cols[i];
    ea.col[nc].type = a.f->types[i];
    ea.col[nc].side = build_a ? 1 : 0;
    nc++;
  }
  for (uint32_t i = 0; i < b.f->ncols; i++) {
    if (i == b.key) continue;
    if (nc >= 16) return fail(VS_ERR_UNSUPPORTED, "join result wider than 16 columns");
    types[nc] = b.f->types[i];
    ea.col[nc].src = b.f->cols[i];
    ea.col[nc].type = b.f->types[i];
    ea.col[nc].side = build_a ? 0 : 1;
    nc++;
  }
  vs_flat *f = nullptr;
  VS_TRY(flat_alloc(nc, types, rows, st, &f));
  for (int i = 0; i < nc; i++) ea.col[i].dst = f->cols[i];
  ea.ncols = nc;
  ea.poff = poff;
  ea.pslot = pslot;
  ea.rows_by_key = rows_by_key;
  ea.t = t;
  ea.n_probe = pr.f->nrows;
  ea.out_rows = rows;
  if (rows) { k_emit<<<(unsigned)((rows + EMIT_ROWS - 1) / EMIT_ROWS), 256, 0, st>>>(ea); vs::note_launch(); }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    vs_flat_free(f);
    return cuda_fail(e, "hash join", __FILE__, __LINE__);
  }
  *out = f;
  return total > max_rows ? fail(VS_ERR_CAPACITY, "join produced %llu rows, bound %llu",
                                 (unsigned long long)total, (unsigned long long)max_rows)
                          : VS_OK;
}

// Count-only Flat x Mat: the flat side's multiplicities against column popcounts.
int count_flat_mat(FlatSide f, const vs_bitmat *m, uint64_t *count, cudaStream_t st) {
  if (f.f->types[f.key] != VS_T_VID) return fail(VS_ERR_ARG, "matrix keys are VIDs; flat key is not");
  Scratch sc{st};
  Table t;
  VS_TRY(table_alloc(sc, f.f->nrows, false, false, &t));
  if (f.f->nrows)
    { k_build<<<grid_for(f.f->nrows), 256, 0, st>>>(t, f.f->cols[f.key], VS_T_VID, f.f->nrows, nullptr); vs::note_launch(); }
  unsigned long long *d_total;
  VS_TRY(sc.get(&d_total, 1));
  VS_CK(cudaMemsetAsync(d_total, 0, 8, st));
  if (m->cols)
    { k_count_mat<<<grid_for((uint64_t)m->cols * 32), 256, 0, st>>>(t, m->words, m->cols, m->wpc,
                                                                 m->col_map, d_total); vs::note_launch(); }
  VS_CK(cudaGetLastError());
  return read_total(d_total, count, st);
}

int count_mat_mat(const vs_bitmat *a, const vs_bitmat *b, uint64_t *count, cudaStream_t st) {
  Scratch sc{st};
  Table t{};
  const bool direct = !a->col_map && !b->col_map;
  if (direct) {
    unsigned long long *d_total;
    VS_TRY(sc.get(&d_total, 1));
    VS_CK(cudaMemsetAsync(d_total, 0, 8, st));
    const uint32_t cols = std::min(a->cols, b->cols);
    if (cols)
      { k_count_direct<<<grid_for(cols), 256, 0, st>>>(reinterpret_cast<const uint4 *>(a->words), a->wpc / 2,
                                                      reinterpret_cast<const uint4 *>(b->words), b->wpc / 2, cols,
                                                      a->colnz, b->colnz, d_total); vs::note_launch(); }
    VS_CK(cudaGetLastError());
    return read_total(d_total, count, st);
  }
  {
    VS_TRY(table_alloc(sc, a->cols, true, false, &t));
    if (a->cols) { k_build_cols<<<grid_for(a->cols), 256, 0, st>>>(t, a->col_map, a->cols); vs::note_launch(); }
  }
  unsigned long long *d_total;
  VS_TRY(sc.get(&d_total, 1));
  VS_CK(cudaMemsetAsync(d_total, 0, 8, st));
  if (b->cols)
    { k_count_mat_mat<<<grid_for((uint64_t)b->cols * 32), 256, 0, st>>>(
        t, a->words, a->cols, a->wpc, b->words, b->cols, b->wpc, b->col_map, direct ? 1 : 0, d_total); vs::note_launch(); }
  VS_CK(cudaGetLastError());
  return read_total(d_total, count, st);
}

}  // namespace jn
}  // namespace vs

// ---------------------------------------------------------------------------
// Allocation-free count-only join.  Its hash table lives in this file-scope
// device array instead of allocated memory; every GPU that loads the library
// holds the array until the process exits.
namespace vs {
namespace jn {

constexpr uint64_t NOALLOC_SLOTS = 1ull << 19;              // hash slots (power of two)
constexpr uint64_t NOALLOC_MAX_BUILD = NOALLOC_SLOTS / 2;   // load factor <= 1/2
// keys [SLOTS + 1] | counts [SLOTS + 1] | total [1]   (8 MiB + 24 B)
constexpr uint64_t NOALLOC_WORDS = 2 * (NOALLOC_SLOTS + 1) + 1;
static __device__ __align__(256) unsigned long long g_noalloc_scratch[NOALLOC_WORDS];

// Device address of the array, looked up once per device with that device
// current (host code may not use the symbol itself as a device pointer).  A
// cached address is checked against the runtime before use: after
// cudaDeviceReset the device's context, and with it the array, is new, and
// the address is looked up again.
int noalloc_scratch(unsigned long long **out) {
  static std::mutex mu;
  static unsigned long long *addr[128] = {};
  int dev = 0;
  VS_CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 128) return fail(VS_ERR_UNSUPPORTED, "device index %d out of range", dev);
  std::lock_guard<std::mutex> lock(mu);
  if (addr[dev]) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, addr[dev]) != cudaSuccess || at.type != cudaMemoryTypeDevice ||
        at.device != dev) {
      cudaGetLastError();  // a stale address is not an error of this call
      addr[dev] = nullptr;
    }
  }
  if (!addr[dev]) {
    void *p = nullptr;
    VS_CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    addr[dev] = static_cast<unsigned long long *>(p);
  }
  *out = addr[dev];
  return VS_OK;
}

// The previous call's table is still in the array: reset the slots this
// call uses (keys to empty, counts and the total to zero).
__global__ void k_noalloc_clear(unsigned long long *keys, unsigned long long *cnt,
                                unsigned long long *total, uint64_t cap) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= cap;
       i += (uint64_t)gridDim.x * blockDim.x) {
    keys[i] = EMPTY;
    cnt[i] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *total = 0;
}

// ---------------------------------------------------------------------------
// Batched join counts over the row blocks of one matrix (batched expand
// results): blockIdx.y is the row block; its warps take chunks of RB_CHUNK
// keys in turn.  A key's column slice of the block (nw words) is read by a
// group of G = min(32, pow2 >= nw) lanes, so narrow blocks put several keys
// in one warp.  The table of blocks travels as a kernel parameter.
constexpr int RB_CHUNK = 256;
struct RowBlocks {
  vs_row_block b[VS_MAX_ROW_BLOCKS];
};

__global__ void __launch_bounds__(256) k_count_row_blocks(const __grid_constant__ RowBlocks tab,
                                                          const uint32_t *__restrict__ keys,
                                                          const uint64_t *__restrict__ w, uint32_t wpc,
                                                          uint32_t cols, const uint32_t *__restrict__ colnz,
                                                          unsigned long long *__restrict__ counts) {
  const vs_row_block rb = tab.b[blockIdx.y];
  if (rb.row_end <= rb.row_begin || rb.key_end <= rb.key_begin) return;
  const uint32_t w0 = rb.row_begin >> 6, nw = ((rb.row_end - 1) >> 6) - w0 + 1;
  const uint64_t m_first = ~0ull << (rb.row_begin & 63);
  const uint64_t m_last = ~0ull >> (63 - ((rb.row_end - 1) & 63));
  uint32_t G = 1;
  while (G < 32 && G < nw) G <<= 1;
  const uint32_t lane = threadIdx.x & 31, grp = lane / G, gl = lane % G, ngrp = 32 / G;
  const uint64_t nkeys = rb.key_end - rb.key_begin;
  const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  const uint32_t *kp = keys + rb.key_begin;
  unsigned long long s = 0;
  for (uint64_t base = ((uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * RB_CHUNK;
       base < nkeys; base += nwarps * RB_CHUNK) {
    const uint64_t end = min(base + RB_CHUNK, nkeys);
    for (uint64_t k = base + grp; k < end; k += ngrp) {
      const uint32_t key = __ldg(kp + k);
      if (key >= cols || (colnz && !__ldg(colnz + key))) continue;  // no such vertex / empty column
      const uint64_t *col = w + (size_t)key * wpc + w0;
      for (uint32_t j = gl; j < nw; j += G) {
        uint64_t x = __ldg(col + j);
        if (j == 0) x &= m_first;
        if (j == nw - 1) x &= m_last;
        s += __popcll(x);
      }
    }
  }
  block_add(s, counts + blockIdx.y);
}

}  // namespace jn
}  // namespace vs

using namespace vs;
using namespace vs::jn;

extern "C" {

int vs_hash_join(vs_table_ref a, vs_table_ref b, int only_count, uint64_t max_rows,
                 vs_flat **out, uint64_t *count, vs_stream_t stream) {
  if (!count || (!only_count && !out)) return fail(VS_ERR_ARG, "vs_hash_join: null output");
  if ((!a.flat == !a.mat) || (!b.flat == !b.mat))
    return fail(VS_ERR_ARG, "each join operand is exactly one of a flat table or a matrix");
  cudaStream_t st = S(stream);
  if (out) *out = nullptr;
  *count = 0;
  for (const vs_table_ref *r : {&a, &b}) {
    if (r->flat && r->key_col >= r->flat->ncols) return fail(VS_ERR_ARG, "key column out of range");
    // a matrix joins on its column variable (join.cpp:49-71 assert the key is column 1)
    if (r->mat && r->key_col != 1) return fail(VS_ERR_ARG, "a matrix operand joins on column 1");
  }
  if (only_count) {
    if (a.flat && b.flat) return join_flat_flat({a.flat, a.key_col}, {b.flat, b.key_col}, true, 0, nullptr, count, st);
    if (a.flat && b.mat) return count_flat_mat({a.flat, a.key_col}, b.mat, count, st);
    if (a.mat && b.flat) return count_flat_mat({b.flat, b.key_col}, a.mat, count, st);
    return count_mat_mat(a.mat, b.mat, count, st);
  }
  // materialise: matrix operands become (row value, key) pair tables
  vs_flat *fa = nullptr, *fb = nullptr;
  int rc = VS_OK;
  if (a.mat && (rc = bitmat_to_flat(a.mat, st, &fa)) != VS_OK) return rc;
  if (b.mat && (rc = bitmat_to_flat(b.mat, st, &fb)) != VS_OK) {
    vs_flat_free(fa);
    return rc;
  }
  FlatSide sa{a.flat ? a.flat : fa, a.flat ? a.key_col : 1u};
  FlatSide sb{b.flat ? b.flat : fb, b.flat ? b.key_col : 1u};
  rc = join_flat_flat(sa, sb, false, max_rows, out, count, st);
  cudaStreamSynchronize(st);
  vs_flat_free(fa);
  vs_flat_free(fb);
  return rc;
}


// Count-only join without allocating (see the header): the smaller key column
// is the build side; at most NOALLOC_MAX_BUILD rows.
int vs_hash_join_count_noalloc(const void *keys_a, uint64_t na, const void *keys_b, uint64_t nb,
                               int key_type, uint64_t *count, vs_stream_t stream) {
  if (!count || (na && !keys_a) || (nb && !keys_b))
    return fail(VS_ERR_ARG, "vs_hash_join_count_noalloc: null argument");
  if (key_type != VS_T_VID && key_type != VS_T_I64)
    return fail(VS_ERR_ARG, "vs_hash_join_count_noalloc: unknown key type %d", key_type);
  // the kernels read the keys directly: a host pointer is refused before any launch
  for (const void *p : {na ? keys_a : nullptr, nb ? keys_b : nullptr}) {
    if (!p) continue;
    cudaPointerAttributes at{};
    VS_CK(cudaPointerGetAttributes(&at, p));
    if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
      return fail(VS_ERR_ARG, "vs_hash_join_count_noalloc: keys_a and keys_b must be device memory");
  }
  const bool build_a = na < nb;
  const void *bk = build_a ? keys_a : keys_b, *pk = build_a ? keys_b : keys_a;
  const uint64_t nbld = build_a ? na : nb, nprb = build_a ? nb : na;
  if (nbld > NOALLOC_MAX_BUILD)
    return fail(VS_ERR_CAPACITY,
                "vs_hash_join_count_noalloc: the smaller side has %llu rows; the fixed table holds at most "
                "%llu (use vs_hash_join)",
                (unsigned long long)nbld, (unsigned long long)NOALLOC_MAX_BUILD);
  unsigned long long *base = nullptr;
  VS_TRY(noalloc_scratch(&base));
  cudaStream_t st = S(stream);
  Table t{};
  t.cap = ht_capacity(std::max<uint64_t>(nbld, 1));
  t.keys = base;
  t.cnt = base + (NOALLOC_SLOTS + 1);
  unsigned long long *total = base + 2 * (NOALLOC_SLOTS + 1);
  { k_noalloc_clear<<<grid_for(t.cap + 1), 256, 0, st>>>(t.keys, t.cnt, total, t.cap); vs::note_launch(); }
  if (nbld) { k_build<<<grid_for(nbld), 256, 0, st>>>(t, bk, key_type, nbld, nullptr); vs::note_launch(); }
  if (nprb) { k_probe<<<grid_for(nprb), 256, 0, st>>>(t, pk, key_type, nprb, nullptr, nullptr, total); vs::note_launch(); }
  VS_CK(cudaGetLastError());
  VS_CK(cudaMemcpyAsync(count, total, sizeof(unsigned long long), cudaMemcpyDefault, st));
  VS_CK(cudaStreamSynchronize(st));
  return VS_OK;
}

int vs_hash_join_count_row_blocks(const vs_bitmat *m, const uint32_t *keys, const vs_row_block *blocks,
                                  uint32_t nblocks, uint64_t *counts, vs_stream_t stream) {
  if (!m || !blocks || !counts || nblocks == 0)
    return fail(VS_ERR_ARG, "vs_hash_join_count_row_blocks: null argument or no block");
  if (nblocks > VS_MAX_ROW_BLOCKS)
    return fail(VS_ERR_ARG, "%u row blocks; at most %d per call", nblocks, VS_MAX_ROW_BLOCKS);
  if (m->kind != VS_KIND_VARROW || m->col_map)
    return fail(VS_ERR_ARG, "row-block join counts need a VarRow matrix whose columns are vertex ids");
  RowBlocks tab{};
  uint64_t max_keys = 0;
  for (uint32_t q = 0; q < nblocks; q++) {
    const vs_row_block &b = blocks[q];
    if (b.row_begin > b.row_end || b.row_end > m->rows || b.key_begin > b.key_end)
      return fail(VS_ERR_ARG, "row block %u: rows [%u, %u) of %u, keys [%llu, %llu)", q, b.row_begin,
                  b.row_end, m->rows, (unsigned long long)b.key_begin, (unsigned long long)b.key_end);
    tab.b[q] = b;
    max_keys = std::max<uint64_t>(max_keys, b.key_end - b.key_begin);
  }
  if (max_keys && !keys) return fail(VS_ERR_ARG, "vs_hash_join_count_row_blocks: null keys");
  for (const void *p : {(const void *)keys, (const void *)counts}) {
    if (!p) continue;
    cudaPointerAttributes at{};
    VS_CK(cudaPointerGetAttributes(&at, p));
    if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
      return fail(VS_ERR_ARG, "vs_hash_join_count_row_blocks: keys and counts must be device memory");
  }
  cudaStream_t st = S(stream);
  VS_CK(cudaMemsetAsync(counts, 0, sizeof(uint64_t) * nblocks, st));
  if (max_keys == 0 || m->rows == 0) return VS_OK;
  const uint64_t warps_needed = (max_keys + RB_CHUNK - 1) / RB_CHUNK;
  const uint32_t gx = (uint32_t)std::min<uint64_t>((warps_needed + 7) / 8, (uint64_t)sm_count() * 8);
  { k_count_row_blocks<<<dim3(gx, nblocks), 256, 0, st>>>(tab, keys, m->words, m->wpc, m->cols, m->colnz,
                                                          reinterpret_cast<unsigned long long *>(counts));
    vs::note_launch(); }
  VS_CK(cudaGetLastError());
  return VS_OK;
}

}  // extern "C"
