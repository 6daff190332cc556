// Multi-way intersection: Mintersect (src/objects/operator/mintersect.cpp:14-345)
// re-designed for sm_103a.
//
// A warp owns one base tuple.  Each dependency yields, for the vertex u the
// tuple holds in that dependency's base column, a set of new vertices:
//   matrix     column u of a ColMain matrix (rows = new vertices); when every
//              dependency is a matrix the warp ANDs the columns word by word,
//              popcounts and extracts the bits (the reference's and_col_from +
//              count_bits_in_col + BitmapIterator, mintersect.cpp:244-333);
//   adjacency  u's sorted out-list in the graph CSR;
//   flat       the (u, new) pairs of a flat edge table, grouped by u on the
//              device (counting sort) and de-duplicated through a pair hash set.
// With a list dependency the warp walks the shortest list (32 candidates per
// step) and tests each candidate against the others: pair-hash lookup for
// flat tables, one bit load for matrices, and for sorted adjacency one of
//   bitmap   one bit load in the list vertex's adjacency bitmap (hubs only),
//   merge    a warp-wide window of 32 list entries slides forward with the
//            candidates; each candidate finds its place by a shuffle search,
//   binary   a binary search of the whole list,
// chosen per base tuple (bitmap when the list's vertex has one, merge for two
// long lists of similar length, else binary search), fixed by the caller, or
// chosen per call by a trained network (k_isect_decide).
// Counting and emitting are two passes over the same code; a prefix sum of
// the per-tuple counts places every tuple's output.
#include <algorithm>
#include <cstring>

#include "dev_util.cuh"
#include "hash.cuh"
#include "picker.cuh"
#include "vs_internal.cuh"

namespace vs {
namespace is {

enum { DEP_MAT = 0, DEP_SORTED = 1, DEP_HASHED = 2 };
enum { M_OTHER = 0, M_BINARY = 1, M_MERGE = 2, M_BITMAP = 3 };
constexpr int MAX_DEPS = 8;
constexpr uint32_t HUB_MIN_DEG = 1024;           // adjacency bitmaps only for lists this long
constexpr uint64_t HUB_BUDGET = 1ull << 30;      // bitmap bytes per graph and direction

struct Dep {
  int kind;
  const uint32_t *base_u;  // base column holding u
  // matrix
  const uint64_t *words;
  uint32_t wpc, rows, cols;
  int has_cmap;
  HashTable cmap;  // col value -> first column (val)
  // lists
  const int64_t *off;
  const uint32_t *adj;
  uint64_t n_u;
  HashTable pairs;  // DEP_HASHED: (u << 32 | new) membership
  // DEP_SORTED: membership method (VS_ISECT_*) and hub bitmaps
  int algo;
  const int32_t *hub_slot;
  const uint64_t *hub_bm;
  uint32_t hub_words;
};

struct OutCol {
  void *dst;
  const void *src;
  int type;
};

struct Args {
  Dep dep[MAX_DEPS];
  int ndeps, all_mat, emit;
  uint64_t nbase;
  uint32_t cache_rows;
  const uint32_t *target_row_map;
  unsigned long long *tcnt, *total;
  const unsigned long long *toff;
  uint64_t max_rows;
  OutCol col[16];
  int nbcols;
  uint32_t *out_new;
  const int *method;  // learned method for AUTO adjacency deps (VS_ISECT_*), or NULL
  unsigned long long *next;  // work queue head: next base tuple to hand out (zeroed per launch)
};

constexpr int ISECT_CHUNK = 4;  // base tuples a warp takes from the queue at a time

__device__ __forceinline__ bool in_sorted(const uint32_t *a, int64_t lo, int64_t hi, uint32_t x) {
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    const uint32_t v = a[mid];
    if (v == x) return true;
    if (v < x)
      lo = mid + 1;
    else
      hi = mid;
  }
  return false;
}

__device__ __forceinline__ void emit_row(const Args &a, uint64_t t, uint64_t pos, uint32_t x) {
  if (pos >= a.max_rows) return;
  for (int c = 0; c < a.nbcols; c++) {
    const OutCol &oc = a.col[c];
    if (oc.type == VS_T_I64)
      ((long long *)oc.dst)[pos] = ((const long long *)oc.src)[t];
    else
      ((uint32_t *)oc.dst)[pos] = ((const uint32_t *)oc.src)[t];
  }
  a.out_new[pos] = a.target_row_map ? a.target_row_map[x] : x;
}

// Base tuples differ by orders of magnitude in cost (hub lists), so warps
// take small chunks from a queue instead of a fixed stride, and each warp adds
// its count on its own (no block-wide barrier waiting for the slowest warp).
__global__ void __launch_bounds__(256) k_isect(Args a) {
  const int lane = threadIdx.x & 31;
  unsigned long long tot = 0;
  for (;;) {
  unsigned long long t0 = 0;
  if (lane == 0) t0 = atomicAdd(a.next, (unsigned long long)ISECT_CHUNK);
  t0 = __shfl_sync(FULLMASK, t0, 0);
  if (t0 >= a.nbase) break;
  const uint64_t t1 = t0 + ISECT_CHUNK < a.nbase ? t0 + ISECT_CHUNK : a.nbase;
  for (uint64_t t = t0; t < t1; t++) {
    uint32_t col[MAX_DEPS];
    int64_t lo[MAX_DEPS], hi[MAX_DEPS];
    uint32_t uu[MAX_DEPS];
    bool empty = false;
    int best = -1;
    int64_t best_len = 0;
#pragma unroll
    for (int i = 0; i < MAX_DEPS; i++) {
      if (i >= a.ndeps) break;
      const Dep &d = a.dep[i];
      const uint32_t u = d.base_u[t];
      uu[i] = u;
      col[i] = 0;
      lo[i] = hi[i] = 0;
      if (d.kind == DEP_MAT) {
        if (d.has_cmap) {
          const uint64_t s = ht_find(d.cmap, u);
          if (s == ~0ull)
            empty = true;
          else
            col[i] = d.cmap.val[s];
        } else if (u < d.cols) {
          col[i] = u;
        } else {
          empty = true;
        }
      } else {
        if (u < d.n_u) {
          lo[i] = d.off[u];
          hi[i] = d.off[u + 1];
        }
        if (lo[i] == hi[i]) empty = true;
        if (best < 0 || hi[i] - lo[i] < best_len) {
          best = i;
          best_len = hi[i] - lo[i];
        }
      }
    }
    unsigned long long count = 0;
    const unsigned long long base_pos = a.emit ? a.toff[t] : 0ull;
    if (!empty && a.all_mat) {
      const uint32_t lw = (a.cache_rows + 63) / 64;
      for (uint32_t q0 = 0; q0 < lw; q0 += 32) {
        const uint32_t q = q0 + lane;
        uint64_t w = 0;
        if (q < lw) {
          w = ~0ull;
          for (int i = 0; i < a.ndeps; i++) w &= a.dep[i].words[(size_t)col[i] * a.dep[i].wpc + q];
          if (q == lw - 1 && (a.cache_rows & 63)) w &= (1ull << (a.cache_rows & 63)) - 1;
        }
        const unsigned n = __popcll(w);
        unsigned incl = n;
        for (int o = 1; o < 32; o <<= 1) {
          const unsigned y = __shfl_up_sync(FULLMASK, incl, o);
          if (lane >= o) incl += y;
        }
        if (a.emit) {
          uint64_t pos = base_pos + count + incl - n;
          while (w) {
            const uint32_t x = q * 64 + (__ffsll((long long)w) - 1);
            w &= w - 1;
            emit_row(a, t, pos++, x);
          }
        }
        count += __shfl_sync(FULLMASK, incl, 31);
      }
    } else if (!empty) {
      const int learned = a.method ? *a.method : VS_ISECT_AUTO;
      // membership method per dependency for this tuple (warp-uniform)
      int meth[MAX_DEPS];
      int64_t cur[MAX_DEPS];
      int32_t hs[MAX_DEPS];
#pragma unroll
      for (int i = 0; i < MAX_DEPS; i++) {
        meth[i] = M_OTHER;
        cur[i] = 0;
        hs[i] = -1;
        if (i >= a.ndeps) break;
        const Dep &d = a.dep[i];
        if (d.kind != DEP_SORTED || i == best) continue;
        const int64_t len = hi[i] - lo[i];
        const int32_t slot = d.hub_slot ? __ldg(d.hub_slot + uu[i]) : -1;
        cur[i] = lo[i];
        hs[i] = slot;
        const int algo = d.algo == VS_ISECT_AUTO ? learned : d.algo;
        if (algo == VS_ISECT_BINARY)
          meth[i] = M_BINARY;
        else if (algo == VS_ISECT_MERGE)
          meth[i] = M_MERGE;
        else if (algo == VS_ISECT_BITMAP)
          meth[i] = slot >= 0 ? M_BITMAP : M_BINARY;
        else  // measured on GB300: a bitmap probe wins whenever one exists; merging pays only for long lists of similar length
          meth[i] = slot >= 0 ? M_BITMAP : (best_len >= 512 && len <= 4 * best_len) ? M_MERGE : M_BINARY;
      }
      const Dep &L = a.dep[best];
      for (int64_t j0 = lo[best]; j0 < hi[best]; j0 += 32) {
        const int64_t j = j0 + lane;
        const bool valid = j < hi[best];
        const uint32_t x = valid ? L.adj[j] : 0xffffffffu;
        bool keep = valid && x < a.cache_rows;
        // the chunk's candidates ascend with the lane: its largest is the last valid lane's
        const uint32_t cmax = __reduce_max_sync(FULLMASK, valid ? x : 0u);
#pragma unroll
        for (int i = 0; i < MAX_DEPS; i++) {
          if (i >= a.ndeps) break;
          if (i == best) continue;
          const Dep &d = a.dep[i];
          if (meth[i] == M_MERGE) {  // all lanes: windows of 32 list entries from the cursor on
            bool found = false;
            for (;;) {
              const int64_t p = cur[i];
              if (p >= hi[i]) break;
              const uint32_t y = p + lane < hi[i] ? __ldg(d.adj + p + lane) : 0xffffffffu;
              int pos = 0;  // first window entry >= x (31 when all are smaller)
#pragma unroll
              for (int step = 16; step; step >>= 1)
                if (__shfl_sync(FULLMASK, y, pos + step - 1) < x) pos += step;
              found |= __shfl_sync(FULLMASK, y, pos) == x;
              if (__shfl_sync(FULLMASK, y, 31) >= cmax) break;  // later candidates start in this window
              cur[i] = p + 32;
            }
            keep = keep && found;
          } else if (keep) {
            if (d.kind == DEP_MAT) {
              keep = x < d.rows && ((d.words[(size_t)col[i] * d.wpc + (x >> 6)] >> (x & 63)) & 1ull);
            } else if (meth[i] == M_BITMAP) {
              keep = (__ldg(d.hub_bm + (size_t)hs[i] * d.hub_words + (x >> 6)) >> (x & 63)) & 1ull;
            } else if (d.kind == DEP_SORTED) {
              keep = in_sorted(d.adj, lo[i], hi[i], x);
            } else {
              keep = ht_find(d.pairs, ((unsigned long long)uu[i] << 32) | x) != ~0ull;
            }
          }
        }
        const unsigned m = __ballot_sync(FULLMASK, keep);
        if (a.emit && keep) emit_row(a, t, base_pos + count + __popc(m & lanemask_lt()), x);
        count += __popc(m);
      }
    }
    if (!a.emit && lane == 0) {
      if (a.tcnt) a.tcnt[t] = count;
      tot += count;
    }
  }
  }
  if (!a.emit && lane == 0 && tot) atomicAdd(a.total, tot);
}

// Count-only intersection of two sorted adjacency dependencies (triangle
// closing, the pattern query's T), in two kernels.
//
// k_isect_pair_count: a warp takes 32 base tuples at a time, lane j loading
// tuple j's two list bounds, so the tuples' dependent loads overlap.  The
// candidates of the walked (shorter) lists of up to PAIR_INLINE entries are
// laid end to end and dealt one per lane per round, so short lists leave no
// lane idle; a lane finds its candidate's tuple by a shuffle search over the
// lanes' first candidate positions.  A longer walk is cut into pieces of
// PAIR_PIECE candidates listed for the second kernel, so the 32 neighbours of
// a hub in one chunk do not make one warp the critical path.
// k_isect_pair_pieces: a warp per piece.
// Either tests a candidate against the other list with one bit of that
// vertex's adjacency bitmap where it has one (and the method allows), else a
// binary search.  When the piece list is full the caller reruns the general
// kernel; the count always equals the general kernel's.
constexpr int PAIR_INLINE = 64;
constexpr int PAIR_PIECE = 256;

struct PairTuple {
  int64_t wlo, wn, olo, ohi;  // walked list [wlo, wlo + wn) of dep w1, other list [olo, ohi)
  int w1, hs;                 // hs: the other vertex's bitmap slot (-1: binary search)
};

__device__ __forceinline__ PairTuple pair_tuple(const Args &a, uint64_t t, int learned) {
  const Dep &d0 = a.dep[0], &d1 = a.dep[1];
  PairTuple p{0, 0, 0, 0, 0, -1};
  const uint32_t u0 = d0.base_u[t], u1 = d1.base_u[t];
  int64_t lo0 = 0, hi0 = 0, lo1 = 0, hi1 = 0;
  if (u0 < d0.n_u) {
    lo0 = d0.off[u0];
    hi0 = d0.off[u0 + 1];
  }
  if (u1 < d1.n_u) {
    lo1 = d1.off[u1];
    hi1 = d1.off[u1 + 1];
  }
  if (lo0 < hi0 && lo1 < hi1) {
    p.w1 = hi1 - lo1 < hi0 - lo0;  // the shorter list; dep 0 on a tie, as the general kernel
    const Dep &o = p.w1 ? d0 : d1;
    p.wlo = p.w1 ? lo1 : lo0;
    p.wn = p.w1 ? hi1 - lo1 : hi0 - lo0;
    p.olo = p.w1 ? lo0 : lo1;
    p.ohi = p.w1 ? hi0 : hi1;
    const int algo = o.algo == VS_ISECT_AUTO ? learned : o.algo;
    if (o.hub_slot && algo != VS_ISECT_BINARY) p.hs = __ldg(o.hub_slot + (p.w1 ? u0 : u1));
  }
  return p;
}

// Candidate x of a walked list in the other list of its tuple.
__device__ __forceinline__ bool pair_member(const Args &a, int w1, int hs, int64_t olo, int64_t ohi, uint32_t x) {
  if (x >= a.cache_rows) return false;
  const Dep &o = w1 ? a.dep[0] : a.dep[1];
  return hs >= 0 ? ((__ldg(o.hub_bm + (size_t)hs * o.hub_words + (x >> 6)) >> (x & 63)) & 1ull)
                 : in_sorted(o.adj, olo, ohi, x);
}

__global__ void __launch_bounds__(256) k_isect_pair_count(Args a, ulonglong2 *pieces, uint64_t piece_cap,
                                                          unsigned long long *piece_n, int *overflow) {
  const int lane = threadIdx.x & 31;
  const int learned = a.method ? *a.method : VS_ISECT_AUTO;
  unsigned long long cnt = 0;
  for (;;) {
    unsigned long long t0 = 0;
    if (lane == 0) t0 = atomicAdd(a.next, 32ull);
    t0 = __shfl_sync(FULLMASK, t0, 0);
    if (t0 >= a.nbase) break;
    const uint64_t t = t0 + lane;
    PairTuple p{0, 0, 0, 0, 0, -1};
    if (t < a.nbase) p = pair_tuple(a, t, learned);
    if (p.wn > PAIR_INLINE) {  // a long walk: its pieces go to the second kernel
      const uint64_t np = (uint64_t)(p.wn + PAIR_PIECE - 1) / PAIR_PIECE;
      const unsigned long long b = atomicAdd(piece_n, (unsigned long long)np);
      if (b + np <= piece_cap) {
        for (uint64_t k = 0; k < np; k++) pieces[b + k] = make_ulonglong2(t, k * PAIR_PIECE);
      } else {
        *overflow = 1;
      }
      p.wn = 0;
    }
    unsigned long long incl = (unsigned long long)p.wn;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(FULLMASK, incl, o);
      if (lane >= o) incl += y;
    }
    const unsigned long long total = __shfl_sync(FULLMASK, incl, 31);
    const unsigned long long start = incl - (unsigned long long)p.wn;
    for (unsigned long long c0 = 0; c0 < total; c0 += 32) {
      const unsigned long long c = c0 + lane;
      int own = 0;  // the last lane whose first candidate is at or below c (it owns c when c < total)
#pragma unroll
      for (int step = 16; step; step >>= 1)
        if (__shfl_sync(FULLMASK, start, own + step) <= c) own += step;
      const unsigned long long ost = __shfl_sync(FULLMASK, start, own);
      const int64_t owlo = __shfl_sync(FULLMASK, p.wlo, own);
      const int64_t oolo = __shfl_sync(FULLMASK, p.olo, own);
      const int64_t oohi = __shfl_sync(FULLMASK, p.ohi, own);
      const int ow1 = __shfl_sync(FULLMASK, p.w1, own);
      const int ohs = __shfl_sync(FULLMASK, p.hs, own);
      if (c < total) {
        const Dep &w = ow1 ? a.dep[1] : a.dep[0];
        const uint32_t x = __ldg(w.adj + owlo + (int64_t)(c - ost));
        cnt += pair_member(a, ow1, ohs, oolo, oohi, x);
      }
    }
  }
  for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(FULLMASK, cnt, o);
  if (lane == 0 && cnt) atomicAdd(a.total, cnt);
}

__global__ void __launch_bounds__(256) k_isect_pair_pieces(Args a, const ulonglong2 *pieces, uint64_t piece_cap,
                                                           const unsigned long long *piece_n, const int *overflow) {
  // a full list holds unwritten entries (a reservation that crossed the end
  // is not written): the caller counts again with room for every piece
  if (*overflow) return;
  const int lane = threadIdx.x & 31;
  const int learned = a.method ? *a.method : VS_ISECT_AUTO;
  const uint64_t n = *piece_n < piece_cap ? *piece_n : piece_cap;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  unsigned long long cnt = 0;
  for (uint64_t k = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < n; k += warps) {
    const ulonglong2 pc = pieces[k];
    const PairTuple p = pair_tuple(a, pc.x, learned);
    const Dep &w = p.w1 ? a.dep[1] : a.dep[0];
    const int64_t end = min(p.wn, (int64_t)pc.y + PAIR_PIECE);
    for (int64_t j = (int64_t)pc.y + lane; j < end; j += 32)
      cnt += pair_member(a, p.w1, p.hs, p.olo, p.ohi, __ldg(w.adj + p.wlo + j));
  }
  for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(FULLMASK, cnt, o);
  if (lane == 0 && cnt) atomicAdd(a.total, cnt);
}

// Features of one call for the learned membership method, from up to
// ISECT_SAMPLE base tuples spread over the base table: list lengths of the
// walked (shortest) list and of the other adjacency lists, their ratios and how
// often the other list's vertex has an adjacency bitmap.  With a picker the
// block then runs the network and stores its choice (class 0 the per-tuple
// rule, 1 binary search everywhere, 2 hub bitmap wherever one exists) for
// k_isect.
constexpr int ISECT_SAMPLE = 4096;

// One sample per thread over ISECT_SAMPLE / 256 blocks; each block writes its
// sums to part[block][32] and the last block to finish (counted in ctl[1])
// adds them in block order, so the features do not depend on timing.
constexpr int ISECT_DECIDE_THREADS = 256;
constexpr int ISECT_DECIDE_BLOCKS = ISECT_SAMPLE / ISECT_DECIDE_THREADS;

__global__ void __launch_bounds__(ISECT_DECIDE_THREADS) k_isect_decide(Args a, uint32_t V, uint64_t E, int has_hubs,
                                                                       const void *picker, float *feat_out, int *ctl,
                                                                       float *part) {
  __shared__ float wsum[ISECT_DECIDE_THREADS / 32][32];
  __shared__ float acc[32];
  __shared__ float f[pk::NF], out[pk::NO];
  __shared__ int s_last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint64_t n = a.nbase < (uint64_t)ISECT_SAMPLE ? a.nbase : (uint64_t)ISECT_SAMPLE;
  // loc: 0 samples, 1 empty, 2 sum log len_walk, 3 sum log len_other, 4 sum log ratio, 5 hub, 6 ratio<=8,
  //      7 bitmap rule, 8 other-list count, 16..23 hist log len_walk, 24..31 hist log ratio
  float loc[32];
#pragma unroll
  for (int j = 0; j < 32; j++) loc[j] = 0.f;
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) {
    const uint64_t t = n == a.nbase ? k : k * a.nbase / n;
    // every sorted dependency's list length and hub flag, loaded once
    int64_t len[MAX_DEPS];
    bool hub[MAX_DEPS], sorted[MAX_DEPS];
    int64_t walk = -1;
    bool empty = false;
#pragma unroll
    for (int i = 0; i < MAX_DEPS; i++) {
      len[i] = 0;
      hub[i] = sorted[i] = false;
      if (i >= a.ndeps) break;
      const Dep &d = a.dep[i];
      if (d.kind != DEP_SORTED) continue;
      sorted[i] = true;
      const uint32_t u = d.base_u[t];
      if (u < d.n_u) {
        len[i] = d.off[u + 1] - d.off[u];
        hub[i] = d.hub_slot && d.hub_slot[u] >= 0;
      }
      if (len[i] == 0) empty = true;
      if (walk < 0 || len[i] < walk) walk = len[i];
    }
    loc[0] = 1.f;
    if (walk >= 0 && empty) loc[1] = 1.f;
    if (walk >= 0 && !empty) {
      const float lw = log2f(1.f + (float)walk);
      loc[2] = lw;
      const int hb = min(7, (int)(lw * 0.5f));
#pragma unroll
      for (int b = 0; b < 8; b++) loc[16 + b] = hb == b ? 1.f : 0.f;
      bool walked = false;
#pragma unroll
      for (int i = 0; i < MAX_DEPS; i++) {
        if (i >= a.ndeps) break;
        if (!sorted[i]) continue;
        if (len[i] == walk && !walked) {
          walked = true;
          continue;
        }
        const float lo = log2f(1.f + (float)len[i]), lr = log2f((float)len[i] / (float)walk);
        loc[3] += lo;
        loc[4] += lr;
        loc[8] += 1.f;
        if (hub[i]) loc[5] += 1.f;
        if (walk >= 512 && len[i] <= 4 * walk) loc[6] += 1.f;
        if (hub[i]) loc[7] += 1.f;
        const int rb = max(0, min(7, (int)lr));
#pragma unroll
        for (int b = 0; b < 8; b++) loc[24 + b] += rb == b ? 1.f : 0.f;
      }
    }
  }
  // warp sums, then the block's in warp order, then the blocks' in block order
#pragma unroll
  for (int j = 0; j < 32; j++) {
    float v = loc[j];
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == j) wsum[wid][j] = v;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = 0.f;
    for (int w = 0; w < ISECT_DECIDE_THREADS / 32; w++) v += wsum[w][threadIdx.x];
    part[blockIdx.x * 32 + threadIdx.x] = v;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd((unsigned *)&ctl[1], 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  if (threadIdx.x < 32) {
    float v = 0.f;
    for (unsigned b = 0; b < gridDim.x; b++) v += __ldcg(part + b * 32 + threadIdx.x);
    acc[threadIdx.x] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const float ns = fmaxf(acc[0], 1.f), nw = fmaxf(acc[0] - acc[1], 1.f), no = fmaxf(acc[8], 1.f);
    int nsorted = 0;
    for (int i = 0; i < a.ndeps; i++) nsorted += a.dep[i].kind == DEP_SORTED;
    f[0] = log2f(1.f + (float)a.nbase) / 40.f;
    f[1] = a.ndeps / 8.f;
    f[2] = log2f(1.f + (float)V) / 32.f;
    f[3] = log2f(1.f + (float)E) / 40.f;
    f[4] = (float)E / fmaxf(1.f, (float)V) / 64.f;
    f[5] = nsorted / 8.f;
    f[6] = acc[1] / ns;
    f[7] = acc[2] / nw / 32.f;
    f[8] = acc[3] / no / 32.f;
    f[9] = acc[4] / no / 32.f;
    f[10] = acc[5] / no;
    f[11] = acc[6] / no;
    f[12] = acc[7] / no;
    f[13] = (float)has_hubs;
    f[14] = (float)a.all_mat;
    f[15] = 0.f;
    for (int b = 0; b < 8; b++) {
      f[16 + b] = acc[16 + b] / nw;
      f[24 + b] = acc[24 + b] / no;
    }
    if (feat_out)
      for (int i = 0; i < pk::NF; i++) feat_out[i] = f[i];
  }
  __syncthreads();
  if (!picker) return;
  pk::mlp_block(picker, f, out);
  if (threadIdx.x == 0) {
    int best = 0;
    for (int c = 1; c < pk::NO; c++)
      if (out[c] > out[best]) best = c;
    ctl[0] = best == 0 ? VS_ISECT_AUTO : best == 1 ? VS_ISECT_BINARY : VS_ISECT_BITMAP;
  }
}

// Flat dependency -> CSR over u with duplicate pairs removed.
__global__ void k_max_u(const uint32_t *u, uint64_t n, unsigned *mx) {
  unsigned m = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    m = max(m, u[i]);
  for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(FULLMASK, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(mx, m);
}

__global__ void k_flat_dedup(HashTable pairs, const uint32_t *u, const uint32_t *nv, uint64_t n,
                             unsigned long long *cnt_u, uint8_t *isnew) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t s = ht_insert(pairs, ((unsigned long long)u[i] << 32) | nv[i]);
    const bool first = atomicCAS(&pairs.val[s], 0xffffffffu, 0u) == 0xffffffffu;
    isnew[i] = first;
    if (first) atomicAdd(&cnt_u[u[i]], 1ull);
  }
}

__global__ void k_flat_scatter(const uint32_t *u, const uint32_t *nv, uint64_t n,
                               const uint8_t *isnew, const unsigned long long *off,
                               unsigned long long *cur, uint32_t *adj) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    if (isnew[i]) adj[off[u[i]] + atomicAdd(&cur[u[i]], 1ull)] = nv[i];
}

__global__ void k_build_cols(HashTable t, const uint32_t *col_map, uint32_t cols) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += gridDim.x * blockDim.x) {
    const uint64_t s = ht_insert(t, col_map[c]);
    atomicMin(&t.val[s], c);
  }
}

// Hub adjacency bitmaps: degree histogram (log2 bins), hub slots, bitmap fill.
__global__ void k_deg_bins(const int64_t *__restrict__ off, uint32_t V, unsigned long long *bins) {
  __shared__ unsigned long long b[64];
  if (threadIdx.x < 64) b[threadIdx.x] = 0;
  __syncthreads();
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int64_t d = off[v + 1] - off[v];
    if (d > 0) atomicAdd(&b[63 - __clzll((unsigned long long)d)], 1ull);
  }
  __syncthreads();
  if (threadIdx.x < 64 && b[threadIdx.x]) atomicAdd(&bins[threadIdx.x], b[threadIdx.x]);
}

__global__ void k_hub_slots(const int64_t *__restrict__ off, uint32_t V, uint32_t min_deg, uint32_t cap,
                            int32_t *slot, uint32_t *hubs, unsigned *count) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    int32_t s = -1;
    if (off[v + 1] - off[v] >= (int64_t)min_deg) {
      const unsigned k = atomicAdd(count, 1u);
      if (k < cap) {
        s = (int32_t)k;
        hubs[k] = v;
      }
    }
    slot[v] = s;
  }
}

__global__ void k_hub_fill(const int64_t *__restrict__ off, const uint32_t *__restrict__ adj,
                           const uint32_t *__restrict__ hubs, uint32_t n, uint64_t *bm, uint32_t words) {
  for (uint32_t b = blockIdx.x; b < n; b += gridDim.x) {
    const uint32_t v = hubs[b];
    unsigned long long *row = reinterpret_cast<unsigned long long *>(bm + (size_t)b * words);
    for (int64_t j = off[v] + threadIdx.x; j < off[v + 1]; j += blockDim.x) {
      const uint32_t x = adj[j];
      atomicOr(row + (x >> 6), 1ull << (x & 63));
    }
  }
}

struct Scratch {
  cudaStream_t st;
  void *p[64] = {};
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

int grid_for(uint64_t n, int per_block = 256) {
  return (int)std::max<uint64_t>(1, std::min<uint64_t>((n + per_block - 1) / per_block,
                                                       (uint64_t)sm_count() * 16));
}

// The hub bitmaps of one list direction of g, built once (the smallest
// power-of-two degree threshold >= HUB_MIN_DEG whose hubs fit HUB_BUDGET).
int hub_index(vs_graph *g, bool fwd, cudaStream_t st, const vs_hub_index **out) {
  std::lock_guard<std::mutex> lock(g->hub_mu);
  vs_hub_index &h = g->hub[fwd ? 0 : 1];
  *out = &h;
  if (h.built) return VS_OK;
  const int64_t *off = fwd ? g->fwd_off : g->rev_off;
  const uint32_t *adj = fwd ? g->fwd_dst : g->rev_src;
  const uint32_t V = g->V;
  h.words = (V + 63) / 64;
  const uint64_t per = (uint64_t)h.words * 8;
  const uint64_t cap = std::min<uint64_t>(HUB_BUDGET / std::max<uint64_t>(per, 1), 1u << 20);
  unsigned long long *bins = nullptr;
  VS_TRY(dalloc_n(&bins, 64, st));
  VS_CK(cudaMemsetAsync(bins, 0, 64 * 8, st));
  if (V) { k_deg_bins<<<grid_for(V), 256, 0, st>>>(off, V, bins); vs::note_launch(); }
  unsigned long long hb[64];
  VS_CK(cudaMemcpyAsync(hb, bins, sizeof(hb), cudaMemcpyDeviceToHost, st));
  VS_CK(cudaStreamSynchronize(st));
  dfree(bins, st);
  // bin k holds degrees in [2^k, 2^(k+1)): hubs with degree >= 2^k number sum(hb[k..])
  int k = 0;
  while ((1ull << k) < HUB_MIN_DEG) k++;
  uint64_t n = 0;
  for (int b = k; b < 64; b++) n += hb[b];
  while (k < 63 && n > cap) n -= hb[k++];
  h.min_deg = (uint32_t)std::min<uint64_t>(1ull << k, 0xffffffffull);
  h.n = (uint32_t)n;
  h.built = true;
  if (n == 0 || cap == 0) {
    h.n = 0;
    return VS_OK;
  }
  uint32_t *hubs = nullptr;
  unsigned *cnt = nullptr;
  VS_TRY(dalloc_n(&h.slot, V, st));
  VS_TRY(dalloc_n(&h.bm, (size_t)n * h.words, st));
  VS_TRY(dalloc_n(&hubs, n, st));
  VS_TRY(dalloc_n(&cnt, 1, st));
  VS_CK(cudaMemsetAsync(cnt, 0, 4, st));
  VS_CK(cudaMemsetAsync(h.bm, 0, (size_t)n * per, st));
  { k_hub_slots<<<grid_for(V), 256, 0, st>>>(off, V, h.min_deg, (uint32_t)n, h.slot, hubs, cnt); vs::note_launch(); }
  { k_hub_fill<<<(unsigned)std::min<uint64_t>(n, (uint64_t)sm_count() * 8), 256, 0, st>>>(off, adj, hubs, (uint32_t)n,
                                                                                      h.bm, h.words); vs::note_launch(); }
  VS_CK(cudaGetLastError());
  VS_CK(cudaStreamSynchronize(st));  // other streams may use the bitmaps next
  dfree(hubs, st);
  dfree(cnt, st);
  return VS_OK;
}

int hash_alloc(Scratch &sc, uint64_t n, HashTable *t) {
  t->cap = ht_capacity(std::max<uint64_t>(n, 1));
  VS_TRY(sc.get(&t->keys, t->cap + 1));
  VS_TRY(sc.get(&t->val, t->cap + 1));
  VS_CK(cudaMemsetAsync(t->keys, 0xff, 8 * (t->cap + 1), sc.st));
  VS_CK(cudaMemsetAsync(t->val, 0xff, 4 * (t->cap + 1), sc.st));
  t->cnt = t->off = t->cur = nullptr;
  return VS_OK;
}

int prepare_flat_dep(Scratch &sc, const vs_flat *f, uint32_t ucol, uint32_t nvcol, Dep *d) {
  if (ucol >= f->ncols || nvcol >= f->ncols || ucol == nvcol)
    return fail(VS_ERR_ARG, "flat dependency columns out of range");
  if (f->types[ucol] != VS_T_VID || f->types[nvcol] != VS_T_VID)
    return fail(VS_ERR_ARG, "Mintersect dependency columns must be VIDs (mintersect.cpp:22-27)");
  cudaStream_t st = sc.st;
  const uint32_t *u = (const uint32_t *)f->cols[ucol], *nv = (const uint32_t *)f->cols[nvcol];
  const uint64_t n = f->nrows;
  unsigned *dmx;
  VS_TRY(sc.get(&dmx, 1));
  VS_CK(cudaMemsetAsync(dmx, 0, 4, st));
  if (n) { k_max_u<<<grid_for(n), 256, 0, st>>>(u, n, dmx); vs::note_launch(); }
  unsigned mx = 0;
  VS_CK(cudaMemcpyAsync(&mx, dmx, 4, cudaMemcpyDeviceToHost, st));
  VS_CK(cudaStreamSynchronize(st));
  const uint64_t n_u = n ? (uint64_t)mx + 1 : 0;
  if (n_u > (1ull << 31)) return fail(VS_ERR_UNSUPPORTED, "flat dependency vertex ids above 2^31");
  d->kind = DEP_HASHED;
  d->n_u = n_u;
  VS_TRY(hash_alloc(sc, n, &d->pairs));
  unsigned long long *cnt, *off, *cur;
  uint8_t *isnew;
  uint32_t *adj;
  VS_TRY(sc.get(&cnt, n_u + 1));
  VS_TRY(sc.get(&off, n_u + 2));
  VS_TRY(sc.get(&cur, n_u + 1));
  VS_TRY(sc.get(&isnew, n));
  VS_TRY(sc.get(&adj, n));
  VS_CK(cudaMemsetAsync(cnt, 0, 8 * (n_u + 1), st));
  VS_CK(cudaMemsetAsync(cur, 0, 8 * (n_u + 1), st));
  if (n) { k_flat_dedup<<<grid_for(n), 256, 0, st>>>(d->pairs, u, nv, n, cnt, isnew); vs::note_launch(); }
  VS_TRY(exclusive_scan_u64(cnt, off, n_u, st));
  if (n) { k_flat_scatter<<<grid_for(n), 256, 0, st>>>(u, nv, n, isnew, off, cur, adj); vs::note_launch(); }
  // offsets are read as int64 by the kernel
  d->off = reinterpret_cast<const int64_t *>(off);
  d->adj = adj;
  VS_CK(cudaGetLastError());
  return VS_OK;
}

}  // namespace is
}  // namespace vs

using namespace vs;
using namespace vs::is;

extern "C" {

int vs_mintersect(vs_table_ref base, const vs_isect_dep *deps, uint32_t ndeps,
                  uint32_t new_vertex_count, int only_count, uint64_t max_rows, vs_flat **out,
                  uint64_t *count, vs_stream_t stream) {
  return vs_mintersect_ex(base, deps, ndeps, new_vertex_count, only_count, max_rows, nullptr, nullptr, out,
                          count, stream);
}

int vs_mintersect_ex(vs_table_ref base, const vs_isect_dep *deps, uint32_t ndeps,
                     uint32_t new_vertex_count, int only_count, uint64_t max_rows, const vs_picker *method_picker,
                     float *features, vs_flat **out, uint64_t *count, vs_stream_t stream) {
  if (!count || (!only_count && !out)) return fail(VS_ERR_ARG, "vs_mintersect: null output");
  if (!base.flat == !base.mat) return fail(VS_ERR_ARG, "base is exactly one of a flat table or a matrix");
  if (ndeps == 0 || ndeps > (uint32_t)MAX_DEPS || !deps)
    return fail(VS_ERR_ARG, "Mintersect takes 1..%d dependencies", MAX_DEPS);
  cudaStream_t st = S(stream);
  *count = 0;
  if (out) *out = nullptr;
  Scratch sc{st};
  // base tuples as a flat table
  vs_flat *bf_owned = nullptr;
  const vs_flat *bf = base.flat;
  if (base.mat) {
    VS_TRY(bitmat_to_flat(base.mat, st, &bf_owned));
    bf = bf_owned;
  }
  struct Owned {
    vs_flat *f;
    ~Owned() { vs_flat_free(f); }
  } owned{bf_owned};
  Args a{};
  a.ndeps = (int)ndeps;
  a.nbase = bf->nrows;
  uint32_t nmat = 0, mat_rows = 0;
  for (uint32_t i = 0; i < ndeps; i++) {
    const vs_isect_dep &d = deps[i];
    Dep &D = a.dep[i];
    const int nkinds = (d.mat != nullptr) + (d.flat != nullptr) + (d.graph != nullptr);
    if (nkinds != 1) return fail(VS_ERR_ARG, "dependency %u must name exactly one source", i);
    if (d.base_col >= bf->ncols) return fail(VS_ERR_ARG, "dependency %u base column out of range", i);
    if (bf->types[d.base_col] != VS_T_VID)
      return fail(VS_ERR_ARG, "base column of dependency %u is not a VID", i);
    D.base_u = (const uint32_t *)bf->cols[d.base_col];
    if (d.mat) {
      const vs_bitmat *m = d.mat;
      if (nmat && m->rows != mat_rows)
        return fail(VS_ERR_ARG, "matrix dependencies differ in row count (mintersect.cpp:69-76)");
      if (!nmat) a.target_row_map = m->row_map;
      mat_rows = m->rows;
      nmat++;
      D.kind = DEP_MAT;
      D.words = m->words;
      D.wpc = m->wpc;
      D.rows = m->rows;
      D.cols = m->cols;
      D.has_cmap = m->col_map != nullptr;
      if (D.has_cmap) {
        VS_TRY(hash_alloc(sc, m->cols, &D.cmap));
        if (m->cols) { k_build_cols<<<grid_for(m->cols), 256, 0, st>>>(D.cmap, m->col_map, m->cols); vs::note_launch(); }
      }
    } else if (d.graph) {
      const vs_graph *g = d.graph;
      if (d.direction == VS_DIR_BOTH && g->directed)
        return fail(VS_ERR_UNSUPPORTED, "adjacency dependency needs one direction");
      const bool fwd = !g->directed || d.direction == VS_DIR_FORWARD;
      if (d.algo < VS_ISECT_AUTO || d.algo > VS_ISECT_BITMAP)
        return fail(VS_ERR_ARG, "dependency %u: unknown intersection method %d", i, d.algo);
      D.kind = DEP_SORTED;
      D.off = fwd ? g->fwd_off : g->rev_off;
      D.adj = fwd ? g->fwd_dst : g->rev_src;
      D.n_u = g->V;
      D.algo = d.algo;
      D.hub_slot = nullptr;
      D.hub_bm = nullptr;
      if (d.algo == VS_ISECT_AUTO || d.algo == VS_ISECT_BITMAP) {
        const vs_hub_index *hx = nullptr;
        VS_TRY(hub_index(const_cast<vs_graph *>(g), fwd, st, &hx));
        if (hx->n) {
          D.hub_slot = hx->slot;
          D.hub_bm = hx->bm;
          D.hub_words = hx->words;
        }
      }
    } else {
      VS_TRY(prepare_flat_dep(sc, d.flat, d.u_col, d.nv_col, &D));
    }
  }
  a.all_mat = nmat == ndeps;
  a.cache_rows = a.all_mat ? mat_rows : new_vertex_count;
  // learned membership method (AUTO adjacency dependencies) and/or its features
  const vs_graph *fg = nullptr;
  bool hubs = false;
  for (uint32_t i = 0; i < ndeps; i++)
    if (deps[i].graph) {
      fg = deps[i].graph;
      hubs |= a.dep[i].hub_slot != nullptr;
    }
  if ((method_picker || features) && fg && !a.all_mat) {
    int *d_ctl = nullptr;  // [0] the method (VS_ISECT_AUTO until the network decides), [1] blocks done
    float *d_feat = nullptr, *d_part = nullptr;
    VS_TRY(sc.get(&d_ctl, 2));
    VS_TRY(sc.get(&d_feat, pk::NF));
    VS_TRY(sc.get(&d_part, ISECT_DECIDE_BLOCKS * 32));
    VS_CK(cudaMemsetAsync(d_ctl, 0, 2 * sizeof(int), st));
    const uint64_t ns = std::min<uint64_t>(a.nbase, ISECT_SAMPLE);
    const int gblocks = std::max<int>(1, (int)((ns + ISECT_DECIDE_THREADS - 1) / ISECT_DECIDE_THREADS));
    { k_isect_decide<<<gblocks, ISECT_DECIDE_THREADS, 0, st>>>(
          a, fg->V, fg->E, hubs ? 1 : 0, method_picker ? vs_picker_device_weights(method_picker) : nullptr, d_feat,
          d_ctl, d_part); vs::note_launch(); }
    a.method = method_picker ? d_ctl : nullptr;
    if (features) VS_CK(cudaMemcpyAsync(features, d_feat, sizeof(float) * pk::NF, cudaMemcpyDefault, st));
  } else if (features) {
    std::memset(features, 0, sizeof(float) * pk::NF);
  }
  unsigned long long *d_total, *tcnt = nullptr, *toff = nullptr;
  VS_TRY(sc.get(&d_total, 3));  // [0] count, [1] pieces of long walks (pair kernels), [2] their overflow flag
  VS_CK(cudaMemsetAsync(d_total, 0, 24, st));
  if (!only_count) {
    VS_TRY(sc.get(&tcnt, a.nbase));
    VS_TRY(sc.get(&toff, a.nbase + 1));
  }
  a.tcnt = tcnt;
  a.total = d_total;
  a.emit = 0;
  const int grid = grid_for(a.nbase * 32);
  VS_TRY(sc.get(&a.next, 1));
  VS_CK(cudaMemsetAsync(a.next, 0, 8, st));
  // two adjacency lists and only a count: the tuple-flattening kernel (a
  // forced window merge keeps the general kernel, which implements it)
  const bool pair_count = only_count && a.ndeps == 2 && a.dep[0].kind == DEP_SORTED && a.dep[1].kind == DEP_SORTED &&
                          a.dep[0].algo != VS_ISECT_MERGE && a.dep[1].algo != VS_ISECT_MERGE;
  unsigned long long res[3] = {0, 0, 0};
  if (a.nbase && pair_count) {
    // a first pass with room for 2 pieces per tuple; when the long walks need
    // more, the pass counted exactly how many, and a second pass gets that room
    uint64_t piece_cap = std::max<uint64_t>(65536, 2 * a.nbase);
    int *overflow = reinterpret_cast<int *>(d_total + 2);
    for (int pass = 0; pass < 2; pass++) {
      ulonglong2 *pieces = nullptr;
      if (pass && sc.get(&pieces, piece_cap) != VS_OK) {  // no room: the general kernel below
        cudaGetLastError();
        break;
      }
      if (!pass) VS_TRY(sc.get(&pieces, piece_cap));
      if (pass) {
        VS_CK(cudaMemsetAsync(d_total, 0, 24, st));
        VS_CK(cudaMemsetAsync(a.next, 0, 8, st));
      }
      { k_isect_pair_count<<<grid_for(a.nbase * 8), 256, 0, st>>>(a, pieces, piece_cap, d_total + 1, overflow);
        vs::note_launch(); }
      { k_isect_pair_pieces<<<sm_count() * 8, 256, 0, st>>>(a, pieces, piece_cap, d_total + 1, overflow);
        vs::note_launch(); }
      VS_CK(cudaGetLastError());
      VS_CK(cudaMemcpyAsync(res, d_total, 24, cudaMemcpyDeviceToHost, st));
      VS_CK(cudaStreamSynchronize(st));
      if (!res[2]) break;
      piece_cap = res[1];
    }
  } else if (a.nbase) {
    { k_isect<<<grid, 256, 0, st>>>(a); vs::note_launch(); }
    VS_CK(cudaGetLastError());
    VS_CK(cudaMemcpyAsync(res, d_total, 24, cudaMemcpyDeviceToHost, st));
    VS_CK(cudaStreamSynchronize(st));
  }
  if (res[2]) {  // the long walks did not fit the piece list: count again with the general kernel
    VS_CK(cudaMemsetAsync(d_total, 0, 8, st));
    VS_CK(cudaMemsetAsync(a.next, 0, 8, st));
    { k_isect<<<grid, 256, 0, st>>>(a); vs::note_launch(); }
    VS_CK(cudaGetLastError());
    VS_CK(cudaMemcpyAsync(res, d_total, 8, cudaMemcpyDeviceToHost, st));
    VS_CK(cudaStreamSynchronize(st));
  }
  unsigned long long total = res[0];
  *count = total;
  if (only_count) return VS_OK;
  VS_TRY(exclusive_scan_u64(tcnt, toff, a.nbase, st));
  const uint64_t rows = std::min<uint64_t>(total, max_rows);
  int32_t types[16];
  if (bf->ncols + 1 > 16) return fail(VS_ERR_UNSUPPORTED, "result wider than 16 columns");
  for (uint32_t c = 0; c < bf->ncols; c++) types[c] = bf->types[c];
  types[bf->ncols] = VS_T_VID;
  vs_flat *f = nullptr;
  VS_TRY(flat_alloc(bf->ncols + 1, types, rows, st, &f));
  a.nbcols = (int)bf->ncols;
  for (uint32_t c = 0; c < bf->ncols; c++) {
    a.col[c].dst = f->cols[c];
    a.col[c].src = bf->cols[c];
    a.col[c].type = bf->types[c];
  }
  a.out_new = (uint32_t *)f->cols[bf->ncols];
  a.toff = toff;
  a.max_rows = rows;
  a.emit = 1;
  VS_CK(cudaMemsetAsync(a.next, 0, 8, st));
  if (a.nbase && rows) { k_isect<<<grid, 256, 0, st>>>(a); vs::note_launch(); }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    vs_flat_free(f);
    return cuda_fail(e, "mintersect", __FILE__, __LINE__);
  }
  *out = f;
  return total > max_rows ? fail(VS_ERR_CAPACITY, "intersection produced %llu rows, bound %llu",
                                 (unsigned long long)total, (unsigned long long)max_rows)
                          : VS_OK;
}

}  // extern "C"
