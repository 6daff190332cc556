// Multi-source bit-matrix expand: VExpand + Expand<DenseVarStackMatrix>
// (src/objects/operator/vexpand.cpp, src/objects/operator/expand.cpp,
// src/include/operator/expand_impl.hh) re-designed for sm_103a.
//
// Data layout in HBM.  Every matrix is vertex-major: vertex v owns W
// consecutive uint64 words (W = ceil(S/64) rounded up to even), bit i of the
// row is source i.  This is the reference's DenseVarStackMatrix with a single
// stack as tall as S (rows padded to 128 instead of 1024), so one hop gathers
// 8W bytes per active edge instead of a padded 128-byte stack slice per stack.
//
// Buffers: two frontier buffers (layer h-1 and layer h ping-pong), the
// visited matrix (Shortest/FindShortest) and the accumulator (the union of
// layers k_min..k_max when it differs from visited).  Each frontier buffer
// has one uint32 flag per vertex with the invariant "flag == 0 => row is
// zero", which lets a hop skip inactive rows and clear only what it wrote
// (flag 2: a non-zero short row kept only in its short-row slot, the buffer
// row being zero; see the short-row notes at the PULL kernels).
//
// Per hop one of three strategies runs; the choice is made ON THE DEVICE by a
// one-block decide kernel from the previous hop's counters, so a whole query
// is a fixed launch sequence that can be captured in a CUDA graph:
//   SPARSE  (vertex, source) pair lists, one atomicOr per (pair, edge): the
//           reference's CSR strategy (expand.cpp:43-131) as an exact
//           bit-matrix update; used from the sources and while frontiers are tiny.
//   PULL    every vertex ORs the rows of its active in-neighbours with 16-byte
//           coalesced loads (sub-warp groups for narrow rows), fused with the
//           visited AND-NOT, the [k_min,k_max] accumulation and the popcounts
//           (dedup_and_update_visit_and_count, bitmap.cpp:1054-1096, and
//           merge_to_MT's union, vexpand.cpp:298-354, folded into the hop).
//           Vertices above the hub threshold get a whole CTA.
//   PUSH    active rows OR-ed into their out-neighbours with 64-bit atomics,
//           followed by a fused dedup/accumulate pass over the touched rows.
#include <algorithm>
#include <atomic>
#include <mutex>
#include <cstring>
#include <vector>

#include "expand_internal.cuh"
#include "picker.cuh"
#include "vs_internal.cuh"

namespace vs {
namespace ex {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

template <typename T> __device__ __forceinline__ T warp_sum(T v) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

// Block-wide sum of per-thread counters, one atomic per block.
__device__ __forceinline__ void block_add(unsigned long long v, unsigned long long *dst) {
  __shared__ unsigned long long part[32];
  v = warp_sum(v);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0ull;
    v = warp_sum(v);
    if (threadIdx.x == 0 && v) atomicAdd(dst, v);
  }
}

// ---------------------------------------------------------------------------
// Run start: clear both frontier buffers (flagged rows only) and the counters.
__global__ void k_clear_flagged(uint4 *__restrict__ buf, uint32_t *__restrict__ flag, uint32_t V,
                                uint32_t Q, const Ctr *ctr, int h, int mode) {
  // mode 0: unconditional; mode 1: only when hop h runs SPARSE or PUSH, or a
  // multi-slice PULL (those write with atomics / partially and need clean rows)
  if (mode == 1) {
    int s = ctr->hop[h].strategy;
    if (!(s == ST_SPARSE || s == ST_PUSH || (s == ST_PULL && ctr->multislice))) return;
  }
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  // four flags per lane (16-byte loads of the 16-byte aligned flag array):
  // a warp step covers 128 vertices, so the scan is a quarter as many
  // dependent loads; flag 2 means the row lives in its slot (buffer row zero)
  uint4 *flag4 = reinterpret_cast<uint4 *>(flag);
  const uint32_t nq = V / 4;
  for (uint32_t base = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; base < nq; base += warps * 32) {
    const uint32_t g = base + lane;
    const uint4 f = g < nq ? flag4[g] : make_uint4(0, 0, 0, 0);
    if (f.x | f.y | f.z | f.w) flag4[g] = make_uint4(0, 0, 0, 0);
    const uint32_t fv[4] = {f.x, f.y, f.z, f.w};
#pragma unroll
    for (int k = 0; k < 4; k++) {
      unsigned m = __ballot_sync(FULL, fv[k] == 1);
      while (m) {
        const int b = __ffs(m) - 1;
        m &= m - 1;
        uint4 *row = buf + (size_t)((base + b) * 4u + k) * Q;
        for (uint32_t q = lane; q < Q; q += 32) row[q] = make_uint4(0, 0, 0, 0);
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x < 32) {  // the last V % 4 vertices
    for (uint32_t v = nq * 4; v < V; v++) {
      const uint32_t f = flag[v];
      if (f == 1)
        for (uint32_t q = lane; q < Q; q += 32) buf[(size_t)v * Q + q] = make_uint4(0, 0, 0, 0);
      __syncwarp();
      if (lane == 0 && f) flag[v] = 0;
    }
  }
}

// Layer 0 (ExpandStatus::init_first_m_layer, expand_impl.hh:252-277).
__device__ __forceinline__ int degree_bin(unsigned long long d) {
  return min(pk::NHIST - 1, 63 - __clzll((long long)(d + 1)));
}

__global__ void k_seed(SeedArgs a) {
  __shared__ unsigned s_hist[pk::NHIST];  // hop 1's frontier statistics (a.stats)
  if (threadIdx.x < pk::NHIST) s_hist[threadIdx.x] = 0;
  __syncthreads();
  unsigned long long pe = 0, nv = 0, ae = 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) {  // counters set on the device: the run has no host copies
    a.ctr->multislice = a.multislice;
    a.ctr->hop[0].pairs = a.S;
    a.ctr->hop[0].new_bits = a.S;
    if (a.rowk && a.rowk[1]) atomicOr(&a.ctr->error, 2);  // a device-set row limit exceeded k_max
  }
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.S; i += gridDim.x * blockDim.x) {
    uint32_t v = a.sources[i];
    if (v >= a.V) {  // reported as VS_ERR_ARG; the pair stays in range
      a.ctr->error = 1;
      a.pairs0[i] = make_uint2(0, i);
      a.pdeg0[i] = 0;
      continue;
    }
    size_t idx = (size_t)v * a.W + (i >> 6);
    unsigned long long bit = 1ull << (i & 63);
    atomicOr((unsigned long long *)&a.buf0[idx], bit);
    const bool first = atomicOr(&a.flag0[v], 1u) == 0;
    if (first) nv++;
    if (a.vis) atomicOr((unsigned long long *)&a.vis[idx], bit);
    if (a.acc) atomicOr((unsigned long long *)&a.acc[idx], bit);
    if ((a.vis && a.res_vis) || a.acc) a.resflag[v] = 1;
    a.pairs0[i] = make_uint2(v, i);
    unsigned long long d = 0;
    _Pragma("unroll") for (int l = 0; l < 2; l++) if (l < a.out.n) d += (unsigned long long)(a.out.off[l][v + 1] - a.out.off[l][v]);
    a.pdeg0[i] = d;
    pe += d;
    if (a.stats && first) {  // each distinct source vertex once, as the stats pass counts rows
      ae += d;
      atomicAdd(&s_hist[degree_bin(d)], 1u);
    }
  }
  block_add(pe, &a.ctr->hop[0].pair_edges);
  block_add(nv, &a.ctr->hop[0].active_vertices);
  if (a.stats) {
    block_add(ae, &a.ctr->hop[1].active_edges);
    if (threadIdx.x < pk::NHIST && s_hist[threadIdx.x])
      atomicAdd(&a.ctr->hop[1].hist[threadIdx.x], (unsigned long long)s_hist[threadIdx.x]);
  }
}

// FindShortest bookkeeping before hop 1 (VExpand::before_execution, vexpand.cpp:179-195).
__global__ void k_dist_init(const uint32_t *__restrict__ src, const uint32_t *__restrict__ tgt,
                            int32_t *__restrict__ dist, uint32_t S, uint32_t V, Ctr *ctr) {
  unsigned long long f = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < S; i += gridDim.x * blockDim.x) {
    if (tgt[i] >= V) ctr->error = 1;
    bool eq = src[i] == tgt[i];
    dist[i] = eq ? 0 : -1;
    f += eq;
  }
  block_add(f, &ctr->found);
}

// with_distance export: layer h (the frontier buffer just written) into its
// own zeroed matrix, flagged rows only; a hop that did not run copies nothing.
__global__ void k_copy_layer(const uint4 *__restrict__ buf, const uint32_t *__restrict__ flag, uint4 *__restrict__ out,
                             uint32_t V, uint32_t Q, const Ctr *ctr, int h) {
  if (h > 0 && ctr->hop[h].strategy == 0) return;
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t base = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; base < V; base += warps * 32) {
    const uint32_t v = base + lane;
    unsigned m = __ballot_sync(FULL, v < V && flag[v]);
    while (m) {
      const int b = __ffs(m) - 1;
      m &= m - 1;
      const size_t row = (size_t)(base + b) * Q;
      for (uint32_t q = lane; q < Q; q += 32) out[row + q] = buf[row + q];
    }
  }
}

// Per-hop row masks of batched queries from per-row hop limits: word w of
// hop h has bit r set when row 64w+r may still grow at hop h.
__global__ void k_row_mask(const uint8_t *__restrict__ lim, uint32_t n, uint32_t K, uint32_t W,
                           uint64_t *__restrict__ hmask, uint32_t *rowk) {
  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= W) return;
  uint32_t kmax = 0, over = 0;
  for (uint32_t r = 0; r < 64; r++) {
    const uint32_t i = w * 64 + r;
    const uint32_t l = i < n ? lim[i] : 0u;
    over |= l > K;
    kmax = max(kmax, min(l, K));
  }
  for (uint32_t h = 0; h <= K; h++) {
    uint64_t m = 0;
    for (uint32_t r = 0; h > 0 && r < 64; r++) {
      const uint32_t i = w * 64 + r;
      if (i < n && min((uint32_t)lim[i], K) >= h) m |= 1ull << r;
    }
    hmask[(size_t)h * W + w] = m;
  }
  if (kmax) atomicMax(&rowk[0], kmax);
  if (over) rowk[1] = 1;
}

// One block of 256 threads: early-stop checks of hop h-1 (VExpand::after_child,
// vexpand.cpp:222-284), the fixed planner's choice for hop h, and — when a
// picker is loaded or features are logged — the feature vector of hop h and
// the picker network's choice.
__global__ void __launch_bounds__(256) k_decide(DecideArgs a) {
  __shared__ float f[pk::NF], out[pk::NO];
  __shared__ int s_run, s_choice, s_pairs_ok;
  const int t = threadIdx.x;
  Ctr *c = a.ctr;
  HopCtr &prev = c->hop[a.h - 1];
  HopCtr &cur = c->hop[a.h];
  const bool use_picker = a.picker && a.picker_on && a.forced == 0;
  // the network's parameters load while thread 0 reads the counters
  const __nv_bfloat16 *w = use_picker ? pk::mlp_stage(a.picker) : nullptr;
  if (t == 0) {
    if (!c->done && a.rowk && (uint32_t)a.h > a.rowk[0]) c->done = 1;  // every row is past its last hop
    if (!c->done && a.h >= 2) {
      if (a.path != VS_PATH_ANY && prev.new_bits == 0) c->done = 1;
      if (a.path == VS_PATH_FIND_SHORTEST && c->found >= a.S) c->done = 1;
    }
    s_run = !c->done;
    s_choice = 0;
    s_pairs_ok = 0;
    if (s_run) {
      c->hops_run = a.h;
      const bool pairs_ok = (a.h == 1) || (prev.strategy == ST_SPARSE && !prev.overflow &&
                                           prev.pairs <= a.pair_cap);
      s_pairs_ok = pairs_ok;
      int s = a.forced;
      if (s == ST_SPARSE && !pairs_ok) s = ST_PULL;
      if (s == 0) {
        // fixed planner: pair lists while their edge work is a small fraction
        // of a dense pass, then push while few rows are active, then pull
        const double pe = (double)prev.pair_edges;
        if (pairs_ok && pe < (double)a.E * a.sparse_frac)
          s = ST_SPARSE;
        else if ((double)prev.active_vertices < (double)a.V * a.push_frac && prev.strategy != 0)
          s = ST_PUSH;
        else
          s = ST_PULL;
      }
      s_choice = s;
    }
  }
  __syncthreads();
  if (!s_run) {
    if (t == 0) cur.strategy = 0;
    return;
  }
  if (use_picker || a.log_features) {
    if (t == 0) {
      pk::HopFeatIn in;
      in.S = (float)a.S;
      in.V = (float)a.V;
      in.E = (float)a.E;
      in.W = (float)a.W;
      in.h = (float)a.h;
      in.k_min = (float)a.k_min;
      in.k_max = (float)a.k_max;
      in.new_bits_prev = (float)prev.new_bits;
      in.active_prev = (float)prev.active_vertices;
      unsigned long long vis = 0;
      for (int i = 0; i < a.h; i++) vis += c->hop[i].new_bits;
      in.visited_bits = (float)vis;
      in.active_edges = (float)cur.active_edges;
      in.pair_edges = s_pairs_ok ? (float)prev.pair_edges : 0.f;
      in.pairs_ok = (float)s_pairs_ok;
      in.shortest = a.path != VS_PATH_ANY ? 1.f : 0.f;
      in.both = (float)a.both;
      in.hist = cur.hist;
      pk::hop_features(in, f);
      if (a.log_features)
        for (int i = 0; i < pk::NF; i++) c->feat[a.h][i] = f[i];
    }
    __syncthreads();
    // one choice left (no pair list, no PUSH in the plan): PULL without the network
    if (use_picker && (s_pairs_ok || a.push_ok)) {
      pk::mlp_run(w, f, out);
      if (t == 0) {
        int best = -1;
        for (int k = 0; k < pk::NO; k++) {
          const int st = pk::class_to_strategy(k);
          if (st == ST_SPARSE && !s_pairs_ok) continue;  // no pair list to expand from
          if (st == ST_PUSH && !a.push_ok) continue;      // the plan launches no PUSH kernels
          if (best < 0 || out[k] > out[best]) best = k;
        }
        s_choice = pk::class_to_strategy(best);
      }
    }
  }
  if (t == 0) {
    cur.strategy = s_choice;
    // short mode: enough short rows in a frontier that L2 does not already
    // hold (a layer from a PULL hop counted them; from SPARSE or PUSH, a few
    // bits per row on average stand in for the count)
    bool sp = false;
    if (s_choice == ST_PULL && a.short_min > 0 && !c->multislice) {
      const double act = (double)prev.active_vertices;
      if (a.short_min > 1.0)
        sp = true;
      else if (act * 8.0 * (double)a.W > (double)a.l2_half)
        sp = prev.strategy == ST_PULL ? (double)(prev.short_rows & 0xFFFFFFFFull) >= a.short_min * act
                                      : (double)prev.new_bits <= 4.0 * act;
    }
    cur.short_pull = sp;
    // a frontier of mostly 4..15-bit rows reads slots instead of words
    cur.short_slots = sp && prev.strategy == ST_PULL &&
                      (double)(prev.short_rows >> 32) < 0.5 * (double)(prev.short_rows & 0xFFFFFFFFull);
  }
}

// Per-hop frontier statistics of layer h-1: E_active (out-degrees of its
// non-zero rows) and the log2(out-degree + 1) histogram of those rows.
// Layers written by the seed or by a SPARSE hop already have these counts
// (counted as their rows became non-zero), so the pass exits at once; so it
// does when only the picker reads them (picker_only) and the hop has a single
// choice: no pair list after a PULL or PUSH hop, and no PUSH in the plan.
__global__ void k_hop_stats(const uint32_t *__restrict__ flagF, Lists out, uint32_t V, Ctr *ctr, int h,
                            int picker_only, int push_ok) {
  if (ctr->done || h == 1 || ctr->hop[h - 1].strategy == ST_SPARSE) return;
  if (picker_only && !push_ok) return;
  __shared__ unsigned long long hist[pk::NHIST];
  if (threadIdx.x < pk::NHIST) hist[threadIdx.x] = 0;
  __syncthreads();
  unsigned long long s = 0;
  // warp-uniform loop; lanes with the same bin add once through their leader
  for (uint32_t v0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; v0 < V; v0 += gridDim.x * blockDim.x) {
    const uint32_t v = v0 + (threadIdx.x & 31);
    int b = -1;
    if (v < V && flagF[v]) {
      unsigned long long d = 0;
      _Pragma("unroll") for (int l = 0; l < 2; l++) if (l < out.n) d += (unsigned long long)(out.off[l][v + 1] - out.off[l][v]);
      s += d;
      b = degree_bin(d);
    }
    const unsigned peers = __match_any_sync(FULL, b);
    if (b >= 0 && (peers & lanemask_lt()) == 0) atomicAdd(&hist[b], (unsigned long long)__popc(peers));
  }
  __syncthreads();
  if (threadIdx.x < pk::NHIST && hist[threadIdx.x]) atomicAdd(&ctr->hop[h].hist[threadIdx.x], hist[threadIdx.x]);
  block_add(s, &ctr->hop[h].active_edges);
}

// SPARSE: (vertex u, source i) pairs of layer h-1; every out-neighbour v gets
// bit i.  Shortest dedups through the visited bit (atomicOr returns the old
// word), Any through the next-layer bit.  New pairs form layer h's list.
// The work is balanced over edges, not pairs: a prefix sum of the pairs'
// out-degrees (k_pscan*) lays all their out-lists end to end, and each warp
// takes fixed chunks of that edge range, so a pair on a 50k-degree hub is
// spread over many warps instead of serialising one.
constexpr int SPARSE_CHUNK = 256;  // edges per warp task
constexpr int SPARSE_K = 2;        // edges per lane per round

// Pairs the SPARSE hop h scans (0 when the hop runs another strategy).
__device__ __forceinline__ uint64_t scan_len(const Ctr *ctr, int h, uint64_t cap) {
  if (ctr->hop[h].strategy != ST_SPARSE) return 0;
  const unsigned long long npr = ctr->hop[h - 1].pairs;
  return npr < cap ? npr : cap;
}

__global__ void k_pscan1(const unsigned long long *__restrict__ pdeg, unsigned long long *__restrict__ doff,
                         unsigned long long *__restrict__ bsum, const Ctr *ctr, int h, uint64_t cap) {
  const uint64_t np = scan_len(ctr, h, cap);
  if (!np) return;
  __shared__ unsigned long long wt[8];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  for (uint64_t b = blockIdx.x; b * 1024 < np; b += gridDim.x) {
    const uint64_t base = b * 1024;
    unsigned long long v[4], run = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const uint64_t i = base + (uint64_t)t * 4 + k;
      v[k] = i < np ? pdeg[i] : 0ull;
      run += v[k];
    }
    unsigned long long incl = run;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) wt[w] = incl;
    __syncthreads();
    unsigned long long pre = 0;
    for (int k = 0; k < w; k++) pre += wt[k];
    pre += incl - run;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const uint64_t i = base + (uint64_t)t * 4 + k;
      if (i < np) doff[i] = pre;
      pre += v[k];
    }
    if (t == 255) bsum[b] = pre;  // block total (pre ends at the block's inclusive sum)
    __syncthreads();
  }
}

__global__ void k_pscan2(unsigned long long *__restrict__ bsum, unsigned long long *__restrict__ doff,
                         const Ctr *ctr, int h, uint64_t cap) {
  const uint64_t np = scan_len(ctr, h, cap);
  if (!np) return;
  const uint64_t nb = (np + 1023) / 1024;
  __shared__ unsigned long long carry, wt[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  if (t == 0) carry = 0;
  __syncthreads();
  for (uint64_t b0 = 0; b0 < nb; b0 += blockDim.x) {
    const uint64_t i = b0 + t;
    const unsigned long long x = i < nb ? bsum[i] : 0ull;
    unsigned long long xi = x;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(FULL, xi, o);
      if (lane >= o) xi += y;
    }
    if (lane == 31) wt[w] = xi;
    __syncthreads();
    unsigned long long pre = carry;
    for (int k = 0; k < w; k++) pre += wt[k];
    if (i < nb) bsum[i] = pre + xi - x;
    __syncthreads();
    if (t == blockDim.x - 1) carry = pre + xi;
    __syncthreads();
  }
  if (t == 0) doff[np] = carry;
}

__global__ void k_pscan3(unsigned long long *__restrict__ doff, const unsigned long long *__restrict__ bsum,
                         const Ctr *ctr, int h, uint64_t cap) {
  const uint64_t np = scan_len(ctr, h, cap);
  if (!np) return;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < np; i += (uint64_t)gridDim.x * blockDim.x)
    doff[i] += bsum[i / 1024];
}

__device__ __forceinline__ unsigned long long out_degree(const Lists &L, uint32_t v) {
  unsigned long long d = 0;
  _Pragma("unroll") for (int l = 0; l < 2; l++) if (l < L.n) d += (unsigned long long)(L.off[l][v + 1] - L.off[l][v]);
  return d;
}

// Largest p in [0, np) with doff[p] <= x for x0 (lanes 0-15) and x1 (lanes
// 16-31), doff ascending with doff[0] = 0 <= x: each step a half-warp probes
// 15 positions spread over its range at once and keeps the part between the
// last probe at or below x and the next, so a range shrinks 16-fold per
// dependent load instead of 2-fold.  Every lane receives both answers.
__device__ __forceinline__ void owner_pairs(const unsigned long long *__restrict__ doff, uint64_t np,
                                            unsigned long long x0, unsigned long long x1, int lane, uint64_t &p0,
                                            uint64_t &p1) {
  const int hl = lane & 15;
  const unsigned long long x = lane < 16 ? x0 : x1;
  uint64_t lo = 0, hi = np;  // doff[lo] <= x, and doff[hi] > x unless hi == np
  while (__any_sync(FULL, hi - lo > 1)) {
    const uint64_t span = hi - lo;
    const uint64_t pos = lo + (span * (uint64_t)hl + 15) / 16;  // probe hl; probe 0 is lo itself
    const bool ok = span > 1 && (hl == 0 || (pos < hi && doff[pos] <= x));
    const unsigned b = __ballot_sync(FULL, ok);
    const unsigned half = lane < 16 ? (b & 0xFFFFu) : (b >> 16);
    if (span > 1) {
      const int k = 31 - __clz(half);
      const uint64_t nhi = k == 15 ? hi : lo + (span * (uint64_t)(k + 1) + 15) / 16;
      lo = lo + (span * (uint64_t)k + 15) / 16;
      hi = nhi < hi ? nhi : hi;
    }
  }
  p0 = __shfl_sync(FULL, lo, 0);
  p1 = __shfl_sync(FULL, lo, 16);
}

__global__ void __launch_bounds__(256, 4) k_sparse(SparseArgs a) {
  Ctr *c = a.ctr;
  if (c->hop[a.h].strategy != ST_SPARSE) return;
  __shared__ uint2 s_new[8][SPARSE_CHUNK];  // a warp's new pairs of its current chunk
  __shared__ unsigned s_hist[pk::NHIST];    // hop h+1's frontier statistics (a.stats)
  if (threadIdx.x < pk::NHIST) s_hist[threadIdx.x] = 0;
  __syncthreads();
  const unsigned long long np_raw = c->hop[a.h - 1].pairs;
  const uint64_t np = np_raw < a.cap ? np_raw : a.cap;
  const unsigned long long T = a.doff[np];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  const uint64_t nchunks = (T + SPARSE_CHUNK - 1) / SPARSE_CHUNK;
  unsigned long long nb = 0, nv = 0, pe = 0, ae = 0;
  for (uint64_t ck = (uint64_t)blockIdx.x * (blockDim.x >> 5) + wib; ck < nchunks; ck += warps) {
    const unsigned long long e0 = ck * SPARSE_CHUNK;
    const unsigned long long e1 = min(e0 + SPARSE_CHUNK, T);
    // pairs owning the chunk's first and last edge: largest p with doff[p] <= e,
    // both found at once by a 16-way search per half-warp
    uint64_t plo, phi;
    owner_pairs(a.doff, np, e0, e1 - 1, lane, plo, phi);
    uint32_t nloc = 0;  // new pairs of this chunk so far (s_new)
    // the chunk's pairs 32 at a time: lane j holds pair g0 + j (its first
    // edge, source id, and its vertex's list starts and first-list length),
    // and an edge of the group's range finds its pair by a shuffle search over
    // the lanes' first edges instead of loading it
    for (uint64_t g0 = plo; g0 <= phi; g0 += 32) {
      unsigned long long dj = ~0ull;  // lanes past the last pair never own an edge
      uint32_t pi = 0;
      int64_t pb0 = 0, pd0 = 0, pb1 = 0;
      if (g0 + lane <= phi) {
        dj = a.doff[g0 + lane];
        const uint2 pr = a.pin[g0 + lane];
        pi = pr.y;
        pb0 = a.out.off[0][pr.x];
        pd0 = a.out.off[0][pr.x + 1] - pb0;
        if (a.out.n > 1) pb1 = a.out.off[1][pr.x];
      }
      // the group's edges inside the chunk
      const unsigned long long d0j = __shfl_sync(FULL, dj, 0);
      const unsigned long long gs = d0j > e0 ? d0j : e0;
      unsigned long long ge = e1;
      if (g0 + 32 <= phi) {
        const unsigned long long nx = a.doff[g0 + 32];
        ge = nx < e1 ? nx : e1;
      }
      // SPARSE_K edges per lane per round, each phase issued for all of them
      // before the next: the adjacency loads, then the returning atomics on
      // the visited (or next-layer) words, then the row flags, so a lane keeps
      // SPARSE_K dependent chains in flight instead of one
      for (unsigned long long eb = gs; eb < ge; eb += 32 * SPARSE_K) {
        uint32_t v[SPARSE_K], i[SPARSE_K];
        bool act[SPARSE_K];
#pragma unroll
        for (int k = 0; k < SPARSE_K; k++) {
          const unsigned long long e = eb + k * 32 + lane;
          int own = 0;  // the last pair whose first edge is at or below e (starts ascend with the lane)
#pragma unroll
          for (int step = 16; step; step >>= 1)
            if (__shfl_sync(FULL, dj, own + step) <= e) own += step;
          i[k] = __shfl_sync(FULL, pi, own);
          const int64_t b0 = __shfl_sync(FULL, pb0, own);
          const int64_t d0 = __shfl_sync(FULL, pd0, own);
          const int64_t b1 = __shfl_sync(FULL, pb1, own);
          const unsigned long long j = e - __shfl_sync(FULL, dj, own);  // the edge's index in its pair's out-lists
          v[k] = 0;
          act[k] = e < ge && (!a.hmask || ((__ldg(a.hmask + (i[k] >> 6)) >> (i[k] & 63)) & 1ull));
          if (act[k]) v[k] = (int64_t)j < d0 ? a.out.adj[0][b0 + j] : a.out.adj[1][b1 + (int64_t)j - d0];
        }
        unsigned long long old[SPARSE_K];
#pragma unroll
        for (int k = 0; k < SPARSE_K; k++) {
          old[k] = ~0ull;  // an inactive edge sets nothing
          if (act[k]) {
            const size_t idx = (size_t)v[k] * a.W + (i[k] >> 6);
            // Shortest dedups through the visited bit, Any through the next-layer bit
            old[k] = atomicOr(a.shortest ? &a.vis[idx] : &a.N[idx], 1ull << (i[k] & 63));
          }
        }
        bool fresh[SPARSE_K];
#pragma unroll
        for (int k = 0; k < SPARSE_K; k++) {
          fresh[k] = !((old[k] >> (i[k] & 63)) & 1ull);
          if (fresh[k]) {
            const size_t idx = (size_t)v[k] * a.W + (i[k] >> 6);
            const unsigned long long bit = 1ull << (i[k] & 63);
            if (a.shortest && !a.last && !a.defer) atomicOr(&a.N[idx], bit);
            if (a.acc_on) atomicOr(&a.acc[idx], bit);
            nb++;
          }
        }
        bool first[SPARSE_K];
#pragma unroll
        for (int k = 0; k < SPARSE_K; k++) {
          // a last layer's rows stay zero in the buffer (flag 2: the run start skips them)
          first[k] = fresh[k] && atomicOr(&a.flagN[v[k]], a.last ? 2u : 1u) == 0;
          nv += first[k];
          // the result column is marked once per row and hop, by the bit that made the row non-zero
          if (first[k] && (a.res_vis || a.acc_on)) a.resflag[v[k]] = 1;
        }
        // the chunk's new pairs gather in shared memory (one list append per chunk);
        // bit 31 of the source id (S < 2^31) marks the pair that made its row non-zero
#pragma unroll
        for (int k = 0; k < SPARSE_K; k++) {
          const unsigned m = __ballot_sync(FULL, fresh[k]);
          if (fresh[k])
            s_new[wib][nloc + __popc(m & lanemask_lt())] = make_uint2(v[k], i[k] | (first[k] ? 0x80000000u : 0u));
          nloc += __popc(m);
        }
      }
    }
    __syncwarp();
    if (nloc && a.last) {  // a last layer's pairs are counted, not kept
      if (lane == 0) atomicAdd(&c->hop[a.h].pairs, (unsigned long long)nloc);
    } else if (nloc) {  // append the chunk's new pairs (with their out-degrees) to layer h's list
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(&c->hop[a.h].pairs, (unsigned long long)nloc);
      base = __shfl_sync(FULL, base, 0);
      for (uint32_t j = lane; j < nloc; j += 32) {
        const uint2 pf = s_new[wib][j];
        const uint2 pr = make_uint2(pf.x, pf.y & 0x7FFFFFFFu);
        const unsigned long long d = out_degree(a.out, pr.x);
        pe += d;
        if (a.stats && (pf.y >> 31)) {  // each row of layer h once, as the stats pass counts them
          ae += d;
          atomicAdd(&s_hist[degree_bin(d)], 1u);
        }
        const unsigned long long slot = base + j;
        if (slot < a.cap) {
          a.pout[slot] = pr;
          a.pdeg_out[slot] = d;
        } else {
          c->hop[a.h].overflow = 1;
          // a deferred row gets the bit a full list cannot hold
          if (a.defer) atomicOr(&a.N[(size_t)pr.x * a.W + (pr.y >> 6)], 1ull << (pr.y & 63));
        }
      }
      __syncwarp();
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) c->hop[a.h].work_edges = T;
  block_add(nb, &c->hop[a.h].new_bits);
  block_add(nv, &c->hop[a.h].active_vertices);
  block_add(pe, &c->hop[a.h].pair_edges);
  if (a.stats) {
    block_add(ae, &c->hop[a.h + 1].active_edges);
    if (threadIdx.x < pk::NHIST && s_hist[threadIdx.x])
      atomicAdd(&c->hop[a.h + 1].hist[threadIdx.x], (unsigned long long)s_hist[threadIdx.x]);
  }
}

// ---------------------------------------------------------------------------
// L2 cache policies for the PULL kernels (variant H = 1): adjacency lists,
// offsets and the visited / next-layer streams are read or written once per
// hop and marked evict-first, so L2 keeps the frontier rows, which power-law
// hubs make the only reused data (marked evict-last).
template <int H> struct L2Pol {
  uint64_t first = 0, last = 0;
  __device__ __forceinline__ L2Pol() {
    if (H) {
      asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(first));
      asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(last));
    }
  }
  __device__ __forceinline__ uint32_t ld_stream(const uint32_t *p) const {
    if (!H) return __ldg(p);
    uint32_t r;
    asm("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(r) : "l"(p), "l"(first));
    return r;
  }
  __device__ __forceinline__ int64_t ld_stream(const int64_t *p) const {
    if (!H) return __ldg(p);
    int64_t r;
    asm("ld.global.nc.L2::cache_hint.s64 %0, [%1], %2;" : "=l"(r) : "l"(p), "l"(first));
    return r;
  }
  __device__ __forceinline__ uint4 ld_row(const uint4 *p) const {
    if (!H) return __ldg(p);
    uint4 r;
    asm("ld.global.nc.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "l"(p), "l"(last));
    return r;
  }
  __device__ __forceinline__ uint4 ld_rw(const uint4 *p) const {
    if (!H) return *p;
    uint4 r;
    asm volatile("ld.global.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "l"(p), "l"(first) : "memory");
    return r;
  }
  __device__ __forceinline__ void st(uint4 *p, uint4 v) const {
    if (!H) {
      *p = v;
      return;
    }
    asm volatile("st.global.L2::cache_hint.v4.u32 [%0], {%1, %2, %3, %4}, %5;"
                 :: "l"(p), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w), "l"(first) : "memory");
  }
};

// ---------------------------------------------------------------------------
// PULL.  A warp owns one target vertex; its lanes form G = 32/L groups of L
// lanes, each group ORs one whole active in-neighbour row (Q uint4 = L * UPL
// per lane at most) at a time.  In-neighbour ids are read 32 at a time,
// filtered by the frontier flags with a ballot and compacted through shared
// memory, so inactive rows cost one flag load and no gather.
//
// Short rows.  In the later hops of a many-source expand over a power-law
// graph most frontier rows hold a handful of sources, and a whole-row gather
// then moves mostly zero words.  Every PULL hop with a successor therefore
// also writes, for every vertex, a tiny word (uint32: the ids of a row of one
// or two bits, else its saturated bit count) and a slot of
// slot_n uint16 (entry 0: the count; entries 1..count: the ids, for up to
// slot_n - 1 bits; slot_n = 16, 32 or 64 as the rows are up to 512 B, 1 KB or
// wider).  A later PULL hop in short mode reads, per in-neighbour, either its
// tiny word (word mode: 4 bytes per vertex, an array L2 can hold, loaded with
// an evict-last hint; the slot follows only for rows of more than TINY_MAX
// bits) or its slot alone (slot mode, for frontiers of mostly longer rows):
// count 0 is an empty row, short rows OR their ids into a per-warp
// shared-memory row with 32-bit atomics, and only longer rows are gathered
// whole.  Short rows of a layer with a successor stay in their slots only
// (flag 2, buffer row zero) unless the layer's rows are read directly;
// k_materialize writes them out before a hop that reads rows.  Layers
// written by SPARSE or the seed get their words and slots from the hop's
// pair list (k_pairs_*), layers written by PUSH or an overflowed SPARSE hop
// from their rows (k_slot_build), when the next hop reads them.
// A tiny word is 0 for an empty row; otherwise its top two bits are a class:
// 1 = one id in bits 0..14, 2 = two ids in bits 0..14 and 15..29, 3 = the
// row's bit count (saturated at 0xFFFF) in bits 0..15, its ids in the slot
// when the count is below slot_n.  Short mode runs only for rows of at most
// 512 words (S <= 32768), so source ids fit 15 bits.
using Tiny = uint32_t;
constexpr uint32_t TINY_MAX = 2;    // ids a tiny word holds
constexpr uint32_t CHUNK_IDS = 16;  // uint16 entries per 32-byte chunk of a slot

// Tiny word of a row of `total` bits; part = its first two ids (bits 0..14,
// 15..29) when total <= TINY_MAX.
__host__ __device__ __forceinline__ Tiny tiny_word(uint32_t total, uint32_t part) {
  return total == 0 ? 0u
         : total <= TINY_MAX ? (total << 30) | part
                             : (3u << 30) | (total < 0xFFFFu ? total : 0xFFFFu);
}
// Bit count of a row from its tiny word: exact up to TINY_MAX, else the
// saturated count.
__device__ __forceinline__ uint32_t tiny_count(Tiny t) {
  const uint32_t cls = t >> 30;
  return cls < 3 ? cls : (t & 0xFFFFu);
}

// Bulk prefetch of `bytes` (a multiple of 16, 16-byte aligned) into L2.
__device__ __forceinline__ void prefetch_l2(const void *p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" :: "l"(p), "r"(bytes) : "memory");
}

// Read-only tiny-word load that asks L2 to keep the line (evict-last).
__device__ __forceinline__ Tiny ld_keep(const Tiny *p) {
  uint64_t pol;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  if constexpr (sizeof(Tiny) == 8) {
    uint64_t r;
    asm("ld.global.nc.L2::cache_hint.b64 %0, [%1], %2;" : "=l"(r) : "l"(p), "l"(pol));
    return (Tiny)r;
  } else {
    uint32_t r;
    asm("ld.global.nc.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(r) : "l"(p), "l"(pol));
    return (Tiny)r;
  }
}

// OR the ids of a tiny word (count in [1, TINY_MAX]) into a shared row
__device__ __forceinline__ void or_tiny_ids(uint32_t *row32, Tiny t, uint32_t cnt) {
  const uint32_t id0 = t & 0x7FFFu;
  atomicOr(row32 + (id0 >> 5), 1u << (id0 & 31));
  if (cnt > 1) {
    const uint32_t id1 = (t >> 15) & 0x7FFFu;
    atomicOr(row32 + (id1 >> 5), 1u << (id1 & 31));
  }
}

// OR entries first..last (last < CHUNK_IDS) of one 32-byte slot chunk into
// a shared row; the loop leaves at the warp's longest list
__device__ __forceinline__ void or_chunk_ids(uint32_t *row32, const uint4 s0, const uint4 s1, uint32_t first,
                                             uint32_t last) {
  const uint32_t w[8] = {s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, s1.z, s1.w};
#pragma unroll
  for (uint32_t i = 0; i < CHUNK_IDS; i++) {
    if (i > last) break;
    if (i < first) continue;
    const uint32_t id = (w[i >> 1] >> ((i & 1) * 16)) & 0xFFFFu;
    atomicOr(row32 + (id >> 5), 1u << (id & 31));
  }
}

// OR the ids of a slot (count in [1, slot_n - 1]) whose first chunk is s0/s1
__device__ __forceinline__ void or_slot_ids(uint32_t *row32, const uint4 *sp, const uint4 s0, const uint4 s1,
                                            uint32_t cnt) {
  or_chunk_ids(row32, s0, s1, 1, cnt < CHUNK_IDS - 1 ? cnt : CHUNK_IDS - 1);
  for (uint32_t c0 = CHUNK_IDS; c0 <= cnt; c0 += CHUNK_IDS) {
    const uint32_t left = cnt - c0;  // entries c0..cnt remain
    or_chunk_ids(row32, __ldg(sp + c0 / 8), __ldg(sp + c0 / 8 + 1), 0, left < CHUNK_IDS - 1 ? left : CHUNK_IDS - 1);
  }
}

// One chunk of up to 32 in-neighbours, u / act per lane.  Dense mode: act =
// the row is non-zero (flag).  Short mode: act = the lane holds an
// in-neighbour and tv is its tiny word; short rows OR their ids into row32,
// the others are gathered whole.
template <int L, int UPL, int H, bool SHORT>
__device__ __forceinline__ void gather_chunk(const PullArgs &a, const L2Pol<H> &pol, uint32_t *s_u, uint32_t *row32,
                                             const uint32_t q0, const uint32_t qn, uint4 (&acc)[UPL], uint32_t u,
                                             bool act, Tiny tv, bool slotmode, unsigned long long &se,
                                             const uint4 *pre = nullptr) {
  constexpr int G = 32 / L;
  const int lane = threadIdx.x & 31, g = lane / L, gl = lane % L;
  if (SHORT && act) {
    // slot mode (frontiers of mostly 4..15-bit rows): the slot alone, its
    // entry 0 holds the count (pre: its first chunk, loaded ahead); word
    // mode: the word, then the slot when the row has more ids than the word
    // holds
    const uint4 *sp = a.slot_in + (size_t)u * (a.slot_n / 8);
    uint4 s0 = make_uint4(0, 0, 0, 0), s1 = s0;
    uint32_t cnt;
    if (slotmode) {
      if (pre) {
        s0 = pre[0];
        s1 = pre[1];
      } else {
        s0 = __ldg(sp);
        s1 = __ldg(sp + 1);
      }
      cnt = s0.x & 0xFFFFu;
    } else {
      cnt = tiny_count(tv);
    }
    if (cnt == 0) {
      act = false;
    } else if (!slotmode && cnt <= TINY_MAX) {
      or_tiny_ids(row32, tv, cnt);
      act = false;
      se++;
    } else if (cnt < a.slot_n) {
      if (!slotmode) {
        s0 = __ldg(sp);
        s1 = __ldg(sp + 1);
      }
      or_slot_ids(row32, sp, s0, s1, cnt);
      act = false;
      se++;
    }
  }
  const unsigned m = __ballot_sync(FULL, act);
  if (!m) return;
  if (act) s_u[__popc(m & lanemask_lt())] = u;
  __syncwarp();
  const int n = __popc(m);
  int t = g;
  for (; t + 3 * G < n; t += 4 * G) {
    const uint4 *r0 = a.F + (size_t)s_u[t] * a.Q + q0;
    const uint4 *r1 = a.F + (size_t)s_u[t + G] * a.Q + q0;
    const uint4 *r2 = a.F + (size_t)s_u[t + 2 * G] * a.Q + q0;
    const uint4 *r3 = a.F + (size_t)s_u[t + 3 * G] * a.Q + q0;
#pragma unroll
    for (int k = 0; k < UPL; k++) {
      const uint32_t q = gl + k * L;
      if (q < qn) {
        uint4 x0 = pol.ld_row(r0 + q), x1 = pol.ld_row(r1 + q), x2 = pol.ld_row(r2 + q), x3 = pol.ld_row(r3 + q);
        acc[k] = or4(acc[k], or4(or4(x0, x1), or4(x2, x3)));
      }
    }
  }
  for (; t < n; t += G) {
    const uint4 *r0 = a.F + (size_t)s_u[t] * a.Q + q0;
#pragma unroll
    for (int k = 0; k < UPL; k++) {
      const uint32_t q = gl + k * L;
      if (q < qn) acc[k] = or4(acc[k], pol.ld_row(r0 + q));
    }
  }
  __syncwarp();
}

template <int L, int UPL, int H, bool SHORT>
__device__ __forceinline__ void gather_rows(const PullArgs &a, const L2Pol<H> &pol, uint32_t *s_u, uint32_t *row32,
                                            const uint32_t q0, const uint32_t qn, uint4 (&acc)[UPL],
                                            const uint32_t *adj, int64_t beg, int64_t end,
                                            int64_t step_start, int64_t step, unsigned long long &se,
                                            bool slotmode = false) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = beg + step_start; base < end; base += step) {
    const int64_t j = base + lane;
    uint32_t u = 0;
    bool act = false;
    Tiny tv = 0;
    if (j < end) {
      u = pol.ld_stream(adj + j);
      if (SHORT) {
        if (!slotmode) tv = ld_keep(a.tiny_in + u);
        act = true;
      } else {
        act = __ldg(a.flagF + u) != 0;
      }
    }
    gather_chunk<L, UPL, H, SHORT>(a, pol, s_u, row32, q0, qn, acc, u, act, tv, slotmode, se);
  }
}

// The tiny word and the slot (ids for up to slot_n - 1 bits) of the
// non-zero row of v held by lanes 0..L-1 (uint4 q = lane + k * L).  A short
// row's ids are gathered in the warp's staging slot in shared memory and
// stored with one 16-byte store per lane of the slot; stale entries past the
// count are never read.
template <int L, int UPL>
// c: this lane's bit count of the row (0 past the row's lanes), counted by the caller
__device__ __forceinline__ bool write_short(const PullArgs &a, uint32_t v, const uint4 (&acc)[UPL], uint32_t qn,
                                            uint32_t c, unsigned long long &ns) {
  __shared__ uint4 s_stage[16][8];  // a slot per warp (at most 64 entries, 16 warps)
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const uint32_t total = __reduce_add_sync(FULL, c);
  uint16_t *slot = a.slot_out + (size_t)v * a.slot_n;
  if (total >= a.slot_n) {  // a long row: its count alone
    if (lane == 0) {
      a.tiny_out[v] = tiny_word(total, 0);
      slot[0] = (uint16_t)(total < 0xFFFFu ? total : 0xFFFFu);
    }
    return false;
  }
  // position of this lane's first id: exclusive prefix of the bit counts
  uint32_t excl;
  if (__ballot_sync(FULL, c > 1) == 0) {
    excl = __popc(__ballot_sync(FULL, c != 0) & lanemask_lt());
  } else {
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += y;
    }
    excl = incl - c;
  }
  uint16_t *stage = reinterpret_cast<uint16_t *>(s_stage[wib]);
  if (c) {
    uint32_t pos = 1 + excl;
#pragma unroll
    for (int k = 0; k < UPL; k++) {
      const uint32_t q = lane + k * L;
      if (q < qn) {
        const uint32_t w[4] = {acc[k].x, acc[k].y, acc[k].z, acc[k].w};
#pragma unroll
        for (int wi = 0; wi < 4; wi++) {
          uint32_t bits = w[wi];
          while (bits) {
            stage[pos++] = (uint16_t)(q * 128 + wi * 32 + __ffs(bits) - 1);
            bits &= bits - 1;
          }
        }
      }
    }
  }
  if (lane == 0) stage[0] = (uint16_t)total;
  __syncwarp();
  if ((uint32_t)lane < a.slot_n / 8) reinterpret_cast<uint4 *>(slot)[lane] = s_stage[wib][lane];
  if (lane == 0) {
    // up to two ids ride in the word, more stay in the slot
    a.tiny_out[v] = tiny_word(total, total <= TINY_MAX ? stage[1] | (total > 1 ? (uint32_t)stage[2] << 15 : 0u) : 0u);
    // short rows in the low half, rows of at most TINY_MAX bits in the high half
    ns += 1ull + (total <= TINY_MAX ? 1ull << 32 : 0ull);
  }
  __syncwarp();  // the staging slot is free for the warp's next row
  return true;
}

// Fused epilogue for the row of v held by lanes 0..L-1 after the group reduction:
// visited AND-NOT + update, accumulator OR, next-layer write (and its slot),
// flag, counters.
// PRE: the visited words of the row (vpre, lanes 0..L-1) and the row's
// next-layer flag (oldf_pre) were loaded ahead by the caller.
template <int L, int UPL, int H, bool PRE = false>
__device__ __forceinline__ void pull_epilogue(const PullArgs &a, const L2Pol<H> &pol, uint32_t v,
                                              const uint32_t q0, const uint32_t qn, uint4 (&acc)[UPL],
                                              unsigned long long &nb, unsigned long long &nv,
                                              unsigned long long &ns, const uint4 *vpre = nullptr,
                                              uint32_t oldf_pre = 0) {
  const int lane = threadIdx.x & 31;
  const bool leader_group = lane < L;
  bool any = false;
  uint32_t bits = 0;  // this lane's new bits of the row
  if (leader_group) {
#pragma unroll
    for (int k = 0; k < UPL; k++) {
      const uint32_t q = lane + k * L;
      if (q < qn) {
        const size_t idx = (size_t)v * a.Q + q0 + q;
        uint4 x = acc[k];
        if (a.hmask) {
          const uint4 m = __ldg(a.hmask + q0 + q);
          x = make_uint4(x.x & m.x, x.y & m.y, x.z & m.z, x.w & m.w);
        }
        if (a.shortest && nz4(x)) {
          const uint4 vv = PRE ? vpre[k] : pol.ld_rw(a.vis + idx);
          x = andnot4(x, vv);
          if (nz4(x)) pol.st(a.vis + idx, or4(vv, x));
        }
        if (nz4(x)) {
          any = true;
          bits += popc4(x);
          if (a.acc_on) a.acc[idx] = or4(a.acc[idx], x);
        }
        acc[k] = x;
      }
    }
  }
  nb += bits;
  const bool rownz = __any_sync(FULL, any);
  if (lane == 0 && rownz && (a.res_vis || a.acc_on)) a.resflag[v] = 1;
  if (!a.multislice && a.last) {
    // layer k_max is not kept: clear the rows an earlier layer left in this
    // buffer, so the next run finds it clean (a flag-2 row is zero already)
    const uint32_t oldf = PRE ? oldf_pre : a.flagN[v];
    if (leader_group && oldf == 1) {
#pragma unroll
      for (int k = 0; k < UPL; k++) {
        const uint32_t q = lane + k * L;
        if (q < qn) pol.st(a.N + (size_t)v * a.Q + q0 + q, make_uint4(0, 0, 0, 0));
      }
    }
    if (lane == 0) {
      if (oldf) a.flagN[v] = 0;
      if (rownz) nv++;
    }
  } else if (!a.multislice) {
    const uint32_t oldf = PRE ? oldf_pre : a.flagN[v];  // 1: the buffer row holds an older layer's bits
    bool virt = false;                 // the row is left in its slot only (flag 2)
    if (a.tiny_out) {  // every vertex gets a tiny word: the count is 0 for an empty row
      if (rownz)
        virt = write_short<L, UPL>(a, v, acc, qn, bits, ns) && a.virt_out;
      else if (lane == 0) {
        a.tiny_out[v] = 0;
        a.slot_out[(size_t)v * a.slot_n] = 0;
      }
    }
    if (leader_group && ((rownz && !virt) || oldf == 1)) {
#pragma unroll
      for (int k = 0; k < UPL; k++) {
        const uint32_t q = lane + k * L;
        if (q < qn) pol.st(a.N + (size_t)v * a.Q + q0 + q, virt ? make_uint4(0, 0, 0, 0) : acc[k]);
      }
    }
    if (lane == 0) {
      const uint32_t nf = rownz ? (virt ? 2u : 1u) : 0u;
      if (nf != oldf) a.flagN[v] = nf;
      if (rownz) nv++;
    }
  } else if (rownz) {
    if (leader_group) {
#pragma unroll
      for (int k = 0; k < UPL; k++) {
        const uint32_t q = lane + k * L;
        if (q < qn && nz4(acc[k])) a.N[(size_t)v * a.Q + q0 + q] = acc[k];
      }
    }
    if (lane == 0 && atomicOr(&a.flagN[v], 1u) == 0) nv++;
  }
}

__device__ __forceinline__ void pull_counters(const PullArgs &a, unsigned long long nb, unsigned long long nv,
                                              unsigned long long ns, unsigned long long se) {
  block_add(nb, &a.ctr->hop[a.h].new_bits);
  block_add(nv, &a.ctr->hop[a.h].active_vertices);
  if (a.tiny_out) block_add(ns, &a.ctr->hop[a.h].short_rows);
  if (a.tiny_in) block_add(se, &a.ctr->hop[a.h].short_edges);
}

template <int L, int UPL, int H>
__device__ __forceinline__ void pull_vertices(const PullArgs &a) {
  const L2Pol<H> pol;
  __shared__ uint32_t s_u[8][32];
  const int wib = threadIdx.x >> 5;
  const uint32_t q0 = blockIdx.y * a.qslice;
  const uint32_t qn = min(a.qslice, a.Q - q0);
  unsigned long long nb = 0, nv = 0, ns = 0, se = 0;
  for (uint32_t v = blockIdx.x * 8 + wib; v < a.V; v += gridDim.x * 8) {
    if (a.hub_threshold) {
      int64_t d = 0;
      _Pragma("unroll") for (int l = 0; l < 2; l++) if (l < a.in.n) d += a.in.off[l][v + 1] - a.in.off[l][v];
      if (d > (int64_t)a.hub_threshold) continue;  // handled by k_pull_hub
    }
    uint4 acc[UPL];
#pragma unroll
    for (int k = 0; k < UPL; k++) acc[k] = make_uint4(0, 0, 0, 0);
    _Pragma("unroll") for (int l = 0; l < 2; l++) if (l < a.in.n)
      gather_rows<L, UPL, H, false>(a, pol, s_u[wib], nullptr, q0, qn, acc, a.in.adj[l],
                                    pol.ld_stream(a.in.off[l] + v), pol.ld_stream(a.in.off[l] + v + 1), 0, 32, se);
#pragma unroll
    for (int o = L; o < 32; o <<= 1)
#pragma unroll
      for (int k = 0; k < UPL; k++) acc[k] = or4(acc[k], shfl_xor4(acc[k], o));
    pull_epilogue<L, UPL, H>(a, pol, v, q0, qn, acc, nb, nv, ns);
  }
  pull_counters(a, nb, nv, ns, se);
}

// Short mode (one slice).  Software-pipelined over the warp's targets: while
// target v is processed, the next target's list bounds, first 32
// in-neighbours and their tiny words are already in flight.  PRE: so are the
// next target's visited words (in registers of lanes 0..L-1) and its
// next-layer flag, which the epilogue would otherwise wait for, and the list
// bounds run one target further ahead, so the next target's in-neighbours
// are requested when v starts.
template <int L, int UPL, bool PRE = false>
__device__ __forceinline__ void pull_vertices_short(const PullArgs &a) {
  const L2Pol<0> pol;
  __shared__ uint32_t s_u[8][32];
  extern __shared__ uint4 s_short[];  // [8 warps][Q], the ids of short in-neighbour rows
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const uint32_t qn = a.Q;
  uint4 *srow = s_short + (size_t)wib * a.Q;
  uint32_t *row32 = reinterpret_cast<uint32_t *>(srow);
  for (uint32_t q = lane; q < a.Q; q += 32) srow[q] = make_uint4(0, 0, 0, 0);
  __syncwarp();
  const bool slotmode = a.ctr->hop[a.h].short_slots;
  const int64_t *off0 = a.in.off[0];
  const uint32_t *adj0 = a.in.adj[0];
  const uint32_t stride = gridDim.x * 8;
  unsigned long long nb = 0, nv = 0, ns = 0, se = 0;
  uint32_t v = blockIdx.x * 8 + wib;
  int64_t beg = 0, end = 0;  // list 0 of target v
  uint32_t pu = 0;           // this lane's in-neighbour in v's first chunk
  Tiny pt = 0;               // ... and its tiny word (word mode)
  uint4 ps[2] = {make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};  // ... or its slot's first chunk (slot mode)
  bool pact = false;
  const uint32_t sq = a.slot_n / 8;  // uint4 per slot
  uint4 vpre[UPL];       // PRE: visited words of v held by lanes 0..L-1
  uint32_t oldf = 0;     // PRE: next-layer flag of v
#pragma unroll
  for (int k = 0; k < UPL; k++) vpre[k] = make_uint4(0, 0, 0, 0);
  if (PRE && v < a.V) {
    oldf = a.flagN[v];
    if (a.shortest && lane < L)
#pragma unroll
      for (int k = 0; k < UPL; k++)
        if (lane + k * L < qn) vpre[k] = pol.ld_rw(a.vis + (size_t)v * a.Q + lane + k * L);
  }
  int64_t b1 = 0, e1 = 0;  // PRE: list 0 of the next target, loaded one target ahead
  if (PRE && (uint64_t)v + stride < a.V) {
    b1 = __ldg(off0 + v + stride);
    e1 = __ldg(off0 + v + stride + 1);
  }
  if (v < a.V) {
    beg = __ldg(off0 + v);
    end = __ldg(off0 + v + 1);
    if (beg + lane < end) {
      pu = __ldg(adj0 + beg + lane);
      if (slotmode) {
        ps[0] = __ldg(a.slot_in + (size_t)pu * sq);
        ps[1] = __ldg(a.slot_in + (size_t)pu * sq + 1);
      } else {
        pt = ld_keep(a.tiny_in + pu);
      }
      pact = true;
    }
  }
  for (; v < a.V; v += stride) {
    const uint32_t vn = v + stride;
    int64_t nbeg = 0, nend = 0, b2 = 0, e2 = 0;
    if (PRE) {  // the next target's bounds arrived during v - stride; fetch those of vn + stride
      nbeg = b1;
      nend = e1;
      const uint64_t v2 = (uint64_t)vn + stride;
      if (v2 < a.V) {
        b2 = __ldg(off0 + v2);
        e2 = __ldg(off0 + v2 + 1);
      }
    } else if (vn < a.V) {
      nbeg = __ldg(off0 + vn);
      nend = __ldg(off0 + vn + 1);
    }
    int64_t d = end - beg;
    if (a.in.n > 1) d += a.in.off[1][v + 1] - a.in.off[1][v];
    uint32_t pun = 0;
    Tiny ptn = 0;
    uint4 psn[2] = {make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
    const bool pactn = nbeg + lane < nend;
    if (PRE && pactn) pun = __ldg(adj0 + nbeg + lane);  // in flight during all of v
    uint4 vpren[UPL];
    uint32_t oldfn = 0;
#pragma unroll
    for (int k = 0; k < UPL; k++) vpren[k] = make_uint4(0, 0, 0, 0);
    if (PRE && vn < a.V) {  // the next target's visited words and flag, in flight during v
      oldfn = a.flagN[vn];
      if (a.shortest && lane < L)
#pragma unroll
        for (int k = 0; k < UPL; k++)
          if (lane + k * L < qn) vpren[k] = pol.ld_rw(a.vis + (size_t)vn * a.Q + lane + k * L);
    }
    if (!(a.hub_threshold && d > (int64_t)a.hub_threshold)) {  // hubs: k_pull_hub_short
      if (lane == 0) {  // the epilogue's read-modify-write rows, fetched while the gather runs
        if (a.shortest && !PRE) prefetch_l2(a.vis + (size_t)v * a.Q, qn * 16);
        if (a.acc_on) prefetch_l2(a.acc + (size_t)v * a.Q, qn * 16);
      }
      uint4 acc[UPL];
#pragma unroll
      for (int k = 0; k < UPL; k++) acc[k] = make_uint4(0, 0, 0, 0);
      gather_chunk<L, UPL, 0, true>(a, pol, s_u[wib], row32, 0, qn, acc, pu, pact, pt, slotmode, se, ps);
      if (!PRE && pactn) pun = __ldg(adj0 + nbeg + lane);  // in flight during the rest of v
      gather_rows<L, UPL, 0, true>(a, pol, s_u[wib], row32, 0, qn, acc, adj0, beg + 32, end, 0, 32, se, slotmode);
      if (a.in.n > 1)
        gather_rows<L, UPL, 0, true>(a, pol, s_u[wib], row32, 0, qn, acc, a.in.adj[1], a.in.off[1][v],
                                     a.in.off[1][v + 1], 0, 32, se, slotmode);
#pragma unroll
      for (int o = L; o < 32; o <<= 1)
#pragma unroll
        for (int k = 0; k < UPL; k++) acc[k] = or4(acc[k], shfl_xor4(acc[k], o));
      __syncwarp();
      if (lane < L) {
#pragma unroll
        for (int k = 0; k < UPL; k++) {
          const uint32_t q = lane + k * L;
          if (q < qn) {
            acc[k] = or4(acc[k], srow[q]);
            srow[q] = make_uint4(0, 0, 0, 0);
          }
        }
      }
      __syncwarp();
      if (pactn) {  // in flight during the epilogue
        if (slotmode) {
          psn[0] = __ldg(a.slot_in + (size_t)pun * sq);
          psn[1] = __ldg(a.slot_in + (size_t)pun * sq + 1);
        } else {
          ptn = ld_keep(a.tiny_in + pun);
        }
      }
      pull_epilogue<L, UPL, 0, PRE>(a, pol, v, 0, qn, acc, nb, nv, ns, vpre, oldf);
    } else if (pactn) {
      if (!PRE) pun = __ldg(adj0 + nbeg + lane);
      if (slotmode) {
        psn[0] = __ldg(a.slot_in + (size_t)pun * sq);
        psn[1] = __ldg(a.slot_in + (size_t)pun * sq + 1);
      } else {
        ptn = ld_keep(a.tiny_in + pun);
      }
    }
    beg = nbeg;
    end = nend;
    pu = pun;
    pt = ptn;
    ps[0] = psn[0];
    ps[1] = psn[1];
    pact = pactn;
    b1 = b2;
    e1 = e2;
    oldf = oldfn;
#pragma unroll
    for (int k = 0; k < UPL; k++) vpre[k] = vpren[k];
  }
  pull_counters(a, nb, nv, ns, se);
}

template <int L, int UPL, int MINB, int H>
__global__ void __launch_bounds__(256, MINB) k_pull(PullArgs a) {
  if (a.ctr->hop[a.h].strategy != ST_PULL || a.ctr->hop[a.h].short_pull) return;
  pull_vertices<L, UPL, H>(a);
}

// the same in short mode (its own kernel: the slot path's registers stay out
// of the dense kernels' budget)
template <int L, int UPL>
__global__ void __launch_bounds__(256, UPL >= 4 ? 2 : 5) k_pull_short(PullArgs a) {
  if (a.ctr->hop[a.h].strategy != ST_PULL || !a.ctr->hop[a.h].short_pull || !a.tiny_in || a.pre) return;
  pull_vertices_short<L, UPL>(a);
}

// ... with the visited words and flag of the next target loaded ahead
template <int L, int UPL>
__global__ void __launch_bounds__(256, UPL >= 4 ? 2 : UPL == 2 ? 3 : 4) k_pull_short_pre(PullArgs a) {
  if (a.ctr->hop[a.h].strategy != ST_PULL || !a.ctr->hop[a.h].short_pull || !a.tiny_in || !a.pre) return;
  pull_vertices_short<L, UPL, true>(a);
}

// Hub vertices (in-degree above the threshold): one 512-thread CTA per vertex,
// warps stride over the in-list, rows reduced through shared memory (short
// rows through one shared row of the CTA).
template <int L, int UPL, bool SHORT>
__device__ __forceinline__ void pull_hubs(const PullArgs &a) {
  extern __shared__ uint4 s_red[];  // [16 warps][32 lanes][UPL], then SHORT: one row of Q
  const L2Pol<0> pol;
  __shared__ uint32_t s_u[16][32];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const uint32_t q0 = blockIdx.y * a.qslice;
  const uint32_t qn = min(a.qslice, a.Q - q0);
  uint4 *srow = s_red + 16 * 32 * UPL;
  if (SHORT) {
    for (uint32_t q = threadIdx.x; q < a.Q; q += blockDim.x) srow[q] = make_uint4(0, 0, 0, 0);
    __syncthreads();
  }
  unsigned long long nb = 0, nv = 0, ns = 0, se = 0;
  for (uint32_t hi = blockIdx.x; hi < a.nhubs; hi += gridDim.x) {
    const uint32_t v = a.hubs[hi];
    uint4 acc[UPL];
#pragma unroll
    for (int k = 0; k < UPL; k++) acc[k] = make_uint4(0, 0, 0, 0);
    _Pragma("unroll") for (int l = 0; l < 2; l++) if (l < a.in.n)
      gather_rows<L, UPL, 0, SHORT>(a, pol, s_u[wib], reinterpret_cast<uint32_t *>(srow), q0, qn, acc,
                                    a.in.adj[l], a.in.off[l][v], a.in.off[l][v + 1], (int64_t)wib * 32,
                                    (int64_t)nw * 32, se, SHORT && a.ctr->hop[a.h].short_slots);
#pragma unroll
    for (int o = L; o < 32; o <<= 1)
#pragma unroll
      for (int k = 0; k < UPL; k++) acc[k] = or4(acc[k], shfl_xor4(acc[k], o));
    if (lane < L)
#pragma unroll
      for (int k = 0; k < UPL; k++) s_red[(wib * 32 + lane) * UPL + k] = acc[k];
    __syncthreads();
    if (wib == 0) {
      if (lane < L) {
        for (int w = 1; w < nw; w++)
#pragma unroll
          for (int k = 0; k < UPL; k++) acc[k] = or4(acc[k], s_red[(w * 32 + lane) * UPL + k]);
        if (SHORT) {
#pragma unroll
          for (int k = 0; k < UPL; k++) {
            const uint32_t q = lane + k * L;
            if (q < qn) acc[k] = or4(acc[k], srow[q]);
          }
        }
      }
      pull_epilogue<L, UPL, 0>(a, pol, v, q0, qn, acc, nb, nv, ns);
    }
    __syncthreads();
    if (SHORT) {
      for (uint32_t q = threadIdx.x; q < a.Q; q += blockDim.x) srow[q] = make_uint4(0, 0, 0, 0);
      __syncthreads();
    }
  }
  pull_counters(a, nb, nv, ns, se);
}

template <int L, int UPL>
__global__ void __launch_bounds__(512) k_pull_hub(PullArgs a) {
  if (a.ctr->hop[a.h].strategy != ST_PULL || a.ctr->hop[a.h].short_pull || a.nhubs == 0) return;
  pull_hubs<L, UPL, false>(a);
}

template <int L, int UPL>
__global__ void __launch_bounds__(512) k_pull_hub_short(PullArgs a) {
  if (a.ctr->hop[a.h].strategy != ST_PULL || !a.ctr->hop[a.h].short_pull || !a.tiny_in || a.nhubs == 0) return;
  pull_hubs<L, UPL, true>(a);
}

// Rows of layer h-1 left in their slots (flag 2), written out whole when hop
// h reads rows: a dense PULL or a PUSH (a short-mode PULL reads the slots).
// prev_virt: the PULL of hop h-1 was allowed to leave rows in their slots.
__global__ void k_materialize(uint32_t *__restrict__ flagF, uint4 *__restrict__ F, uint32_t V, uint32_t Q,
                              const uint16_t *__restrict__ slots, uint32_t slot_n, const Ctr *ctr, int h,
                              int prev_virt) {
  const HopCtr &p = ctr->hop[h - 1], &c = ctr->hop[h];
  if (!prev_virt || p.strategy != ST_PULL || (p.short_rows & 0xFFFFFFFFull) == 0) return;
  if (c.strategy == 0 || (c.strategy == ST_PULL && c.short_pull)) return;
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t base = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; base < V; base += warps * 32) {
    const uint32_t v = base + lane;
    unsigned m = __ballot_sync(FULL, v < V && flagF[v] == 2);
    while (m) {
      const int b = __ffs(m) - 1;
      m &= m - 1;
      const uint32_t r = base + b;
      const uint16_t *slot = slots + (size_t)r * slot_n;
      const uint32_t cnt = slot[0];
      for (uint32_t q0 = 0; q0 < Q; q0 += 32) {
        const uint32_t q = q0 + lane;
        uint32_t w[4] = {0, 0, 0, 0};
        for (uint32_t i = 1; i <= cnt; i++) {
          const uint32_t id = slot[i];
          if (id >> 7 == q) w[(id >> 5) & 3] |= 1u << (id & 31);
        }
        if (q < Q) F[(size_t)r * Q + q] = make_uint4(w[0], w[1], w[2], w[3]);
      }
      if (lane == 0) flagF[r] = 1;
    }
  }
}

// Word and slot of row r held in one chunk (Q <= 32: lane q holds uint4 q).
__device__ __forceinline__ void short_from_chunk(uint4 x, uint32_t r, Tiny *tiny, uint16_t *slots,
                                                 uint32_t slot_n) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t n = popc4(x);
  uint32_t incl = n;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(FULL, incl, o);
    if (lane >= (uint32_t)o) incl += y;
  }
  const uint32_t total = __shfl_sync(FULL, incl, 31);
  uint32_t part = 0;  // ids 1 and 2 of the row, in tiny-word positions
  uint16_t *slot = slots + (size_t)r * slot_n;
  if (total < slot_n) {
    uint32_t at = 1 + incl - n;
    const uint32_t w[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
    for (int wi = 0; wi < 4; wi++) {
      uint32_t bits = w[wi];
      while (bits) {
        const uint32_t t = __ffs(bits) - 1;
        bits &= bits - 1;
        const uint32_t id = lane * 128 + wi * 32 + t;
        if (at <= TINY_MAX) part |= id << (15 * (at - 1));
        slot[at] = (uint16_t)id;
        at++;
      }
    }
  }
  part = __reduce_or_sync(FULL, part);
  if (lane == 0) {
    tiny[r] = tiny_word(total, part);
    slot[0] = (uint16_t)(total < 0xFFFFu ? total : 0xFFFFu);
  }
}

// Hop h pulls in short mode over a layer that SPARSE (without overflow) or
// the seed wrote: that hop left exactly one (vertex, source) pair per bit, so
// the words and slots are built from the pair list instead of the rows.
__device__ __forceinline__ bool pairs_build(const Ctr *c, int h) {
  const HopCtr &cur = c->hop[h], &p = c->hop[h - 1];
  return cur.strategy == ST_PULL && cur.short_pull && (h == 1 || (p.strategy == ST_SPARSE && !p.overflow));
}

// Rows of a layer a SPARSE hop left in its pair list (Shortest: the hop
// dedups through the visited bits and writes no next-layer words), built
// before hop h reads them.  mode 0, right after hop h's decision: every pair
// when hop h reads whole rows (PUSH, dense or multi-slice PULL) or builds its
// short-row index from rows (the list overflowed); mode 1, after the index
// was built from the pairs: the pairs of rows too long for a slot, which a
// short-mode PULL gathers whole.  SPARSE reads only pairs.
__global__ void k_pairs_rows(const uint2 *__restrict__ pairs, const uint32_t *__restrict__ cnt,
                             unsigned long long *__restrict__ N, uint32_t W, uint32_t slot_n, uint64_t cap,
                             const Ctr *ctr, int h, int mode) {
  if (ctr->hop[h - 1].strategy != ST_SPARSE) return;
  const int s = ctr->hop[h].strategy;
  const bool go = mode == 0 ? (s == ST_PUSH || (s == ST_PULL && !pairs_build(ctr, h))) : pairs_build(ctr, h);
  if (!go) return;
  const unsigned long long np_raw = ctr->hop[h - 1].pairs;
  const uint64_t np = np_raw < cap ? np_raw : cap;
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < np; k += (uint64_t)gridDim.x * blockDim.x) {
    const uint2 pr = pairs[k];
    if (mode == 1 && cnt[pr.x] < slot_n) continue;
    atomicOr(&N[(size_t)pr.x * W + (pr.y >> 6)], 1ull << (pr.y & 63));
  }
}

__global__ void k_pairs_zero(uint32_t *__restrict__ cnt, uint32_t V, const Ctr *ctr, int h) {
  if (!pairs_build(ctr, h)) return;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) cnt[v] = 0;
}

// every pair's source id into its vertex's slot (entries 1.., in any order)
__global__ void k_pairs_slots(const uint2 *__restrict__ pairs, uint32_t *__restrict__ cnt, uint16_t *__restrict__ slots,
                              uint32_t slot_n, uint64_t cap, const Ctr *ctr, int h) {
  if (!pairs_build(ctr, h)) return;
  const unsigned long long np_raw = ctr->hop[h - 1].pairs;
  const uint64_t np = np_raw < cap ? np_raw : cap;
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < np; k += (uint64_t)gridDim.x * blockDim.x) {
    const uint2 pr = pairs[k];
    const uint32_t at = atomicAdd(&cnt[pr.x], 1u) + 1;
    if (at < slot_n) slots[(size_t)pr.x * slot_n + at] = (uint16_t)pr.y;
  }
}

// the tiny word of every vertex from its pair count (0 for an empty row)
__global__ void k_pairs_words(const uint32_t *__restrict__ flagF, const uint32_t *__restrict__ cnt,
                              Tiny *__restrict__ tiny, uint16_t *__restrict__ slots, uint32_t slot_n, uint32_t V,
                              const Ctr *ctr, int h) {
  if (!pairs_build(ctr, h)) return;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const uint32_t c = flagF[v] ? cnt[v] : 0u;
    uint32_t part = 0;
    if (c && c <= TINY_MAX) {
      part = slots[(size_t)v * slot_n + 1];
      if (c > 1) part |= (uint32_t)slots[(size_t)v * slot_n + 2] << 15;
    }
    tiny[v] = tiny_word(c, part);
    if (c) slots[(size_t)v * slot_n] = (uint16_t)(c < 0xFFFFu ? c : 0xFFFFu);
  }
}

// Tiny words and slots of layer h-1 when hop h pulls in short mode and that
// layer was written by PUSH or by a SPARSE hop whose pair list overflowed: a warp per
// flagged row counts its bits and writes its word (and slot); every other
// vertex gets the count 0.
__global__ void k_slot_build(const uint32_t *__restrict__ flagF, const uint4 *__restrict__ F, uint32_t V,
                             uint32_t Q, Tiny *__restrict__ tiny, uint16_t *__restrict__ slots, uint32_t slot_n,
                             const Ctr *ctr, int h) {
  if (ctr->hop[h].strategy != ST_PULL || !ctr->hop[h].short_pull || ctr->hop[h - 1].strategy == ST_PULL ||
      pairs_build(ctr, h))
    return;
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t base = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; base < V; base += warps * 32) {
    const uint32_t v = base + lane;
    const bool f = v < V && flagF[v];
    if (v < V && !f) {  // empty row
      tiny[v] = 0;
      slots[(size_t)v * slot_n] = 0;
    }
    unsigned m = __ballot_sync(FULL, f);
    if (Q <= 32) {  // one chunk per row: four rows' loads in flight at once
      while (m) {
        uint32_t rr[4] = {0, 0, 0, 0};
        int n = 0;
#pragma unroll
        for (int k = 0; k < 4; k++)
          if (m) {
            rr[k] = base + __ffs(m) - 1;
            m &= m - 1;
            n = k + 1;
          }
        uint4 x[4];
#pragma unroll
        for (int k = 0; k < 4; k++)
          x[k] = (k < n && (uint32_t)lane < Q) ? F[(size_t)rr[k] * Q + lane] : make_uint4(0, 0, 0, 0);
#pragma unroll
        for (int k = 0; k < 4; k++)
          if (k < n) short_from_chunk(x[k], rr[k], tiny, slots, slot_n);
      }
      continue;
    }
    while (m) {
      const int b = __ffs(m) - 1;
      m &= m - 1;
      const uint32_t r = base + b;
      const uint4 *row = F + (size_t)r * Q;
      uint32_t c = 0;
      for (uint32_t q = lane; q < Q; q += 32) c += popc4(row[q]);
      const uint32_t total = warp_sum(c);
      uint32_t part = 0;  // ids 1 and 2 of the row, in tiny-word positions
      uint16_t *slot = slots + (size_t)r * slot_n;
      if (total < slot_n) {
        uint32_t pos = 1;
        for (uint32_t q0 = 0; q0 < Q; q0 += 32) {
          const uint32_t q = q0 + lane;
          const uint4 x = q < Q ? row[q] : make_uint4(0, 0, 0, 0);
          const uint32_t n = popc4(x);
          uint32_t incl = n;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
          }
          uint32_t at = pos + incl - n;
          const uint32_t w[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
          for (int wi = 0; wi < 4; wi++) {
            uint32_t bits = w[wi];
            while (bits) {
              const uint32_t t = __ffs(bits) - 1;
              bits &= bits - 1;
              const uint32_t id = q * 128 + wi * 32 + t;
              if (at <= TINY_MAX) part |= id << (15 * (at - 1));
              slot[at] = (uint16_t)id;
              at++;
            }
          }
          pos += __shfl_sync(FULL, incl, 31);
        }
      }
      part = __reduce_or_sync(FULL, part);
      if (lane == 0) {
        tiny[r] = tiny_word(total, part);
        slot[0] = (uint16_t)(total < 0xFFFFu ? total : 0xFFFFu);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// PUSH.  Active rows of layer h-1 (flag set) are compacted into a list; a warp
// per active vertex ORs its row into each out-neighbour's next-layer row with
// 64-bit atomics and records first touches; a second pass over the touched
// list applies the visited AND-NOT and the accumulator (Shortest/Any rules).
__global__ void k_push_compact(const uint32_t *__restrict__ flagF, uint32_t V, uint32_t *list,
                               Ctr *ctr, int h) {
  if (ctr->hop[h].strategy != ST_PUSH) return;
  const int lane = threadIdx.x & 31;
  for (uint32_t v0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; v0 < V;
       v0 += gridDim.x * blockDim.x) {
    const uint32_t v = v0 + lane;
    const bool f = v < V && flagF[v];
    const unsigned m = __ballot_sync(FULL, f);
    if (!m) continue;
    unsigned base = 0;
    if (lane == 0) base = atomicAdd(&ctr->push_active, (unsigned)__popc(m));
    base = __shfl_sync(FULL, base, 0);
    if (f) list[base + __popc(m & lanemask_lt())] = v;
  }
}

__global__ void __launch_bounds__(256) k_push(PushArgs a) {
  Ctr *c = a.ctr;
  if (c->hop[a.h].strategy != ST_PUSH) return;
  const uint32_t n = c->push_active;
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < n; t += warps) {
    const uint32_t u = a.active[t];
    const unsigned long long *row = a.F + (size_t)u * a.W;
    _Pragma("unroll") for (int l = 0; l < 2; l++) if (l < a.out.n) {
      const int64_t beg = a.out.off[l][u], end = a.out.off[l][u + 1];
      for (int64_t j = beg; j < end; j++) {
        const uint32_t v = __ldg(a.out.adj[l] + j);
        unsigned long long *dst = a.N + (size_t)v * a.W;
        for (uint32_t w = lane; w < a.W; w += 32) {
          const unsigned long long x = row[w];
          if (x) atomicOr(dst + w, x);
        }
        if (lane == 0 && atomicOr(&a.flagN[v], 1u) == 0) {
          unsigned s = atomicAdd(&c->push_touched, 1u);
          a.touched[s] = v;
        }
      }
    }
  }
}

__global__ void __launch_bounds__(256) k_push_epilogue(PushArgs a) {
  Ctr *c = a.ctr;
  if (c->hop[a.h].strategy != ST_PUSH) return;
  const uint32_t n = c->push_touched;
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  unsigned long long nb = 0, nv = 0;
  for (uint32_t t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < n; t += warps) {
    const uint32_t v = a.touched[t];
    bool any = false;
    for (uint32_t w = lane; w < a.W; w += 32) {
      const size_t idx = (size_t)v * a.W + w;
      unsigned long long x = a.N[idx];
      const unsigned long long x0 = x;
      if (a.hmask) x &= a.hmask[w];
      if (a.shortest && x) {
        const unsigned long long vv = a.vis[idx];
        x &= ~vv;
        if (x) a.vis[idx] = vv | x;
      }
      if (x != x0) a.N[idx] = x;
      if (x) {
        any = true;
        nb += __popcll(x);
        if (a.acc_on) a.acc[idx] |= x;
      }
    }
    const bool rownz = __any_sync(FULL, any);
    if (lane == 0) {
      if (!rownz)
        a.flagN[v] = 0;  // row is all zero again
      else
        nv++;
      if (rownz && (a.res_vis || a.acc_on)) a.resflag[v] = 1;
    }
  }
  block_add(nb, &c->hop[a.h].new_bits);
  block_add(nv, &c->hop[a.h].active_vertices);
}

__global__ void k_push_reset(Ctr *c) {
  c->push_active = 0;
  c->push_touched = 0;
}

// FindShortest target check of hop h (vexpand.cpp:237-271).
__global__ void k_find_check(const uint64_t *__restrict__ N, const uint32_t *__restrict__ tgt,
                             int32_t *__restrict__ dist, uint32_t S, uint32_t W, uint32_t V,
                             Ctr *ctr, int h) {
  if (ctr->hop[h].strategy == 0) return;
  unsigned long long f = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < S; i += gridDim.x * blockDim.x) {
    if (tgt[i] < V && dist[i] == -1 && ((N[(size_t)tgt[i] * W + (i >> 6)] >> (i & 63)) & 1ull)) {
      dist[i] = h;
      f++;
    }
  }
  block_add(f, &ctr->found);
}

// Shortest with k_min == 1: the result is visited minus layer 0, i.e. the
// source bits (i, s_i) cleared (a source is never re-reached once visited).
__global__ void k_clear_diag(uint64_t *__restrict__ vis, const uint32_t *__restrict__ src,
                             uint32_t S, uint32_t W, uint32_t V) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < S; i += gridDim.x * blockDim.x)
    if (src[i] < V) atomicAnd((unsigned long long *)&vis[(size_t)src[i] * W + (i >> 6)], ~(1ull << (i & 63)));
}

// Hub list of a direction set (degree above the threshold).
__global__ void k_hubs(Lists in, uint32_t V, uint32_t thr, uint32_t *list, unsigned *n) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    int64_t d = 0;
    _Pragma("unroll") for (int l = 0; l < 2; l++) if (l < in.n) d += in.off[l][v + 1] - in.off[l][v];
    if (d > (int64_t)thr) list[atomicAdd(n, 1u)] = v;
  }
}

// ---------------------------------------------------------------------------
// Host side.

Lists pull_lists(const vs_graph *g, int dir) {
  Lists L;
  L.n = 0;
  const bool fwd = !g->directed || dir == VS_DIR_FORWARD || dir == VS_DIR_BOTH;
  const bool bwd = g->directed && (dir == VS_DIR_BACKWARD || dir == VS_DIR_BOTH);
  if (fwd) {  // in-lists of the target: reverse CSR
    L.off[L.n] = g->rev_off;
    L.adj[L.n] = g->rev_src;
    L.n++;
  }
  if (bwd) {
    L.off[L.n] = g->fwd_off;
    L.adj[L.n] = g->fwd_dst;
    L.n++;
  }
  return L;
}

Lists push_lists(const vs_graph *g, int dir) {
  Lists L;
  L.n = 0;
  const bool fwd = !g->directed || dir == VS_DIR_FORWARD || dir == VS_DIR_BOTH;
  const bool bwd = g->directed && (dir == VS_DIR_BACKWARD || dir == VS_DIR_BOTH);
  if (fwd) {
    L.off[L.n] = g->fwd_off;
    L.adj[L.n] = g->fwd_dst;
    L.n++;
  }
  if (bwd) {
    L.off[L.n] = g->rev_off;
    L.adj[L.n] = g->rev_src;
    L.n++;
  }
  return L;
}

using PullFn = void (*)(PullArgs);

struct PullVariant {
  int L, UPL;
  PullFn pull[4], hub;  // pull[k]: bit 0 = 8 blocks per SM, bit 1 = L2 cache policies
  PullFn pull_short, hub_short, pull_short_pre;
};

#define VS_PULLS(L, U) {k_pull<L, U, 1, 0>, k_pull<L, U, 8, 0>, k_pull<L, U, 1, 1>, k_pull<L, U, 8, 1>}
#define VS_VARIANT(L, U) \
  {L, U, VS_PULLS(L, U), k_pull_hub<L, U>, k_pull_short<L, U>, k_pull_hub_short<L, U>, k_pull_short_pre<L, U>}
const PullVariant kVariants[] = {
    VS_VARIANT(1, 1),  VS_VARIANT(2, 1),  VS_VARIANT(4, 1),  VS_VARIANT(8, 1), VS_VARIANT(16, 1),
    VS_VARIANT(32, 1), VS_VARIANT(32, 2), VS_VARIANT(32, 4), VS_VARIANT(32, 8),
};
#undef VS_VARIANT
#undef VS_PULLS

const PullVariant &pick_variant(uint32_t qslice) {
  for (const auto &v : kVariants)
    if ((uint32_t)(v.L * v.UPL) >= qslice) return v;
  return kVariants[sizeof(kVariants) / sizeof(kVariants[0]) - 1];
}

}  // namespace ex
}  // namespace vs

using namespace vs;
using namespace vs::ex;

struct vs_expand_plan {
  vs_graph *g = nullptr;
  vs_expand_params p{};
  uint32_t S = 0, W = 0, Q = 0, qslice = 0, nslices = 1;
  uint64_t *buf[2] = {nullptr, nullptr};
  uint32_t *flag[2] = {nullptr, nullptr};
  uint64_t *vis = nullptr, *acc = nullptr;
  uint2 *pairs[2] = {nullptr, nullptr};
  unsigned long long *pdeg[2] = {nullptr, nullptr}, *doff = nullptr, *bsum = nullptr;
  uint64_t pair_cap = 0;
  uint32_t *push_list = nullptr, *touched = nullptr;
  uint32_t *resflag = nullptr;  // per vertex: result column may be non-zero
  uint32_t *d_src = nullptr, *d_tgt = nullptr;
  int32_t *d_dist = nullptr;
  Ctr *ctr = nullptr;
  uint32_t *hubs = nullptr;
  uint32_t nhubs = 0, hub_threshold = 0;
  bool use_vis = false, use_acc = false, clear_diag = false;
  bool collect_stats = false;
  int grid_pull = 0, grid_hub = 0, grid_sparse = 0, grid_v = 0, grid_push = 0, grid_short = 0, grid_short_pre = 0;
  vs_bitmat result{};
  bool has_result = false;
  // tuning knobs of the fixed planner
  double sparse_frac = 0.02, push_frac = 0.0;
  const void *picker = nullptr;
  bool log_features = false;
  int pull_kind = 0;  // PULL kernel variant (bit 0: 8 blocks/SM bound, bit 1: L2 policies)
  uint64_t *hmask = nullptr;  // (k_max + 1) x W words: rows allowed to grow at hop h
  uint32_t *rowk = nullptr;   // [0] largest row limit, [1] a limit exceeded k_max (device-set limits)
  uint64_t *layer_out[VS_MAX_HOPS + 1] = {};  // with_distance: layer h is copied here (zeroed, V x W words)
  // short-row index of the two frontier buffers' layers; none when S > 32768 or multi-slice
  Tiny *tiny[2] = {nullptr, nullptr};      // short-row words
  uint16_t *slot[2] = {nullptr, nullptr};  // ... and their slots
  uint32_t slot_n = 16;                    // uint16 entries per slot
  double short_min = 0.0;                  // share of short rows for a short-mode PULL (0: off)
  bool use_hmask = false;
  int hop_forced[VS_MAX_HOPS + 1] = {};
  bool timing = false;
  uint32_t timed_hops = 0;
  cudaStream_t last_stream = 0;  // frees are ordered after the last run on it
  cudaEvent_t ev[3 * (VS_MAX_HOPS + 1)] = {};
  // one-shot cache: the caller's parameters, the graph's serial, the plan's
  // device bytes and the event its last user's stream recorded
  vs_expand_params key{};
  uint64_t graph_serial = 0, bytes = 0;
  cudaEvent_t cache_ev = nullptr;
};

namespace vs {
namespace ex {

// Any with k_min == k_max returns layer k_max itself: no accumulator (the last
// frontier buffer is the result).  Any over a range, and Shortest with
// k_min >= 2, union layers k_min..k_max into an accumulator.
inline bool needs_acc(const vs_expand_params &p) {
  return (p.path_type == VS_PATH_ANY && p.k_min != p.k_max) ||
         (p.path_type == VS_PATH_SHORTEST && p.k_min >= 2);
}

// uint16 entries of a short-row slot for rows of W words: a sixteenth of
// the row's bytes at 64 and 128 words, 128 bytes beyond.
inline uint32_t slot_entries(uint32_t W) { return W <= 64 ? 16 : W <= 128 ? 32 : 64; }

// Short-row words and slots (15-bit ids: S <= 32768) need rows in one slice, and short
// mode runs only on frontiers larger than half of L2 (unless forced: share >
// 1): a graph whose whole V x W matrix fits there never uses them.
inline bool short_slots_ok(uint32_t S, uint32_t nslices, double share, uint64_t V, uint32_t W) {
  return share >= 0 && S <= 32768 && nslices == 1 && (share > 1.0 || V * 8ull * W > l2_bytes() / 2);
}

int plan_free(vs_expand_plan *pl) {
  if (!pl) return VS_OK;
  const cudaStream_t st = pl->last_stream;
  void *ptrs[] = {pl->tiny[0], pl->tiny[1], pl->slot[0], pl->slot[1], pl->resflag, pl->pdeg[0], pl->pdeg[1], pl->doff,
                  pl->bsum, pl->hmask, pl->rowk, pl->buf[0], pl->buf[1], pl->flag[0], pl->flag[1], pl->vis, pl->acc,
                  pl->pairs[0], pl->pairs[1], pl->push_list, pl->touched, pl->d_src,
                  pl->d_tgt, pl->d_dist, pl->ctr, pl->hubs};
  for (void *p : ptrs)  // stream-ordered after the plan's last run
    if (p) dfree(p, st);
  for (cudaEvent_t e : pl->ev)
    if (e) cudaEventDestroy(e);
  if (pl->cache_ev) cudaEventDestroy(pl->cache_ev);
  delete pl;
  return VS_OK;
}

// The one-shot vs_expand keeps its plans: a call takes an idle plan built for
// the same graph, source count and parameters (or builds one), runs it and
// hands out the result as a view whose release returns the plan.  Reuse skips
// the allocations, the full-matrix clears of a new plan and its hub list; a
// run clears only what the previous run wrote.  At most kCacheIdle idle plans
// are kept, holding at most a quarter of the device's memory (48 GB at
// least); vs_release_cached frees them all.
constexpr size_t kCacheIdle = 8;

uint64_t cache_bytes_cap() {
  static uint64_t cap = 0;
  if (cap == 0) {
    size_t free_b = 0, total_b = 0;
    cap = 48ull << 30;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) cap = std::max<uint64_t>(cap, total_b / 4);
  }
  return cap;
}

struct PlanCache {
  std::mutex mu;
  std::vector<vs_expand_plan *> idle;  // oldest first
  std::vector<uint64_t> dead;          // serials of freed graphs (plans lent out then are freed on return)
};
PlanCache &plan_cache() {
  static PlanCache c;
  return c;
}

bool same_params(const vs_expand_params &a, const vs_expand_params &b) {
  return a.k_min == b.k_min && a.k_max == b.k_max && a.path_type == b.path_type && a.direction == b.direction &&
         a.strategy == b.strategy && a.use_picker == b.use_picker && a.hub_threshold == b.hub_threshold &&
         a.slice_words == b.slice_words && a.pair_capacity == b.pair_capacity && a.pull_kernel == b.pull_kernel &&
         a.sparse_frac == b.sparse_frac && a.short_share == b.short_share;
}

vs_expand_plan *plan_cache_take(const vs_graph *g, uint32_t S, const vs_expand_params &p) {
  PlanCache &c = plan_cache();
  std::lock_guard<std::mutex> lk(c.mu);
  for (size_t i = c.idle.size(); i-- > 0;) {
    vs_expand_plan *pl = c.idle[i];
    if (pl->graph_serial == g->serial && pl->S == S && same_params(pl->key, p)) {
      c.idle.erase(c.idle.begin() + (long)i);
      return pl;
    }
  }
  return nullptr;
}

void plan_cache_trim(PlanCache &c, std::vector<vs_expand_plan *> &drop) {
  uint64_t bytes = 0;
  for (vs_expand_plan *pl : c.idle) bytes += pl->bytes;
  const uint64_t cap = cache_bytes_cap();
  while (!c.idle.empty() && (c.idle.size() > kCacheIdle || bytes > cap)) {
    bytes -= c.idle.front()->bytes;
    drop.push_back(c.idle.front());
    c.idle.erase(c.idle.begin());
  }
}

}  // namespace ex

uint64_t next_graph_serial() {
  static std::atomic<uint64_t> n{1};
  return n++;
}

void plan_cache_return(vs_expand_plan *pl, cudaStream_t st) {
  using namespace ex;
  if (!pl->cache_ev) cudaEventCreateWithFlags(&pl->cache_ev, cudaEventDisableTiming);
  if (pl->cache_ev) cudaEventRecord(pl->cache_ev, st);  // the next user's stream waits for this one
  pl->last_stream = st;
  std::vector<vs_expand_plan *> drop;
  {
    PlanCache &c = plan_cache();
    std::lock_guard<std::mutex> lk(c.mu);
    if (std::find(c.dead.begin(), c.dead.end(), pl->graph_serial) != c.dead.end() || !pl->cache_ev) {
      drop.push_back(pl);
    } else {
      c.idle.push_back(pl);
      plan_cache_trim(c, drop);
    }
  }
  for (vs_expand_plan *d : drop) plan_free(d);
}

void plan_cache_drop_graph(uint64_t serial) {
  using namespace ex;
  std::vector<vs_expand_plan *> drop;
  {
    PlanCache &c = plan_cache();
    std::lock_guard<std::mutex> lk(c.mu);
    c.dead.push_back(serial);
    for (size_t i = 0; i < c.idle.size();) {
      if (c.idle[i]->graph_serial == serial) {
        drop.push_back(c.idle[i]);
        c.idle.erase(c.idle.begin() + (long)i);
      } else {
        i++;
      }
    }
  }
  for (vs_expand_plan *d : drop) plan_free(d);
}

namespace ex {

template <typename K> int occupancy_grid(K kernel, int threads, size_t smem, int cap_per_sm) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
  if (per_sm <= 0) per_sm = 1;
  if (cap_per_sm > 0 && per_sm > cap_per_sm) per_sm = cap_per_sm;
  return per_sm * sm_count();
}

}  // namespace ex
}  // namespace vs

extern "C" {

int vs_expand_plan_create(vs_graph *g, uint32_t S, const vs_expand_params *p,
                          vs_expand_plan **out) {
  if (!g || !p || !out) return fail(VS_ERR_ARG, "vs_expand_plan_create: null argument");
  if (p->k_min > p->k_max) return fail(VS_ERR_ARG, "k_min %u > k_max %u", p->k_min, p->k_max);
  if (p->k_max > VS_MAX_HOPS) return fail(VS_ERR_ARG, "k_max %u exceeds %d", p->k_max, VS_MAX_HOPS);
  if (p->path_type < VS_PATH_ANY || p->path_type > VS_PATH_FIND_SHORTEST)
    return fail(VS_ERR_ARG, "unknown path type %d", p->path_type);
  if (p->direction < VS_DIR_FORWARD || p->direction > VS_DIR_BOTH)
    return fail(VS_ERR_ARG, "unknown direction %d", p->direction);
  if (p->strategy < VS_STRAT_AUTO || p->strategy > VS_STRAT_SPARSE)
    return fail(VS_ERR_ARG, "unknown strategy %d", p->strategy);
  if (p->pull_kernel < 0 || p->pull_kernel > 7) return fail(VS_ERR_ARG, "pull kernel variant must be 0..7");
  if (p->sparse_frac < 0) return fail(VS_ERR_ARG, "sparse_frac must be >= 0");
  if (S == 0) return fail(VS_ERR_ARG, "no start vertex for VExpand");
  if (S >= 0x80000000u) return fail(VS_ERR_ARG, "VExpand takes fewer than 2^31 start vertices");
  cudaStream_t st = 0;
  vs_expand_plan *pl = new vs_expand_plan();
  pl->g = g;
  pl->p = *p;
  pl->S = S;
  pl->W = words_per_col(S);
  pl->Q = pl->W / 2;
  uint32_t qs = p->slice_words ? (p->slice_words + 1) / 2 : pl->Q;
  qs = std::min(qs, (uint32_t)256);
  if (qs == 0) qs = 1;
  pl->qslice = qs;
  pl->nslices = (pl->Q + qs - 1) / qs;
  const bool shortest = p->path_type != VS_PATH_ANY;
  pl->use_vis = shortest;
  pl->use_acc = needs_acc(*p);
  pl->clear_diag = p->path_type == VS_PATH_SHORTEST && p->k_min == 1;
  const uint32_t V = g->V;
  const size_t rowwords = (size_t)V * pl->W;
  pl->pair_cap = p->pair_capacity ? p->pair_capacity
                                  : std::max<uint64_t>(1u << 20, std::min<uint64_t>((uint64_t)S * V / 8, 1ull << 25));
  pl->pair_cap = std::max<uint64_t>(pl->pair_cap, S);
  int rc = VS_OK;
#define PL_ALLOC(ptr, n)                                          \
  if ((rc = dalloc_n(&(ptr), (n), st)) != VS_OK) {                \
    plan_free(pl);                                                \
    return rc;                                                    \
  }
  PL_ALLOC(pl->buf[0], rowwords);
  PL_ALLOC(pl->buf[1], rowwords);
  PL_ALLOC(pl->flag[0], V);
  PL_ALLOC(pl->flag[1], V);
  if (pl->use_vis) PL_ALLOC(pl->vis, rowwords);
  if (pl->use_acc) PL_ALLOC(pl->acc, rowwords);
  PL_ALLOC(pl->pairs[0], pl->pair_cap);
  PL_ALLOC(pl->pairs[1], pl->pair_cap);
  PL_ALLOC(pl->pdeg[0], pl->pair_cap);
  PL_ALLOC(pl->pdeg[1], pl->pair_cap);
  PL_ALLOC(pl->doff, pl->pair_cap + 1);
  PL_ALLOC(pl->bsum, (pl->pair_cap + 1023) / 1024 + 1);
  PL_ALLOC(pl->push_list, V);
  PL_ALLOC(pl->resflag, V);
  PL_ALLOC(pl->touched, V);
  PL_ALLOC(pl->d_src, S);
  if (p->path_type == VS_PATH_FIND_SHORTEST) {
    PL_ALLOC(pl->d_tgt, S);
    PL_ALLOC(pl->d_dist, S);
  }
  PL_ALLOC(pl->ctr, 1);
  PL_ALLOC(pl->hmask, (size_t)(p->k_max + 1) * pl->W);
  PL_ALLOC(pl->rowk, 2);
  pl->short_min = p->short_share == 0 ? 0.1 : p->short_share;
  if (short_slots_ok(S, pl->nslices, p->short_share, V, pl->W)) {
    PL_ALLOC(pl->tiny[0], V);
    PL_ALLOC(pl->tiny[1], V);
    pl->slot_n = slot_entries(pl->W);
    PL_ALLOC(pl->slot[0], (size_t)V * pl->slot_n);
    PL_ALLOC(pl->slot[1], (size_t)V * pl->slot_n);
  } else {
    pl->short_min = 0;
  }
#undef PL_ALLOC
  cudaError_t e = cudaSuccess;
  // every row starts zero; later runs clear only the rows their flags mark
  if ((e = cudaMemsetAsync(pl->buf[0], 0, rowwords * 8, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(pl->buf[1], 0, rowwords * 8, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(pl->flag[0], 0, 4ull * V, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(pl->flag[1], 0, 4ull * V, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(pl->resflag, 0, 4ull * V, st)) != cudaSuccess ||
      (pl->vis && (e = cudaMemsetAsync(pl->vis, 0, rowwords * 8, st)) != cudaSuccess) ||
      (pl->acc && (e = cudaMemsetAsync(pl->acc, 0, rowwords * 8, st)) != cudaSuccess)) {
    plan_free(pl);
    return cuda_fail(e, "cudaMemsetAsync", __FILE__, __LINE__);
  }
  // hub list for the pull direction set
  pl->hub_threshold = p->hub_threshold ? p->hub_threshold : 2048;
  {
    Lists in = pull_lists(g, p->direction);
    unsigned *dn = nullptr;
    if ((rc = dalloc_n(&pl->hubs, V, st)) != VS_OK || (rc = dalloc_n(&dn, 1, st)) != VS_OK) {
      plan_free(pl);
      return rc;
    }
    cudaMemsetAsync(dn, 0, sizeof(unsigned), st);
    { k_hubs<<<sm_count() * 4, 256, 0, st>>>(in, V, pl->hub_threshold, pl->hubs, dn); vs::note_launch(); }
    unsigned hn = 0;
    cudaMemcpyAsync(&hn, dn, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    e = cudaStreamSynchronize(st);
    dfree(dn, st);
    if (e != cudaSuccess) {
      plan_free(pl);
      return cuda_fail(e, "hub list", __FILE__, __LINE__);
    }
    pl->nhubs = hn;
  }
  pl->pull_kind = p->pull_kernel;
  if (p->sparse_frac > 0) pl->sparse_frac = p->sparse_frac;
  const PullVariant &var = pick_variant(pl->qslice);
  const int hub_smem = 16 * 32 * 16 * var.UPL;
  if (hub_smem > 48 * 1024) cudaFuncSetAttribute(var.hub, cudaFuncAttributeMaxDynamicSharedMemorySize, hub_smem);
  pl->grid_pull = occupancy_grid(var.pull[pl->pull_kind & 3], 256, 0, 8);
  pl->grid_hub = std::max(1, std::min((int)pl->nhubs, occupancy_grid(var.hub, 512, hub_smem, 2)));
  if (pl->slot[0]) {  // short mode: a row of Q uint4 per warp (PULL) or per CTA (hubs)
    const int hs = hub_smem + (int)pl->Q * 16;
    if (hs > 48 * 1024) cudaFuncSetAttribute(var.hub_short, cudaFuncAttributeMaxDynamicSharedMemorySize, hs);
    pl->grid_short = occupancy_grid(var.pull_short, 256, 8 * (size_t)pl->Q * 16, 8);
    pl->grid_short_pre = occupancy_grid(var.pull_short_pre, 256, 8 * (size_t)pl->Q * 16, 8);
  }
  pl->grid_sparse = occupancy_grid(k_sparse, 256, 0, 8);
  pl->grid_push = occupancy_grid(k_push, 256, 0, 8);
  pl->grid_v = sm_count() * 8;
  *out = pl;
  return VS_OK;
}

// Device bytes vs_expand_plan_create allocates for these arguments (the
// serving loop admits queries by this number).
int vs_expand_plan_footprint(const vs_graph *g, uint32_t S, const vs_expand_params *p, uint64_t *bytes) {
  if (!g || !p || !bytes) return fail(VS_ERR_ARG, "null argument");
  const uint64_t V = g->V, W = words_per_col(S);
  const bool use_vis = p->path_type != VS_PATH_ANY;
  const bool use_acc = needs_acc(*p);
  uint64_t cap = p->pair_capacity ? p->pair_capacity
                                  : std::max<uint64_t>(1u << 20, std::min<uint64_t>((uint64_t)S * V / 8, 1ull << 25));
  cap = std::max<uint64_t>(cap, S);
  uint64_t b = (2 + use_vis + use_acc) * V * W * 8;             // frontier pair, visited, accumulator
  b += 6 * V * 4;                                                 // flags x2, resflag, push list, touched, hubs
  b += cap * (2 * 8 + 2 * 8 + 8) + ((cap + 1023) / 1024 + 1) * 8;  // pair lists, degrees, offsets, block sums
  b += (uint64_t)S * 4 * 3 + sizeof(Ctr) + (uint64_t)(p->k_max + 1) * W * 8;
  uint32_t qs = p->slice_words ? (p->slice_words + 1) / 2 : (uint32_t)(W / 2);
  qs = std::max<uint32_t>(1, std::min<uint32_t>(qs, 256));
  const uint32_t nslices = (uint32_t)((W / 2 + qs - 1) / qs);
  if (short_slots_ok(S, nslices, p->short_share, V, (uint32_t)W))
    b += 2 * V * (2 * slot_entries((uint32_t)W) + sizeof(Tiny));  // short-row words and slots of both buffers
  *bytes = b;
  return VS_OK;
}

int vs_expand_plan_free(vs_expand_plan *plan) { return plan_free(plan); }

int vs_expand_plan_run(vs_expand_plan *pl, const uint32_t *sources, const uint32_t *targets,
                       int32_t *distances, vs_stream_t stream) {
  if (!pl || !sources) return fail(VS_ERR_ARG, "vs_expand_plan_run: null argument");
  const vs_expand_params &p = pl->p;
  if (p.path_type == VS_PATH_FIND_SHORTEST && (!targets || !distances))
    return fail(VS_ERR_ARG, "FindShortest needs targets and distances");
  cudaStream_t st = S(stream);
  if (st != pl->last_stream) {  // earlier work on the plan ran in another stream's order
    VS_CK(cudaStreamSynchronize(pl->last_stream));
    pl->last_stream = st;
  }
  const vs_graph *g = pl->g;
  const uint32_t V = g->V, S_ = pl->S, W = pl->W, Q = pl->Q;
  const size_t rowbytes = (size_t)V * W * 8;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  VS_CK(cudaStreamIsCapturing(st, &cap));
  const bool timing = pl->timing && cap == cudaStreamCaptureStatusNone;  // events are not captured
  VS_TRY(copy_in(pl->d_src, sources, S_, st));
  if (pl->d_tgt) VS_TRY(copy_in(pl->d_tgt, targets, S_, st));
  // run start: clean frontier buffers, zero visited/accumulator/counters
  for (int b = 0; b < 2; b++)
    { k_clear_flagged<<<pl->grid_v, 256, 0, st>>>(reinterpret_cast<uint4 *>(pl->buf[b]), pl->flag[b],
                                                V, Q, pl->ctr, 0, 0); vs::note_launch(); }
  // the result matrix (visited or accumulator): clear the rows the previous
  // run marked in resflag, which also zeroes resflag; a visited matrix beside
  // an accumulator has no row marks and is cleared whole
  if (pl->acc || pl->vis)
    { k_clear_flagged<<<pl->grid_v, 256, 0, st>>>(reinterpret_cast<uint4 *>(pl->acc ? pl->acc : pl->vis),
                                                pl->resflag, V, Q, pl->ctr, 0, 0); vs::note_launch(); }
  if (pl->acc && pl->vis) VS_CK(cudaMemsetAsync(pl->vis, 0, rowbytes, st));
  VS_CK(cudaMemsetAsync(pl->ctr, 0, sizeof(Ctr), st));
  const Lists in = pull_lists(g, p.direction), outl = push_lists(g, p.direction);
  SeedArgs sa;
  sa.sources = pl->d_src;
  sa.S = S_;
  sa.W = W;
  sa.buf0 = pl->buf[0];
  sa.flag0 = pl->flag[0];
  sa.vis = pl->vis;
  sa.acc = (pl->use_acc && p.k_min == 0) ? pl->acc : nullptr;
  sa.pairs0 = pl->pairs[0];
  sa.pdeg0 = pl->pdeg[0];
  sa.resflag = pl->resflag;
  sa.res_vis = pl->use_vis && !pl->use_acc;
  sa.out = outl;
  sa.ctr = pl->ctr;
  sa.V = V;
  sa.multislice = pl->nslices > 1;
  sa.rowk = pl->use_hmask ? pl->rowk : nullptr;
  sa.stats = pl->collect_stats || pl->log_features || (pl->picker && p.use_picker);
  { k_seed<<<std::max(1u, std::min((S_ + 255) / 256, (uint32_t)sm_count() * 4)), 256, 0, st>>>(sa); vs::note_launch(); }
  VS_CK(cudaGetLastError());
  if (pl->layer_out[0])
    { k_copy_layer<<<pl->grid_v, 256, 0, st>>>(reinterpret_cast<const uint4 *>(pl->buf[0]), pl->flag[0],
                                             reinterpret_cast<uint4 *>(pl->layer_out[0]), V, Q, pl->ctr, 0); vs::note_launch(); }
  if (p.path_type == VS_PATH_FIND_SHORTEST)
    { k_dist_init<<<std::max(1u, std::min((S_ + 255) / 256, 1024u)), 256, 0, st>>>(pl->d_src, pl->d_tgt,
                                                                              pl->d_dist, S_, V, pl->ctr); vs::note_launch(); }
  const PullVariant &var = pick_variant(pl->qslice);
  const int forced = p.strategy == VS_STRAT_PULL ? ST_PULL
                     : p.strategy == VS_STRAT_PUSH ? ST_PUSH
                     : p.strategy == VS_STRAT_SPARSE ? ST_SPARSE
                                                     : 0;
  // a PULL hop may leave the short rows of its layer in their slots when the
  // layer has a successor and nothing reads its rows directly (FindShortest
  // checks every layer's rows; a kept layer is copied out)
  auto leave_in_slots = [&](uint32_t hh) {
    return pl->slot[0] != nullptr && hh >= 1 && hh < p.k_max && p.path_type != VS_PATH_FIND_SHORTEST &&
           pl->layer_out[hh] == nullptr;
  };
  // a Shortest SPARSE hop leaves its layer's rows in its pair list when a
  // later hop may build them (not the last hop, not an exported layer, not
  // FindShortest, whose target check reads every layer's rows) and the plan
  // has a short-row index (without one every PULL hop reads whole rows, so
  // building them later only adds a pass)
  auto defer_rows = [&](uint32_t hh) {
    return pl->use_vis && pl->slot[0] != nullptr && hh >= 1 && hh < p.k_max &&
           p.path_type != VS_PATH_FIND_SHORTEST && !pl->layer_out[hh];
  };
  // PUSH runs only when forced (for the run or a hop) or enabled in the
  // fixed planner (push_frac > 0)
  bool any_forced_push = forced == ST_PUSH;
  for (uint32_t hh = 1; hh <= p.k_max; hh++) any_forced_push |= pl->hop_forced[hh] == ST_PUSH;
  // (the picker chooses PUSH only where the plan enables it)
  const bool can_push = any_forced_push || pl->push_frac > 0;
  const bool stats = pl->collect_stats || pl->log_features || (pl->picker && p.use_picker);
  for (uint32_t h = 1; h <= p.k_max; h++) {
    const int fb = (h - 1) & 1, nbuf = h & 1;
    DecideArgs da;
    da.ctr = pl->ctr;
    da.h = h;
    da.path = p.path_type;
    da.S = S_;
    da.V = V;
    da.E = g->E;
    da.forced = pl->hop_forced[h] ? pl->hop_forced[h] : forced;
    da.log_features = pl->log_features;
    da.both = p.direction == VS_DIR_BOTH && g->directed;
    da.pair_cap = pl->pair_cap;
    da.sparse_frac = pl->sparse_frac;
    da.push_frac = pl->push_frac;
    da.picker = pl->picker;
    da.picker_on = p.use_picker;
    da.push_ok = can_push;
    da.rowk = pl->use_hmask ? pl->rowk : nullptr;
    da.short_min = pl->short_min;
    da.l2_half = l2_bytes() / 2;
    da.W = W;
    da.k_min = p.k_min;
    da.k_max = p.k_max;
    // the seed and SPARSE hops count their layer's statistics; after a PULL or
    // PUSH hop only a picker that may choose PUSH (or logging) needs the pass
    const bool picker_only = !pl->collect_stats && !pl->log_features;
    if (stats && h > 1 && !(picker_only && !can_push))
      { k_hop_stats<<<pl->grid_v, 256, 0, st>>>(pl->flag[fb], outl, V, pl->ctr, h, picker_only, can_push);
        vs::note_launch(); }
    { k_decide<<<1, 256, 0, st>>>(da); vs::note_launch(); }
    // hop_ms covers what the chosen strategy costs, not the statistics and decision before it
    if (timing) cudaEventRecord(pl->ev[3 * h], st);
    if (defer_rows(h - 1))  // rows a SPARSE hop h-1 left in its pair list, when hop h reads rows
      { k_pairs_rows<<<pl->grid_v, 256, 0, st>>>(pl->pairs[fb], pl->touched, reinterpret_cast<unsigned long long *>(pl->buf[fb]),
                                               W, pl->slot_n, pl->pair_cap, pl->ctr, h, 0); vs::note_launch(); }
    if (pl->slot[0] && leave_in_slots(h - 1))  // whole rows back for a hop that reads rows
      { k_materialize<<<pl->grid_v, 256, 0, st>>>(pl->flag[fb], reinterpret_cast<uint4 *>(pl->buf[fb]), V, Q,
                                                pl->slot[fb], pl->slot_n, pl->ctr, h, 1); vs::note_launch(); }

    if (h > 1)  // hop 1 writes a buffer the run start cleared
      { k_clear_flagged<<<pl->grid_v, 256, 0, st>>>(reinterpret_cast<uint4 *>(pl->buf[nbuf]),
                                                  pl->flag[nbuf], V, Q, pl->ctr, h, 1); vs::note_launch(); }
    const bool acc_on = pl->use_acc && h >= p.k_min && h <= p.k_max;
    SparseArgs sp;
    sp.ctr = pl->ctr;
    sp.h = h;
    sp.resflag = pl->resflag;
    sp.res_vis = pl->use_vis && !pl->use_acc;
    sp.hmask = pl->use_hmask ? reinterpret_cast<const unsigned long long *>(pl->hmask + (size_t)h * W) : nullptr;
    sp.pin = pl->pairs[fb];
    sp.pout = pl->pairs[nbuf];
    sp.cap = pl->pair_cap;
    sp.out = outl;
    sp.W = W;
    sp.N = reinterpret_cast<unsigned long long *>(pl->buf[nbuf]);
    sp.vis = reinterpret_cast<unsigned long long *>(pl->vis);
    sp.acc = reinterpret_cast<unsigned long long *>(pl->acc);
    sp.flagN = pl->flag[nbuf];
    sp.shortest = pl->use_vis;
    sp.acc_on = acc_on;
    sp.doff = pl->doff;
    sp.pdeg_out = pl->pdeg[nbuf];
    sp.stats = stats && h < p.k_max;
    sp.last = h == p.k_max && pl->use_vis && p.path_type != VS_PATH_FIND_SHORTEST && !pl->layer_out[h];
    sp.defer = defer_rows(h);
    { k_pscan1<<<pl->grid_v, 256, 0, st>>>(pl->pdeg[fb], pl->doff, pl->bsum, pl->ctr, h, pl->pair_cap); vs::note_launch(); }
    { k_pscan2<<<1, 1024, 0, st>>>(pl->bsum, pl->doff, pl->ctr, h, pl->pair_cap); vs::note_launch(); }
    { k_pscan3<<<pl->grid_v, 256, 0, st>>>(pl->doff, pl->bsum, pl->ctr, h, pl->pair_cap); vs::note_launch(); }
    { k_sparse<<<pl->grid_sparse, 256, 0, st>>>(sp); vs::note_launch(); }
    PushArgs pa;
    pa.ctr = pl->ctr;
    pa.h = h;
    pa.resflag = pl->resflag;
    pa.res_vis = pl->use_vis && !pl->use_acc;
    pa.hmask = pl->use_hmask ? reinterpret_cast<const unsigned long long *>(pl->hmask + (size_t)h * W) : nullptr;
    pa.out = outl;
    pa.F = reinterpret_cast<const unsigned long long *>(pl->buf[fb]);
    pa.N = reinterpret_cast<unsigned long long *>(pl->buf[nbuf]);
    pa.vis = reinterpret_cast<unsigned long long *>(pl->vis);
    pa.acc = reinterpret_cast<unsigned long long *>(pl->acc);
    pa.flagN = pl->flag[nbuf];
    pa.active = pl->push_list;
    pa.touched = pl->touched;
    pa.W = W;
    pa.shortest = pl->use_vis;
    pa.acc_on = acc_on;
    if (can_push) {  // PUSH kernels only when the hop can run PUSH
      { k_push_reset<<<1, 1, 0, st>>>(pl->ctr); vs::note_launch(); }
      { k_push_compact<<<pl->grid_v, 256, 0, st>>>(pl->flag[fb], V, pl->push_list, pl->ctr, h); vs::note_launch(); }
      { k_push<<<pl->grid_push, 256, 0, st>>>(pa); vs::note_launch(); }
      { k_push_epilogue<<<pl->grid_push, 256, 0, st>>>(pa); vs::note_launch(); }
    }
    PullArgs a;
    a.resflag = pl->resflag;
    a.res_vis = pl->use_vis && !pl->use_acc;
    a.hmask = pl->use_hmask ? reinterpret_cast<const uint4 *>(pl->hmask + (size_t)h * W) : nullptr;
    a.in = in;
    a.F = reinterpret_cast<const uint4 *>(pl->buf[fb]);
    a.N = reinterpret_cast<uint4 *>(pl->buf[nbuf]);
    a.vis = reinterpret_cast<uint4 *>(pl->vis);
    a.acc = reinterpret_cast<uint4 *>(pl->acc);
    a.flagF = pl->flag[fb];
    a.flagN = pl->flag[nbuf];
    a.V = V;
    a.Q = Q;
    a.qslice = pl->qslice;
    a.multislice = pl->nslices > 1;
    a.shortest = pl->use_vis;
    a.acc_on = acc_on;
    // the last hop's layer is read by nothing when the result is the visited
    // matrix or the accumulator (FindShortest checks every layer's targets)
    a.last = h == p.k_max && (pl->use_vis || pl->use_acc) && p.path_type != VS_PATH_FIND_SHORTEST &&
             !pl->layer_out[h];
    a.hub_threshold = pl->nhubs ? pl->hub_threshold : 0;
    a.hubs = pl->hubs;
    a.nhubs = pl->nhubs;
    a.ctr = pl->ctr;
    a.h = h;
    const bool keep_short = pl->slot[0] && h < p.k_max && !a.last;  // the next hop may read this layer's words
    a.virt_out = keep_short && leave_in_slots(h);
    a.tiny_in = pl->slot[0] ? pl->tiny[fb] : nullptr;
    a.slot_in = pl->slot[0] ? reinterpret_cast<const uint4 *>(pl->slot[fb]) : nullptr;
    a.tiny_out = keep_short ? pl->tiny[nbuf] : nullptr;
    a.slot_out = keep_short ? pl->slot[nbuf] : nullptr;
    a.slot_n = pl->slot_n;
    a.pre = (pl->pull_kind & 4) == 0;
    if (timing) cudaEventRecord(pl->ev[3 * h + 1], st);
    if (pl->slot[0]) {  // words and slots of a layer SPARSE, PUSH or the seed wrote, when this hop reads them
      { k_pairs_zero<<<pl->grid_v, 256, 0, st>>>(pl->touched, V, pl->ctr, h); vs::note_launch(); }
      { k_pairs_slots<<<pl->grid_v, 256, 0, st>>>(pl->pairs[fb], pl->touched, pl->slot[fb], pl->slot_n, pl->pair_cap,
                                                pl->ctr, h); vs::note_launch(); }
      { k_pairs_words<<<pl->grid_v, 256, 0, st>>>(pl->flag[fb], pl->touched, pl->tiny[fb], pl->slot[fb], pl->slot_n, V,
                                                pl->ctr, h); vs::note_launch(); }
      if (defer_rows(h - 1))  // the rows too long for a slot, which the short-mode PULL gathers whole
        { k_pairs_rows<<<pl->grid_v, 256, 0, st>>>(pl->pairs[fb], pl->touched,
                                                 reinterpret_cast<unsigned long long *>(pl->buf[fb]), W, pl->slot_n,
                                                 pl->pair_cap, pl->ctr, h, 1); vs::note_launch(); }
      { k_slot_build<<<pl->grid_v, 256, 0, st>>>(pl->flag[fb], reinterpret_cast<const uint4 *>(pl->buf[fb]), V, Q,
                                               pl->tiny[fb], pl->slot[fb], pl->slot_n, pl->ctr, h); vs::note_launch(); }
    }
    { var.pull[pl->pull_kind & 3]<<<dim3(pl->grid_pull, pl->nslices), 256, 0, st>>>(a); vs::note_launch(); }
    if (pl->nhubs)
      { var.hub<<<dim3(pl->grid_hub, pl->nslices), 512, 16 * 32 * 16 * var.UPL, st>>>(a); vs::note_launch(); }
    if (pl->slot[0]) {
      if (a.pre)
        { var.pull_short_pre<<<pl->grid_short_pre, 256, 8 * (size_t)Q * 16, st>>>(a); vs::note_launch(); }
      else
        { var.pull_short<<<pl->grid_short, 256, 8 * (size_t)Q * 16, st>>>(a); vs::note_launch(); }
      if (pl->nhubs)
        { var.hub_short<<<pl->grid_hub, 512, 16 * 32 * 16 * var.UPL + (size_t)Q * 16, st>>>(a); vs::note_launch(); }
    }
    if (p.path_type == VS_PATH_FIND_SHORTEST)
      { k_find_check<<<std::max(1u, std::min((S_ + 255) / 256, 1024u)), 256, 0, st>>>(
          pl->buf[nbuf], pl->d_tgt, pl->d_dist, S_, W, V, pl->ctr, h); vs::note_launch(); }
    if (pl->layer_out[h])
      { k_copy_layer<<<pl->grid_v, 256, 0, st>>>(reinterpret_cast<const uint4 *>(pl->buf[nbuf]), pl->flag[nbuf],
                                               reinterpret_cast<uint4 *>(pl->layer_out[h]), V, Q, pl->ctr, h); vs::note_launch(); }
    if (timing) cudaEventRecord(pl->ev[3 * h + 2], st);
    VS_CK(cudaGetLastError());
  }
  pl->timed_hops = timing ? p.k_max : 0;
  if (pl->clear_diag)
    { k_clear_diag<<<std::max(1u, std::min((S_ + 255) / 256, 1024u)), 256, 0, st>>>(pl->vis, pl->d_src,
                                                                                S_, W, V); vs::note_launch(); }
  if (p.path_type == VS_PATH_FIND_SHORTEST)
    VS_TRY(copy_in(distances, (const int32_t *)pl->d_dist, S_, st));
  VS_CK(cudaGetLastError());
  // result view
  vs_bitmat &r = pl->result;
  r = vs_bitmat{};
  r.rows = S_;
  r.cols = V;
  r.wpc = W;
  r.kind = VS_KIND_VARROW;
  const int lb = p.k_max & 1;  // buffer of layer k_max (the result of Any [k, k])
  r.words = pl->use_acc ? pl->acc : pl->use_vis ? pl->vis : pl->buf[lb];
  r.row_map = pl->d_src;
  r.col_map = nullptr;
  r.colnz = (pl->use_acc || pl->use_vis) ? pl->resflag : pl->flag[lb];
  r.owns_words = false;
  r.view = true;
  pl->has_result = p.path_type != VS_PATH_FIND_SHORTEST;
  return VS_OK;
}

int vs_expand_plan_result(vs_expand_plan *pl, vs_bitmat **view) {
  if (!pl || !view) return fail(VS_ERR_ARG, "null argument");
  if (!pl->has_result) return fail(VS_ERR_ARG, "plan has no matrix result");
  vs_bitmat *m = new vs_bitmat(pl->result);
  m->view = true;
  *view = m;
  return VS_OK;
}

int vs_expand_plan_stats(vs_expand_plan *pl, vs_expand_stats *stats, vs_stream_t stream) {
  if (!pl || !stats) return fail(VS_ERR_ARG, "null argument");
  Ctr h;
  VS_CK(cudaMemcpyAsync(&h, pl->ctr, sizeof(Ctr), cudaMemcpyDeviceToHost, S(stream)));
  VS_CK(cudaStreamSynchronize(S(stream)));
  std::memset(stats, 0, sizeof(*stats));
  if (h.error & 2) return fail(VS_ERR_ARG, "a row hop limit set on the device exceeds k_max %u", pl->p.k_max);
  if (h.error) return fail(VS_ERR_ARG, "a source or target vertex id is >= V (%u)", pl->g->V);
  stats->hops_run = (uint32_t)h.hops_run;
  stats->found = (uint32_t)h.found;
  uint64_t vc = pl->S;
  for (int i = 0; i <= VS_MAX_HOPS; i++) {
    stats->new_bits[i] = h.hop[i].new_bits;
    stats->active_vertices[i] = h.hop[i].active_vertices;
    stats->active_edges[i] = h.hop[i].active_edges;
    stats->pairs[i] = h.hop[i].pairs;
    stats->strategy[i] = h.hop[i].strategy;
    stats->short_pull[i] = h.hop[i].short_pull ? (h.hop[i].short_slots ? 2 : 1) : 0;
    stats->short_rows[i] = h.hop[i].short_rows & 0xFFFFFFFFull;
    stats->tiny_rows[i] = h.hop[i].short_rows >> 32;
    stats->short_edges[i] = h.hop[i].short_edges;
    if (i >= 1 && i <= h.hops_run) vc += h.hop[i].new_bits;
  }
  for (uint32_t i = 1; i <= pl->timed_hops && i <= VS_MAX_HOPS; i++) {
    float a = 0, b = 0;
    if (cudaEventElapsedTime(&a, pl->ev[3 * i], pl->ev[3 * i + 2]) == cudaSuccess) stats->hop_ms[i] = a;
    if (cudaEventElapsedTime(&b, pl->ev[3 * i + 1], pl->ev[3 * i + 2]) == cudaSuccess) stats->pull_ms[i] = b;
  }
  stats->visit_count = pl->use_vis ? vc : 0;
  return VS_OK;
}

int vs_expand_plan_set_tuning(vs_expand_plan *pl, double sparse_frac, double push_frac,
                              int collect_stats, int timing) {
  if (!pl) return fail(VS_ERR_ARG, "null plan");
  if (sparse_frac >= 0) pl->sparse_frac = sparse_frac;
  if (push_frac >= 0) pl->push_frac = push_frac;
  pl->collect_stats = collect_stats != 0;
  if (timing && !pl->timing) {
    for (cudaEvent_t &e : pl->ev)
      if (!e) VS_CK(cudaEventCreate(&e));
  }
  pl->timing = timing != 0;
  return VS_OK;
}

int vs_expand_plan_set_picker(vs_expand_plan *pl, const vs_picker *p) {
  if (!pl) return fail(VS_ERR_ARG, "null plan");
  pl->picker = p ? vs_picker_device_weights(p) : nullptr;
  return VS_OK;
}

int vs_expand_plan_set_hop_strategies(vs_expand_plan *pl, const int32_t *strategies, uint32_t n) {
  if (!pl) return fail(VS_ERR_ARG, "null plan");
  for (int h = 0; h <= VS_MAX_HOPS; h++) pl->hop_forced[h] = 0;
  for (uint32_t h = 1; strategies && h < n && h <= VS_MAX_HOPS; h++) {
    const int s = strategies[h];
    if (s < VS_STRAT_AUTO || s > VS_STRAT_SPARSE) return fail(VS_ERR_ARG, "unknown strategy %d", s);
    pl->hop_forced[h] = s == VS_STRAT_PULL ? ST_PULL : s == VS_STRAT_PUSH ? ST_PUSH : s == VS_STRAT_SPARSE ? ST_SPARSE : 0;
  }
  return VS_OK;
}

// Batched queries: row i of the plan belongs to a query whose hop range ends
// at row_kmax[i] (<= the plan's k_max).  Rows stop growing after their own
// last hop, so every query's rows equal the result of running it alone.
int vs_expand_plan_set_row_limits(vs_expand_plan *pl, const uint8_t *row_kmax, uint32_t n) {
  if (!pl) return fail(VS_ERR_ARG, "null plan");
  if (!row_kmax) {
    pl->use_hmask = false;
    return VS_OK;
  }
  if (n != pl->S) return fail(VS_ERR_ARG, "row limits need one entry per source row (%u)", pl->S);
  const uint32_t K = pl->p.k_max, W = pl->W;
  std::vector<uint64_t> m((size_t)(K + 1) * W, 0);
  bool all = true;
  uint32_t rk[2] = {0, 0};
  for (uint32_t i = 0; i < n; i++) {
    if (row_kmax[i] > K) return fail(VS_ERR_ARG, "row %u hop limit %u exceeds k_max %u", i, row_kmax[i], K);
    all &= row_kmax[i] == K;
    rk[0] = std::max<uint32_t>(rk[0], row_kmax[i]);
    for (uint32_t h = 1; h <= row_kmax[i]; h++) m[(size_t)h * W + i / 64] |= 1ull << (i % 64);
  }
  if (!all && !pl->use_acc && !pl->use_vis)
    return fail(VS_ERR_UNSUPPORTED, "row limits need an accumulating plan (Any with k_min < k_max, or Shortest)");
  // the mask is written even when unused, so a run captured with limits stays right
  VS_CK(cudaStreamSynchronize(pl->last_stream));  // no earlier run still reads the mask
  VS_CK(cudaMemcpy(pl->hmask, m.data(), 8 * m.size(), cudaMemcpyHostToDevice));
  VS_CK(cudaMemcpy(pl->rowk, rk, sizeof(rk), cudaMemcpyHostToDevice));
  pl->use_hmask = !all;
  return VS_OK;
}

// Row limits from a device array, stream-ordered (capturable): the mask of
// every hop is built by k_row_mask; rows at index >= n get limit 0 (they
// never grow).  A limit above k_max is clamped and reported as VS_ERR_ARG by
// the next run.
int vs_expand_plan_set_row_limits_device(vs_expand_plan *pl, const uint8_t *row_kmax, uint32_t n,
                                         vs_stream_t stream) {
  if (!pl || !row_kmax) return fail(VS_ERR_ARG, "vs_expand_plan_set_row_limits_device: null argument");
  if (n > pl->S) return fail(VS_ERR_ARG, "%u row limits for a plan of %u rows", n, pl->S);
  if (!pl->use_acc && !pl->use_vis)
    return fail(VS_ERR_UNSUPPORTED, "row limits need an accumulating plan (Any with k_min < k_max, or Shortest)");
  cudaStream_t st = S(stream);
  if (st != pl->last_stream) {
    VS_CK(cudaStreamSynchronize(pl->last_stream));
    pl->last_stream = st;
  }
  VS_CK(cudaMemsetAsync(pl->rowk, 0, 2 * sizeof(uint32_t), st));
  const uint32_t W = pl->W;
  { k_row_mask<<<(W + 255) / 256, 256, 0, st>>>(row_kmax, n, pl->p.k_max, W, pl->hmask, pl->rowk); vs::note_launch(); }
  VS_CK(cudaGetLastError());
  pl->use_hmask = true;
  return VS_OK;
}

// Kernel shape of the PULL hops (chosen by the autotuner): bit 0 asks for 8
// resident 256-thread blocks per SM (32 registers), bit 1 adds L2 cache
// policies (streams evict-first, frontier rows evict-last), bit 2 runs
// short-mode hops without loading the next target's visited words and flag
// ahead.
int vs_expand_plan_set_pull_kernel(vs_expand_plan *pl, int kind) {
  if (!pl || kind < 0 || kind > 7) return fail(VS_ERR_ARG, "pull kernel variant must be 0..7");
  pl->pull_kind = kind;
  const PullVariant &var = pick_variant(pl->qslice);
  pl->grid_pull = occupancy_grid(var.pull[kind & 3], 256, 0, 8);
  return VS_OK;
}

int vs_expand_plan_log_features(vs_expand_plan *pl, int on) {
  if (!pl) return fail(VS_ERR_ARG, "null plan");
  pl->log_features = on != 0;
  return VS_OK;
}

int vs_expand_plan_features(vs_expand_plan *pl, float *features, vs_stream_t stream) {
  if (!pl || !features) return fail(VS_ERR_ARG, "null argument");
  VS_CK(cudaMemcpyAsync(features, pl->ctr->feat, sizeof(float) * 32 * (VS_MAX_HOPS + 1), cudaMemcpyDefault,
                        S(stream)));
  VS_CK(cudaStreamSynchronize(S(stream)));
  return VS_OK;
}

// VExpand with_distance, Dense strategy (copy_to_multi_MT, vexpand.cpp:356-378):
// layers k_min..k_actual each as a VarRow matrix with the sources as row map.
int vs_expand_layers(vs_graph *g, const uint32_t *sources, uint32_t S, const vs_expand_params *p,
                     vs_bitmat **layers, uint32_t *nlayers, vs_stream_t stream) {
  if (!g || !p || !layers || !nlayers) return fail(VS_ERR_ARG, "vs_expand_layers: null argument");
  if (p->path_type == VS_PATH_FIND_SHORTEST)
    return fail(VS_ERR_ARG, "FindShortest reports distances per pair, not layers");
  if (p->k_min > p->k_max || p->k_max > VS_MAX_HOPS) return fail(VS_ERR_ARG, "bad hop range [%u, %u]", p->k_min, p->k_max);
  const uint32_t n = p->k_max - p->k_min + 1;
  *nlayers = 0;
  for (uint32_t i = 0; i < n; i++) layers[i] = nullptr;
  if (S == 0) return VS_OK;  // no start vertex: no layer (VExpand::before_execution)
  cudaStream_t st = vs::S(stream);
  vs_expand_plan *pl = nullptr;
  VS_TRY(vs_expand_plan_create(g, S, p, &pl));
  pl->collect_stats = true;
  int rc = VS_OK;
  for (uint32_t i = 0; i < n && rc == VS_OK; i++) {
    rc = bitmat_alloc(S, g->V, VS_KIND_VARROW, st, &layers[i]);
    if (rc == VS_OK) {
      pl->layer_out[p->k_min + i] = layers[i]->words;
      rc = vs_bitmat_set_maps(layers[i], sources, nullptr, stream);
    }
  }
  if (rc == VS_OK) {
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_fail(e, "vs_expand_layers", __FILE__, __LINE__);
  }
  if (rc == VS_OK) rc = vs_expand_plan_run(pl, sources, nullptr, nullptr, stream);
  vs_expand_stats stt{};
  if (rc == VS_OK) rc = vs_expand_plan_stats(pl, &stt, stream);
  plan_free(pl);
  uint32_t keep = 0;
  if (rc == VS_OK) {
    const uint32_t k_actual = stt.hops_run;  // last hop run (VExpand::after_child, vexpand.cpp:223)
    keep = k_actual >= p->k_min ? std::min(k_actual, p->k_max) - p->k_min + 1 : 0;
  }
  for (uint32_t i = keep; i < n; i++) {
    vs_bitmat_free(layers[i]);
    layers[i] = nullptr;
  }
  *nlayers = keep;
  return rc;
}

int vs_expand(vs_graph *g, const uint32_t *sources, uint32_t S, const vs_expand_params *p,
              const uint32_t *targets, int32_t *distances, vs_bitmat **out, vs_expand_stats *stats,
              vs_stream_t stream) {
  if (!g || !p) return fail(VS_ERR_ARG, "vs_expand: null argument");
  if (S == 0) {
    // VExpand::before_execution returns false on an empty start list: empty result
    if (out && p->path_type != VS_PATH_FIND_SHORTEST)
      return bitmat_alloc(0, g->V, VS_KIND_VARROW, vs::S(stream), out);
    if (stats) std::memset(stats, 0, sizeof(*stats));
    return VS_OK;
  }
  cudaStream_t st = vs::S(stream);
  vs_expand_plan *pl = plan_cache_take(g, S, *p);
  if (pl) {
    if (pl->cache_ev) VS_CK(cudaStreamWaitEvent(st, pl->cache_ev, 0));
  } else {
    int rc0 = vs_expand_plan_create(g, S, p, &pl);
    if (rc0 == VS_ERR_OOM) {  // the cached plans may hold the memory: release them and retry once
      vs_release_cached();
      rc0 = vs_expand_plan_create(g, S, p, &pl);
    }
    if (rc0 != VS_OK) return rc0;
    pl->key = *p;
    pl->graph_serial = g->serial;
    vs_expand_plan_footprint(g, S, p, &pl->bytes);
  }
  pl->collect_stats = stats != nullptr;
  int rc = vs_expand_plan_run(pl, sources, targets, distances, stream);
  if (rc == VS_OK && stats) rc = vs_expand_plan_stats(pl, stats, stream);
  if (rc == VS_OK && !stats) {
    int err = 0;
    cudaError_t e = cudaMemcpyAsync(&err, &pl->ctr->error, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
      rc = cuda_fail(e, "vs_expand", __FILE__, __LINE__);
    else if (err)
      rc = fail(VS_ERR_ARG, "a source or target vertex id is >= V (%u)", g->V);
  }
  if (rc != VS_OK) {  // a failed run leaves the plan out of the cache
    plan_free(pl);
    return rc;
  }
  if (out && p->path_type != VS_PATH_FIND_SHORTEST) {
    // the result is the plan's own result matrix, lent until the handle is freed
    vs_bitmat *m = new vs_bitmat(pl->result);
    m->view = true;
    m->owns_words = false;
    m->pool_plan = pl;
    m->st = st;
    *out = m;
    return VS_OK;
  }
  plan_cache_return(pl, st);
  return VS_OK;
}

int vs_release_cached(void) {
  std::vector<vs_expand_plan *> drop;
  {
    PlanCache &c = plan_cache();
    std::lock_guard<std::mutex> lk(c.mu);
    drop.swap(c.idle);
  }
  for (vs_expand_plan *d : drop) plan_free(d);
  return VS_OK;
}

}  // extern "C"
