// Argument blocks and counters of the expand kernels.
#pragma once
#include <stdint.h>

#include "vs_internal.cuh"

namespace vs {
namespace ex {

enum { ST_NONE = 0, ST_PULL = 1, ST_PUSH = 2, ST_SPARSE = 3 };

// Per-hop device counters (hop 0 describes the seeded layer 0).
struct HopCtr {
  unsigned long long new_bits;         // bits set in layer h (Shortest: newly visited)
  unsigned long long active_vertices;  // non-zero rows of layer h
  unsigned long long active_edges;     // edges leaving non-zero rows of layer h-1 (stats pass)
  unsigned long long pairs;            // SPARSE: (vertex, source) pairs of layer h
  unsigned long long pair_edges;       // SPARSE: sum of out-degrees over those pairs
  unsigned long long work_edges;       // SPARSE: edges scanned by the hop
  unsigned long long hist[16];         // log2(out-degree + 1) histogram of layer h-1's active rows
  int overflow;                        // SPARSE: pair list overflowed
  int strategy;                        // strategy run at hop h (0 = not run)
  int short_pull;                      // PULL reads the short rows of layer h-1 through their slots
  int short_slots;                     // ... reading slots (count in entry 0) instead of tiny words
  unsigned long long short_rows;       // rows of layer h with 1..slot_n-1 bits (low 32 bits) and with at most
                                       // TINY_MAX bits (high 32 bits), counted when its words are written
  unsigned long long short_edges;      // active in-edges of a short-mode PULL served from a slot
};

struct Ctr {
  HopCtr hop[VS_MAX_HOPS + 1];
  unsigned long long found;  // FindShortest
  int done;                  // early stop reached: later hops are no-ops
  int hops_run;              // k_actual_max
  int multislice;            // PULL runs in several source slices
  unsigned push_active, push_touched;
  int error;  // bit 0: a source or target id was >= V (entry skipped); bit 1: a row limit > k_max
  float feat[VS_MAX_HOPS + 1][32];  // picker features of every hop (when logged)
};

// Up to two adjacency lists (Direction::Both uses both CSRs).
struct Lists {
  const int64_t *off[2];
  const uint32_t *adj[2];
  int n;
};

struct SeedArgs {
  uint32_t *resflag;  // result column may be non-zero (colnz of the result view)
  int res_vis;        // the result is the visited matrix (else the accumulator)
  const uint32_t *sources;
  uint32_t S, W, V;
  uint64_t *buf0;
  uint32_t *flag0;
  uint64_t *vis, *acc;
  uint2 *pairs0;
  unsigned long long *pdeg0;  // out-degree of every seeded pair's vertex
  Lists out;
  Ctr *ctr;
  int multislice;  // PULL runs in several source slices
  const uint32_t *rowk;  // row-limit words of the plan (NULL: no row limits)
  int stats;  // also count hop 1's frontier statistics (active_edges, hist) of layer 0
};

struct DecideArgs {
  Ctr *ctr;
  int h, path, forced, picker_on, log_features, both;
  int push_ok;  // the plan launches PUSH kernels (the picker may choose PUSH)
  uint32_t S, V, W, k_min, k_max;
  uint64_t E, pair_cap;
  double sparse_frac, push_frac;
  const void *picker;  // bf16 weights of a vs_picker (NULL = fixed planner)
  const uint32_t *rowk;  // [0] largest row hop limit (NULL: no row limits)
  double short_min;      // short-mode PULL when at least this share of the frontier's rows are short (0: off; > 1: always)
  uint64_t l2_half;       // ... and the frontier's rows exceed this many bytes (smaller ones stay in L2)
};

struct SparseArgs {
  uint32_t *resflag;  // result column may be non-zero (colnz of the result view)
  int res_vis;        // the result is the visited matrix (else the accumulator)
  Ctr *ctr;
  int h;
  const unsigned long long *hmask;  // rows that may still grow at hop h (NULL = all)
  const uint2 *pin;
  uint2 *pout;
  const unsigned long long *doff;  // exclusive prefix of the input pairs' out-degrees (+ total)
  unsigned long long *pdeg_out;    // out-degree of every output pair's vertex
  uint64_t cap;
  Lists out;
  uint32_t W;
  unsigned long long *N, *vis, *acc;
  uint32_t *flagN;
  int shortest, acc_on;
  int stats;  // also count hop h+1's frontier statistics (active_edges, hist) of the layer it writes
  int last;   // Shortest, and layer h is read by nothing: no next-layer rows or pairs, rows flagged 2
  int defer;  // Shortest: layer h's rows are built from its pair list by the hop that reads rows (k_pairs_rows)
};

struct PushArgs {
  uint32_t *resflag;  // result column may be non-zero (colnz of the result view)
  int res_vis;        // the result is the visited matrix (else the accumulator)
  Ctr *ctr;
  int h;
  const unsigned long long *hmask;
  Lists out;
  const unsigned long long *F;
  unsigned long long *N, *vis, *acc;
  uint32_t *flagN;
  const uint32_t *active;
  uint32_t *touched;
  uint32_t W;
  int shortest, acc_on;
};

struct PullArgs {
  uint32_t *resflag;  // result column may be non-zero (colnz of the result view)
  int res_vis;        // the result is the visited matrix (else the accumulator)
  const uint4 *hmask;  // rows that may still grow at hop h, Q uint4 (NULL = all)
  Lists in;
  const uint4 *F;
  uint4 *N, *vis, *acc;
  const uint32_t *flagF;
  uint32_t *flagN;  // 0: empty row; 1: non-zero row in the buffer; 2: non-zero row held in its slot only
  uint32_t V, Q, qslice;
  int multislice, shortest, acc_on;
  int last;  // the run's last hop and nothing reads its layer: zero the buffer instead of writing it
  const uint32_t *tiny_in;  // short-row words of layer h-1, one per vertex (NULL: no short mode)
  const uint4 *slot_in;     // slots of layer h-1 (two uint4 per vertex)
  uint32_t *tiny_out;       // words of layer h, written for every vertex (NULL: not kept)
  uint16_t *slot_out;       // slots of layer h (count, then the ids of a row of < slot_n bits)
  uint32_t slot_n;          // uint16 entries per slot (16, 32 or 64)
  int virt_out;             // short rows of layer h may stay in their slots (flag 2, buffer row zero)
  int pre;                  // short mode: the next target's visited words and flag are loaded ahead
  uint32_t hub_threshold;
  const uint32_t *hubs;
  uint32_t nhubs;
  Ctr *ctr;
  int h;
};


}  // namespace ex
}  // namespace vs
