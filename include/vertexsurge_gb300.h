/*
 * vertexsurge_gb300 — C ABI of the GB300 (sm_103a) implementation of
 * VertexSurge's variable-length graph pattern matching hot path:
 * the bit-matrix multi-source BFS expand (VExpand), the vertex-id hash join
 * (HashJoin), the multi-way intersection (Mintersect) and the glue operators
 * between them (MatrixTableSelect, TableConvert, Count).
 *
 * Conventions
 *  - Every call returns a status (VS_OK == 0); vs_last_error() gives the
 *    message of the calling thread's last failure.
 *  - Handles own device memory.  Pointers passed in (sources, columns, maps)
 *    may be host or device memory; they are borrowed for the duration of the
 *    call only.
 *  - Calls are ordered on the stream passed (a cudaStream_t, NULL = legacy
 *    default stream).  Calls that return a host-visible result (counts,
 *    downloads, statistics) synchronise that stream.
 *  - A handle is not thread-safe; independent handles are.
 *
 * Logical matrices.  A bit matrix has `rows` x `cols` logical elements;
 * column c is stored as `wpc` consecutive uint64 words (wpc >= ceil(rows/64),
 * even), element (r, c) is bit r % 64 of word c * wpc + r / 64.  An expand
 * result has one row per source (in input order) and one column per vertex:
 * column v is the set of sources that reach v.  Downloads produce the packed
 * logical form with ceil(rows/64) words per column.
 */
#ifndef VERTEXSURGE_GB300_H
#define VERTEXSURGE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference reports errors with assert/exit, e.g.
 *      src/objects/operator/vexpand.cpp:88-91, join.cpp:82-85) ------------ */
#define VS_OK 0
#define VS_ERR_ARG 1         /* invalid argument or shape                   */
#define VS_ERR_OOM 2         /* device allocation failed                    */
#define VS_ERR_CUDA 3        /* a CUDA runtime call failed                  */
#define VS_ERR_TIMEOUT 4     /* a bounded device-side wait gave up          */
#define VS_ERR_UNSUPPORTED 5 /* combination the operator does not support   */
#define VS_ERR_CAPACITY 6    /* output exceeded the caller's row bound      */

/* Direction (src/include/common/common.hh, rules src/objects/meta/schema.cpp:261-302) */
#define VS_DIR_FORWARD 0
#define VS_DIR_BACKWARD 1
#define VS_DIR_BOTH 2

/* ExpandPathType (src/include/operator/expand.hh:24-28) */
#define VS_PATH_ANY 0
#define VS_PATH_SHORTEST 1
#define VS_PATH_FIND_SHORTEST 2

/* Per-hop expansion strategy */
#define VS_STRAT_AUTO 0   /* fixed planner, or the learned picker when enabled */
#define VS_STRAT_PULL 1   /* dense: every vertex ORs its active in-neighbour rows */
#define VS_STRAT_PUSH 2   /* active rows OR-ed into out-neighbours with atomics */
#define VS_STRAT_SPARSE 3 /* (vertex, source) pair lists, one bit per edge */

/* Table kinds (src/include/execution/tuple.hh:9-18 TableType) */
#define VS_KIND_VARROW 1
#define VS_KIND_COLMAIN 2

/* Flat column types (src/include/meta/type.hh: VID = uint32, Int64) */
#define VS_T_VID 0
#define VS_T_I64 1

typedef void *vs_stream_t;
typedef struct vs_graph vs_graph;
typedef struct vs_bitmat vs_bitmat;
typedef struct vs_flat vs_flat;
typedef struct vs_expand_plan vs_expand_plan;

const char *vs_last_error(void);
/* Select the CUDA device for the calling thread and set up the stream-ordered
 * allocator pool. */
int vs_init(int device);
const char *vs_version(void);
/* Number of CUDA kernels this library has launched since it was loaded
 * (diagnostics; no counterpart in the reference). */
uint64_t vs_kernel_launches(void);

/* CUDA-graph capture (no counterpart in the reference): the calls made on
 * `stream` between vs_capture_begin and vs_capture_end are recorded, not run,
 * and vs_captured_launch replays them as one graph launch.  Capturable calls:
 * vs_expand_plan_run with device sources (the plan's host-side settings —
 * row limits set from the host, tuning, picker, forced strategies — are fixed
 * at capture), vs_expand_plan_set_row_limits_device and
 * vs_hash_join_count_row_blocks.  Run a plan once on `stream` before
 * capturing it.  The stream must not be the legacy default stream.
 * vs_kernel_launches counts a captured kernel once per replay. */
typedef struct vs_captured vs_captured;
int vs_capture_begin(vs_stream_t stream);
int vs_capture_end(vs_stream_t stream, vs_captured **out);
int vs_captured_launch(vs_captured *g, vs_stream_t stream);
/* Kernel nodes of the captured graph. */
uint64_t vs_captured_kernels(const vs_captured *g);
int vs_captured_free(vs_captured *g);

/* ---- graph (replaces Graph::load + Graph::get_edges_refs CSR requests,
 *      src/objects/storage/graph_store.cpp:48-73, :75-110, :142-189) ------
 * fwd: out-lists (u -> v), rev: in-lists (v <- u), both int64 offsets [V+1]
 * and uint32 ids, every list sorted.  directed == 0 marks an undirected edge
 * type stored both ways, for which direction has no effect. */
int vs_graph_upload(uint32_t V, uint64_t E, const int64_t *fwd_off, const uint32_t *fwd_dst,
                    const int64_t *rev_off, const uint32_t *rev_src, int directed,
                    vs_stream_t stream, vs_graph **out);
int vs_graph_info(const vs_graph *g, uint32_t *V, uint64_t *E, int *directed);
int vs_graph_free(vs_graph *g);

/* ---- bit matrices (replaces DenseVarStackMatrix / DenseColMainMatrix and
 *      VarRowMatrixTable / ColMainMatrixTable, src/include/storage/bitmap.hh:262-425,
 *      src/include/execution/matrix_table.hh) ------------------------------ */
typedef struct vs_bitmat_info {
  uint32_t rows, cols, wpc;
  int32_t kind;
  int32_t has_row_map, has_col_map;
  uint64_t *words; /* device pointer, cols * wpc words (borrowed) */
} vs_bitmat_info;

int vs_bitmat_create(uint32_t rows, uint32_t cols, int kind, vs_stream_t stream, vs_bitmat **out);
int vs_bitmat_upload(vs_bitmat *m, const uint64_t *logical_words, vs_stream_t stream);
int vs_bitmat_download(const vs_bitmat *m, uint64_t *logical_words, vs_stream_t stream);
/* row_map[r] / col_map[c] give the vertex id of a physical row / column
 * (MatrixTable::row_map / col_map); NULL leaves the map absent. */
int vs_bitmat_set_maps(vs_bitmat *m, const uint32_t *row_map, const uint32_t *col_map,
                       vs_stream_t stream);
int vs_bitmat_get_maps(const vs_bitmat *m, uint32_t *row_map, uint32_t *col_map,
                       vs_stream_t stream);
int vs_bitmat_get_info(const vs_bitmat *m, vs_bitmat_info *info);
int vs_bitmat_free(vs_bitmat *m);

/* Count / Table::tuple_count on a matrix table: popcount
 * (src/objects/operator/big_operators2.cpp:5-14, bitmap.cpp:1098-1125). */
int vs_bitmat_count(const vs_bitmat *m, uint64_t *count, vs_stream_t stream);

/* MatrixTableSelect on a VarRow table (big_operators2.cpp:138-213): the
 * result keeps columns targets[0..T) (duplicates kept) and has col_map =
 * targets, row_map inherited. */
int vs_matrix_select(const vs_bitmat *m, const uint32_t *targets, uint32_t T, vs_bitmat **out,
                     vs_stream_t stream);

/* TableConvert VarRow -> ColMain (big_operators2.cpp:16-86); transpose
 * swaps rows and columns together with their maps. */
int vs_table_convert(const vs_bitmat *m, int transpose, vs_bitmat **out, vs_stream_t stream);

/* TableConvert(Flat) / matrix iterators (bit_matrix_table.cpp:133-289):
 * one (row value, column value) VID pair per set bit, maps applied. */
int vs_bitmat_to_flat(const vs_bitmat *m, vs_flat **out, vs_stream_t stream);

/* ---- flat tables (replaces FlatTable, src/include/execution/flat_table.hh) */
int vs_flat_create(uint32_t ncols, const int32_t *types, uint64_t nrows, vs_flat **out);
int vs_flat_upload(vs_flat *f, uint32_t col, const void *data, vs_stream_t stream);
int vs_flat_download(const vs_flat *f, uint32_t col, void *data, vs_stream_t stream);
int vs_flat_info(const vs_flat *f, uint32_t *ncols, uint64_t *nrows, int32_t *types);
int vs_flat_free(vs_flat *f);
/* Device address of column col (valid until the table is freed). */
int vs_flat_column(const vs_flat *f, uint32_t col, const void **device_ptr);

/* ---- expand (replaces VExpand + Expand<DenseVarStackMatrix> with
 *      ExpandStrategy::Dense: src/objects/operator/vexpand.cpp:45-483,
 *      src/objects/operator/expand.cpp:210-414,
 *      src/include/operator/expand_impl.hh:135-277) ----------------------- */
typedef struct vs_expand_params {
  uint32_t k_min, k_max;   /* hop range [k_min, k_max]; FindShortest uses k_max as the cap */
  int32_t path_type;       /* VS_PATH_* */
  int32_t direction;       /* VS_DIR_* */
  int32_t strategy;        /* VS_STRAT_*: AUTO lets the planner choose per hop */
  int32_t use_picker;      /* 1: the learned picker chooses under AUTO (when loaded); it may choose
                              PUSH only where the plan runs PUSH (push_frac > 0 or a forced hop) */
  uint32_t hub_threshold;  /* in-degree above which a vertex gets a whole CTA (0 = tuned default) */
  uint32_t slice_words;    /* source words per pass (0 = whole row up to 256 words) */
  uint64_t pair_capacity;  /* sparse (vertex, source) list capacity (0 = default) */
  int32_t pull_kernel;     /* PULL kernel shape 0..7, see vs_expand_plan_set_pull_kernel */
  int32_t reserved;
  double sparse_frac;      /* fixed planner: SPARSE while pair-list edges < this x E (0 = 0.02) */
  double short_share;      /* short-mode PULL: rows of the frontier with few bits (at most 15, or 31
                              / 63 for rows of 128 / more words) are read from a slot of their
                              source ids instead of whole, on hops where at least this share of
                              the frontier's rows are short and the frontier exceeds half of L2
                              (0 = 0.1; < 0 = never; > 1 = every PULL hop); needs S <= 32768 and
                              whole-row passes, and keeps 36 to 132 B per vertex, except in plans
                              whose V x S matrix fits in half of L2 (short mode never runs there) */
} vs_expand_params;

#define VS_MAX_HOPS 64
typedef struct vs_expand_stats {
  uint32_t hops_run;              /* k_actual_max of the reference */
  uint32_t found;                 /* FindShortest: targets found */
  uint64_t visit_count;           /* Shortest: visited bits at the end */
  uint64_t new_bits[VS_MAX_HOPS + 1];       /* bits set in layer h (Shortest: new bits) */
  uint64_t active_vertices[VS_MAX_HOPS + 1];/* non-zero columns of layer h */
  uint64_t active_edges[VS_MAX_HOPS + 1];   /* edges leaving non-zero columns of layer h-1 */
  uint64_t pairs[VS_MAX_HOPS + 1];          /* sparse hops: pairs produced */
  int32_t strategy[VS_MAX_HOPS + 1];        /* strategy run at hop h */
  float hop_ms[VS_MAX_HOPS + 1];            /* device time of hop h (plans with timing on) */
  float pull_ms[VS_MAX_HOPS + 1];           /* device time of hop h's pull kernels */
  int32_t short_pull[VS_MAX_HOPS + 1];      /* the PULL of hop h ran in short mode: 1 reading words, 2 slots */
  uint64_t short_rows[VS_MAX_HOPS + 1];     /* rows of layer h short enough for a slot (when a PULL
                                               hop wrote its slots) */
  uint64_t short_edges[VS_MAX_HOPS + 1];    /* active in-edges of hop h's PULL served from a slot */
  uint64_t tiny_rows[VS_MAX_HOPS + 1];      /* rows of layer h with one or two bits (ids inline in the word) */
} vs_expand_stats;

/* A plan owns the frontier, next, visited and accumulator matrices for S
 * sources and can be re-run; vs_expand_plan_run enqueues work only (no host
 * synchronisation, no allocation), so it may be captured in a CUDA graph when
 * sources/targets/distances are device pointers. */
int vs_expand_plan_create(vs_graph *g, uint32_t S, const vs_expand_params *p,
                          vs_expand_plan **out);
int vs_expand_plan_run(vs_expand_plan *plan, const uint32_t *sources, const uint32_t *targets,
                       int32_t *distances, vs_stream_t stream);
/* Result of the last run as a borrowed VarRow matrix view (rows = sources,
 * row_map = sources, cols = vertices), valid until the next run or free. */
int vs_expand_plan_result(vs_expand_plan *plan, vs_bitmat **view);
int vs_expand_plan_stats(vs_expand_plan *plan, vs_expand_stats *stats, vs_stream_t stream);
int vs_expand_plan_free(vs_expand_plan *plan);
/* Device bytes a plan for S sources with these parameters allocates
 * (admission control of the serving loop; no counterpart in the reference). */
int vs_expand_plan_footprint(const vs_graph *g, uint32_t S, const vs_expand_params *p, uint64_t *bytes);
/* Planner knobs: fraction of E below which pair lists (SPARSE) run, fraction
 * of V below which PUSH runs (negative = keep), per-hop E_active statistics
 * (an extra pass per hop) and per-hop CUDA-event timing (not for capture). */
int vs_expand_plan_set_tuning(vs_expand_plan *plan, double sparse_frac, double push_frac,
                              int collect_stats, int timing);

/* VExpand with path_params.with_distance, Dense strategy (replaces
 * VExpand::copy_to_multi_MT, vexpand.cpp:356-378, and MultipleMatrixTable,
 * matrix_table.hh:132-149): every layer h in [k_min, k_actual] as its own
 * VarRow matrix (rows = sources with them as row map, columns = vertices):
 * Shortest, the vertices first reached at hop h; Any, the ends of the walks of
 * exactly h hops.  k_actual is the last hop run (a Shortest expand stops when
 * a hop adds no vertex).  layers: caller array of k_max - k_min + 1 handles;
 * *nlayers = layers returned, from k_min up.  Not for FindShortest. */
int vs_expand_layers(vs_graph *g, const uint32_t *sources, uint32_t S, const vs_expand_params *p,
                     vs_bitmat **layers, uint32_t *nlayers, vs_stream_t stream);
/* (row value, column value, distance) tuples of layer matrices, layer by layer
 * (MultipleMatrixTable::output_to_flat, bit_matrix_table.cpp:302-340);
 * distance column I64. */
int vs_layers_to_flat(const vs_bitmat *const *layers, const int32_t *distances, uint32_t n, vs_flat **out,
                      vs_stream_t stream);
/* The same with each (row value, column value) pair once, at the smallest
 * distance it appears (VExpand::merge_to_Flat for Any paths,
 * vexpand.cpp:383-405, which de-duplicates pairs across layers k_min..k_actual;
 * Shortest layers are disjoint, so both calls agree there).  Layers of one
 * shape, distances ascending. */
int vs_layers_to_flat_first(const vs_bitmat *const *layers, const int32_t *distances, uint32_t n, vs_flat **out,
                            vs_stream_t stream);
/* One-shot expand (VExpand::run_internal, vexpand.cpp:448-483): plan, run,
 * hand the result matrix to the caller.  FindShortest: targets[i] is the
 * target of source i, distances[i] receives the hop count (0 when source ==
 * target, -1 when not found) and *out may be NULL.  The library keeps the
 * plans of one-shot calls (at most 8 idle, a quarter of the device's memory
 * and at least 48 GB): a call with the same
 * graph, source count and parameters reuses one, and the returned matrix is
 * that plan's result, lent until vs_bitmat_free (treat it as read-only). */
int vs_expand(vs_graph *g, const uint32_t *sources, uint32_t S, const vs_expand_params *p,
              const uint32_t *targets, int32_t *distances, vs_bitmat **out,
              vs_expand_stats *stats, vs_stream_t stream);
/* Frees the idle plans kept for one-shot expands (no reference counterpart). */
int vs_release_cached(void);

/* ---- hash join (replaces HashJoin, src/objects/operator/join.cpp:26-449) --
 * A table operand is a flat table with the key in column key_col, or a
 * ColMain matrix whose column variable is the key (rows are its payload).
 * The result has join_schema order (src/objects/execution/tuple.cpp:317-342):
 * every column of a, then every non-key column of b; a matrix operand
 * contributes the columns (row value, key).  count is always the exact
 * number of result tuples; at most max_rows are written to *out (the result
 * holds min(count, max_rows) rows and the call returns VS_ERR_CAPACITY when
 * it had to drop tuples).  only_count != 0 computes count only. */
typedef struct vs_table_ref {
  const vs_flat *flat;
  const vs_bitmat *mat;
  uint32_t key_col;
} vs_table_ref;

int vs_hash_join(vs_table_ref a, vs_table_ref b, int only_count, uint64_t max_rows,
                 vs_flat **out, uint64_t *count, vs_stream_t stream);

/* Count-only join of two key columns that allocates no memory (no counterpart
 * in the reference).  For callers that cannot call cudaMalloc: an engine or
 * serving loop that hands all device memory to its own allocator up front,
 * where an allocation mid-query could fail under memory pressure, take the
 * driver's allocation lock or synchronise the device and stall other work.
 * keys_a / keys_b are device arrays of na / nb keys (VS_T_VID = uint32,
 * VS_T_I64 = int64; a host pointer is refused with VS_ERR_ARG before any
 * launch); *count (host or device memory) receives
 * sum_k multiplicity_a(k) * multiplicity_b(k), the same number as
 * vs_hash_join(only_count = 1) on tables holding these key columns.
 * The hash table lives in a fixed device array of this library: 2^19 slots,
 * 8 MiB per GPU, held from the first call on that GPU until process exit.
 * The smaller side may have at most 262,144 rows; larger inputs are rejected
 * with VS_ERR_CAPACITY before any work is queued.  The first call on a device
 * looks up the array's device address (make it before any stream capture);
 * after cudaDeviceReset the next call looks it up again.
 * Every call reuses the same array and clears the part it needs: calls whose
 * work overlaps on the GPU (concurrent streams, or host threads sharing a
 * device) race on it and must be serialised by the caller. */
int vs_hash_join_count_noalloc(const void *keys_a, uint64_t na, const void *keys_b, uint64_t nb,
                               int key_type, uint64_t *count, vs_stream_t stream);

/* Batched join counts (no counterpart in the reference, which joins one
 * query's result at a time).  The VarRow matrix m (a batched expand result,
 * columns = vertex ids) holds several queries in row blocks; block q covers
 * rows [row_begin, row_end) and is joined on the vertex id with the vertex-id
 * keys[key_begin, key_end), count only:
 *   counts[q] = sum over those keys k < V of popcount(column k, rows of q),
 * the count HashJoin gives for (query q's matrix) x (a flat table with that
 * key column).  keys and counts are device memory; counts (nblocks uint64)
 * are overwritten in stream order without a host sync (capturable).  At most
 * VS_MAX_ROW_BLOCKS blocks per call. */
#define VS_MAX_ROW_BLOCKS 512
typedef struct vs_row_block {
  uint32_t row_begin, row_end;
  uint64_t key_begin, key_end;
} vs_row_block;
int vs_hash_join_count_row_blocks(const vs_bitmat *m, const uint32_t *keys, const vs_row_block *blocks,
                                  uint32_t nblocks, uint64_t *counts, vs_stream_t stream);

/* ---- multi-way intersection (replaces Mintersect,
 *      src/objects/operator/mintersect.cpp:14-345) ---------------------------
 * base: flat table or VarRow matrix (columns row value, column value).
 * Each dependency supplies, for the vertex u found in base column base_col,
 * a set of new vertices: a ColMain matrix (rows = new vertex, columns = u,
 * maps optional), a flat edge table (columns u_col -> nv_col) or the graph's
 * adjacency (u's out-list along direction).  For every base tuple the
 * intersection of its dependencies' sets is emitted as (base columns...,
 * new vertex); new_vertex_count bounds the new vertex ids when no dependency
 * is a matrix. */
typedef struct vs_isect_dep {
  const vs_bitmat *mat;
  const vs_flat *flat;
  const vs_graph *graph;
  int32_t direction;
  uint32_t u_col, nv_col;
  uint32_t base_col;
  /* Membership test against a graph adjacency list (VS_ISECT_*; 0 = AUTO).
   * Every choice gives the same result.  AUTO decides per base tuple: the
   * adjacency bitmap when the list's vertex is a hub, a warp-window merge when
   * the walked list has at least 512 entries and this one at most 4x that,
   * else a binary search.  Hub bitmaps (the highest-degree vertices, degree
   * >= 1024, at most 1 GiB per graph and direction) are built on first use
   * and kept with the graph. */
  int32_t algo;
} vs_isect_dep;
#define VS_ISECT_AUTO 0
#define VS_ISECT_BINARY 1
#define VS_ISECT_MERGE 2
#define VS_ISECT_BITMAP 3

int vs_mintersect(vs_table_ref base, const vs_isect_dep *deps, uint32_t ndeps,
                  uint32_t new_vertex_count, int only_count, uint64_t max_rows, vs_flat **out,
                  uint64_t *count, vs_stream_t stream);
/* The same with the learned choice of the adjacency membership method (no
 * counterpart in the reference): method_picker (a vs_picker trained on
 * intersection timings; class 0 = the per-tuple rule of VS_ISECT_AUTO,
 * 1 = binary search, 2 = hub bitmap) decides on the device, from 32 features
 * sampled over up to 4096 base tuples, for every graph dependency whose algo
 * is VS_ISECT_AUTO.
 * features (nullable, 32 floats, host or device) receives those features.
 * Results do not depend on the choice. */
typedef struct vs_picker vs_picker;
int vs_mintersect_ex(vs_table_ref base, const vs_isect_dep *deps, uint32_t ndeps,
                     uint32_t new_vertex_count, int only_count, uint64_t max_rows, const vs_picker *method_picker,
                     float *features, vs_flat **out, uint64_t *count, vs_stream_t stream);

/* ---- result consumers (replace MatrixColumnCount, MatrixRowOrSum and
 *      SemiJoin<N>, src/include/operator/big_operators2.hh,
 *      src/objects/operator/matrix_column_count.cpp:6-87,
 *      matrix_row_or_sum.cpp:7-54, semi_join.cpp:7-262) ------------------ */
/* One (column value, bit count) row per column of a VarRow or ColMain matrix,
 * zero counts included; order 0 = column order, 1 = ascending, 2 = descending
 * by the (count, column value) pair.  Output columns: VID, I64 (the reference's
 * count column is Int32; the values are the same). */
int vs_matrix_column_count(const vs_bitmat *m, int order, vs_flat **out, vs_stream_t stream);
/* The values of the columns holding any bit, in column order (one VID column). */
int vs_matrix_row_or_sum(const vs_bitmat *m, vs_flat **out, vs_stream_t stream);
/* SemiJoin over nkeys (1 or 2) key columns: a's rows (flat a) or bits
 * (VarRow a, key columns 0 = row value, 1 = column value) whose key tuple
 * occurs in b (flat or VarRow).  Two key columns must be vertex ids.  Output:
 * a flat table with a's columns (flat a) or a matrix of a's shape and maps
 * with the other bits cleared (VarRow a); count = rows or bits kept.  ColMain
 * inputs are VS_ERR_UNSUPPORTED, as in the reference. */
int vs_semi_join(vs_table_ref a, vs_table_ref b, uint32_t nkeys, const uint32_t *a_key_cols,
                 const uint32_t *b_key_cols, int only_count, vs_flat **out_flat, vs_bitmat **out_mat,
                 uint64_t *count, vs_stream_t stream);

/* MatrixTableFilter (replaces MatrixTableFilter<F>, big_operators2.hh:53-61,
 * 142-170, over VarRowMatrixTable::filter / ColMainMatrixTable::filter,
 * matrix_table.hh:153-200): clears, in place, every bit (r, c) of m for which
 * the predicate is false, r and c being the row and column VALUES (row_map[r]
 * and col_map[c] when the maps exist, else the indices).  The reference takes
 * a host predicate f(r, c); here it is the AND of up to three device forms:
 *   row_keep   bitset over row values: keep when bit r is set (values at or
 *              above row_values fail); NULL = no row condition
 *   col_keep   the same over column values (col_values bits); NULL = none
 *   pairs      npairs keys (r << 32 | c) sorted ascending (checked; an
 *              unsorted list is VS_ERR_ARG); pairs_mode 1 keeps only listed
 *              pairs, 2 drops listed pairs, 0 ignores the list.
 * The arrays are device or host memory (host arrays are copied in and the
 * call syncs the stream before returning).  A MultipleMatrixTable is filtered
 * layer by layer (one call per layer matrix).  With device arrays and no pair
 * list the call is stream-ordered; a pair list is checked for order with one
 * host sync. */
int vs_matrix_filter(vs_bitmat *m, const uint64_t *row_keep, uint32_t row_values, const uint64_t *col_keep,
                     uint32_t col_values, const uint64_t *pairs, uint64_t npairs, int pairs_mode,
                     vs_stream_t stream);
/* Column predicate of the reference's LDBC-FinBench tcr1 plan
 * (src/objects/testify/ldbc-finbench/tcr1.cpp:46-57, a VertexNeighborFetcher
 * and a VertexPropertyFetcher): mask bit v (g->V bits, ceil(V/64) words) is
 * set when some neighbour u of v in g (out-lists for VS_DIR_FORWARD, in-lists
 * for VS_DIR_BACKWARD) has prop[u] == value.  Vertices of several types share
 * g's id space (e.g. mediums numbered after the accounts).  prop holds nprop
 * uint8 values, host or device; a neighbour id >= nprop is VS_ERR_ARG.  mask
 * is host or device memory; the call syncs the stream once. */
int vs_vertex_mask_any_neighbor(const vs_graph *g, int direction, const uint8_t *prop, uint32_t nprop,
                                uint8_t value, uint64_t *mask, vs_stream_t stream);

/* Scan with a range filter (replaces Scan + VariableFilter over a vertex
 * property, big_operators.hh:21-38, scan.cpp:31-70): the vertex ids i < n with
 * lo <= values[i] <= hi, ascending, as one VID column.  values: device array
 * of n unsigned 1-, 2- or 4-byte or signed 8-byte properties; NULL selects
 * every id (no filter). */
int vs_select_ids_in_range(const void *values, int value_bytes, uint32_t n, int64_t lo, int64_t hi, vs_flat **out,
                           vs_stream_t stream);

/* ---- learned per-hop strategy picker (no counterpart in the reference; it
 *      replaces the fixed Adaptive coverage thresholds of expand.cpp:346-414)
 * A 32-64-64-3 ReLU network, bf16 weights, fp32 accumulation, trained with
 * softmax cross-entropy and Adam by this library's own CUDA kernels.  Input:
 * the 32 features the expand logs per hop (vs_expand_plan_features); output
 * class 0 = PULL, 1 = PUSH, 2 = SPARSE.  Feature rows X are n x 32 floats,
 * labels y are n int32 classes; pointers may be host or device memory. */
int vs_picker_create(uint64_t seed, vs_picker **out);
int vs_picker_free(vs_picker *p);
int vs_picker_num_params(void);
int vs_picker_set_params(vs_picker *p, const float *params);
int vs_picker_get_params(const vs_picker *p, float *params);
int vs_picker_forward(const vs_picker *p, const float *X, uint64_t n, float *logits, vs_stream_t stream);
int vs_picker_backward(const vs_picker *p, const float *X, const int32_t *y, uint64_t n, float *grads,
                       float *loss, vs_stream_t stream);
int vs_picker_train(vs_picker *p, const float *X, const int32_t *y, uint64_t n, uint32_t epochs,
                    uint32_t batch, float lr, uint64_t seed, float *final_loss, vs_stream_t stream);
int vs_picker_predict(const vs_picker *p, const float *X, uint64_t n, int32_t *cls, vs_stream_t stream);
/* Let a plan's AUTO hops be chosen by the picker (NULL restores the fixed planner). */
int vs_expand_plan_set_picker(vs_expand_plan *plan, const vs_picker *p);
/* Per-hop overrides: strategies[h] (h = 1..k_max) forces hop h; 0 = planner's choice. */
int vs_expand_plan_set_hop_strategies(vs_expand_plan *plan, const int32_t *strategies, uint32_t n);
/* Batched queries: the plan's S rows hold the sources of several queries
 * that share path type, direction and k_min; row i stops growing after hop
 * row_kmax[i] (<= k_max), so each query's rows equal its result when run
 * alone.  NULL removes the limits.  (No counterpart in the reference, which
 * runs one VExpand per query.) */
int vs_expand_plan_set_row_limits(vs_expand_plan *plan, const uint8_t *row_kmax, uint32_t n);
/* The same from a device array of n <= S limits, stream-ordered and
 * capturable (rows n..S-1 get limit 0 and never grow; a limit above k_max
 * makes the next run fail with VS_ERR_ARG).  Runs stop after the largest
 * row limit. */
int vs_expand_plan_set_row_limits_device(vs_expand_plan *plan, const uint8_t *row_kmax, uint32_t n,
                                         vs_stream_t stream);
/* Kernel shape of PULL hops (the autotuner's knob): kind 0..7, bit 0 = eight
 * resident 256-thread blocks per SM, bit 1 = L2 cache policies that keep
 * frontier rows and stream everything else, bit 2 = short-mode hops without
 * loading the next target's visited words and flag ahead.  Results never
 * depend on it. */
int vs_expand_plan_set_pull_kernel(vs_expand_plan *plan, int kind);
/* Feature logging: when on, every run records the 32 features of each hop;
 * vs_expand_plan_features copies (VS_MAX_HOPS + 1) x 32 floats (row h = hop h). */
int vs_expand_plan_log_features(vs_expand_plan *plan, int on);
int vs_expand_plan_features(vs_expand_plan *plan, float *features, vs_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* VERTEXSURGE_GB300_H */
