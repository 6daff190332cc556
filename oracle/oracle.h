/*
 * ORACLE — test infrastructure only.
 *
 * A portable CPU restatement (C++17 + OpenMP, no SIMD) of VertexSurge's
 * variable-length graph pattern matching operators, the reference the parity
 * tests compare the CUDA path with and the timed CPU baseline.  Only tests/, the smoke check
 * in __graft_entry__.py and bench.py's CPU-baseline leg may load it; nothing
 * in the product links or calls it.
 *
 * It follows the reference's scalar (use_simd == false) branches:
 *   bit matrices  src/objects/storage/bitmap.cpp (DenseVarStackMatrix,
 *                 DenseColMainMatrix), layout src/include/storage/bitmap.hh:329-425
 *   expand        src/objects/operator/expand.cpp:210-344 (the BlockHilbert
 *                 hop and its edge layout, and a CSR pull with the same result),
 *                 src/include/operator/expand_impl.hh:135-277,
 *                 src/objects/operator/vexpand.cpp:166-354
 *   select/count/convert  src/objects/operator/big_operators2.cpp:6-86,152-213
 *   hash join     src/objects/operator/join.cpp:26-449
 *   mintersect    src/objects/operator/mintersect.cpp:48-345
 *   directions    src/objects/meta/schema.cpp:261-302
 *
 * The reference itself cannot be compiled in this environment (TBB, fmt,
 * spdlog, xxHash, googletest and the antlr4 runtime are absent, and its
 * AVX-512 paths do not build on aarch64), so parity of the restatement is
 * pinned against the known answers of the reference's own unit tests
 * (join.cpp:451-920, mintersect.cpp:347-511, big_operators2.cpp:215-296,
 * bit_matrix_table.cpp:363-483) and, for expand, against an independent
 * per-source breadth-first search.
 *
 * Matrices cross this interface in LOGICAL column-major form: column c of an
 * R x C matrix is ceil(R/64) little-endian uint64 words, bit (r % 64) of word
 * r / 64 is element (r, c).
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { OR_ANY = 0, OR_SHORTEST = 1, OR_FIND_SHORTEST = 2 };
enum { OR_FORWARD = 0, OR_BACKWARD = 1, OR_BOTH = 2 };
enum { OR_T_VID = 0, OR_T_I64 = 1 };
enum { OR_FLAT = 0, OR_VARROW = 1, OR_COLMAIN = 2 };

/* Expand.  Graph: forward CSR (u -> v lists) and reverse CSR (v <- u lists).
 * directed == 0 means the edge type is undirected and stored both ways, in
 * which case dir is ignored (schema.cpp:280-292).
 * out_words: V columns x ceil(S/64) words (row = source index, col = vertex).
 * targets/dist: FindShortest only (S entries).
 * hop_stats (nullable, 4 x 64 entries): [0][h] = visited count after hop h,
 * [1][h] = popcount of layer h, [2][h] = E_active of hop h (edges whose
 * source row is non-zero in layer h-1), [3][0] = hops actually run. */
int oracle_vexpand(uint32_t V, const int64_t *fwd_off, const uint32_t *fwd_dst,
                   const int64_t *rev_off, const uint32_t *rev_src, int directed,
                   const uint32_t *sources, uint32_t S, uint32_t k_min, uint32_t k_max,
                   int path_type, int dir, uint32_t stack_row_count,
                   const uint32_t *targets, int32_t *dist, uint64_t *out_words,
                   uint64_t *hop_stats);

/* The reference's default dense hop, ExpandDenseStrategy::BlockHilbert
 * (big_operators.hh:44-46, expand.cpp:263-311), over its edge layout
 * (graph_loader.hh:239-276): the (u, v) pairs of the direction (base column u
 * OR-ed into column v) cut into n_blocks blocks by target with the
 * reference's partition rule, each block in the order of the curve index
 * (graph_concepts.hh:164-174); blocks run in parallel, and each pair's columns
 * are prefetched in runs of 20 pairs.  oracle_flat_blocks returns a handle
 * (NULL on bad arguments) for oracle_vexpand_blocks, which takes the
 * remaining arguments of oracle_vexpand and gives the same results.
 * oracle_flat_blocks_export copies out the n_blocks + 1 block offsets and the
 * pairs (u, v interleaved) when the pointers are not NULL, and returns the
 * pair count. */
void *oracle_flat_blocks(uint32_t V, const int64_t *fwd_off, const uint32_t *fwd_dst,
                         const int64_t *rev_off, const uint32_t *rev_src, int directed, int dir,
                         uint32_t n_blocks);
void oracle_flat_blocks_free(void *blocks);
uint64_t oracle_flat_blocks_export(const void *blocks, uint64_t *off, uint32_t *pairs);
int oracle_vexpand_blocks(const void *blocks, const uint32_t *sources, uint32_t S, uint32_t k_min,
                          uint32_t k_max, int path_type, uint32_t stack_row_count,
                          const uint32_t *targets, int32_t *dist, uint64_t *out_words,
                          uint64_t *hop_stats);

/* A table crossing the oracle interface. */
typedef struct or_table {
  int kind;              /* OR_FLAT / OR_VARROW / OR_COLMAIN */
  uint32_t ncols;        /* flat: number of columns; matrix: 2 */
  const int32_t *var;    /* variable id of every column (matrix: row var, col var) */
  const int32_t *type;   /* flat: OR_T_VID / OR_T_I64 per column */
  const void *const *cols;
  uint64_t nrows;        /* flat tuple count */
  uint32_t mrows, mcols; /* matrix shape */
  const uint64_t *words; /* matrix, logical column-major */
  const uint32_t *row_map, *col_map; /* nullable */
} or_table;

/* A flat result owned by the oracle. */
typedef struct or_result {
  uint32_t ncols;
  uint64_t nrows;
  int32_t var[16];
  int32_t type[16];
  void *cols[16];
  int64_t count; /* only_count result */
} or_result;

void oracle_free_result(or_result *r);

/* HashJoin(key, only_count) over deps a (deps[0]) and b (deps[1]). */
int oracle_hash_join(const or_table *a, const or_table *b, int32_t key_var, int only_count,
                     or_result *out);

/* Mintersect(new_var, new_type_count, only_count): deps[0] = base, deps[1..] */
int oracle_mintersect(const or_table *base, const or_table *deps, uint32_t ndeps,
                      int32_t new_var, uint32_t new_type_vertex_count, int only_count,
                      or_result *out);

/* MatrixTableSelect: keep columns targets[0..T) of a VarRow matrix
 * (rows x cols, no col_map); out: rows x T logical words. */
int oracle_matrix_select(uint32_t rows, uint32_t cols, const uint64_t *words,
                         uint32_t stack_row_count, const uint32_t *targets, uint32_t T,
                         uint64_t *out_words);

/* TableConvert VarRow -> ColMain; transpose swaps rows and columns.
 * out: (transpose ? cols x rows : rows x cols) logical words. */
int oracle_table_convert(uint32_t rows, uint32_t cols, const uint64_t *words,
                         uint32_t stack_row_count, int transpose, uint64_t *out_words);

/* Count over a matrix (VarRowMatrixTable::tuple_count). */
uint64_t oracle_matrix_count(uint32_t rows, uint32_t cols, const uint64_t *words,
                             uint32_t stack_row_count);

/* VarRowMatrixTable::Iterator / TableConvert(Flat): emit mapped (r, c) pairs
 * of every set bit. Returns the number of pairs; out arrays sized by caller
 * (pass NULL to count only). */
uint64_t oracle_matrix_iterate(uint32_t rows, uint32_t cols, const uint64_t *words,
                               uint32_t stack_row_count, const uint32_t *row_map,
                               const uint32_t *col_map, uint32_t *out_r, uint32_t *out_c);

/* MatrixColumnCount(count_name, ord) over a VarRow or ColMain matrix
 * (matrix_column_count.cpp:6-87): one (column value, popcount of the column)
 * row per column, zero counts included.  ord 0 = column order, 1 = ascending,
 * 2 = descending by the (count, column value) pair.  out arrays: mcols each. */
int oracle_matrix_column_count(const or_table *m, int ord, uint32_t *out_col, int64_t *out_count);

/* MatrixRowOrSum (matrix_row_or_sum.cpp:7-54): the values of the columns
 * holding any bit, in column order.  Returns their number (out nullable). */
uint64_t oracle_matrix_row_or_sum(const or_table *m, uint32_t *out_col);

/* SemiJoin<N>(key_vars, only_count) (semi_join.cpp:7-262): a = left input,
 * b = right input (Flat or VarRow).  Flat a: the rows of a whose key tuple
 * occurs in b.  VarRow a: the bits (r, c) of a whose key tuple occurs in b;
 * with only_count == 0 the masked matrix goes to out_words (a's logical
 * shape).  out->count is the number of kept rows or bits. */
int oracle_semi_join(const or_table *a, const or_table *b, const int32_t *key_vars, uint32_t N,
                     int only_count, or_result *out, uint64_t *out_words);

/* MatrixTableFilter<F>::run_internal (big_operators2.hh:142-170) over
 * VarRowMatrixTable::Iterator::filter / ColMainMatrixTable::Iterator::filter
 * (matrix_table.hh:153-200): every set bit (r, c) of m is mapped through
 * row_map / col_map and cleared, in place in m->words, when the predicate is
 * false.  The predicate is the device forms of vs_matrix_filter: row_keep /
 * col_keep bitsets over values (NULL = no condition; values at or above
 * row_values / col_values fail) and a sorted (r << 32 | c) pair list, mode 1
 * keep listed, 2 drop listed, 0 none.  Returns the number of bits cleared. */
uint64_t oracle_matrix_filter(const or_table *m, const uint64_t *row_keep, uint32_t row_values,
                              const uint64_t *col_keep, uint32_t col_values, const uint64_t *pairs,
                              uint64_t npairs, int pairs_mode);

/* tcr1's column predicate (ldbc-finbench/tcr1.cpp:46-57): bit v of mask set
 * when a neighbour u of v (CSR off[V+1], adj) has prop[u] == value. */
void oracle_vertex_mask_any_neighbor(const int64_t *off, const uint32_t *adj, uint32_t V, const uint8_t *prop,
                                     uint8_t value, uint64_t *mask);

/* Thread count used by every parallel region (0 = OpenMP default). */
void oracle_set_threads(int n);
int oracle_get_threads(void);

#ifdef __cplusplus
}
#endif
