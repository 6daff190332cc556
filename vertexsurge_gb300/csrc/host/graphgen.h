/*
 * Synthetic graph generators and CSR construction (host C++, OpenMP).
 *
 * The reference loads graphs written by its offline importer
 * (src/objects/importer.cpp, src/include/meta/graph_loader.hh:163-200 writes
 * CSR as int64 offsets + uint32 targets).  The synthetic workloads used here
 * (R-MAT and Zipf out-degree graphs) are produced directly in that CSR form:
 * self-loops and duplicate edges removed, every adjacency list sorted.
 *
 * All random draws come from a counter-based hash (splitmix64 finaliser over
 * (seed, edge index, level)), so a graph depends only on its parameters and
 * not on the thread count or the machine.  The R-MAT path uses integer
 * thresholds only and is bit-identical on x86-64 and aarch64.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Counts of a generated graph: V vertices, E directed edges after cleaning. */
typedef struct vsg_graph {
  uint32_t V;
  uint64_t E;
  int64_t *fwd_off;  /* V+1 */
  uint32_t *fwd_dst; /* E, each list sorted ascending */
  int64_t *rev_off;  /* V+1 */
  uint32_t *rev_src; /* E, each list sorted ascending */
} vsg_graph;

/* Directed R-MAT: 2^scale vertices, edge_factor * 2^scale edges attempted,
 * quadrant probabilities a, b, c (d = 1 - a - b - c).  undirected != 0 adds
 * the reverse of every edge before cleaning (reference behaviour for
 * undirected edge types, graph_loader.hh:64-66). */
int vsg_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
             uint64_t seed, int undirected, vsg_graph *out);

/* Power-law out-degree graph: V vertices, out-degree ~ discrete power law
 * with exponent alpha (P(d) ~ d^-alpha), capped at max_deg, scaled so the
 * expected edge count is target_edges; targets uniform over [0, V). */
int vsg_zipf(uint32_t V, uint64_t target_edges, double alpha, uint32_t max_deg,
             uint64_t seed, vsg_graph *out);

/* Build a cleaned CSR pair from an explicit edge list (src[i] -> dst[i]). */
int vsg_from_edges(uint32_t V, uint64_t M, const uint32_t *src,
                   const uint32_t *dst, int undirected, vsg_graph *out);

void vsg_free(vsg_graph *g);

/* Uniform sample of n distinct vertex ids from [0, V), in ascending order
 * (same contract as the reference's uniform_random_numbers,
 * src/include/utils/utils.hh:75-95, which returns a sorted std::set when
 * 2n <= V). */
int vsg_sample_sources(uint32_t V, uint32_t n, uint64_t seed, uint32_t *out);
/* Community tags (uint8) of n vertices as the reference's social-network
 * importer assigns them (std::mt19937(seed) + std::shuffle). */
int vsg_sn_communities(uint64_t n, uint32_t seed, uint8_t *out);

/* The counter-based hash used by every generator (exposed for tests). */
uint64_t vsg_hash(uint64_t seed, uint64_t a, uint64_t b);

#ifdef __cplusplus
}
#endif
