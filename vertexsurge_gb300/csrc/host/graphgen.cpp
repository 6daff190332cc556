// Synthetic graph generators and CSR construction.  See graphgen.h.
#include "graphgen.h"

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <random>
#include <set>
#include <vector>

namespace {

inline uint64_t mix64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xBF58476D1CE4E5B9ULL;
  x ^= x >> 27;
  x *= 0x94D049BB133111EBULL;
  x ^= x >> 31;
  return x;
}

inline uint64_t hash3(uint64_t seed, uint64_t a, uint64_t b) {
  return mix64(mix64(seed + 0x9E3779B97F4A7C15ULL) ^ mix64(a * 0xD6E8FEB86659FD93ULL + b));
}

template <typename T> T *alloc_array(uint64_t n) {
  void *p = std::malloc(sizeof(T) * (n ? n : 1));
  return static_cast<T *>(p);
}

// Exclusive prefix sum of counts[0..n) into off[0..n]; parallel two-pass.
void prefix_sum(const uint32_t *counts, uint64_t n, int64_t *off) {
  int nt = omp_get_max_threads();
  std::vector<int64_t> part(nt + 1, 0);
#pragma omp parallel num_threads(nt)
  {
    int t = omp_get_thread_num();
    uint64_t lo = n * t / nt, hi = n * (t + 1) / nt;
    int64_t s = 0;
    for (uint64_t i = lo; i < hi; i++) s += counts[i];
    part[t + 1] = s;
#pragma omp barrier
#pragma omp single
    for (int i = 0; i < nt; i++) part[i + 1] += part[i];
    int64_t run = part[t];
    for (uint64_t i = lo; i < hi; i++) {
      off[i] = run;
      run += counts[i];
    }
  }
  off[n] = part[nt];
}

// Group (src, dst) pairs by src into a CSR, then sort + dedup every list and
// drop self loops.  get(i, &s, &d) returns the i-th pair; returns false to skip.
template <typename Get>
void build_clean_csr(uint32_t V, uint64_t M, Get get, int64_t **off_out, uint32_t **adj_out,
                     uint64_t *E_out) {
  uint32_t *cnt = alloc_array<uint32_t>(V);
  std::memset(cnt, 0, sizeof(uint32_t) * V);
#pragma omp parallel for schedule(static)
  for (uint64_t i = 0; i < M; i++) {
    uint32_t s, d;
    if (get(i, &s, &d) && s != d) __atomic_fetch_add(&cnt[s], 1u, __ATOMIC_RELAXED);
  }
  int64_t *off = alloc_array<int64_t>((uint64_t)V + 1);
  prefix_sum(cnt, V, off);
  uint64_t raw = (uint64_t)off[V];
  uint32_t *adj = alloc_array<uint32_t>(raw);
  std::memset(cnt, 0, sizeof(uint32_t) * V);
#pragma omp parallel for schedule(static)
  for (uint64_t i = 0; i < M; i++) {
    uint32_t s, d;
    if (get(i, &s, &d) && s != d) {
      uint32_t pos = __atomic_fetch_add(&cnt[s], 1u, __ATOMIC_RELAXED);
      adj[off[s] + pos] = d;
    }
  }
  // sort + unique each list, record the cleaned length
#pragma omp parallel for schedule(dynamic, 1024)
  for (uint64_t v = 0; v < V; v++) {
    uint32_t *b = adj + off[v], *e = adj + off[v + 1];
    std::sort(b, e);
    cnt[v] = (uint32_t)(std::unique(b, e) - b);
  }
  int64_t *off2 = alloc_array<int64_t>((uint64_t)V + 1);
  prefix_sum(cnt, V, off2);
  uint64_t E = (uint64_t)off2[V];
  uint32_t *adj2 = alloc_array<uint32_t>(E);
#pragma omp parallel for schedule(dynamic, 1024)
  for (uint64_t v = 0; v < V; v++) {
    std::memcpy(adj2 + off2[v], adj + off[v], sizeof(uint32_t) * cnt[v]);
  }
  std::free(adj);
  std::free(off);
  std::free(cnt);
  *off_out = off2;
  *adj_out = adj2;
  *E_out = E;
}

// Reverse CSR of a cleaned forward CSR; lists come out sorted.
void reverse_csr(uint32_t V, const int64_t *off, const uint32_t *adj, int64_t **roff_out,
                 uint32_t **radj_out) {
  uint64_t E = (uint64_t)off[V];
  uint32_t *cnt = alloc_array<uint32_t>(V);
  std::memset(cnt, 0, sizeof(uint32_t) * V);
#pragma omp parallel for schedule(static)
  for (uint64_t i = 0; i < E; i++) __atomic_fetch_add(&cnt[adj[i]], 1u, __ATOMIC_RELAXED);
  int64_t *roff = alloc_array<int64_t>((uint64_t)V + 1);
  prefix_sum(cnt, V, roff);
  uint32_t *radj = alloc_array<uint32_t>(E);
  std::memset(cnt, 0, sizeof(uint32_t) * V);
#pragma omp parallel for schedule(dynamic, 1024)
  for (uint64_t u = 0; u < V; u++) {
    for (int64_t j = off[u]; j < off[u + 1]; j++) {
      uint32_t v = adj[j];
      uint32_t pos = __atomic_fetch_add(&cnt[v], 1u, __ATOMIC_RELAXED);
      radj[roff[v] + pos] = (uint32_t)u;
    }
  }
#pragma omp parallel for schedule(dynamic, 1024)
  for (uint64_t v = 0; v < V; v++) std::sort(radj + roff[v], radj + roff[v + 1]);
  std::free(cnt);
  *roff_out = roff;
  *radj_out = radj;
}

void finish(uint32_t V, int64_t *off, uint32_t *adj, uint64_t E, vsg_graph *out) {
  out->V = V;
  out->E = E;
  out->fwd_off = off;
  out->fwd_dst = adj;
  reverse_csr(V, off, adj, &out->rev_off, &out->rev_src);
}

}  // namespace

extern "C" {

uint64_t vsg_hash(uint64_t seed, uint64_t a, uint64_t b) { return hash3(seed, a, b); }

int vsg_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
             int undirected, vsg_graph *out) {
  if (!out || scale == 0 || scale > 31 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return 1;
  const uint32_t V = 1u << scale;
  const uint64_t M = (uint64_t)edge_factor * V;
  // integer thresholds on a 32-bit uniform draw: no floating point per edge
  const uint64_t ta = (uint64_t)std::floor(a * 4294967296.0);
  const uint64_t tb = (uint64_t)std::floor((a + b) * 4294967296.0);
  const uint64_t tc = (uint64_t)std::floor((a + b + c) * 4294967296.0);
  uint32_t *src = alloc_array<uint32_t>(M), *dst = alloc_array<uint32_t>(M);
#pragma omp parallel for schedule(static)
  for (uint64_t e = 0; e < M; e++) {
    uint32_t u = 0, v = 0;
    for (uint32_t l = 0; l < scale; l += 2) {
      uint64_t h = hash3(seed, e, l);
      for (uint32_t k = 0; k < 2 && l + k < scale; k++) {
        uint64_t r = (h >> (32 * k)) & 0xFFFFFFFFULL;
        uint32_t bu = 0, bv = 0;
        if (r < ta) {
        } else if (r < tb) {
          bv = 1;
        } else if (r < tc) {
          bu = 1;
        } else {
          bu = 1;
          bv = 1;
        }
        u = (u << 1) | bu;
        v = (v << 1) | bv;
      }
    }
    src[e] = u;
    dst[e] = v;
  }
  int rc = vsg_from_edges(V, M, src, dst, undirected, out);
  std::free(src);
  std::free(dst);
  return rc;
}

int vsg_from_edges(uint32_t V, uint64_t M, const uint32_t *src, const uint32_t *dst,
                   int undirected, vsg_graph *out) {
  if (!out || V == 0) return 1;
  for (uint64_t i = 0; i < M; i++)
    if (src[i] >= V || dst[i] >= V) return 1;
  int64_t *off;
  uint32_t *adj;
  uint64_t E;
  if (undirected) {
    build_clean_csr(
        V, 2 * M,
        [&](uint64_t i, uint32_t *s, uint32_t *d) {
          uint64_t j = i >> 1;
          if (i & 1) {
            *s = dst[j];
            *d = src[j];
          } else {
            *s = src[j];
            *d = dst[j];
          }
          return true;
        },
        &off, &adj, &E);
  } else {
    build_clean_csr(
        V, M,
        [&](uint64_t i, uint32_t *s, uint32_t *d) {
          *s = src[i];
          *d = dst[i];
          return true;
        },
        &off, &adj, &E);
  }
  finish(V, off, adj, E, out);
  return 0;
}

int vsg_zipf(uint32_t V, uint64_t target_edges, double alpha, uint32_t max_deg, uint64_t seed,
             vsg_graph *out) {
  if (!out || V < 2 || alpha <= 1.0 || max_deg == 0) return 1;
  // Continuous power law d = floor(x_min * U^(-1/(alpha-1))) capped at max_deg;
  // x_min is calibrated by bisection on a fixed prefix of vertices so the
  // expected total matches target_edges.
  const double inv = -1.0 / (alpha - 1.0);
  auto degree = [&](uint64_t v, double xmin) -> uint32_t {
    uint64_t h = hash3(seed, v, 0xD3);
    double u = ((h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    double x = xmin * std::pow(u, inv);
    if (x > (double)max_deg) return max_deg;
    uint32_t d = (uint32_t)x;
    return d;
  };
  const uint64_t probe = std::min<uint64_t>(V, 1u << 20);
  double lo = 0.01, hi = 1000.0;
  for (int it = 0; it < 60; it++) {
    double mid = 0.5 * (lo + hi);
    double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (uint64_t v = 0; v < probe; v++) s += degree(v, mid);
    double est = s * ((double)V / (double)probe);
    if (est < (double)target_edges)
      lo = mid;
    else
      hi = mid;
  }
  const double xmin = 0.5 * (lo + hi);
  uint32_t *deg = alloc_array<uint32_t>(V);
#pragma omp parallel for schedule(static)
  for (uint64_t v = 0; v < V; v++) deg[v] = degree(v, xmin);
  int64_t *off = alloc_array<int64_t>((uint64_t)V + 1);
  prefix_sum(deg, V, off);
  uint64_t raw = (uint64_t)off[V];
  uint32_t *adj = alloc_array<uint32_t>(raw);
  uint32_t *cnt = deg;  // reuse as cleaned lengths
#pragma omp parallel for schedule(dynamic, 256)
  for (uint64_t v = 0; v < V; v++) {
    uint32_t *b = adj + off[v];
    uint32_t d = (uint32_t)(off[v + 1] - off[v]), n = 0;
    for (uint32_t j = 0; j < d; j++) {
      uint32_t t = (uint32_t)(hash3(seed ^ 0x5A5A5A5AULL, v, j) % V);
      if (t != v) b[n++] = t;
    }
    std::sort(b, b + n);
    cnt[v] = (uint32_t)(std::unique(b, b + n) - b);
  }
  int64_t *off2 = alloc_array<int64_t>((uint64_t)V + 1);
  prefix_sum(cnt, V, off2);
  uint64_t E = (uint64_t)off2[V];
  uint32_t *adj2 = alloc_array<uint32_t>(E);
#pragma omp parallel for schedule(dynamic, 1024)
  for (uint64_t v = 0; v < V; v++) std::memcpy(adj2 + off2[v], adj + off[v], sizeof(uint32_t) * cnt[v]);
  std::free(adj);
  std::free(off);
  std::free(deg);
  finish(V, off2, adj2, E, out);
  return 0;
}

void vsg_free(vsg_graph *g) {
  if (!g) return;
  std::free(g->fwd_off);
  std::free(g->fwd_dst);
  std::free(g->rev_off);
  std::free(g->rev_src);
  std::memset(g, 0, sizeof(*g));
}

int vsg_sample_sources(uint32_t V, uint32_t n, uint64_t seed, uint32_t *out) {
  if (n > V || !out) return 1;
  if ((uint64_t)2 * n <= V) {
    std::set<uint32_t> s;
    uint64_t i = 0;
    while (s.size() < n) s.insert((uint32_t)(hash3(seed, i++, 0x50) % V));
    uint32_t k = 0;
    for (uint32_t x : s) out[k++] = x;
  } else {
    std::vector<uint32_t> all(V);
    for (uint32_t i = 0; i < V; i++) all[i] = i;
    for (uint32_t i = V - 1; i > 0; i--) {  // Fisher-Yates with the same hash
      uint32_t j = (uint32_t)(hash3(seed, i, 0x51) % (i + 1));
      std::swap(all[i], all[j]);
    }
    std::sort(all.begin(), all.begin() + n);
    std::memcpy(out, all.data(), sizeof(uint32_t) * n);
  }
  return 0;
}

// Community tags of n vertices in id order, as the reference's social-network
// importer assigns them (SocialNetworkImporter::set_random_community,
// src/objects/meta/graph_loader.cpp:229-260): consecutive blocks of
// 2048 x {1,1,1,10,10,10,100,100,100,1000,1000,1000} vertices get the tags
// 0..11, the rest tag 12, then the tags are shuffled by std::shuffle with a
// std::mt19937 seeded as given (the standard library's own shuffle, so the
// tags equal the reference importer's when both use the same library).
int vsg_sn_communities(uint64_t n, uint32_t seed, uint8_t *out) {
  if (!out && n) return 1;
  static const size_t block = 2048;
  static const size_t sel[] = {1, 1, 1, 10, 10, 10, 100, 100, 100, 1000, 1000, 1000};
  const size_t nsel = sizeof(sel) / sizeof(sel[0]);
  std::vector<uint8_t> tag(n);
  size_t idx = 0;
  for (size_t c = 0; c < nsel; c++)
    for (size_t x = 0; x < block * sel[c] && idx < n; x++) tag[idx++] = (uint8_t)c;
  while (idx < n) tag[idx++] = (uint8_t)nsel;
  std::mt19937 gen(seed);
  std::shuffle(tag.begin(), tag.end(), gen);
  if (n) std::memcpy(out, tag.data(), n);
  return 0;
}

}  // extern "C"
