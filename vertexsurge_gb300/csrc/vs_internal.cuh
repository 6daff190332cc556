// Internal definitions shared by the CUDA translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/vertexsurge_gb300.h"

namespace vs {

// Kernels launched by this library since load (vs_kernel_launches).
extern std::atomic<unsigned long long> g_launches;
inline void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void set_error(const char *fmt, ...);
int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);

// Return a status from the enclosing function when a CUDA call fails.
#define VS_CK(call)                                                      \
  do {                                                                   \
    cudaError_t _e = (call);                                             \
    if (_e != cudaSuccess) return ::vs::cuda_fail(_e, #call, __FILE__, __LINE__); \
  } while (0)

#define VS_TRY(call)        \
  do {                      \
    int _rc = (call);       \
    if (_rc != VS_OK) return _rc; \
  } while (0)

inline cudaStream_t S(vs_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

// Stream-ordered allocation from the device pool (kept warm by vs_init).
int dalloc(void **p, size_t bytes, cudaStream_t st);
void dfree(void *p, cudaStream_t st);
template <typename T> int dalloc_n(T **p, size_t n, cudaStream_t st) {
  return dalloc(reinterpret_cast<void **>(p), sizeof(T) * (n ? n : 1), st);
}

// Copy n elements from a host or device pointer (unified addressing).
template <typename T> int copy_in(T *dst, const T *src, size_t n, cudaStream_t st) {
  if (n == 0) return VS_OK;
  VS_CK(cudaMemcpyAsync(dst, src, sizeof(T) * n, cudaMemcpyDefault, st));
  return VS_OK;
}

int sm_count();
size_t l2_bytes();  // the device's L2 cache size

inline uint32_t words_per_col(uint32_t rows) {
  uint32_t w = (rows + 63) / 64;
  return (w + 1) & ~1u;  // even: every column starts on a 16-byte boundary
}

}  // namespace vs

// Adjacency bitmaps of a graph's highest-degree vertices for one list
// direction (membership tests of the intersection), built on first use.
struct vs_hub_index {
  int32_t *slot = nullptr;  // per vertex: bitmap index, or -1
  uint64_t *bm = nullptr;   // n bitmaps of `words` uint64 (bit x = x is in the list)
  uint32_t n = 0, words = 0, min_deg = 0;
  bool built = false;
};

struct vs_graph {
  uint64_t serial;  // unique per upload (never reused): keys cached plans of this graph
  uint32_t V;
  uint64_t E;
  int directed;
  int64_t *fwd_off;
  uint32_t *fwd_dst;
  int64_t *rev_off;
  uint32_t *rev_src;
  vs_hub_index hub[2];  // [0] forward lists, [1] reverse lists
  std::mutex hub_mu;
};

struct vs_bitmat {
  uint32_t rows, cols, wpc;
  int kind;
  uint64_t *words;
  uint32_t *row_map, *col_map;
  uint32_t *colnz;  // optional: colnz[c] == 0 => column c is all zero (expand results)
  cudaStream_t st;  // stream of the last work on the handle; frees are ordered on it
  bool owns_words;
  bool view;  // borrowed view: vs_bitmat_free only releases the struct
  vs_expand_plan *pool_plan = nullptr;  // a one-shot expand result: freeing it returns this plan to the cache
};

struct vs_flat {
  uint32_t ncols;
  uint64_t nrows;
  int32_t types[16];
  void *cols[16];
  cudaStream_t st;  // stream of the last work on the handle; frees are ordered on it
};

namespace vs {
// Cache of expand plans behind the one-shot vs_expand (expand.cu).
void plan_cache_return(vs_expand_plan *pl, cudaStream_t st);  // a result handle was freed
void plan_cache_drop_graph(uint64_t serial);                   // the graph is being freed
uint64_t next_graph_serial();

inline size_t type_size(int t) { return t == VS_T_I64 ? 8 : 4; }
int exclusive_scan_u64(const unsigned long long *in, unsigned long long *out, size_t n,
                       cudaStream_t st);
int popcount_words(const uint64_t *w, size_t n, uint64_t *count, cudaStream_t st);
int bitmat_popcount(const vs_bitmat *m, uint64_t *count, cudaStream_t st);
int bitmat_to_flat(const vs_bitmat *m, cudaStream_t st, vs_flat **out);
int validate_ids(const uint32_t *d_ids, uint32_t n, uint32_t bound, cudaStream_t st, bool *ok);
extern "C" const void *vs_picker_device_weights(const vs_picker *p);
int flat_alloc(uint32_t ncols, const int32_t *types, uint64_t nrows, cudaStream_t st, vs_flat **out);
int bitmat_alloc(uint32_t rows, uint32_t cols, int kind, cudaStream_t st, vs_bitmat **out);

// Device-side helpers -------------------------------------------------------
__device__ __forceinline__ uint4 or4(uint4 a, uint4 b) {
  return make_uint4(a.x | b.x, a.y | b.y, a.z | b.z, a.w | b.w);
}
__device__ __forceinline__ uint4 andnot4(uint4 a, uint4 b) {
  return make_uint4(a.x & ~b.x, a.y & ~b.y, a.z & ~b.z, a.w & ~b.w);
}
__device__ __forceinline__ bool nz4(uint4 a) { return (a.x | a.y | a.z | a.w) != 0; }
__device__ __forceinline__ int popc4(uint4 a) {
  return __popc(a.x) + __popc(a.y) + __popc(a.z) + __popc(a.w);
}
__device__ __forceinline__ uint4 shfl_xor4(uint4 a, int m) {
  a.x = __shfl_xor_sync(0xffffffffu, a.x, m);
  a.y = __shfl_xor_sync(0xffffffffu, a.y, m);
  a.z = __shfl_xor_sync(0xffffffffu, a.z, m);
  a.w = __shfl_xor_sync(0xffffffffu, a.w, m);
  return a;
}
// Read-only, streaming-friendly 16-byte load.
__device__ __forceinline__ uint4 ldg4(const uint4 *p) { return __ldg(p); }

}  // namespace vs
