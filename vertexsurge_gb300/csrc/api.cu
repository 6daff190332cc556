// Handles, errors, allocation, graph upload, bit-matrix and flat-table basics.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "vs_internal.cuh"

namespace vs {

static thread_local std::string g_last_error;
std::atomic<unsigned long long> g_launches{0};

void set_error(const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

int fail(int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
  set_error("%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();  // clear the sticky-free allocation error
    return VS_ERR_OOM;
  }
  return VS_ERR_CUDA;
}

int dalloc(void **p, size_t bytes, cudaStream_t st) {
  cudaError_t e = cudaMallocAsync(p, bytes, st);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    *p = nullptr;
    return fail(VS_ERR_OOM, "device allocation of %zu bytes failed", bytes);
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaMallocAsync", __FILE__, __LINE__);
  return VS_OK;
}

void dfree(void *p, cudaStream_t st) {
  if (p) cudaFreeAsync(p, st);
}

int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

size_t l2_bytes() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrL2CacheSize, dev);
    if (n <= 0) n = 1 << 20;
  }
  return (size_t)n;
}

int flat_alloc(uint32_t ncols, const int32_t *types, uint64_t nrows, cudaStream_t st,
               vs_flat **out) {
  if (ncols == 0 || ncols > 16) return fail(VS_ERR_ARG, "flat table needs 1..16 columns");
  vs_flat *f = new vs_flat();
  f->ncols = ncols;
  f->nrows = nrows;
  f->st = st;
  for (uint32_t i = 0; i < ncols; i++) {
    if (types[i] != VS_T_VID && types[i] != VS_T_I64) {
      delete f;
      return fail(VS_ERR_ARG, "column %u has unknown type %d", i, types[i]);
    }
    f->types[i] = types[i];
    int rc = dalloc(&f->cols[i], type_size(types[i]) * (nrows ? nrows : 1), st);
    if (rc != VS_OK) {
      for (uint32_t j = 0; j < i; j++) dfree(f->cols[j], st);
      delete f;
      return rc;
    }
  }
  *out = f;
  return VS_OK;
}

int bitmat_alloc(uint32_t rows, uint32_t cols, int kind, cudaStream_t st, vs_bitmat **out) {
  if (kind != VS_KIND_VARROW && kind != VS_KIND_COLMAIN)
    return fail(VS_ERR_ARG, "unknown matrix kind %d", kind);
  vs_bitmat *m = new vs_bitmat();
  m->rows = rows;
  m->cols = cols;
  m->wpc = words_per_col(rows);
  m->kind = kind;
  m->owns_words = true;
  m->st = st;
  size_t n = (size_t)m->wpc * cols;
  int rc = dalloc_n(&m->words, n, st);
  if (rc != VS_OK) {
    delete m;
    return rc;
  }
  cudaError_t e = cudaMemsetAsync(m->words, 0, sizeof(uint64_t) * (n ? n : 1), st);
  if (e != cudaSuccess) {
    dfree(m->words, st);
    delete m;
    return cuda_fail(e, "cudaMemsetAsync", __FILE__, __LINE__);
  }
  *out = m;
  return VS_OK;
}

// popcount over a word array, 64-bit result accumulated with one atomic per block
__global__ void popcount_kernel(const uint64_t *__restrict__ w, size_t n,
                                unsigned long long *__restrict__ out) {
  unsigned long long s = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    s += __popcll(w[i]);
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ unsigned long long part[32];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < blockDim.x / 32 ? part[threadIdx.x] : 0;
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0 && s) atomicAdd(out, s);
  }
}

__global__ void mask_last_word_kernel(uint64_t *w, uint32_t cols, uint32_t wpc, uint32_t last,
                                      uint64_t mask) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += gridDim.x * blockDim.x)
    w[(size_t)c * wpc + last] &= mask;
}

// popcount of the columns whose colnz flag is set: a warp loads 32 flags at
// once and walks only the flagged columns (16-byte loads).
__global__ void popcount_cols_kernel(const uint4 *__restrict__ w, uint32_t cols, uint32_t q_per_col,
                                     const uint32_t *__restrict__ colnz, unsigned long long *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  unsigned long long s = 0;
  for (uint32_t c0 = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; c0 < cols; c0 += warps * 32) {
    const uint32_t c = c0 + lane;
    unsigned m = __ballot_sync(0xffffffffu, c < cols && colnz[c]);
    while (m) {
      const uint32_t cc = c0 + __ffs(m) - 1;
      m &= m - 1;
      for (uint32_t q = lane; q < q_per_col; q += 32) {
        const uint4 x = __ldg(w + (size_t)cc * q_per_col + q);
        s += __popc(x.x) + __popc(x.y) + __popc(x.z) + __popc(x.w);
      }
    }
  }
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ unsigned long long part[32];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < blockDim.x / 32 ? part[threadIdx.x] : 0;
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0 && s) atomicAdd(out, s);
  }
}

int bitmat_popcount(const vs_bitmat *m, uint64_t *count, cudaStream_t st) {
  if (!m->colnz) return popcount_words(m->words, (size_t)m->wpc * m->cols, count, st);
  unsigned long long *d;
  VS_TRY(dalloc_n(&d, 1, st));
  VS_CK(cudaMemsetAsync(d, 0, sizeof(*d), st));
  if (m->cols) {
    int blocks = (int)std::min<size_t>(((size_t)m->cols + 255) / 256, (size_t)sm_count() * 8);
    { popcount_cols_kernel<<<blocks, 256, 0, st>>>(reinterpret_cast<const uint4 *>(m->words), m->cols, m->wpc / 2,
                                                    m->colnz, d); vs::note_launch(); }
    VS_CK(cudaGetLastError());
  }
  unsigned long long h = 0;
  VS_CK(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, st));
  dfree(d, st);
  VS_CK(cudaStreamSynchronize(st));
  *count = h;
  return VS_OK;
}

int popcount_words(const uint64_t *w, size_t n, uint64_t *count, cudaStream_t st) {
  unsigned long long *d;
  VS_TRY(dalloc_n(&d, 1, st));
  VS_CK(cudaMemsetAsync(d, 0, sizeof(*d), st));
  if (n) {
    int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)sm_count() * 8);
    { popcount_kernel<<<blocks, 256, 0, st>>>(w, n, d); vs::note_launch(); }
    VS_CK(cudaGetLastError());
  }
  unsigned long long h = 0;
  VS_CK(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, st));
  dfree(d, st);
  VS_CK(cudaStreamSynchronize(st));
  *count = h;
  return VS_OK;
}

// Exclusive prefix sum over n uint64 values: out[0..n] with out[n] = total.
// Three passes: per-block scans of 1024 values, a one-block scan of the block
// totals, then the block offsets added back.
__global__ void k_scan_block(const unsigned long long *__restrict__ in,
                             unsigned long long *__restrict__ out, size_t n,
                             unsigned long long *__restrict__ sums) {
  __shared__ unsigned long long warp_tot[32];
  const size_t base = (size_t)blockIdx.x * 1024;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  unsigned long long v[4], run = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    size_t i = base + (size_t)t * 4 + k;
    v[k] = i < n ? in[i] : 0ull;
    run += v[k];
  }
  unsigned long long incl = run;
  for (int o = 1; o < 32; o <<= 1) {
    unsigned long long y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_tot[w] = incl;
  __syncthreads();
  if (w == 0) {
    unsigned long long x = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0ull, xi = x;
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long y = __shfl_up_sync(0xffffffffu, xi, o);
      if (lane >= o) xi += y;
    }
    warp_tot[lane] = xi - x;
    if (lane == 31) sums[blockIdx.x] = xi;
  }
  __syncthreads();
  unsigned long long pre = warp_tot[w] + incl - run;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    size_t i = base + (size_t)t * 4 + k;
    if (i < n) out[i] = pre;
    pre += v[k];
  }
}

__global__ void k_scan_sums(unsigned long long *sums, size_t nb, unsigned long long *total) {
  __shared__ unsigned long long carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __shared__ unsigned long long wt[32];
  for (size_t b0 = 0; b0 < nb; b0 += blockDim.x) {
    size_t i = b0 + threadIdx.x;
    unsigned long long x = i < nb ? sums[i] : 0ull, xi = x;
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long y = __shfl_up_sync(0xffffffffu, xi, o);
      if (lane >= o) xi += y;
    }
    if (lane == 31) wt[w] = xi;
    __syncthreads();
    if (w == 0) {
      unsigned long long a = lane < (int)(blockDim.x >> 5) ? wt[lane] : 0ull, ai = a;
      for (int o = 1; o < 32; o <<= 1) {
        unsigned long long y = __shfl_up_sync(0xffffffffu, ai, o);
        if (lane >= o) ai += y;
      }
      wt[lane] = ai - a;
    }
    __syncthreads();
    const unsigned long long c = carry;
    if (i < nb) sums[i] = c + wt[w] + xi - x;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = c + wt[w] + xi;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(unsigned long long *__restrict__ out, size_t n,
                           const unsigned long long *__restrict__ sums,
                           const unsigned long long *__restrict__ total) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] += sums[i / 1024];
  if (i == 0) out[n] = *total;
}

int exclusive_scan_u64(const unsigned long long *in, unsigned long long *out, size_t n,
                       cudaStream_t st) {
  const size_t nb = (n + 1023) / 1024;
  unsigned long long *sums, *total;
  VS_TRY(dalloc_n(&sums, nb ? nb : 1, st));
  VS_TRY(dalloc_n(&total, 1, st));
  if (n) {
    { k_scan_block<<<(unsigned)nb, 256, 0, st>>>(in, out, n, sums); vs::note_launch(); }
    { k_scan_sums<<<1, 1024, 0, st>>>(sums, nb, total); vs::note_launch(); }
    { k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, n, sums, total); vs::note_launch(); }
  } else {
    VS_CK(cudaMemsetAsync(out, 0, sizeof(unsigned long long), st));
  }
  dfree(sums, st);
  dfree(total, st);
  VS_CK(cudaGetLastError());
  return VS_OK;
}

}  // namespace vs

using namespace vs;

extern "C" {

const char *vs_last_error(void) { return g_last_error.c_str(); }

const char *vs_version(void) { return "vertexsurge_gb300 0.1 sm_103a"; }

uint64_t vs_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

struct vs_captured {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint64_t kernels = 0;
};

int vs_capture_begin(vs_stream_t stream) {
  cudaStream_t st = vs::S(stream);
  if (st == 0) return fail(VS_ERR_ARG, "capture needs a created stream, not the default stream");
  // relaxed: the library's own host calls (stream syncs of a plan's previous
  // stream) stay legal while the stream records
  VS_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
  return VS_OK;
}

int vs_capture_end(vs_stream_t stream, vs_captured **out) {
  if (!out) return fail(VS_ERR_ARG, "vs_capture_end: null argument");
  cudaStream_t st = vs::S(stream);
  cudaGraph_t graph = nullptr;
  VS_CK(cudaStreamEndCapture(st, &graph));
  if (!graph) return fail(VS_ERR_ARG, "vs_capture_end: nothing was captured");
  size_t n = 0;
  cudaError_t e = cudaGraphGetNodes(graph, nullptr, &n);
  std::vector<cudaGraphNode_t> nodes(n);
  if (e == cudaSuccess && n) e = cudaGraphGetNodes(graph, nodes.data(), &n);
  uint64_t kernels = 0;
  for (size_t i = 0; e == cudaSuccess && i < n; i++) {
    cudaGraphNodeType t;
    e = cudaGraphNodeGetType(nodes[i], &t);
    kernels += t == cudaGraphNodeTypeKernel;
  }
  vs_captured *g = new vs_captured();
  g->graph = graph;
  g->kernels = kernels;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    delete g;
    return cuda_fail(e, "vs_capture_end", __FILE__, __LINE__);
  }
  g_launches.fetch_sub(kernels, std::memory_order_relaxed);  // recorded, not run
  *out = g;
  return VS_OK;
}

int vs_captured_launch(vs_captured *g, vs_stream_t stream) {
  if (!g) return fail(VS_ERR_ARG, "null captured graph");
  VS_CK(cudaGraphLaunch(g->exec, vs::S(stream)));
  g_launches.fetch_add(g->kernels, std::memory_order_relaxed);
  return VS_OK;
}

uint64_t vs_captured_kernels(const vs_captured *g) { return g ? g->kernels : 0; }

int vs_captured_free(vs_captured *g) {
  if (!g) return VS_OK;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
  return VS_OK;
}

int vs_init(int device) {
  VS_CK(cudaSetDevice(device));
  cudaMemPool_t pool;
  VS_CK(cudaDeviceGetDefaultMemPool(&pool, device));
  uint64_t threshold = UINT64_MAX;  // keep freed blocks for reuse
  VS_CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold));
  sm_count();
  return VS_OK;
}

// A CSR is well formed when off[0] = 0, off[V] = E, offsets never decrease
// and every target is a vertex id; any violation sets *bad.
__global__ void k_check_csr(const int64_t *__restrict__ off, const uint32_t *__restrict__ adj, uint32_t V,
                            uint64_t E, unsigned *bad) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool ok = true;
  if (i0 == 0) ok = off[0] == 0 && off[V] == (int64_t)E;
  for (uint64_t i = i0; i < V; i += stride) ok &= off[i] <= off[i + 1];
  for (uint64_t i = i0; i < E; i += stride) ok &= adj[i] < V;
  if (!ok) atomicExch(bad, 1u);
}

int vs_graph_upload(uint32_t V, uint64_t E, const int64_t *fwd_off, const uint32_t *fwd_dst,
                    const int64_t *rev_off, const uint32_t *rev_src, int directed,
                    vs_stream_t stream, vs_graph **out) {
  if (!out || V == 0 || !fwd_off || !rev_off || (E && (!fwd_dst || !rev_src)))
    return fail(VS_ERR_ARG, "vs_graph_upload: missing CSR arrays");
  cudaStream_t st = S(stream);
  vs_graph *g = new vs_graph();
  g->serial = vs::next_graph_serial();
  g->V = V;
  g->E = E;
  g->directed = directed ? 1 : 0;
  int rc = VS_OK;
  if ((rc = dalloc_n(&g->fwd_off, (size_t)V + 1, st)) != VS_OK ||
      (rc = dalloc_n(&g->rev_off, (size_t)V + 1, st)) != VS_OK ||
      (rc = dalloc_n(&g->fwd_dst, E, st)) != VS_OK ||
      (rc = dalloc_n(&g->rev_src, E, st)) != VS_OK ||
      (rc = copy_in(g->fwd_off, fwd_off, (size_t)V + 1, st)) != VS_OK ||
      (rc = copy_in(g->rev_off, rev_off, (size_t)V + 1, st)) != VS_OK ||
      (rc = copy_in(g->fwd_dst, fwd_dst, E, st)) != VS_OK ||
      (rc = copy_in(g->rev_src, rev_src, E, st)) != VS_OK) {
    vs_graph_free(g);
    return rc;
  }
  // every later kernel indexes rows and lists by these arrays: reject malformed input here
  unsigned *bad = nullptr;
  if ((rc = dalloc_n(&bad, 1, st)) != VS_OK) {
    vs_graph_free(g);
    return rc;
  }
  unsigned hbad = 0;
  cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(unsigned), st);
  const int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>((std::max<uint64_t>(V, E) + 255) / 256,
                                                                   (uint64_t)sm_count() * 8));
  if (e == cudaSuccess) {
    k_check_csr<<<blocks, 256, 0, st>>>(g->fwd_off, g->fwd_dst, V, E, bad);
    vs::note_launch();
    k_check_csr<<<blocks, 256, 0, st>>>(g->rev_off, g->rev_src, V, E, bad);
    vs::note_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hbad, bad, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  dfree(bad, st);
  if (e != cudaSuccess) {
    vs_graph_free(g);
    return cuda_fail(e, "vs_graph_upload", __FILE__, __LINE__);
  }
  if (hbad) {
    vs_graph_free(g);
    return fail(VS_ERR_ARG, "malformed CSR: offsets must rise from 0 to E and every target must be < V (%u)", V);
  }
  *out = g;
  return VS_OK;
}

int vs_graph_info(const vs_graph *g, uint32_t *V, uint64_t *E, int *directed) {
  if (!g) return fail(VS_ERR_ARG, "null graph");
  if (V) *V = g->V;
  if (E) *E = g->E;
  if (directed) *directed = g->directed;
  return VS_OK;
}

int vs_graph_free(vs_graph *g) {
  if (!g) return VS_OK;
  vs::plan_cache_drop_graph(g->serial);
  cudaFree(g->fwd_off);
  cudaFree(g->rev_off);
  cudaFree(g->fwd_dst);
  cudaFree(g->rev_src);
  for (vs_hub_index &h : g->hub) {
    if (h.slot) cudaFree(h.slot);
    if (h.bm) cudaFree(h.bm);
  }
  delete g;
  return VS_OK;
}

int vs_bitmat_create(uint32_t rows, uint32_t cols, int kind, vs_stream_t stream, vs_bitmat **out) {
  if (!out) return fail(VS_ERR_ARG, "null output");
  return bitmat_alloc(rows, cols, kind, S(stream), out);
}

int vs_bitmat_upload(vs_bitmat *m, const uint64_t *logical_words, vs_stream_t stream) {
  if (!m || (!logical_words && m->rows && m->cols)) return fail(VS_ERR_ARG, "null argument");
  if (m->view) return fail(VS_ERR_ARG, "vs_bitmat_upload: the matrix is a read-only view (an expand result)");
  cudaStream_t st = S(stream);
  if (st != m->st) {  // the matrix was allocated in another stream's order
    VS_CK(cudaStreamSynchronize(m->st));
    m->st = st;
  }
  const size_t lw = (m->rows + 63) / 64;
  VS_CK(cudaMemsetAsync(m->words, 0, sizeof(uint64_t) * (size_t)m->wpc * m->cols, st));
  if (lw && m->cols) {
    VS_CK(cudaMemcpy2DAsync(m->words, m->wpc * 8, logical_words, lw * 8, lw * 8, m->cols,
                            cudaMemcpyDefault, st));
    if (m->rows % 64) {  // bits past the last row must stay zero
      const uint64_t mask = (1ull << (m->rows % 64)) - 1;
      { mask_last_word_kernel<<<std::max(1u, std::min((m->cols + 255) / 256, 4096u)), 256, 0, st>>>(
          m->words, m->cols, m->wpc, (uint32_t)(lw - 1), mask); vs::note_launch(); }
      VS_CK(cudaGetLastError());
    }
  }
  return VS_OK;
}

int vs_bitmat_download(const vs_bitmat *m, uint64_t *logical_words, vs_stream_t stream) {
  if (!m || (!logical_words && m->rows && m->cols)) return fail(VS_ERR_ARG, "null argument");
  cudaStream_t st = S(stream);
  const size_t lw = (m->rows + 63) / 64;
  if (lw && m->cols)
    VS_CK(cudaMemcpy2DAsync(logical_words, lw * 8, m->words, m->wpc * 8, lw * 8, m->cols,
                            cudaMemcpyDefault, st));
  VS_CK(cudaStreamSynchronize(st));
  return VS_OK;
}

int vs_bitmat_set_maps(vs_bitmat *m, const uint32_t *row_map, const uint32_t *col_map,
                       vs_stream_t stream) {
  if (!m) return fail(VS_ERR_ARG, "null matrix");
  cudaStream_t st = S(stream);
  if (row_map) {
    if (!m->row_map) VS_TRY(dalloc_n(&m->row_map, m->rows, st));
    VS_TRY(copy_in(m->row_map, row_map, m->rows, st));
  }
  if (col_map) {
    if (!m->col_map) VS_TRY(dalloc_n(&m->col_map, m->cols, st));
    VS_TRY(copy_in(m->col_map, col_map, m->cols, st));
  }
  return VS_OK;
}

int vs_bitmat_get_maps(const vs_bitmat *m, uint32_t *row_map, uint32_t *col_map,
                       vs_stream_t stream) {
  if (!m) return fail(VS_ERR_ARG, "null matrix");
  cudaStream_t st = S(stream);
  if (row_map && m->row_map)
    VS_CK(cudaMemcpyAsync(row_map, m->row_map, 4ull * m->rows, cudaMemcpyDefault, st));
  if (col_map && m->col_map)
    VS_CK(cudaMemcpyAsync(col_map, m->col_map, 4ull * m->cols, cudaMemcpyDefault, st));
  VS_CK(cudaStreamSynchronize(st));
  return VS_OK;
}

int vs_bitmat_get_info(const vs_bitmat *m, vs_bitmat_info *info) {
  if (!m || !info) return fail(VS_ERR_ARG, "null argument");
  info->rows = m->rows;
  info->cols = m->cols;
  info->wpc = m->wpc;
  info->kind = m->kind;
  info->has_row_map = m->row_map != nullptr;
  info->has_col_map = m->col_map != nullptr;
  info->words = m->words;
  return VS_OK;
}

int vs_bitmat_free(vs_bitmat *m) {
  if (!m) return VS_OK;
  if (m->pool_plan) {  // a one-shot expand result: its plan goes back to the cache
    vs::plan_cache_return(m->pool_plan, m->st);
    delete m;
    return VS_OK;
  }
  if (!m->view) {  // stream-ordered after the handle's last work, no device-wide wait
    if (m->owns_words) dfree(m->words, m->st);
    dfree(m->row_map, m->st);
    dfree(m->col_map, m->st);
    dfree(m->colnz, m->st);
  }
  delete m;
  return VS_OK;
}

int vs_bitmat_count(const vs_bitmat *m, uint64_t *count, vs_stream_t stream) {
  if (!m || !count) return fail(VS_ERR_ARG, "null argument");
  return bitmat_popcount(m, count, S(stream));
}

int vs_flat_create(uint32_t ncols, const int32_t *types, uint64_t nrows, vs_flat **out) {
  if (!out || !types) return fail(VS_ERR_ARG, "null argument");
  VS_TRY(flat_alloc(ncols, types, nrows, 0, out));
  // allocated in legacy-stream order: make it usable from any stream
  VS_CK(cudaStreamSynchronize(0));
  return VS_OK;
}

int vs_flat_upload(vs_flat *f, uint32_t col, const void *data, vs_stream_t stream) {
  if (!f || col >= f->ncols || (!data && f->nrows)) return fail(VS_ERR_ARG, "bad column");
  f->st = S(stream);
  if (f->nrows)
    VS_CK(cudaMemcpyAsync(f->cols[col], data, type_size(f->types[col]) * f->nrows,
                          cudaMemcpyDefault, S(stream)));
  return VS_OK;
}

int vs_flat_download(const vs_flat *f, uint32_t col, void *data, vs_stream_t stream) {
  if (!f || col >= f->ncols || (!data && f->nrows)) return fail(VS_ERR_ARG, "bad column");
  if (f->nrows)
    VS_CK(cudaMemcpyAsync(data, f->cols[col], type_size(f->types[col]) * f->nrows,
                          cudaMemcpyDefault, S(stream)));
  VS_CK(cudaStreamSynchronize(S(stream)));
  return VS_OK;
}

int vs_flat_info(const vs_flat *f, uint32_t *ncols, uint64_t *nrows, int32_t *types) {
  if (!f) return fail(VS_ERR_ARG, "null table");
  if (ncols) *ncols = f->ncols;
  if (nrows) *nrows = f->nrows;
  if (types)
    for (uint32_t i = 0; i < f->ncols; i++) types[i] = f->types[i];
  return VS_OK;
}

int vs_flat_column(const vs_flat *f, uint32_t col, const void **device_ptr) {
  if (!f || !device_ptr) return fail(VS_ERR_ARG, "vs_flat_column: null argument");
  if (col >= f->ncols) return fail(VS_ERR_ARG, "column %u of %u", col, f->ncols);
  *device_ptr = f->cols[col];
  return VS_OK;
}

int vs_flat_free(vs_flat *f) {
  if (!f) return VS_OK;
  for (uint32_t i = 0; i < f->ncols; i++) dfree(f->cols[i], f->st);
  delete f;
  return VS_OK;
}

}  // extern "C"
