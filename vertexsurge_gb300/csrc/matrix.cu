// Glue operators between the expand and the join/intersection:
// MatrixTableSelect, TableConvert (copy and 64x64 bit-block transpose),
// TableConvert(Flat) / matrix iterators.
// Reference: src/objects/operator/big_operators2.cpp:16-86,138-213,
// src/objects/execution/bit_matrix_table.cpp:133-289.
#include <algorithm>
#include <vector>

#include "vs_internal.cuh"

namespace vs {
namespace mx {

constexpr unsigned FULL = 0xffffffffu;

// Column gather: out[:, j] = in[:, targets[j]] (whole columns of wpc words).
__global__ void k_select(const uint4 *__restrict__ in, uint4 *__restrict__ out,
                         const uint32_t *__restrict__ targets, uint32_t T, uint32_t q_per_col) {
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); j < T; j += warps) {
    const uint4 *src = in + (size_t)targets[j] * q_per_col;
    uint4 *dst = out + (size_t)j * q_per_col;
    for (uint32_t q = lane; q < q_per_col; q += 32) dst[q] = __ldg(src + q);
  }
}

__global__ void k_count_invalid(const uint32_t *__restrict__ ids, uint32_t n, uint32_t bound,
                                unsigned *__restrict__ bad) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (ids[i] >= bound) atomicAdd(bad, 1u);
}

// 64x64 bit-block transpose.  Block (bw, bc) covers input rows 64*bw..+63 and
// input columns 64*bc..+63; lane l holds input columns bc*64+l and bc*64+32+l.
// Output column r = 64*bw + j receives word bc: bit c = input (r, 64*bc + c).
__global__ void k_transpose(const uint64_t *__restrict__ in, uint64_t *__restrict__ out,
                            uint32_t in_rows, uint32_t in_cols, uint32_t wpc_in,
                            uint32_t wpc_out, uint32_t tiles_r, uint32_t tiles_c) {
  const int lane = threadIdx.x & 31;
  const uint64_t ntiles = (uint64_t)tiles_r * tiles_c;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  for (uint64_t t = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < ntiles;
       t += warps) {
    const uint32_t bw = (uint32_t)(t % tiles_r), bc = (uint32_t)(t / tiles_r);
    const uint32_t c_lo = bc * 64 + lane, c_hi = c_lo + 32;
    const uint64_t a = c_lo < in_cols ? in[(size_t)c_lo * wpc_in + bw] : 0ull;
    const uint64_t b = c_hi < in_cols ? in[(size_t)c_hi * wpc_in + bw] : 0ull;
    uint64_t mine_lo = 0, mine_hi = 0;  // output rows 64bw+lane and 64bw+32+lane
#pragma unroll 8
    for (int j = 0; j < 64; j++) {
      const unsigned lo = __ballot_sync(FULL, (a >> j) & 1ull);
      const unsigned hi = __ballot_sync(FULL, (b >> j) & 1ull);
      const uint64_t w = (uint64_t)lo | ((uint64_t)hi << 32);
      if (j == lane) mine_lo = w;
      if (j == lane + 32) mine_hi = w;
    }
    const uint32_t r_lo = bw * 64 + lane, r_hi = r_lo + 32;
    if (r_lo < in_rows) out[(size_t)r_lo * wpc_out + bc] = mine_lo;
    if (r_hi < in_rows) out[(size_t)r_hi * wpc_out + bc] = mine_hi;
  }
}

// Set bits -> (row value, column value) pairs.  A warp owns a column; lanes
// take consecutive words, an exclusive warp scan orders the bits, one
// atomicAdd per column reserves the output range.
__global__ void k_to_flat(const uint64_t *__restrict__ w, uint32_t rows, uint32_t cols,
                          uint32_t wpc, const uint32_t *__restrict__ row_map,
                          const uint32_t *__restrict__ col_map, uint32_t *__restrict__ out_r,
                          uint32_t *__restrict__ out_c, unsigned long long *__restrict__ cursor,
                          unsigned long long total, const uint32_t *__restrict__ colnz) {
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  const uint32_t lw = (rows + 63) / 64;
  // a warp takes 32 columns at a time and walks the ones that may hold bits
  for (uint32_t c0 = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; c0 < cols; c0 += warps * 32) {
   unsigned cm = __ballot_sync(FULL, c0 + lane < cols && (!colnz || colnz[c0 + lane]));
   while (cm) {
    const uint32_t c = c0 + __ffs(cm) - 1;
    cm &= cm - 1;
    const uint32_t cv = col_map ? col_map[c] : c;
    for (uint32_t w0 = 0; w0 < lw; w0 += 32) {
      const uint32_t wi = w0 + lane;
      uint64_t x = wi < lw ? w[(size_t)c * wpc + wi] : 0ull;
      unsigned n = __popcll(x);
      unsigned incl = n;
      for (int o = 1; o < 32; o <<= 1) {
        unsigned y = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += y;
      }
      const unsigned wtot = __shfl_sync(FULL, incl, 31);
      if (!wtot) continue;
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(cursor, (unsigned long long)wtot);
      base = __shfl_sync(FULL, base, 0);
      unsigned long long pos = base + incl - n;
      while (x) {
        const uint32_t r = wi * 64 + (__ffsll((long long)x) - 1);
        x &= x - 1;
        if (pos >= total || r >= rows) break;  // words past the logical rows are zero
        out_r[pos] = row_map ? row_map[r] : r;
        out_c[pos] = cv;
        pos++;
      }
    }
   }
  }
}

}  // namespace mx

int validate_ids(const uint32_t *d_ids, uint32_t n, uint32_t bound, cudaStream_t st, bool *ok) {
  unsigned *bad;
  VS_TRY(dalloc_n(&bad, 1, st));
  VS_CK(cudaMemsetAsync(bad, 0, sizeof(unsigned), st));
  if (n) { mx::k_count_invalid<<<std::max(1u, std::min((n + 255) / 256, 4096u)), 256, 0, st>>>(d_ids, n, bound, bad); vs::note_launch(); }
  unsigned h = 0;
  VS_CK(cudaMemcpyAsync(&h, bad, sizeof(h), cudaMemcpyDeviceToHost, st));
  dfree(bad, st);
  VS_CK(cudaStreamSynchronize(st));
  *ok = h == 0;
  return VS_OK;
}

int bitmat_to_flat(const vs_bitmat *m, cudaStream_t st, vs_flat **out) {
  uint64_t total = 0;
  VS_TRY(bitmat_popcount(m, &total, st));
  const int32_t types[2] = {VS_T_VID, VS_T_VID};
  vs_flat *f = nullptr;
  VS_TRY(flat_alloc(2, types, total, st, &f));
  unsigned long long *cur;
  int rc = dalloc_n(&cur, 1, st);
  if (rc != VS_OK) {
    vs_flat_free(f);
    return rc;
  }
  cudaMemsetAsync(cur, 0, sizeof(*cur), st);
  if (total && m->cols) {
    int blocks = std::max(1, std::min((int)((m->cols + 255) / 256), sm_count() * 8));
    { mx::k_to_flat<<<blocks, 256, 0, st>>>(m->words, m->rows, m->cols, m->wpc, m->row_map, m->col_map,
                                          (uint32_t *)f->cols[0], (uint32_t *)f->cols[1], cur, total, m->colnz); vs::note_launch(); }
  }
  dfree(cur, st);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    vs_flat_free(f);
    return cuda_fail(e, "k_to_flat", __FILE__, __LINE__);
  }
  *out = f;
  return VS_OK;
}

__global__ void k_fill_i64(long long *dst, uint64_t n, long long v) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    dst[i] = v;
}

// The bits of a layer not seen in an earlier one (first = layer & ~seen),
// then seen |= layer; n uint4 of each matrix.
__global__ void k_first_bits(const uint4 *__restrict__ layer, uint4 *__restrict__ seen, uint4 *__restrict__ first,
                             uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint4 l = layer[i], s = seen[i];
    first[i] = andnot4(l, s);
    seen[i] = or4(s, l);
  }
}

// (row value, column value, distance) tuples of the parts, part i with distances[i].
int concat_parts(const std::vector<vs_flat *> &parts, const int32_t *distances, cudaStream_t st, vs_flat **out) {
  uint64_t total = 0;
  for (auto *p : parts) total += p->nrows;
  const int32_t types[3] = {VS_T_VID, VS_T_VID, VS_T_I64};
  vs_flat *f = nullptr;
  VS_TRY(flat_alloc(3, types, total, st, &f));
  uint64_t off = 0;
  for (size_t i = 0; i < parts.size(); i++) {
    const uint64_t k = parts[i]->nrows;
    if (!k) continue;
    cudaError_t e = cudaMemcpyAsync((uint32_t *)f->cols[0] + off, parts[i]->cols[0], 4 * k, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync((uint32_t *)f->cols[1] + off, parts[i]->cols[1], 4 * k, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) {
      const int blocks = (int)std::min<uint64_t>((k + 255) / 256, (uint64_t)sm_count() * 8);
      k_fill_i64<<<blocks, 256, 0, st>>>((long long *)f->cols[2] + off, k, distances[i]);
      vs::note_launch();
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
      vs_flat_free(f);
      return cuda_fail(e, "layers to flat", __FILE__, __LINE__);
    }
    off += k;
  }
  const cudaError_t e = cudaStreamSynchronize(st);  // the parts are freed on return
  if (e != cudaSuccess) {
    vs_flat_free(f);
    return cuda_fail(e, "layers to flat", __FILE__, __LINE__);
  }
  *out = f;
  return VS_OK;
}

}  // namespace vs

using namespace vs;

extern "C" {

int vs_layers_to_flat(const vs_bitmat *const *layers, const int32_t *distances, uint32_t n, vs_flat **out,
                      vs_stream_t stream) {
  if (!out || (n && (!layers || !distances))) return fail(VS_ERR_ARG, "vs_layers_to_flat: null argument");
  cudaStream_t st = S(stream);
  std::vector<vs_flat *> parts(n, nullptr);
  struct Free {
    std::vector<vs_flat *> &p;
    ~Free() {
      for (auto *f : p) vs_flat_free(f);
    }
  } fr{parts};
  for (uint32_t i = 0; i < n; i++) {
    if (!layers[i]) return fail(VS_ERR_ARG, "layer %u is null", i);
    VS_TRY(bitmat_to_flat(layers[i], st, &parts[i]));
  }
  return concat_parts(parts, distances, st, out);
}

int vs_layers_to_flat_first(const vs_bitmat *const *layers, const int32_t *distances, uint32_t n, vs_flat **out,
                            vs_stream_t stream) {
  if (!out || (n && (!layers || !distances))) return fail(VS_ERR_ARG, "vs_layers_to_flat_first: null argument");
  for (uint32_t i = 0; i < n; i++) {
    if (!layers[i]) return fail(VS_ERR_ARG, "layer %u is null", i);
    const vs_bitmat *l0 = layers[0], *l = layers[i];
    if (l->rows != l0->rows || l->cols != l0->cols || l->wpc != l0->wpc || l->kind != l0->kind)
      return fail(VS_ERR_ARG, "layer %u differs in shape from layer 0", i);
    if (i && distances[i] <= distances[i - 1]) return fail(VS_ERR_ARG, "distances must ascend");
  }
  cudaStream_t st = S(stream);
  std::vector<vs_flat *> parts(n, nullptr);
  struct Free {
    std::vector<vs_flat *> &p;
    uint64_t *seen = nullptr, *first = nullptr;
    cudaStream_t st;
    ~Free() {
      for (auto *f : p) vs_flat_free(f);
      dfree(seen, st);
      dfree(first, st);
    }
  } fr{parts, nullptr, nullptr, st};
  if (n) {
    const uint64_t words = (uint64_t)layers[0]->wpc * layers[0]->cols;  // wpc is even: whole uint4
    VS_TRY(dalloc_n(&fr.seen, words, st));
    VS_TRY(dalloc_n(&fr.first, words, st));
    VS_CK(cudaMemsetAsync(fr.seen, 0, 8 * words, st));
    const int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>((words / 2 + 255) / 256, (uint64_t)sm_count() * 8));
    for (uint32_t i = 0; i < n; i++) {
      if (words) {
        k_first_bits<<<blocks, 256, 0, st>>>(reinterpret_cast<const uint4 *>(layers[i]->words),
                                                 reinterpret_cast<uint4 *>(fr.seen),
                                                 reinterpret_cast<uint4 *>(fr.first), words / 2);
        vs::note_launch();
        VS_CK(cudaGetLastError());
      }
      vs_bitmat view = *layers[i];  // the layer's maps over the new bits
      view.words = fr.first;
      view.colnz = nullptr;
      view.owns_words = false;
      view.view = true;
      view.pool_plan = nullptr;
      VS_TRY(bitmat_to_flat(&view, st, &parts[i]));
    }
  }
  return concat_parts(parts, distances, st, out);
}

int vs_matrix_select(const vs_bitmat *m, const uint32_t *targets, uint32_t T, vs_bitmat **out,
                     vs_stream_t stream) {
  if (!m || !out || (T && !targets)) return fail(VS_ERR_ARG, "vs_matrix_select: null argument");
  if (m->col_map)  // the reference asserts here (big_operators2.cpp:165-168)
    return fail(VS_ERR_UNSUPPORTED, "MatrixTableSelect on a matrix that already has a col_map");
  cudaStream_t st = S(stream);
  vs_bitmat *r = nullptr;
  VS_TRY(bitmat_alloc(m->rows, T, m->kind, st, &r));
  int rc = VS_OK;
  if (T) {
    if ((rc = dalloc_n(&r->col_map, T, st)) != VS_OK || (rc = copy_in(r->col_map, targets, T, st)) != VS_OK) {
      vs_bitmat_free(r);
      return rc;
    }
    bool ok = false;
    if ((rc = validate_ids(r->col_map, T, m->cols, st, &ok)) != VS_OK) {
      vs_bitmat_free(r);
      return rc;
    }
    if (!ok) {
      vs_bitmat_free(r);
      return fail(VS_ERR_ARG, "MatrixTableSelect target outside [0, %u)", m->cols);
    }
    int blocks = std::max(1, std::min((int)((T + 7) / 8), sm_count() * 8));
    { mx::k_select<<<blocks, 256, 0, st>>>(reinterpret_cast<const uint4 *>(m->words),
                                         reinterpret_cast<uint4 *>(r->words), r->col_map, T, m->wpc / 2); vs::note_launch(); }
  }
  if (m->row_map) {
    if ((rc = dalloc_n(&r->row_map, m->rows, st)) != VS_OK) {
      vs_bitmat_free(r);
      return rc;
    }
    cudaMemcpyAsync(r->row_map, m->row_map, 4ull * m->rows, cudaMemcpyDeviceToDevice, st);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    vs_bitmat_free(r);
    return cuda_fail(e, "k_select", __FILE__, __LINE__);
  }
  *out = r;
  return VS_OK;
}

int vs_table_convert(const vs_bitmat *m, int transpose, vs_bitmat **out, vs_stream_t stream) {
  if (!m || !out) return fail(VS_ERR_ARG, "vs_table_convert: null argument");
  cudaStream_t st = S(stream);
  vs_bitmat *r = nullptr;
  const uint32_t rows = transpose ? m->cols : m->rows, cols = transpose ? m->rows : m->cols;
  VS_TRY(bitmat_alloc(rows, cols, VS_KIND_COLMAIN, st, &r));
  int rc = VS_OK;
  if (!transpose) {
    if (m->rows && m->cols)
      cudaMemcpyAsync(r->words, m->words, 8ull * m->wpc * m->cols, cudaMemcpyDeviceToDevice, st);
  } else if (m->rows && m->cols) {
    const uint32_t tiles_r = (m->rows + 63) / 64, tiles_c = (m->cols + 63) / 64;
    uint64_t tiles = (uint64_t)tiles_r * tiles_c;
    int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>((tiles + 7) / 8, (uint64_t)sm_count() * 16));
    { mx::k_transpose<<<blocks, 256, 0, st>>>(m->words, r->words, m->rows, m->cols, m->wpc, r->wpc,
                                            tiles_r, tiles_c); vs::note_launch(); }
  }
  const uint32_t *rm = transpose ? m->col_map : m->row_map;
  const uint32_t *cm = transpose ? m->row_map : m->col_map;
  if (rm) {
    if ((rc = dalloc_n(&r->row_map, r->rows, st)) != VS_OK) {
      vs_bitmat_free(r);
      return rc;
    }
    cudaMemcpyAsync(r->row_map, rm, 4ull * r->rows, cudaMemcpyDeviceToDevice, st);
  }
  if (cm) {
    if ((rc = dalloc_n(&r->col_map, r->cols, st)) != VS_OK) {
      vs_bitmat_free(r);
      return rc;
    }
    cudaMemcpyAsync(r->col_map, cm, 4ull * r->cols, cudaMemcpyDeviceToDevice, st);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    vs_bitmat_free(r);
    return cuda_fail(e, "vs_table_convert", __FILE__, __LINE__);
  }
  *out = r;
  return VS_OK;
}

int vs_bitmat_to_flat(const vs_bitmat *m, vs_flat **out, vs_stream_t stream) {
  if (!m || !out) return fail(VS_ERR_ARG, "vs_bitmat_to_flat: null argument");
  return bitmat_to_flat(m, S(stream), out);
}

}  // extern "C"
