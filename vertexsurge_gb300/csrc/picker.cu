// Learned strategy picker: training and batch inference kernels.
//
// A 32 -> 64 -> 64 -> 3 ReLU network with bf16 weights and fp32 accumulation,
// trained with softmax cross-entropy and Adam on fp32 master weights (the
// forward and backward passes read the bf16 copies; gradients flow to the
// masters unchanged).  A training block holds 64 samples and the full
// parameter set in shared memory and runs both passes as small matrix
// products over the block's samples, so each gradient entry is summed inside
// the block and added to global memory once per block.  The network is tiny
// (6.4k parameters): plain FMA work, far below anything worth a tensor-core
// pipeline.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "picker.cuh"
#include "vs_internal.cuh"

using namespace vs;
using namespace vs::pk;

struct vs_picker {
  float *master = nullptr;         // NPARAM fp32
  __nv_bfloat16 *w = nullptr;      // NPARAM bf16 (used by forward/backward and the expand planner)
  float *m = nullptr, *v = nullptr;  // Adam moments
  float *grad = nullptr;
  int step = 0;
};

namespace vs {
namespace pk {

constexpr int TB = 64;  // samples per training block

__global__ void k_to_bf16(const float *__restrict__ src, __nv_bfloat16 *__restrict__ dst, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    dst[i] = __float2bfloat16_rn(src[i]);
}

// Forward (+ optional backward) for blocks of TB samples.
// smem: weights (float) NPARAM, X TB*NF, H1 TB*H1, H2 TB*H2, dL TB*NO, dH2 TB*H2, dH1 TB*H1
__global__ void __launch_bounds__(256) k_train_block(const __nv_bfloat16 *__restrict__ wb,
                                                     const float *__restrict__ X,
                                                     const int32_t *__restrict__ y, uint64_t n,
                                                     float inv_total, float *__restrict__ logits_out,
                                                     float *__restrict__ grad, float *__restrict__ loss) {
  extern __shared__ float sm[];
  float *W = sm;
  float *x = W + NPARAM;
  float *h1 = x + TB * NF;
  float *h2 = h1 + TB * H1;
  float *dl = h2 + TB * H2;
  float *dh2 = dl + TB * NO;
  float *dh1 = dh2 + TB * H2;
  const int t = threadIdx.x, nt = blockDim.x;
  for (int i = t; i < NPARAM; i += nt) W[i] = __bfloat162float(wb[i]);
  const uint64_t s0 = (uint64_t)blockIdx.x * TB;
  const int ns = (int)((n - s0) < (uint64_t)TB ? (n - s0) : (uint64_t)TB);
  for (int i = t; i < TB * NF; i += nt) {
    const int s = i / NF;
    x[i] = s < ns ? X[(s0 + s) * NF + (i % NF)] : 0.f;
  }
  __syncthreads();
  for (int i = t; i < TB * H1; i += nt) {
    const int s = i / H1, j = i % H1;
    float a = W[OFF_B1 + j];
    for (int k = 0; k < NF; k++) a += W[OFF_W1 + j * NF + k] * x[s * NF + k];
    h1[i] = a > 0.f ? a : 0.f;
  }
  __syncthreads();
  for (int i = t; i < TB * H2; i += nt) {
    const int s = i / H2, j = i % H2;
    float a = W[OFF_B2 + j];
    for (int k = 0; k < H1; k++) a += W[OFF_W2 + j * H1 + k] * h1[s * H1 + k];
    h2[i] = a > 0.f ? a : 0.f;
  }
  __syncthreads();
  float lsum = 0.f;
  for (int s = t; s < ns; s += nt) {
    float z[NO];
    for (int j = 0; j < NO; j++) {
      float a = W[OFF_B3 + j];
      for (int k = 0; k < H2; k++) a += W[OFF_W3 + j * H2 + k] * h2[s * H2 + k];
      z[j] = a;
      if (logits_out) logits_out[(s0 + s) * NO + j] = a;
    }
    if (grad) {
      const float mx = fmaxf(z[0], fmaxf(z[1], z[2]));
      float e[NO], se = 0.f;
      for (int j = 0; j < NO; j++) {
        e[j] = expf(z[j] - mx);
        se += e[j];
      }
      const int label = y[s0 + s];
      for (int j = 0; j < NO; j++) dl[s * NO + j] = (e[j] / se - (j == label ? 1.f : 0.f)) * inv_total;
      lsum += -(z[label] - mx - logf(se));
    }
  }
  if (!grad) return;
  for (int s = ns + t; s < TB; s += nt)
    for (int j = 0; j < NO; j++) dl[s * NO + j] = 0.f;
  if (lsum != 0.f) atomicAdd(loss, lsum * inv_total);
  __syncthreads();
  // dW3 = dl^T h2, db3
  for (int i = t; i < NO * H2 + NO; i += nt) {
    float a = 0.f;
    if (i < NO * H2) {
      const int j = i / H2, k = i % H2;
      for (int s = 0; s < ns; s++) a += dl[s * NO + j] * h2[s * H2 + k];
      atomicAdd(&grad[OFF_W3 + i], a);
    } else {
      const int j = i - NO * H2;
      for (int s = 0; s < ns; s++) a += dl[s * NO + j];
      atomicAdd(&grad[OFF_B3 + j], a);
    }
  }
  // dh2 = (dl W3) . relu'(h2)
  for (int i = t; i < TB * H2; i += nt) {
    const int s = i / H2, k = i % H2;
    float a = 0.f;
    for (int j = 0; j < NO; j++) a += dl[s * NO + j] * W[OFF_W3 + j * H2 + k];
    dh2[i] = h2[i] > 0.f ? a : 0.f;
  }
  __syncthreads();
  // dW2 = dh2^T h1, db2
  for (int i = t; i < H2 * H1 + H2; i += nt) {
    float a = 0.f;
    if (i < H2 * H1) {
      const int j = i / H1, k = i % H1;
      for (int s = 0; s < ns; s++) a += dh2[s * H2 + j] * h1[s * H1 + k];
      atomicAdd(&grad[OFF_W2 + i], a);
    } else {
      const int j = i - H2 * H1;
      for (int s = 0; s < ns; s++) a += dh2[s * H2 + j];
      atomicAdd(&grad[OFF_B2 + j], a);
    }
  }
  // dh1 = (dh2 W2) . relu'(h1)
  for (int i = t; i < TB * H1; i += nt) {
    const int s = i / H1, k = i % H1;
    float a = 0.f;
    for (int j = 0; j < H2; j++) a += dh2[s * H2 + j] * W[OFF_W2 + j * H1 + k];
    dh1[i] = h1[i] > 0.f ? a : 0.f;
  }
  __syncthreads();
  // dW1 = dh1^T x, db1
  for (int i = t; i < H1 * NF + H1; i += nt) {
    float a = 0.f;
    if (i < H1 * NF) {
      const int j = i / NF, k = i % NF;
      for (int s = 0; s < ns; s++) a += dh1[s * H1 + j] * x[s * NF + k];
      atomicAdd(&grad[OFF_W1 + i], a);
    } else {
      const int j = i - H1 * NF;
      for (int s = 0; s < ns; s++) a += dh1[s * H1 + j];
      atomicAdd(&grad[OFF_B1 + j], a);
    }
  }
}

constexpr size_t TRAIN_SMEM = sizeof(float) * (NPARAM + TB * NF + TB * H1 + TB * H2 + TB * NO + TB * H2 + TB * H1);

__global__ void k_adam(float *__restrict__ master, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, __nv_bfloat16 *__restrict__ wb, int n, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float p = master[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    master[i] = p;
    wb[i] = __float2bfloat16_rn(p);
  }
}

__global__ void k_gather_rows(const float *__restrict__ X, const int32_t *__restrict__ y,
                              const uint32_t *__restrict__ perm, uint64_t n, float *__restrict__ Xo,
                              int32_t *__restrict__ yo) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n * NF;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t r = i / NF, c = i % NF;
    Xo[i] = X[(uint64_t)perm[r] * NF + c];
    if (c == 0) yo[r] = y[perm[r]];
  }
}

__global__ void k_argmax(const float *__restrict__ logits, uint64_t n, int32_t *__restrict__ cls) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const float *z = logits + i * NO;
    int b = 0;
    for (int j = 1; j < NO; j++)
      if (z[j] > z[b]) b = j;
    cls[i] = b;
  }
}

inline uint64_t mix(uint64_t x) {
  x ^= x >> 30;
  x *= 0xBF58476D1CE4E5B9ULL;
  x ^= x >> 27;
  x *= 0x94D049BB133111EBULL;
  x ^= x >> 31;
  return x;
}

int run_blocks(const vs_picker *p, const float *dX, const int32_t *dy, uint64_t n, float *logits, float *grad,
               float *loss, float inv_total, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    VS_CK(cudaFuncSetAttribute(k_train_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TRAIN_SMEM));
    attr = true;
  }
  if (!n) return VS_OK;
  const unsigned blocks = (unsigned)((n + TB - 1) / TB);
  { k_train_block<<<blocks, 256, TRAIN_SMEM, st>>>(p->w, dX, dy, n, inv_total, logits, grad, loss); vs::note_launch(); }
  VS_CK(cudaGetLastError());
  return VS_OK;
}

struct Buf {
  cudaStream_t st;
  void *p[8] = {};
  int k = 0;
  template <typename T> int get(T **o, size_t n) {
    int rc = dalloc_n(o, n, st);
    if (rc == VS_OK) p[k++] = *o;
    return rc;
  }
  ~Buf() {
    for (int i = 0; i < k; i++) dfree(p[i], st);
  }
};

}  // namespace pk
}  // namespace vs

extern "C" {

int vs_picker_create(uint64_t seed, vs_picker **out) {
  if (!out) return fail(VS_ERR_ARG, "null output");
  vs_picker *p = new vs_picker();
  int rc = VS_OK;
  if ((rc = dalloc_n(&p->master, NPARAM, 0)) || (rc = dalloc_n(&p->w, NPARAM, 0)) ||
      (rc = dalloc_n(&p->m, NPARAM, 0)) || (rc = dalloc_n(&p->v, NPARAM, 0)) ||
      (rc = dalloc_n(&p->grad, NPARAM, 0))) {
    vs_picker_free(p);
    return rc;
  }
  // He-uniform initialisation from a counter hash; zero biases
  std::vector<float> h(NPARAM, 0.f);
  auto fill = [&](int off, int fan_out, int fan_in) {
    const float lim = std::sqrt(6.f / (float)fan_in);
    for (int i = 0; i < fan_out * fan_in; i++) {
      const double u = (double)(mix(seed * 0x9E3779B97F4A7C15ULL + (uint64_t)(off + i)) >> 11) / 9007199254740992.0;
      h[off + i] = (float)((2.0 * u - 1.0) * lim);
    }
  };
  fill(OFF_W1, H1, NF);
  fill(OFF_W2, H2, H1);
  fill(OFF_W3, NO, H2);
  rc = vs_picker_set_params(p, h.data());
  if (rc != VS_OK) {
    vs_picker_free(p);
    return rc;
  }
  *out = p;
  return VS_OK;
}

int vs_picker_free(vs_picker *p) {
  if (!p) return VS_OK;
  cudaFree(p->master);
  cudaFree(p->w);
  cudaFree(p->m);
  cudaFree(p->v);
  cudaFree(p->grad);
  delete p;
  return VS_OK;
}

int vs_picker_num_params(void) { return NPARAM; }

int vs_picker_set_params(vs_picker *p, const float *params) {
  if (!p || !params) return fail(VS_ERR_ARG, "null argument");
  VS_CK(cudaMemcpy(p->master, params, sizeof(float) * NPARAM, cudaMemcpyDefault));
  VS_CK(cudaMemset(p->m, 0, sizeof(float) * NPARAM));
  VS_CK(cudaMemset(p->v, 0, sizeof(float) * NPARAM));
  p->step = 0;
  { k_to_bf16<<<(NPARAM + 255) / 256, 256>>>(p->master, p->w, NPARAM); vs::note_launch(); }
  VS_CK(cudaDeviceSynchronize());
  return VS_OK;
}

int vs_picker_get_params(const vs_picker *p, float *params) {
  if (!p || !params) return fail(VS_ERR_ARG, "null argument");
  VS_CK(cudaMemcpy(params, p->master, sizeof(float) * NPARAM, cudaMemcpyDefault));
  return VS_OK;
}

// logits[n x 3] for n feature rows X[n x 32] (host or device pointers).
int vs_picker_forward(const vs_picker *p, const float *X, uint64_t n, float *logits, vs_stream_t stream) {
  if (!p || (n && (!X || !logits))) return fail(VS_ERR_ARG, "null argument");
  cudaStream_t st = S(stream);
  Buf b{st};
  float *dX, *dL;
  VS_TRY(b.get(&dX, n * NF));
  VS_TRY(b.get(&dL, n * NO));
  VS_TRY(copy_in(dX, X, n * NF, st));
  VS_TRY(run_blocks(p, dX, nullptr, n, dL, nullptr, nullptr, 0.f, st));
  VS_CK(cudaMemcpyAsync(logits, dL, sizeof(float) * n * NO, cudaMemcpyDefault, st));
  VS_CK(cudaStreamSynchronize(st));
  return VS_OK;
}

// Gradient of the mean cross-entropy over the n rows with respect to the
// parameters (layout of picker.cuh), and the loss.
int vs_picker_backward(const vs_picker *p, const float *X, const int32_t *y, uint64_t n, float *grads,
                       float *loss, vs_stream_t stream) {
  if (!p || !grads || !n || !X || !y) return fail(VS_ERR_ARG, "null argument");
  cudaStream_t st = S(stream);
  Buf b{st};
  float *dX, *dG, *dLoss;
  int32_t *dy;
  VS_TRY(b.get(&dX, n * NF));
  VS_TRY(b.get(&dy, n));
  VS_TRY(b.get(&dG, NPARAM));
  VS_TRY(b.get(&dLoss, 1));
  VS_TRY(copy_in(dX, X, n * NF, st));
  VS_TRY(copy_in(dy, y, n, st));
  VS_CK(cudaMemsetAsync(dG, 0, sizeof(float) * NPARAM, st));
  VS_CK(cudaMemsetAsync(dLoss, 0, sizeof(float), st));
  VS_TRY(run_blocks(p, dX, dy, n, nullptr, dG, dLoss, 1.f / (float)n, st));
  VS_CK(cudaMemcpyAsync(grads, dG, sizeof(float) * NPARAM, cudaMemcpyDefault, st));
  float h = 0.f;
  VS_CK(cudaMemcpyAsync(&h, dLoss, sizeof(float), cudaMemcpyDeviceToHost, st));
  VS_CK(cudaStreamSynchronize(st));
  if (loss) *loss = h;
  return VS_OK;
}

// Adam over shuffled mini-batches; returns the mean loss of the last epoch.
int vs_picker_train(vs_picker *p, const float *X, const int32_t *y, uint64_t n, uint32_t epochs,
                    uint32_t batch, float lr, uint64_t seed, float *final_loss, vs_stream_t stream) {
  if (!p || !X || !y || !n || !batch) return fail(VS_ERR_ARG, "bad training arguments");
  cudaStream_t st = S(stream);
  Buf b{st};
  float *dX, *dXs, *dLoss;
  int32_t *dy, *dys;
  uint32_t *dperm;
  VS_TRY(b.get(&dX, n * NF));
  VS_TRY(b.get(&dXs, n * NF));
  VS_TRY(b.get(&dy, n));
  VS_TRY(b.get(&dys, n));
  VS_TRY(b.get(&dperm, n));
  VS_TRY(b.get(&dLoss, 1));
  VS_TRY(copy_in(dX, X, n * NF, st));
  VS_TRY(copy_in(dy, y, n, st));
  std::vector<uint32_t> perm(n);
  float last = 0.f;
  for (uint32_t e = 0; e < epochs; e++) {
    for (uint64_t i = 0; i < n; i++) perm[i] = (uint32_t)i;
    for (uint64_t i = n - 1; i > 0; i--) std::swap(perm[i], perm[mix(seed ^ (e * 0x51ED27ULL) ^ i) % (i + 1)]);
    VS_CK(cudaMemcpyAsync(dperm, perm.data(), 4 * n, cudaMemcpyHostToDevice, st));
    { k_gather_rows<<<(unsigned)std::min<uint64_t>((n * NF + 255) / 256, 4096), 256, 0, st>>>(dX, dy, dperm, n, dXs, dys); vs::note_launch(); }
    VS_CK(cudaMemsetAsync(dLoss, 0, sizeof(float), st));
    for (uint64_t b0 = 0; b0 < n; b0 += batch) {
      const uint64_t nb = std::min<uint64_t>(batch, n - b0);
      VS_CK(cudaMemsetAsync(p->grad, 0, sizeof(float) * NPARAM, st));
      VS_TRY(run_blocks(p, dXs + b0 * NF, dys + b0, nb, nullptr, p->grad, dLoss, 1.f / (float)nb, st));
      p->step++;
      const float c1 = 1.f - std::pow(0.9f, (float)p->step), c2 = 1.f - std::pow(0.999f, (float)p->step);
      { k_adam<<<(NPARAM + 255) / 256, 256, 0, st>>>(p->master, p->grad, p->m, p->v, p->w, NPARAM, lr, 0.9f, 0.999f, 1e-8f, c1, c2); vs::note_launch(); }
    }
    float h = 0.f;
    VS_CK(cudaMemcpyAsync(&h, dLoss, sizeof(float), cudaMemcpyDeviceToHost, st));
    VS_CK(cudaStreamSynchronize(st));
    last = h * (float)batch / (float)n;  // mean of the per-batch mean losses (approximately)
  }
  if (final_loss) *final_loss = last;
  return VS_OK;
}

int vs_picker_predict(const vs_picker *p, const float *X, uint64_t n, int32_t *cls, vs_stream_t stream) {
  if (!p || (n && (!X || !cls))) return fail(VS_ERR_ARG, "null argument");
  cudaStream_t st = S(stream);
  Buf b{st};
  float *dX, *dL;
  int32_t *dc;
  VS_TRY(b.get(&dX, n * NF));
  VS_TRY(b.get(&dL, n * NO));
  VS_TRY(b.get(&dc, n));
  VS_TRY(copy_in(dX, X, n * NF, st));
  VS_TRY(run_blocks(p, dX, nullptr, n, dL, nullptr, nullptr, 0.f, st));
  if (n) { k_argmax<<<(unsigned)std::min<uint64_t>((n + 255) / 256, 4096), 256, 0, st>>>(dL, n, dc); vs::note_launch(); }
  VS_CK(cudaMemcpyAsync(cls, dc, 4 * n, cudaMemcpyDefault, st));
  VS_CK(cudaStreamSynchronize(st));
  return VS_OK;
}

const void *vs_picker_device_weights(const vs_picker *p) { return p ? p->w : nullptr; }

}  // extern "C"
