// Learned per-hop strategy picker: features and MLP inference (device side).
//
// The network is 32 -> 64 -> 64 -> 3 with ReLU, bf16 weights and fp32
// accumulation.  Its input is a fixed feature vector of the frontier entering
// hop h, computed on the device from the previous hop's counters and the
// out-degree histogram of the active rows; its output scores PULL, PUSH and
// SPARSE.  It only chooses a strategy, never a result: every strategy yields
// the same bit matrix.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace vs {
namespace pk {

constexpr int NF = 32, H1 = 64, H2 = 64, NO = 3;
// parameter layout (row-major, out x in): W1, b1, W2, b2, W3, b3
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + H1 * NF, OFF_W2 = OFF_B1 + H1, OFF_B2 = OFF_W2 + H2 * H1,
              OFF_W3 = OFF_B2 + H2, OFF_B3 = OFF_W3 + NO * H2, NPARAM = OFF_B3 + NO;
constexpr int NHIST = 16;
static_assert((NF & (NF - 1)) == 0 && (H1 & (H1 - 1)) == 0, "rotated dot products need power-of-two widths");

// class index -> strategy code of the expand kernels
__host__ __device__ inline int class_to_strategy(int c) { return c == 0 ? 1 : (c == 1 ? 2 : 3); }
__host__ __device__ inline int strategy_to_class(int s) { return s == 1 ? 0 : (s == 2 ? 1 : 2); }

struct HopFeatIn {
  float S, V, E, W, h, k_min, k_max;
  float new_bits_prev, active_prev, visited_bits, active_edges, pair_edges;
  float pairs_ok, shortest, both;
  const unsigned long long *hist;  // NHIST bins of log2(out-degree + 1) over active rows
};

__device__ __forceinline__ float lg(float x) { return log2f(1.f + x); }

// Single-precision throughout: the features are fp32 network inputs, and a
// hop's decide block runs on the critical path of the run.
__device__ inline void hop_features(const HopFeatIn &in, float *f) {
  const float SV = in.S * in.V;
  f[0] = in.new_bits_prev / SV;
  f[1] = in.active_prev / in.V;
  f[2] = lg(in.active_prev) / 32.f;
  f[3] = in.visited_bits / SV;
  f[4] = lg(in.S) / 16.f;
  f[5] = in.W / 256.f;
  f[6] = lg(in.V) / 32.f;
  f[7] = lg(in.E) / 40.f;
  f[8] = in.E / in.V / 64.f;
  f[9] = in.h / 8.f;
  f[10] = in.active_edges / in.E;
  f[11] = lg(in.active_edges) / 40.f;
  f[12] = in.pairs_ok;
  f[13] = in.shortest;
  f[14] = in.both;
  f[15] = lg(in.pair_edges) / 40.f;
  unsigned long long tot = 0;
  for (int b = 0; b < NHIST; b++) tot += in.hist[b];
  const float r = tot ? 1.f / (float)tot : 0.f;
  for (int b = 0; b < NHIST; b++) f[16 + b] = (float)in.hist[b] * r;
}

// Inference by a whole block, in two calls every thread makes.
// mlp_stage starts copying the bf16 parameters (16-byte aligned) into shared
// memory with asynchronous 16-byte copies and returns the buffer; a kernel
// can call it first and compute its features while the copies are in flight.
// mlp_run (blockDim.x = P * H1, P a power of two, 2..16) waits for them, then
// splits each hidden unit's dot product over P adjacent lanes, each starting
// at its own offset so a warp's lanes read different banks, sums them by
// shuffles, and computes each output unit in one warp.  out[NO] must be
// shared memory.
__device__ inline __nv_bfloat16 *mlp_stage(const void *params) {
  __shared__ __align__(16) __nv_bfloat16 w[(NPARAM + 7) / 8 * 8];
  const int t = threadIdx.x;
  const __nv_bfloat16 *gw = (const __nv_bfloat16 *)params;
  constexpr int NV = NPARAM / 8;
  // asynchronous 16-byte copies: no thread waits for them before mlp_run
  for (int i = t; i < NV; i += blockDim.x) {
    const unsigned dst = (unsigned)__cvta_generic_to_shared(reinterpret_cast<uint4 *>(w) + i);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(reinterpret_cast<const uint4 *>(gw) + i)
                 : "memory");
  }
  // the few tail elements by the block's last threads (thread 0 often has other work)
  for (int i = NV * 8 + (int)(blockDim.x - 1 - t); i < NPARAM; i += blockDim.x) w[i] = gw[i];
  return w;
}

__device__ inline void mlp_run(const __nv_bfloat16 *w, const float *f, float *out) {
  __shared__ float h1[H1], h2[H2];
  const int t = threadIdx.x, lane = t & 31;
  asm volatile("cp.async.wait_all;" ::: "memory");
  __syncthreads();
  const int P = blockDim.x / H1, u = t / P, p = t & (P - 1);
  {
    const int n = NF / P;
    float acc = 0.f;
    for (int k = 0; k < n; k++) {
      const int i = p * n + ((k + u) & (n - 1));
      acc += __bfloat162float(w[OFF_W1 + u * NF + i]) * f[i];
    }
    for (int o = P >> 1; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (p == 0) {
      acc += __bfloat162float(w[OFF_B1 + u]);
      h1[u] = acc > 0.f ? acc : 0.f;
    }
  }
  __syncthreads();
  {
    const int n = H1 / P;
    float acc = 0.f;
    for (int k = 0; k < n; k++) {
      const int i = p * n + ((k + 2 * u) & (n - 1));
      acc += __bfloat162float(w[OFF_W2 + u * H1 + i]) * h1[i];
    }
    for (int o = P >> 1; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (p == 0) {
      acc += __bfloat162float(w[OFF_B2 + u]);
      h2[u] = acc > 0.f ? acc : 0.f;
    }
  }
  __syncthreads();
  if (t < NO * 32) {
    const int o3 = t >> 5;
    float acc = 0.f;
    for (int i = lane; i < H2; i += 32) acc += __bfloat162float(w[OFF_W3 + o3 * H2 + i]) * h2[i];
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) out[o3] = acc + __bfloat162float(w[OFF_B3 + o3]);
  }
  __syncthreads();
}

__device__ inline void mlp_block(const void *params, const float *f, float *out) {
  mlp_run(mlp_stage(params), f, out);
}

// One sample through the network, computed by one thread (64 FMAs per
// output unit).  w: bf16 parameters in the layout above.
__device__ inline void mlp_forward_1(const __nv_bfloat16 *__restrict__ w, const float *x, float *h1,
                                     float *h2, float *out) {
  for (int j = 0; j < H1; j++) {
    float s = __bfloat162float(w[OFF_B1 + j]);
    for (int i = 0; i < NF; i++) s += __bfloat162float(w[OFF_W1 + j * NF + i]) * x[i];
    h1[j] = s > 0.f ? s : 0.f;
  }
  for (int j = 0; j < H2; j++) {
    float s = __bfloat162float(w[OFF_B2 + j]);
    for (int i = 0; i < H1; i++) s += __bfloat162float(w[OFF_W2 + j * H1 + i]) * h1[i];
    h2[j] = s > 0.f ? s : 0.f;
  }
  for (int j = 0; j < NO; j++) {
    float s = __bfloat162float(w[OFF_B3 + j]);
    for (int i = 0; i < H2; i++) s += __bfloat162float(w[OFF_W3 + j * H2 + i]) * h2[i];
    out[j] = s;
  }
}

}  // namespace pk
}  // namespace vs
