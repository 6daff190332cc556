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

// class index -> strategy code of the expand kernels
__host__ __device__ inline int class_to_strategy(int c) { return c == 0 ? 1 : (c == 1 ? 2 : 3); }
__host__ __device__ inline int strategy_to_class(int s) { return s == 1 ? 0 : (s == 2 ? 1 : 2); }

struct HopFeatIn {
  double S, V, E, W, h, k_min, k_max;
  double new_bits_prev, active_prev, visited_bits, active_edges, pair_edges;
  double pairs_ok, shortest, both;
  const unsigned long long *hist;  // NHIST bins of log2(out-degree + 1) over active rows
};

__device__ __forceinline__ float lg(double x) { return (float)log2(1.0 + x); }

__device__ inline void hop_features(const HopFeatIn &in, float *f) {
  const double SV = in.S * in.V;
  f[0] = (float)(in.new_bits_prev / SV);
  f[1] = (float)(in.active_prev / in.V);
  f[2] = lg(in.active_prev) / 32.f;
  f[3] = (float)(in.visited_bits / SV);
  f[4] = lg(in.S) / 16.f;
  f[5] = (float)(in.W / 256.0);
  f[6] = lg(in.V) / 32.f;
  f[7] = lg(in.E) / 40.f;
  f[8] = (float)(in.E / in.V / 64.0);
  f[9] = (float)(in.h / 8.0);
  f[10] = (float)(in.active_edges / in.E);
  f[11] = lg(in.active_edges) / 40.f;
  f[12] = (float)in.pairs_ok;
  f[13] = (float)in.shortest;
  f[14] = (float)in.both;
  f[15] = lg(in.pair_edges) / 40.f;
  double tot = 0;
  for (int b = 0; b < NHIST; b++) tot += (double)in.hist[b];
  for (int b = 0; b < NHIST; b++) f[16 + b] = tot > 0 ? (float)((double)in.hist[b] / tot) : 0.f;
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
