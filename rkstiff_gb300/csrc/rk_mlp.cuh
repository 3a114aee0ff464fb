// Learned step-size controller: MLP layout and the in-kernel inference routine.
#pragma once

#include <cuda_bf16.h>

#include "rk_common.cuh"

namespace rk {

constexpr int MLP_IN = RK_MLP_IN;
constexpr int MLP_H = RK_MLP_H;
// offsets into the FP32 training parameter vector
constexpr int MP_W1 = 0;
constexpr int MP_B1 = MP_W1 + MLP_H * MLP_IN;
constexpr int MP_W2 = MP_B1 + MLP_H;
constexpr int MP_B2 = MP_W2 + MLP_H * MLP_H;
constexpr int MP_W3 = MP_B2 + MLP_H;
constexpr int MP_B3 = MP_W3 + MLP_H;
static_assert(MP_B3 + 1 == RK_MLP_NPARAM, "parameter layout");
// inference buffer: floats mu[IN], inv_sd[IN], b1[H], b2[H], b3, pad[3]; then bf16 weights
constexpr int PK_FLOATS = 2 * MLP_IN + 2 * MLP_H + 4;
static_assert(PK_FLOATS * 4 + (MLP_H * MLP_IN + MLP_H * MLP_H + MLP_H) * 2 == RK_MLP_PACK_BYTES, "pack layout");

// floats of per-group shared scratch the inference uses: features, two hidden layers, sum
constexpr int MLP_SCRATCH_FLOATS = MLP_IN + 2 * MLP_H + 40;

// y = MLP(feat) with bf16 weights and FP32 accumulation, evaluated by the whole group.
// `feat` (MLP_IN floats, raw features) and `s` (MLP_SCRATCH_FLOATS) are shared memory.
RK_DEV float mlp_infer(const Group& g, const unsigned char* __restrict__ pk, const float* feat, float* s) {
  const float* mu = reinterpret_cast<const float*>(pk);
  const float* isd = mu + MLP_IN;
  const float* b1 = isd + MLP_IN;
  const float* b2 = b1 + MLP_H;
  const float b3 = b2[MLP_H];
  const __nv_bfloat16* W1 = reinterpret_cast<const __nv_bfloat16*>(pk + PK_FLOATS * 4);
  const __nv_bfloat16* W2 = W1 + MLP_H * MLP_IN;
  const __nv_bfloat16* w3 = W2 + MLP_H * MLP_H;
  float* h1 = s;
  float* h2 = s + MLP_H;
  float* part = s + 2 * MLP_H;
  for (int j = g.tid; j < MLP_H; j += g.nthr) {
    float z = b1[j];
#pragma unroll
    for (int c = 0; c < MLP_IN; ++c) z += __bfloat162float(W1[j * MLP_IN + c]) * ((feat[c] - mu[c]) * isd[c]);
    h1[j] = tanhf(z);
  }
  g.sync();
  for (int j = g.tid; j < MLP_H; j += g.nthr) {
    float z = b2[j];
    // W2 is packed transposed (entry k * MLP_H + j = W2[j][k]): a warp reads 32 consecutive
    // weights per k
#pragma unroll 8
    for (int k = 0; k < MLP_H; ++k) z += __bfloat162float(W2[k * MLP_H + j]) * h1[k];
    h2[j] = tanhf(z);
  }
  g.sync();
  float acc = 0.f;
  for (int j = g.tid; j < MLP_H; j += g.nthr) acc += __bfloat162float(w3[j]) * h2[j];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  const int nw = g.nthr >> 5;
  if (nw > 1) {
    if ((g.tid & 31) == 0) part[g.tid >> 5] = acc;
    g.sync();
    acc = 0.f;
    for (int w = 0; w < nw; ++w) acc += part[w];
  }
  g.sync();
  return acc + b3;
}

}  // namespace rk
