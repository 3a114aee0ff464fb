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
// `feat` (MLP_IN floats, raw features) and `s` (MLP_SCRATCH_FLOATS) are shared memory; `pk`
// is the inference buffer, normally the block's shared-memory copy of it.  The hidden layer
// runs on every thread of the group: P = nthr / MLP_H consecutive lanes share an output, each
// over MLP_H / P inputs, combined by shuffles (one-warp groups: two outputs per lane).
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
  float* out = s + 2 * MLP_H;
  for (int j = g.tid; j < MLP_H; j += g.nthr) {
    float z = b1[j];
#pragma unroll
    for (int c = 0; c < MLP_IN; ++c) z += __bfloat162float(W1[j * MLP_IN + c]) * ((feat[c] - mu[c]) * isd[c]);
    h1[j] = tanhf(z);
  }
  g.sync();
  // W2 is packed transposed (entry k * MLP_H + j = W2[j][k])
  const int P = g.nthr >= 2 * MLP_H ? (g.nthr / MLP_H > 8 ? 8 : g.nthr / MLP_H) : 1;
  const int KP = MLP_H / P;
  for (int t = g.tid; t < MLP_H * P; t += g.nthr) {
    const int j = t / P, p = t - j * P;
    float z = 0.f;
#pragma unroll 8
    for (int k = p * KP; k < (p + 1) * KP; ++k) z += __bfloat162float(W2[k * MLP_H + j]) * h1[k];
    // every lane of a warp is in this iteration when P > 1 (MLP_H * P = nthr)
    for (int o = P >> 1; o > 0; o >>= 1) z += __shfl_xor_sync(0xffffffffu, z, o);
    if (p == 0) h2[j] = tanhf(b2[j] + z);
  }
  g.sync();
  if (g.tid < 32) {
    float acc = 0.f;
    for (int j = g.tid; j < MLP_H; j += 32) acc += __bfloat162float(w3[j]) * h2[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (g.tid == 0) out[0] = acc + b3;
  }
  g.sync();
  return out[0];
}

}  // namespace rk
