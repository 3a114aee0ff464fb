// Training kernels of the learned step-size controller (forward, backward with gradient
// accumulation, Adam) and the packing of the BF16 inference buffer.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "rk_launch.h"
#include "rk_mlp.cuh"

namespace rk {

constexpr int MB = 64;  // samples per block (one thread per sample / per hidden unit)

// Forward (and, with T != nullptr, backward) of one block of MB samples.  Hidden units are
// mapped to threads, so every matrix product runs over shared-memory rows.
__global__ void __launch_bounds__(MB) mlp_kernel(const float* __restrict__ p, const float* __restrict__ X,
                                                 const float* __restrict__ T, int64_t batch, float norm,
                                                 float* __restrict__ Y, float* __restrict__ grad,
                                                 float* __restrict__ loss) {
  __shared__ float xs[MB][MLP_IN];
  __shared__ float ha[MB][MLP_H + 1];  // h1, then dz1
  __shared__ float hb[MB][MLP_H + 1];  // h2, then dz2
  __shared__ float dy[MB];
  __shared__ float red[MB];
  const int t = threadIdx.x;
  const int64_t base = (int64_t)blockIdx.x * MB;
  const int nv = (int)(batch - base < MB ? batch - base : MB);
  for (int e = t; e < MB * MLP_IN; e += MB) {
    const int i = e / MLP_IN, c = e % MLP_IN;
    xs[i][c] = i < nv ? X[(base + i) * MLP_IN + c] : 0.f;
  }
  __syncthreads();
  const int j = t;  // hidden unit of this thread
  for (int i = 0; i < MB; ++i) {
    float z = p[MP_B1 + j];
#pragma unroll
    for (int c = 0; c < MLP_IN; ++c) z += p[MP_W1 + j * MLP_IN + c] * xs[i][c];
    ha[i][j] = tanhf(z);
  }
  __syncthreads();
  for (int i = 0; i < MB; ++i) {
    float z = p[MP_B2 + j];
    for (int k = 0; k < MLP_H; ++k) z += p[MP_W2 + j * MLP_H + k] * ha[i][k];
    hb[i][j] = tanhf(z);
  }
  __syncthreads();
  {
    const int i = t;  // sample of this thread
    float y = p[MP_B3];
    for (int k = 0; k < MLP_H; ++k) y += p[MP_W3 + k] * hb[i][k];
    if (Y && i < nv) Y[base + i] = y;
    if (T) {
      const float r = i < nv ? y - T[base + i] : 0.f;
      dy[i] = 2.f * r / norm;
      red[i] = r * r / norm;
    }
  }
  if (!T) return;
  __syncthreads();
  // output layer
  float gw3 = 0.f;
  for (int i = 0; i < MB; ++i) gw3 += hb[i][j] * dy[i];
  atomicAdd(&grad[MP_W3 + j], gw3);
  if (t == 0) {
    float gb3 = 0.f, l = 0.f;
    for (int i = 0; i < MB; ++i) {
      gb3 += dy[i];
      l += red[i];
    }
    atomicAdd(&grad[MP_B3], gb3);
    atomicAdd(loss, l);
  }
  const float w3j = p[MP_W3 + j];
  for (int i = 0; i < MB; ++i) hb[i][j] = dy[i] * w3j * (1.f - hb[i][j] * hb[i][j]);  // dz2
  __syncthreads();
  // second layer: dW2[j][k] = sum_i dz2[i][j] h1[i][k]
  float gb2 = 0.f;
  for (int i = 0; i < MB; ++i) gb2 += hb[i][j];
  atomicAdd(&grad[MP_B2 + j], gb2);
  for (int k = 0; k < MLP_H; ++k) {
    float gk = 0.f;
    for (int i = 0; i < MB; ++i) gk += hb[i][j] * ha[i][k];
    atomicAdd(&grad[MP_W2 + j * MLP_H + k], gk);
  }
  __syncthreads();
  // back to the first layer: dz1[i][k] = (sum_j dz2[i][j] W2[j][k]) (1 - h1[i][k]^2), k = t
  {
    const int k = t;
    for (int i = 0; i < MB; ++i) {
      float dh = 0.f;
      for (int jj = 0; jj < MLP_H; ++jj) dh += hb[i][jj] * p[MP_W2 + jj * MLP_H + k];
      ha[i][k] = dh * (1.f - ha[i][k] * ha[i][k]);
    }
  }
  __syncthreads();
  float gb1 = 0.f;
  float gw1[MLP_IN];
#pragma unroll
  for (int c = 0; c < MLP_IN; ++c) gw1[c] = 0.f;
  for (int i = 0; i < MB; ++i) {
    const float d = ha[i][j];
    gb1 += d;
#pragma unroll
    for (int c = 0; c < MLP_IN; ++c) gw1[c] += d * xs[i][c];
  }
  atomicAdd(&grad[MP_B1 + j], gb1);
#pragma unroll
  for (int c = 0; c < MLP_IN; ++c) atomicAdd(&grad[MP_W1 + j * MLP_IN + c], gw1[c]);
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1,
                            float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void pack_kernel(const float* __restrict__ p, const float* __restrict__ mu, const float* __restrict__ sd,
                            unsigned char* __restrict__ out) {
  float* f = reinterpret_cast<float*>(out);
  __nv_bfloat16* w = reinterpret_cast<__nv_bfloat16*>(out + PK_FLOATS * 4);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < MLP_IN) {
    f[t] = mu[t];
    f[MLP_IN + t] = 1.f / sd[t];
  }
  if (t < MLP_H) {
    f[2 * MLP_IN + t] = p[MP_B1 + t];
    f[2 * MLP_IN + MLP_H + t] = p[MP_B2 + t];
  }
  if (t == 0) {
    f[2 * MLP_IN + 2 * MLP_H] = p[MP_B3];
    f[2 * MLP_IN + 2 * MLP_H + 1] = f[2 * MLP_IN + 2 * MLP_H + 2] = f[2 * MLP_IN + 2 * MLP_H + 3] = 0.f;
  }
  const int nw = MLP_H * MLP_IN + MLP_H * MLP_H + MLP_H;
  for (int e = t; e < nw; e += gridDim.x * blockDim.x) {
    float v;
    if (e < MLP_H * MLP_IN) v = p[MP_W1 + e];
    else if (e < MLP_H * MLP_IN + MLP_H * MLP_H) {
      // W2 transposed: entry k * MLP_H + j holds W2[j][k]
      const int q = e - MLP_H * MLP_IN, k = q / MLP_H, j = q % MLP_H;
      v = p[MP_W2 + j * MLP_H + k];
    }
    else v = p[MP_W3 + e - MLP_H * MLP_IN - MLP_H * MLP_H];
    w[e] = __float2bfloat16_rn(v);
  }
}

}  // namespace rk

using namespace rk;

extern "C" {

int rk_mlp_forward(const float* params, const float* X, int64_t batch, float* Y, void* stream) {
  if (!params || !X || !Y || batch < 0) {
    set_error("rk_mlp_forward: invalid argument");
    return RK_E_ARG;
  }
  if (batch == 0) return RK_OK;
  mlp_kernel<<<(unsigned)((batch + MB - 1) / MB), MB, 0, (cudaStream_t)stream>>>(params, X, nullptr, batch, 1.f, Y,
                                                                                 nullptr, nullptr);
  return cuda_check(cudaGetLastError(), "mlp forward launch");
}

int rk_mlp_grad(const float* params, const float* X, const float* T, int64_t batch, float norm, float* grad,
                float* loss, void* stream) {
  if (!params || !X || !T || !grad || !loss || batch < 0 || !(norm > 0.f)) {
    set_error("rk_mlp_grad: invalid argument");
    return RK_E_ARG;
  }
  if (batch == 0) return RK_OK;
  mlp_kernel<<<(unsigned)((batch + MB - 1) / MB), MB, 0, (cudaStream_t)stream>>>(params, X, T, batch, norm, nullptr,
                                                                                 grad, loss);
  return cuda_check(cudaGetLastError(), "mlp grad launch");
}

int rk_mlp_adam(float* params, const float* grad, float* m, float* v, int64_t step, float lr, float beta1,
                float beta2, float eps, void* stream) {
  if (!params || !grad || !m || !v || step < 1) {
    set_error("rk_mlp_adam: invalid argument");
    return RK_E_ARG;
  }
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  adam_kernel<<<(RK_MLP_NPARAM + 255) / 256, 256, 0, (cudaStream_t)stream>>>(params, grad, m, v, RK_MLP_NPARAM, lr,
                                                                             beta1, beta2, eps, c1, c2);
  return cuda_check(cudaGetLastError(), "mlp adam launch");
}

int rk_mlp_pack(const float* params, const float* mu, const float* sd, void* out, void* stream) {
  if (!params || !mu || !sd || !out) {
    set_error("rk_mlp_pack: invalid argument");
    return RK_E_ARG;
  }
  pack_kernel<<<8, 256, 0, (cudaStream_t)stream>>>(params, mu, sd, reinterpret_cast<unsigned char*>(out));
  return cuda_check(cudaGetLastError(), "mlp pack launch");
}

}  // extern "C"
