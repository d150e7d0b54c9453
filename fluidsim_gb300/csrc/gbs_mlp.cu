// Training and inference kernels of the learned subgrid-stress closure.
//
// Network: x = g * in_scale (9) -> h1 = tanh(W1 x + b1) (64)
//          -> h2 = tanh(W2 h1 + b2) (64) -> y = W3 h2 + b3 (6),
//          tau = y * out_scale.  Weights are read as BF16, arithmetic and
//          accumulation are FP32.  Loss: mean over samples and outputs of
//          (y - tau_target / out_scale)^2, plus pi_weight times the mean over
//          samples of (Pi(tau) - Pi(tau_target))^2 with the subgrid
//          dissipation Pi(tau) = tau_ij S_ij, S_ij = (d_j u_i + d_i u_j) / 2
//          (pointwise energy transfer to the unresolved scales).
//
// Data are structure-of-arrays fields: g[c * ld + i] (9 rows), tau[o * ld + i]
// (6 rows), so the gradient and stress fields of the LES / filtered DNS are
// used in place.  A minibatch is a list of point indices.
//
// Gradient: one thread per sample computes the forward pass and the
// back-propagated deltas and stores (x, h1, h2, dz1, dz2, dy) in a
// workspace; the weight gradients are then reduced over the batch in
// chunks (shared-memory tiles, fixed order, one partial row per block) and
// summed over blocks in a fixed order, so the result is deterministic.
#include <cuda_bf16.h>

#include "gbs_internal.cuh"
#include "gbs_turb.h"
#include "gbs_mlp_eval.cuh"
#include "gbs_mlp_mma.cuh"

namespace gbs {

constexpr int kNP = kH * kIn + kH + kH * kH + kH + kOut * kH + kOut;  // 5190
constexpr int kFeat = kIn + kH + kH + kH + kH + kOut;                 // per-sample rows
constexpr int kOffW1 = 0, kOffB1 = kH * kIn, kOffW2 = kOffB1 + kH;
constexpr int kOffB2 = kOffW2 + kH * kH, kOffW3 = kOffB2 + kH, kOffB3 = kOffW3 + kOut * kH;
// workspace rows (each of length B)
constexpr int kRX = 0, kRH1 = kIn, kRH2 = kRH1 + kH, kRZ1 = kRH2 + kH, kRZ2 = kRZ1 + kH,
              kRDY = kRZ2 + kH;
constexpr int kChunk = 2048;  // samples per block in the weight-gradient reduction
constexpr int kTile = 32;

// strain-rate component o (xx yy zz xy xz yz) of the gradient g[3 i + j],
// times the multiplicity of tau_o in tau_ij S_ij (1 on the diagonal, 2 off)
__device__ __forceinline__ void strain_weighted(const float* gr, float* s) {
  s[0] = gr[0];
  s[1] = gr[4];
  s[2] = gr[8];
  s[3] = gr[1] + gr[3];
  s[4] = gr[2] + gr[6];
  s[5] = gr[5] + gr[7];
}

__global__ void __launch_bounds__(256)
k_mlp_fwd_bwd(MLPWeights w, const float* __restrict__ g, const float* __restrict__ tau,
              int64_t ld, const int64_t* __restrict__ idx, int64_t B, float pi_weight,
              float* __restrict__ ws, float* __restrict__ loss) {
  __shared__ MLPShared sm;
  __shared__ float red[8];
  mlp_stage(sm, w);
  __syncthreads();
  float lsum = 0.f;
  const float inv = 2.f / (float)(B * kOut);
  const float invB = 1.f / (float)B;
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < B;
       b += (int64_t)gridDim.x * blockDim.x) {
    const int o = opaque_zero();  // keeps the weight reads inside the loop
    const int64_t i = idx[b];
    float x[kInPad], sw[kOut];
    {
      float gr[kIn];
#pragma unroll
      for (int c = 0; c < kIn; ++c) gr[c] = g[c * ld + i];
      strain_weighted(gr, sw);
#pragma unroll
      for (int c = 0; c < kIn; ++c) {
        x[c] = gr[c] * sm.sin[c];
        ws[(kRX + c) * B + b] = x[c];
      }
#pragma unroll
      for (int c = kIn; c < kInPad; ++c) x[c] = 0.f;
    }
    float h1[kH];
#pragma unroll
    for (int j = 0; j < kH; ++j) {
      float z = sm.b1[j + o];
#pragma unroll
      for (int q = 0; q < kInPad / 4; ++q) {
        const float4 wv = sm.W1[j * (kInPad / 4) + q + o];
        z = fmaf(wv.x, x[4 * q], z);
        z = fmaf(wv.y, x[4 * q + 1], z);
        z = fmaf(wv.z, x[4 * q + 2], z);
        z = fmaf(wv.w, x[4 * q + 3], z);
      }
      h1[j] = tanhf(z);
      ws[(kRH1 + j) * B + b] = h1[j];
    }
    float4 ya = make_float4(sm.b3[0], sm.b3[1], sm.b3[2], sm.b3[3]);
    float4 yb = make_float4(sm.b3[4], sm.b3[5], 0.f, 0.f);
#pragma unroll 2
    for (int j = 0; j < kH; ++j) {
      float z = sm.b2[j + o];
#pragma unroll
      for (int q = 0; q < kH / 4; ++q) {
        const float4 wv = sm.W2[j * (kH / 4) + q + o];
        z = fmaf(wv.x, h1[4 * q], z);
        z = fmaf(wv.y, h1[4 * q + 1], z);
        z = fmaf(wv.z, h1[4 * q + 2], z);
        z = fmaf(wv.w, h1[4 * q + 3], z);
      }
      const float h2 = tanhf(z);
      ws[(kRH2 + j) * B + b] = h2;
      ya = fma4(h2, sm.W3t[2 * j + o], ya);
      yb = fma4(h2, sm.W3t[2 * j + 1 + o], yb);
    }
    const float y[kOut] = {ya.x, ya.y, ya.z, ya.w, yb.x, yb.y};
    float dy[kOut];
    float dpi = 0.f;  // Pi(tau) - Pi(tau_target)
#pragma unroll
    for (int q = 0; q < kOut; ++q) {
      const float t = tau[q * ld + i];
      const float d = y[q] - t / sm.sout[q];
      lsum = fmaf(d, d, lsum);
      dy[q] = inv * d;
      dpi = fmaf(sw[q], fmaf(y[q], sm.sout[q], -t), dpi);
    }
    // the loss accumulates per output: the Pi term is folded in with weight
    // kOut so that lsum / (B kOut) is the total loss
    lsum = fmaf(pi_weight * (float)kOut * dpi, dpi, lsum);
    const float cpi = 2.f * pi_weight * invB * dpi;
#pragma unroll
    for (int q = 0; q < kOut; ++q) {
      dy[q] = fmaf(cpi * sw[q], sm.sout[q], dy[q]);
      ws[(kRDY + q) * B + b] = dy[q];
    }
    // dh1 = W2^T dz2, dz2 = (W3^T dy) * (1 - h2^2); h1 is reused as dh1
#pragma unroll
    for (int c = 0; c < kH; ++c) h1[c] = 0.f;
#pragma unroll 2
    for (int j = 0; j < kH; ++j) {
      const float4 wa = sm.W3t[2 * j + o], wb = sm.W3t[2 * j + 1 + o];
      float dh2 = 0.f;
      dh2 = fmaf(wa.x, dy[0], dh2);
      dh2 = fmaf(wa.y, dy[1], dh2);
      dh2 = fmaf(wa.z, dy[2], dh2);
      dh2 = fmaf(wa.w, dy[3], dh2);
      dh2 = fmaf(wb.x, dy[4], dh2);
      dh2 = fmaf(wb.y, dy[5], dh2);
      const float h2 = ws[(kRH2 + j) * B + b];
      const float dz2 = dh2 * (1.f - h2 * h2);
      ws[(kRZ2 + j) * B + b] = dz2;
#pragma unroll
      for (int q = 0; q < kH / 4; ++q) {
        const float4 wv = sm.W2[j * (kH / 4) + q + o];
        h1[4 * q] = fmaf(wv.x, dz2, h1[4 * q]);
        h1[4 * q + 1] = fmaf(wv.y, dz2, h1[4 * q + 1]);
        h1[4 * q + 2] = fmaf(wv.z, dz2, h1[4 * q + 2]);
        h1[4 * q + 3] = fmaf(wv.w, dz2, h1[4 * q + 3]);
      }
    }
#pragma unroll
    for (int c = 0; c < kH; ++c) {
      const float a = ws[(kRH1 + c) * B + b];
      ws[(kRZ1 + c) * B + b] = h1[c] * (1.f - a * a);
    }
  }
  // block reduction of the loss (fixed order inside the block)
  for (int q = 16; q; q >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, q);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = lsum;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.f;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
    atomicAdd(loss, s / (float)(B * kOut));
  }
}

// parameter p -> (row a of the left operand, row c of the right operand) of
// the outer-product sum  sum_b left[a][b] * right[c][b]  (right row -1: 1)
__device__ __forceinline__ void param_rows(int p, int& a, int& c) {
  if (p < kOffB1) { a = kRZ1 + p / kIn; c = kRX + p % kIn; }
  else if (p < kOffW2) { a = kRZ1 + (p - kOffB1); c = -1; }
  else if (p < kOffB2) { const int q = p - kOffW2; a = kRZ2 + q / kH; c = kRH1 + q % kH; }
  else if (p < kOffW3) { a = kRZ2 + (p - kOffB2); c = -1; }
  else if (p < kOffB3) { const int q = p - kOffW3; a = kRDY + q / kH; c = kRH2 + q % kH; }
  else { a = kRDY + (p - kOffB3); c = -1; }
}

__global__ void __launch_bounds__(256)
k_mlp_wgrad(const float* __restrict__ ws, int64_t B, float* __restrict__ partial) {
  __shared__ float tile[kFeat][kTile + 1];
  constexpr int PPT = (kNP + 255) / 256;
  float acc[PPT];
  int ra[PPT], rc[PPT];
#pragma unroll
  for (int k = 0; k < PPT; ++k) {
    acc[k] = 0.f;
    const int p = threadIdx.x + k * 256;
    if (p < kNP) param_rows(p, ra[k], rc[k]);
    else { ra[k] = 0; rc[k] = -1; }
  }
  const int64_t b0 = (int64_t)blockIdx.x * kChunk;
  const int64_t b1 = b0 + kChunk < B ? b0 + kChunk : B;
  for (int64_t t0 = b0; t0 < b1; t0 += kTile) {
    __syncthreads();
    for (int e = threadIdx.x; e < kFeat * kTile; e += blockDim.x) {
      const int r = e / kTile, s = e % kTile;
      tile[r][s] = t0 + s < b1 ? ws[r * B + t0 + s] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
      if (threadIdx.x + k * 256 >= kNP) continue;
      float sacc = 0.f;
      if (rc[k] < 0) {
        for (int s = 0; s < kTile; ++s) sacc += tile[ra[k]][s];
      } else {
        for (int s = 0; s < kTile; ++s) sacc = fmaf(tile[ra[k]][s], tile[rc[k]][s], sacc);
      }
      acc[k] += sacc;
    }
  }
#pragma unroll
  for (int k = 0; k < PPT; ++k) {
    const int p = threadIdx.x + k * 256;
    if (p < kNP) partial[(int64_t)blockIdx.x * kNP + p] = acc[k];
  }
}

__global__ void k_mlp_sum_partials(const float* __restrict__ partial, int nblocks,
                                   float* __restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kNP) return;
  float s = 0.f;
  for (int b = 0; b < nblocks; ++b) s += partial[(int64_t)b * kNP + p];
  grad[p] = s;
}

// Adam on the FP32 master weights, then the BF16 copies of W1, W2, W3.
__global__ void k_adam(float* __restrict__ master, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ grad, float lr, float beta1, float beta2,
                       float eps, float bc1, float bc2, __nv_bfloat16* W1, __nv_bfloat16* W2,
                       __nv_bfloat16* W3) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kNP) return;
  const float gr = grad[p];
  const float mm = beta1 * m[p] + (1.f - beta1) * gr;
  const float vv = beta2 * v[p] + (1.f - beta2) * gr * gr;
  m[p] = mm;
  v[p] = vv;
  const float w = master[p] - lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
  master[p] = w;
  if (p < kOffB1) W1[p - kOffW1] = __float2bfloat16(w);
  else if (p >= kOffW2 && p < kOffB2) W2[p - kOffW2] = __float2bfloat16(w);
  else if (p >= kOffW3 && p < kOffB3) W3[p - kOffW3] = __float2bfloat16(w);
}

// inference on SoA fields (float): tensor-core tiles of 16 points per warp
// (gbs_mlp_mma.cuh)
__global__ void __launch_bounds__(256)
k_mlp_forward(MLPWeights w, const float* __restrict__ g, int64_t ld, float* __restrict__ tau,
              int64_t n) {
  __shared__ MMAShared sm;
  mma_stage(sm, w);
  __syncthreads();
  mma_eval_all<float, float>(sm, g, tau, ld, n);
}

static MLPWeights to_w(const gbs_mlp_weights* p) {
  MLPWeights w;
  w.W1 = static_cast<const __nv_bfloat16*>(p->W1);
  w.W2 = static_cast<const __nv_bfloat16*>(p->W2);
  w.W3 = static_cast<const __nv_bfloat16*>(p->W3);
  w.b1 = p->b1;
  w.b2 = p->b2;
  w.b3 = p->b3;
  w.in_scale = p->in_scale;
  w.out_scale = p->out_scale;
  return w;
}

}  // namespace gbs

extern "C" {

int64_t gbs_mlp_grad_workspace(int64_t batch) {
  const int64_t nb = (batch + gbs::kChunk - 1) / gbs::kChunk;
  return (int64_t)sizeof(float) * (gbs::kFeat * batch + nb * gbs::kNP);
}

int gbs_mlp_forward(const gbs_mlp_weights* w, const float* g, int64_t ld, float* tau,
                    int64_t n, void* stream) {
  gbs::clear_error();
  if (!w || !g || !tau || n < 0 || ld < n) {
    gbs::set_error("gbs_mlp_forward: invalid argument");
    return GBS_EINVAL;
  }
  if (n == 0) return GBS_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int64_t nb = (n + 127) / 128;  // 8 warps of 16 points
  if (nb > 152 * 8) nb = 152 * 8;
  gbs::k_mlp_forward<<<(int)nb, 256, 0, st>>>(gbs::to_w(w), g, ld, tau, n);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

int gbs_mlp_grad(const gbs_mlp_weights* w, const float* g, const float* tau, int64_t ld,
                 const int64_t* idx, int64_t batch, double pi_weight, void* workspace,
                 float* grad, float* loss, void* stream) {
  gbs::clear_error();
  if (!w || !g || !tau || !idx || batch < 1 || !workspace || !grad || !loss ||
      !(pi_weight >= 0.0)) {
    gbs::set_error("gbs_mlp_grad: invalid argument");
    return GBS_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  float* ws = static_cast<float*>(workspace);
  const int nb = (int)((batch + gbs::kChunk - 1) / gbs::kChunk);
  float* partial = ws + (int64_t)gbs::kFeat * batch;
  GBS_CUDA_TRY(cudaMemsetAsync(loss, 0, sizeof(float), st));
  int64_t g1 = (batch + 255) / 256;
  if (g1 > 152 * 8) g1 = 152 * 8;
  gbs::k_mlp_fwd_bwd<<<(int)g1, 256, 0, st>>>(gbs::to_w(w), g, tau, ld, idx, batch,
                                          (float)pi_weight, ws, loss);
  GBS_CHECK_LAUNCH();
  gbs::k_mlp_wgrad<<<nb, 256, 0, st>>>(ws, batch, partial);
  GBS_CHECK_LAUNCH();
  gbs::k_mlp_sum_partials<<<(gbs::kNP + 255) / 256, 256, 0, st>>>(partial, nb, grad);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

int gbs_mlp_adam(float* master, float* m, float* v, const float* grad, int64_t step,
                 double lr, double beta1, double beta2, double eps,
                 const gbs_mlp_weights* w_bf16, void* stream) {
  gbs::clear_error();
  if (!master || !m || !v || !grad || step < 1 || !w_bf16) {
    gbs::set_error("gbs_mlp_adam: invalid argument");
    return GBS_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const float bc1 = (float)(1.0 - pow(beta1, (double)step));
  const float bc2 = (float)(1.0 - pow(beta2, (double)step));
  gbs::k_adam<<<(gbs::kNP + 255) / 256, 256, 0, st>>>(
      master, m, v, grad, (float)lr, (float)beta1, (float)beta2, (float)eps, bc1, bc2,
      (__nv_bfloat16*)w_bf16->W1, (__nv_bfloat16*)w_bf16->W2, (__nv_bfloat16*)w_bf16->W3);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

}  // extern "C"
