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
// All products run on the tensor cores (mma.sync m16n8k16, BF16 operands,
// FP32 accumulation; FP32 values as three BF16 terms, gbs_mlp_mma.cuh).
// Gradient: each warp takes 16 samples through the forward pass and the
// back-propagated deltas and stores (x, h1, h2, dz1, dz2, dy) in a
// workspace; the weight and bias gradients are then reduced over the batch
// in chunks of kWChunk samples (one partial row per chunk) and summed over
// chunks in a fixed order, so the result is deterministic.
#include <cuda_bf16.h>

#include "gbs_internal.cuh"
#include "gbs_turb.h"
#include "gbs_mlp_mma.cuh"

namespace gbs {

constexpr int kNP = kH * kIn + kH + kH * kH + kH + kOut * kH + kOut;  // 5190
constexpr int kFeat = kIn + kH + kH + kH + kH + kOut;                 // per-sample rows
constexpr int kOffW1 = 0, kOffB1 = kH * kIn, kOffW2 = kOffB1 + kH;
constexpr int kOffB2 = kOffW2 + kH * kH, kOffW3 = kOffB2 + kH, kOffB3 = kOffW3 + kOut * kH;
// workspace rows (each of length B)
constexpr int kRX = 0, kRH1 = kIn, kRH2 = kRH1 + kH, kRZ1 = kRH2 + kH, kRZ2 = kRZ1 + kH,
              kRDY = kRZ2 + kH;

// Forward and backward of 16 samples per warp on the tensor cores
// (gbs_mlp_mma.cuh: BF16 weights, FP32 values as three BF16 terms, FP32
// accumulation).  Writes the workspace rows (x, h1, h2, dz1, dz2, dy) of
// every sample and adds the batch loss.  The backward products
// dh2 = W3^T dy and dh1 = W2^T dz2 use transposed BF16 copies of W3 and W2.
struct MMATrainShared {
  MMAShared f;
  __nv_bfloat16 W2t[kH * kW2S];  // W2t[c][j] = W2[j][c]
  __nv_bfloat16 W3t[kH * kOutP]; // W3t[j][o] = W3[o][j], o < 6 (else 0)
};

__global__ void __launch_bounds__(256, 2)
k_mlp_fwd_bwd_mma(MLPWeights w, const float* __restrict__ g, const float* __restrict__ tau,
                  int64_t ld, const int64_t* __restrict__ idx, int64_t B, float pi_weight,
                  float* __restrict__ ws, float* __restrict__ loss) {
  __shared__ MMATrainShared sm;
  __shared__ float red[8];
  mma_stage(sm.f, w);
  const __nv_bfloat16 zb = __float2bfloat16(0.f);
  for (int i = threadIdx.x; i < kH * kW2S; i += blockDim.x) {
    const int c = i / kW2S, j = i % kW2S;
    sm.W2t[i] = j < kH ? w.W2[j * kH + c] : zb;
  }
  for (int i = threadIdx.x; i < kH * kOutP; i += blockDim.x) {
    const int j = i / kOutP, o = i % kOutP;
    sm.W3t[i] = o < kOut ? w.W3[o * kH + j] : zb;
  }
  __syncthreads();
  const MMAShared& s = sm.f;
  const int lane = threadIdx.x & 31;
  const int gq = lane >> 2, q = lane & 3;
  const float inv = 2.f / (float)(B * kOut);
  const float invB = 1.f / (float)B;
  float lsum = 0.f;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t tt = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tt * 16 < B;
       tt += warps) {
    const int64_t ba = tt * 16 + gq, bb = ba + 8;  // the lane's two samples
    const bool va = ba < B, vb = bb < B;
    const int64_t ia = idx[va ? ba : B - 1], ib = idx[vb ? bb : B - 1];
    // layer 1 input (columns 2q, 2q+1, 2q+8, 2q+9), saved to the workspace
    uint32_t A[3][4];
    {
      float x[2][4];
      const int cols[4] = {2 * q, 2 * q + 1, 2 * q + 8, 2 * q + 9};
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int c = cols[u];
        const bool ok = c < kIn;
        x[0][u] = ok ? g[c * ld + ia] * s.sin[c] : 0.f;
        x[1][u] = ok ? g[c * ld + ib] * s.sin[c] : 0.f;
        if (ok && va) ws[(kRX + c) * B + ba] = x[0][u];
        if (ok && vb) ws[(kRX + c) * B + bb] = x[1][u];
      }
      split3(x[0][0], x[0][1], A[0][0], A[1][0], A[2][0]);
      split3(x[1][0], x[1][1], A[0][1], A[1][1], A[2][1]);
      split3(x[0][2], x[0][3], A[0][2], A[1][2], A[2][2]);
      split3(x[1][2], x[1][3], A[0][3], A[1][3], A[2][3]);
    }
    // layer 1 -> h1 (saved; kept as the three-term A fragments of layer 2)
    uint32_t H[3][4][4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      float c[2][4];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int nt = 2 * t + h;
        const int col = 8 * nt + 2 * q;
        c[h][0] = c[h][2] = s.b1[col];
        c[h][1] = c[h][3] = s.b1[col + 1];
        const __nv_bfloat16* wr = s.W1 + (8 * nt + gq) * kW1S + 2 * q;
        const uint32_t b0 = ld_b32(wr), b1 = ld_b32(wr + 8);
#pragma unroll
        for (int p = 0; p < 3; ++p) mma_bf16(c[h], A[p], b0, b1);
#pragma unroll
        for (int e = 0; e < 4; ++e) c[h][e] = tanh_act(c[h][e]);
        if (va) {
          ws[(kRH1 + col) * B + ba] = c[h][0];
          ws[(kRH1 + col + 1) * B + ba] = c[h][1];
        }
        if (vb) {
          ws[(kRH1 + col) * B + bb] = c[h][2];
          ws[(kRH1 + col + 1) * B + bb] = c[h][3];
        }
      }
      split3(c[0][0], c[0][1], H[0][t][0], H[1][t][0], H[2][t][0]);
      split3(c[0][2], c[0][3], H[0][t][1], H[1][t][1], H[2][t][1]);
      split3(c[1][0], c[1][1], H[0][t][2], H[1][t][2], H[2][t][2]);
      split3(c[1][2], c[1][3], H[0][t][3], H[1][t][3], H[2][t][3]);
    }
    // layer 2 -> h2 (kept and saved), layer 3 -> y
    float h2[8][4];
    float y[4] = {s.b3[2 * q], s.b3[2 * q + 1], s.b3[2 * q], s.b3[2 * q + 1]};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int nt = 2 * t + h;
        const int col = 8 * nt + 2 * q;
        float (&c)[4] = h2[nt];
        c[0] = c[2] = s.b2[col];
        c[1] = c[3] = s.b2[col + 1];
        const __nv_bfloat16* wr = s.W2 + (8 * nt + gq) * kW2S + 2 * q;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
          const uint32_t b0 = ld_b32(wr + 16 * kt), b1 = ld_b32(wr + 16 * kt + 8);
#pragma unroll
          for (int p = 0; p < 3; ++p) mma_bf16(c, H[p][kt], b0, b1);
        }
#pragma unroll
        for (int e = 0; e < 4; ++e) c[e] = tanh_act(c[e]);
        if (va) {
          ws[(kRH2 + col) * B + ba] = c[0];
          ws[(kRH2 + col + 1) * B + ba] = c[1];
        }
        if (vb) {
          ws[(kRH2 + col) * B + bb] = c[2];
          ws[(kRH2 + col + 1) * B + bb] = c[3];
        }
      }
      uint32_t A3[3][4];
      split3(h2[2 * t][0], h2[2 * t][1], A3[0][0], A3[1][0], A3[2][0]);
      split3(h2[2 * t][2], h2[2 * t][3], A3[0][1], A3[1][1], A3[2][1]);
      split3(h2[2 * t + 1][0], h2[2 * t + 1][1], A3[0][2], A3[1][2], A3[2][2]);
      split3(h2[2 * t + 1][2], h2[2 * t + 1][3], A3[0][3], A3[1][3], A3[2][3]);
      const __nv_bfloat16* wr = s.W3 + gq * kW2S + 16 * t + 2 * q;
      const uint32_t b0 = ld_b32(wr), b1 = ld_b32(wr + 8);
#pragma unroll
      for (int p = 0; p < 3; ++p) mma_bf16(y, A3[p], b0, b1);
    }
    // loss and dy: outputs o = 2q, 2q+1 of samples a (y[0..1]) and b (y[2..3])
    float dy[4] = {0.f, 0.f, 0.f, 0.f};
    {
      const bool oq = q < 3;
      float sw[2][2], tg[2][2], dp[2] = {0.f, 0.f};
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        const int64_t i = r == 0 ? ia : ib;
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int o = 2 * q + u;
          // strain-rate component o times its multiplicity in tau_ij S_ij
          float sv = 0.f;
          if (oq) {
            if (o < 3) sv = g[(4 * o) * ld + i];
            else if (o == 3) sv = g[1 * ld + i] + g[3 * ld + i];
            else if (o == 4) sv = g[2 * ld + i] + g[6 * ld + i];
            else sv = g[5 * ld + i] + g[7 * ld + i];
          }
          sw[r][u] = sv;
          tg[r][u] = oq ? tau[o * ld + i] : 0.f;
          dp[r] = fmaf(sv, fmaf(y[2 * r + u], s.sout[o], -tg[r][u]), dp[r]);
        }
      }
#pragma unroll
      for (int r = 0; r < 2; ++r) {  // Pi(tau) - Pi(tau_target) of the sample
        dp[r] += __shfl_xor_sync(0xffffffffu, dp[r], 1);
        dp[r] += __shfl_xor_sync(0xffffffffu, dp[r], 2);
      }
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        const bool vr = r == 0 ? va : vb;
        if (!vr || !oq) continue;
        const float cpi = 2.f * pi_weight * invB * dp[r];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int o = 2 * q + u;
          const float d = y[2 * r + u] - tg[r][u] / s.sout[o];
          lsum = fmaf(d, d, lsum);
          dy[2 * r + u] = fmaf(cpi * sw[r][u], s.sout[o], inv * d);
          ws[(kRDY + o) * B + (r == 0 ? ba : bb)] = dy[2 * r + u];
        }
        if (q == 0) lsum = fmaf(pi_weight * (float)kOut * dp[r], dp[r], lsum);
      }
    }
    // dh2 = W3^T dy (K = outputs, padded to 16), dz2 = dh2 (1 - h2^2)
    uint32_t D[3][4];
    split3(dy[0], dy[1], D[0][0], D[1][0], D[2][0]);
    split3(dy[2], dy[3], D[0][1], D[1][1], D[2][1]);
#pragma unroll
    for (int p = 0; p < 3; ++p) D[p][2] = D[p][3] = 0u;
    uint32_t Z[3][4][4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      float c[2][4];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int nt = 2 * t + h;
        const int col = 8 * nt + 2 * q;
        c[h][0] = c[h][1] = c[h][2] = c[h][3] = 0.f;
        const uint32_t b0 = ld_b32(sm.W3t + (8 * nt + gq) * kOutP + 2 * q);
#pragma unroll
        for (int p = 0; p < 3; ++p) mma_bf16(c[h], D[p], b0, 0u);
#pragma unroll
        for (int e = 0; e < 4; ++e) c[h][e] *= 1.f - h2[nt][e] * h2[nt][e];
        if (va) {
          ws[(kRZ2 + col) * B + ba] = c[h][0];
          ws[(kRZ2 + col + 1) * B + ba] = c[h][1];
        }
        if (vb) {
          ws[(kRZ2 + col) * B + bb] = c[h][2];
          ws[(kRZ2 + col + 1) * B + bb] = c[h][3];
        }
      }
      split3(c[0][0], c[0][1], Z[0][t][0], Z[1][t][0], Z[2][t][0]);
      split3(c[0][2], c[0][3], Z[0][t][1], Z[1][t][1], Z[2][t][1]);
      split3(c[1][0], c[1][1], Z[0][t][2], Z[1][t][2], Z[2][t][2]);
      split3(c[1][2], c[1][3], Z[0][t][3], Z[1][t][3], Z[2][t][3]);
    }
    // dh1 = W2^T dz2, dz1 = dh1 (1 - h1^2) (h1 read back from the workspace)
#pragma unroll 2
    for (int nt = 0; nt < 8; ++nt) {
      const int col = 8 * nt + 2 * q;
      float c[4] = {0.f, 0.f, 0.f, 0.f};
      const __nv_bfloat16* wr = sm.W2t + (8 * nt + gq) * kW2S + 2 * q;
#pragma unroll
      for (int kt = 0; kt < 4; ++kt) {
        const uint32_t b0 = ld_b32(wr + 16 * kt), b1 = ld_b32(wr + 16 * kt + 8);
#pragma unroll
        for (int p = 0; p < 3; ++p) mma_bf16(c, Z[p][kt], b0, b1);
      }
      if (va) {
        const float h0 = ws[(kRH1 + col) * B + ba], h1v = ws[(kRH1 + col + 1) * B + ba];
        ws[(kRZ1 + col) * B + ba] = c[0] * (1.f - h0 * h0);
        ws[(kRZ1 + col + 1) * B + ba] = c[1] * (1.f - h1v * h1v);
      }
      if (vb) {
        const float h0 = ws[(kRH1 + col) * B + bb], h1v = ws[(kRH1 + col + 1) * B + bb];
        ws[(kRZ1 + col) * B + bb] = c[2] * (1.f - h0 * h0);
        ws[(kRZ1 + col + 1) * B + bb] = c[3] * (1.f - h1v * h1v);
      }
    }
  }
  for (int o = 16; o; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if (lane == 0) red[threadIdx.x >> 5] = lsum;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
    atomicAdd(loss, t / (float)(B * kOut));
  }
}

// Weight and bias gradients on the tensor cores: for a chunk of kWChunk
// samples, every output tile of 16 x 8 parameters is sum_b L[a][b] R[c][b]
// over the chunk with L the back-propagated rows (dz1, dz2, dy) and R the
// forward rows (x, h1, h2) of the workspace, plus a column of ones in R that
// gives the bias gradients.  Both operands are FP32 values split into three
// BF16 terms; the six products whose size exceeds 2^-24 of the leading one
// are accumulated in FP32 (a0 b0, a0 b1, a1 b0, a0 b2, a1 b1, a2 b0).  One
// partial row per chunk, summed over chunks in a fixed order: deterministic.
// (65 536-sample gradient: 0.429 ms with 512-sample chunks, 0.194 with 128
// (512 CTAs: latency of the operand loads hidden), 0.205 with 64)
#ifndef GBS_WCHUNK
#define GBS_WCHUNK 128
#endif
constexpr int kWChunk = GBS_WCHUNK;
// output tiles: dW2 (4 m-tiles x 9 n-tiles, n-tile 8 = bias), dW1 (4 x 2,
// column 9 = bias), dW3 (1 x 9, n-tile 8 = bias)
constexpr int kTilesW2 = 36, kTilesW1 = 8, kTilesW3 = 9;
constexpr int kWTiles = kTilesW2 + kTilesW1 + kTilesW3;

__device__ __forceinline__ void split3_1(float x, float& a, float& b, float& c) {
  a = __bfloat162float(__float2bfloat16_rn(x));
  const float r = x - a;
  b = __bfloat162float(__float2bfloat16_rn(r));
  c = r - b;
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&h);
}

__global__ void __launch_bounds__(256)
k_mlp_wgrad_mma(const float* __restrict__ ws, int64_t B, float* __restrict__ partial) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gq = lane >> 2, q = lane & 3;
  const int64_t b0 = (int64_t)blockIdx.x * kWChunk;
  const int64_t b1 = b0 + kWChunk < B ? b0 + kWChunk : B;
  for (int tile = warp; tile < kWTiles; tile += blockDim.x >> 5) {
    // rows of the left operand (m) and right operand (n) of this tile
    int lrow, nrowL, rrow, nrowR, mt, nt, ones_col;  // ones_col: column index of 1s
    if (tile < kTilesW2) {
      mt = tile / 9;
      nt = tile % 9;
      lrow = kRZ2 + 16 * mt;
      nrowL = 16;
      rrow = kRH1 + 8 * nt;
      nrowR = nt < 8 ? 8 : 0;
      ones_col = nt < 8 ? -1 : 0;
    } else if (tile < kTilesW2 + kTilesW1) {
      const int t = tile - kTilesW2;
      mt = t / 2;
      nt = t % 2;
      lrow = kRZ1 + 16 * mt;
      nrowL = 16;
      rrow = kRX + 8 * nt;
      nrowR = nt == 0 ? 8 : 1;  // inputs 0..7, then input 8
      ones_col = nt == 0 ? -1 : 1;
    } else {
      const int t = tile - kTilesW2 - kTilesW1;
      mt = 0;
      nt = t;
      lrow = kRDY;
      nrowL = kOut;
      rrow = kRH2 + 8 * nt;
      nrowR = nt < 8 ? 8 : 0;
      ones_col = nt < 8 ? -1 : 0;
    }
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 2
    for (int64_t k0 = b0; k0 < b1; k0 += 16) {
      // A (16 x 16): rows gq, gq + 8; samples k0 + 2q (+1), k0 + 2q + 8 (+1)
      uint32_t A[3][4];
#pragma unroll
      for (int h = 0; h < 2; ++h) {  // sample columns 2q.. and 2q+8..
        const int64_t kb = k0 + 2 * q + 8 * h;
#pragma unroll
        for (int rr = 0; rr < 2; ++rr) {  // rows gq and gq + 8
          const int m = gq + 8 * rr;
          float v0 = 0.f, v1 = 0.f;
          if (m < nrowL) {
            const float* row = ws + (int64_t)(lrow + m) * B;
            if (kb < b1) v0 = row[kb];
            if (kb + 1 < b1) v1 = row[kb + 1];
          }
          float a0, a1, a2, c0, c1, c2;
          split3_1(v0, a0, a1, a2);
          split3_1(v1, c0, c1, c2);
          A[0][2 * h + rr] = pack_bf16(a0, c0);
          A[1][2 * h + rr] = pack_bf16(a1, c1);
          A[2][2 * h + rr] = pack_bf16(a2, c2);
        }
      }
      // B (16 x 8): samples k0 + 2q (+1) and k0 + 2q + 8 (+1), column gq
      uint32_t Bf[3][2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int64_t kb = k0 + 2 * q + 8 * h;
        float v0 = 0.f, v1 = 0.f;
        if (gq < nrowR) {
          const float* row = ws + (int64_t)(rrow + gq) * B;
          if (kb < b1) v0 = row[kb];
          if (kb + 1 < b1) v1 = row[kb + 1];
        } else if (gq == ones_col) {
          v0 = kb < b1 ? 1.f : 0.f;
          v1 = kb + 1 < b1 ? 1.f : 0.f;
        }
        float a0, a1, a2, c0, c1, c2;
        split3_1(v0, a0, a1, a2);
        split3_1(v1, c0, c1, c2);
        Bf[0][h] = pack_bf16(a0, c0);
        Bf[1][h] = pack_bf16(a1, c1);
        Bf[2][h] = pack_bf16(a2, c2);
      }
      mma_bf16(acc, A[0], Bf[0][0], Bf[0][1]);
      mma_bf16(acc, A[0], Bf[1][0], Bf[1][1]);
      mma_bf16(acc, A[1], Bf[0][0], Bf[0][1]);
      mma_bf16(acc, A[0], Bf[2][0], Bf[2][1]);
      mma_bf16(acc, A[1], Bf[1][0], Bf[1][1]);
      mma_bf16(acc, A[2], Bf[0][0], Bf[0][1]);
    }
    // scatter the tile to parameter indices
    float* out = partial + (int64_t)blockIdx.x * kNP;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int m = gq + (e >= 2 ? 8 : 0);  // row of the tile
      const int n = 2 * q + (e & 1);        // column of the tile
      int pidx = -1;
      if (tile < kTilesW2) {
        const int j = 16 * mt + m;
        pidx = nt < 8 ? kOffW2 + j * kH + 8 * nt + n : (n == 0 ? kOffB2 + j : -1);
      } else if (tile < kTilesW2 + kTilesW1) {
        const int j = 16 * mt + m;
        const int c = 8 * nt + n;
        pidx = c < kIn ? kOffW1 + j * kIn + c : (c == kIn ? kOffB1 + j : -1);
      } else if (m < kOut) {
        pidx = nt < 8 ? kOffW3 + m * kH + 8 * nt + n : (n == 0 ? kOffB3 + m : -1);
      }
      if (pidx >= 0) out[pidx] = acc[e];
    }
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
// (gbs_mlp_mma.cuh), activations as three BF16 terms or one (BF16 form)
template <int TERMS>
__global__ void __launch_bounds__(256, mlp_minb<TERMS>())
k_mlp_forward(MLPWeights w, const float* __restrict__ g, int64_t ld, float* __restrict__ tau,
              int64_t n) {
  __shared__ MMAShared sm;
  mma_stage(sm, w);
  __syncthreads();
  mma_eval_all<TERMS, float, float>(sm, g, tau, ld, n);
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

template <int TERMS>
static int mlp_forward(const gbs_mlp_weights* w, const float* g, int64_t ld, float* tau,
                       int64_t n, void* stream, const char* name) {
  clear_error();
  if (!w || !g || !tau || n < 0 || ld < n) {
    set_error("%s: invalid argument", name);
    return GBS_EINVAL;
  }
  if (n == 0) return GBS_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int64_t nb = (n + 127) / 128;  // 8 warps of 16 points
  if (nb > 152 * 8) nb = 152 * 8;
  k_mlp_forward<TERMS><<<(int)nb, 256, 0, st>>>(to_w(w), g, ld, tau, n);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

}  // namespace gbs

extern "C" {

int64_t gbs_mlp_grad_workspace(int64_t batch) {
  const int64_t nb = (batch + gbs::kWChunk - 1) / gbs::kWChunk;
  return (int64_t)sizeof(float) * (gbs::kFeat * batch + nb * gbs::kNP);
}

int gbs_mlp_forward(const gbs_mlp_weights* w, const float* g, int64_t ld, float* tau,
                    int64_t n, void* stream) {
  return gbs::mlp_forward<3>(w, g, ld, tau, n, stream, "gbs_mlp_forward");
}

int gbs_mlp_forward_bf16(const gbs_mlp_weights* w, const float* g, int64_t ld, float* tau,
                         int64_t n, void* stream) {
  return gbs::mlp_forward<1>(w, g, ld, tau, n, stream, "gbs_mlp_forward_bf16");
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
  const int nb = (int)((batch + gbs::kWChunk - 1) / gbs::kWChunk);
  float* partial = ws + (int64_t)gbs::kFeat * batch;
  GBS_CUDA_TRY(cudaMemsetAsync(loss, 0, sizeof(float), st));
  int64_t g1 = (batch + 127) / 128;  // 8 warps of 16 samples
  if (g1 > 152 * 8) g1 = 152 * 8;
  gbs::k_mlp_fwd_bwd_mma<<<(int)g1, 256, 0, st>>>(gbs::to_w(w), g, tau, ld, idx, batch,
                                              (float)pi_weight, ws, loss);
  GBS_CHECK_LAUNCH();
  gbs::k_mlp_wgrad_mma<<<nb, 256, 0, st>>>(ws, batch, partial);
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
