// Tensor-core evaluation of the closure network 9 -> 64 -> 64 -> 6 (tanh)
// for the inference kernels (the in-solver closure and gbs_mlp_forward).
//
// One warp evaluates 16 points at a time with mma.sync m16n8k16 (BF16
// operands, FP32 accumulation):
//   layer 1: [16 points x 16 inputs (9, zero padded)] x W1^T -> 64 (8 n-tiles)
//   layer 2: [16 x 64] x W2^T -> 64 (8 n-tiles x 4 k-tiles)
//   layer 3: [16 x 64] x W3^T -> 8 (6 outputs, zero padded; 4 k-tiles)
// The weights are BF16 and enter exactly.  The activations (inputs scaled by
// in_scale, then tanh outputs) are FP32 values carried as the sum of three
// BF16 terms a = a0 + a1 + a2 (a0 = bf16(a), a1 = bf16(a - a0), a2 =
// bf16(a - a0 - a1)), so each layer is three MMAs per tile whose FP32 sum
// equals the FP32 product to within the FP32 accumulation error; with the
// tanh below the result matches the FP32 evaluation to ~1e-7 relative.
//
// Fragment layouts (PTX ISA, mma.m16n8k16 .bf16, g = lane / 4, q = lane % 4):
//   A (row-major 16 x 16): a0 = (g, 2q..2q+1), a1 = (g+8, 2q..), a2 = (g,
//   2q+8..), a3 = (g+8, 2q+8..); B (16 x 8, "col"): b0 = (k 2q..2q+1, n g),
//   b1 = (k 2q+8.., n g); C/D: c0,c1 = (g, 2q / 2q+1), c2,c3 = (g+8, ...).
// The C fragments of n-tiles 2t and 2t+1 of one layer are the A fragment of
// k-tile t of the next, so activations stay in registers; layer 2's n-tiles
// are produced in pairs and consumed at once by layer 3.
//
// Shared memory holds the weights as BF16 with row strides of 24 (W1) and
// 72 (W2, W3) elements: the B-fragment loads (32 bits at row n0 + g, column
// k0 + 2q) then fall in 32 distinct banks.
//
// TERMS = 1 is the BF16 form: each activation enters as one BF16 value
// (BF16 operands, FP32 accumulation, the tensor-core precision of mixed-
// precision inference) and tanh is the hardware tanh.approx.f32; a third of
// the MMAs, no splitting, one MUFU operation per tanh instead of two.
// Relative error ~3e-3 against the FP32 evaluation.
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

#include "gbs_turb.h"

// CTAs of 256 threads per SM the inference kernels are compiled for (3 fits
// 80 registers but spills, and measured slower: 0.297 against 0.290 ms for
// 2.1 M points)
#ifndef GBS_MLP_MINB
#define GBS_MLP_MINB 2
#endif
// the same for the BF16 form (TERMS = 1): 4 (64 registers, no spill; 2.1 M
// points 0.109 ms, 0.112 with 3)
#ifndef GBS_MLP_MINB_BF16
#define GBS_MLP_MINB_BF16 4
#endif
template <int TERMS> constexpr int mlp_minb() { return TERMS == 1 ? GBS_MLP_MINB_BF16 : GBS_MLP_MINB; }

namespace gbs {

constexpr int kW1S = 24, kW2S = 72, kOutP = 8;

struct MMAShared {
  __nv_bfloat16 W1[kH * kW1S];
  __nv_bfloat16 W2[kH * kW2S];
  __nv_bfloat16 W3[kOutP * kW2S];
  float b1[kH], b2[kH], b3[kOutP], sin[16], sout[kOutP];
};

// Every thread of the CTA calls it; a __syncthreads() must follow.
__device__ __forceinline__ void mma_stage(MMAShared& s, const MLPWeights& w) {
  const __nv_bfloat16 z = __float2bfloat16(0.f);
  for (int i = threadIdx.x; i < kH * kW1S; i += blockDim.x) {
    const int j = i / kW1S, c = i % kW1S;
    s.W1[i] = c < kIn ? w.W1[j * kIn + c] : z;
  }
  for (int i = threadIdx.x; i < kH * kW2S; i += blockDim.x) {
    const int j = i / kW2S, c = i % kW2S;
    s.W2[i] = c < kH ? w.W2[j * kH + c] : z;
  }
  for (int i = threadIdx.x; i < kOutP * kW2S; i += blockDim.x) {
    const int o = i / kW2S, c = i % kW2S;
    s.W3[i] = (o < kOut && c < kH) ? w.W3[o * kH + c] : z;
  }
  for (int i = threadIdx.x; i < kH; i += blockDim.x) {
    s.b1[i] = w.b1[i];
    s.b2[i] = w.b2[i];
  }
  if (threadIdx.x < kOutP) {
    s.b3[threadIdx.x] = threadIdx.x < kOut ? w.b3[threadIdx.x] : 0.f;
    s.sout[threadIdx.x] = threadIdx.x < kOut ? w.out_scale[threadIdx.x] : 0.f;
  }
  if (threadIdx.x < 16) s.sin[threadIdx.x] = threadIdx.x < kIn ? w.in_scale[threadIdx.x] : 0.f;
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Two FP32 values (lower column first) -> three packed BF16 pairs whose sums
// give back the values: p[0] + p[1] + p[2].
__device__ __forceinline__ void split3(float x, float y, uint32_t& p0, uint32_t& p1,
                                       uint32_t& p2) {
  const __nv_bfloat162 h0 = __floats2bfloat162_rn(x, y);
  const float2 f0 = __bfloat1622float2(h0);
  const float rx = x - f0.x, ry = y - f0.y;
  const __nv_bfloat162 h1 = __floats2bfloat162_rn(rx, ry);
  const float2 f1 = __bfloat1622float2(h1);
  const __nv_bfloat162 h2 = __floats2bfloat162_rn(rx - f1.x, ry - f1.y);
  p0 = *reinterpret_cast<const uint32_t*>(&h0);
  p1 = *reinterpret_cast<const uint32_t*>(&h1);
  p2 = *reinterpret_cast<const uint32_t*>(&h2);
}

// tanh x = 1 - 2 / (exp(2x) + 1) with the hardware exponential and divide
// intrinsics: absolute error ~1e-7 over the whole line (the activations feed
// linear layers, where absolute errors are what count), +-1 in the limits.
__device__ __forceinline__ float tanh_act(float x) {
  return 1.f - __fdividef(2.f, __expf(2.f * x) + 1.f);
}

// TERMS = 3: split3; TERMS = 1: one BF16 pair in p0 (p1, p2 untouched).
template <int TERMS>
__device__ __forceinline__ void split_t(float x, float y, uint32_t& p0, uint32_t& p1,
                                        uint32_t& p2) {
  if constexpr (TERMS == 3) {
    split3(x, y, p0, p1, p2);
  } else {
    const __nv_bfloat162 h0 = __floats2bfloat162_rn(x, y);
    p0 = *reinterpret_cast<const uint32_t*>(&h0);
  }
}

// TERMS = 3: tanh_act; TERMS = 1: the hardware approximation (MUFU.TANH,
// relative error ~2^-11, below the BF16 rounding of its result).
template <int TERMS>
__device__ __forceinline__ float act_t(float x) {
  if constexpr (TERMS == 3) {
    return tanh_act(x);
  } else {
    float r;
    asm("tanh.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }
}

__device__ __forceinline__ uint32_t ld_b32(const __nv_bfloat16* p) {
  return *reinterpret_cast<const uint32_t*>(p);
}

// The network on the 16 points p0 .. p0 + 15 (< n) of SoA fields:
// input c of point i at g[i + c * ld], output o at tau[i + o * ld].
template <int TERMS, typename TI, typename TO>
__device__ __forceinline__ void mma_eval16(const MMAShared& s, const TI* __restrict__ g,
                                           TO* __restrict__ tau, int64_t ld, int64_t p0,
                                           int64_t n) {
  const int lane = threadIdx.x & 31;
  const int gq = lane >> 2, q = lane & 3;
  const int64_t ra = p0 + gq, rb = p0 + gq + 8;
  const int64_t la = ra < n ? ra : n - 1, lb = rb < n ? rb : n - 1;

  // layer 1 input: x = g * in_scale at columns 2q, 2q+1, 2q+8, 2q+9
  uint32_t A[3][4];
  {
    float x[2][4];
    const int cols[4] = {2 * q, 2 * q + 1, 2 * q + 8, 2 * q + 9};
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int c = cols[u];
      const bool ok = c < kIn;
      x[0][u] = ok ? (float)g[la + c * ld] * s.sin[c] : 0.f;
      x[1][u] = ok ? (float)g[lb + c * ld] * s.sin[c] : 0.f;
    }
    split_t<TERMS>(x[0][0], x[0][1], A[0][0], A[1][0], A[2][0]);
    split_t<TERMS>(x[1][0], x[1][1], A[0][1], A[1][1], A[2][1]);
    split_t<TERMS>(x[0][2], x[0][3], A[0][2], A[1][2], A[2][2]);
    split_t<TERMS>(x[1][2], x[1][3], A[0][3], A[1][3], A[2][3]);
  }

  // layer 1 -> h1 as the A fragments of layer 2 (3 terms x 4 k-tiles)
  uint32_t H[3][4][4];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    float c[2][4];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int nt = 2 * t + h;
      const float bx = s.b1[8 * nt + 2 * q], by = s.b1[8 * nt + 2 * q + 1];
      c[h][0] = bx;
      c[h][1] = by;
      c[h][2] = bx;
      c[h][3] = by;
      const __nv_bfloat16* wr = s.W1 + (8 * nt + gq) * kW1S + 2 * q;
      const uint32_t b0 = ld_b32(wr), b1 = ld_b32(wr + 8);
#pragma unroll
      for (int p = 0; p < TERMS; ++p) mma_bf16(c[h], A[p], b0, b1);
#pragma unroll
      for (int e = 0; e < 4; ++e) c[h][e] = act_t<TERMS>(c[h][e]);
    }
    split_t<TERMS>(c[0][0], c[0][1], H[0][t][0], H[1][t][0], H[2][t][0]);
    split_t<TERMS>(c[0][2], c[0][3], H[0][t][1], H[1][t][1], H[2][t][1]);
    split_t<TERMS>(c[1][0], c[1][1], H[0][t][2], H[1][t][2], H[2][t][2]);
    split_t<TERMS>(c[1][2], c[1][3], H[0][t][3], H[1][t][3], H[2][t][3]);
  }

  // layer 2, two n-tiles at a time, each pair feeding k-tile t of layer 3
  float y[4] = {s.b3[2 * q], s.b3[2 * q + 1], s.b3[2 * q], s.b3[2 * q + 1]};
#pragma unroll 1
  for (int t = 0; t < 4; ++t) {
    float c[2][4];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int nt = 2 * t + h;
      const float bx = s.b2[8 * nt + 2 * q], by = s.b2[8 * nt + 2 * q + 1];
      c[h][0] = bx;
      c[h][1] = by;
      c[h][2] = bx;
      c[h][3] = by;
      const __nv_bfloat16* wr = s.W2 + (8 * nt + gq) * kW2S + 2 * q;
#pragma unroll
      for (int kt = 0; kt < 4; ++kt) {
        const uint32_t b0 = ld_b32(wr + 16 * kt), b1 = ld_b32(wr + 16 * kt + 8);
#pragma unroll
        for (int p = 0; p < TERMS; ++p) mma_bf16(c[h], H[p][kt], b0, b1);
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) c[h][e] = act_t<TERMS>(c[h][e]);
    }
    uint32_t A3[3][4];
    split_t<TERMS>(c[0][0], c[0][1], A3[0][0], A3[1][0], A3[2][0]);
    split_t<TERMS>(c[0][2], c[0][3], A3[0][1], A3[1][1], A3[2][1]);
    split_t<TERMS>(c[1][0], c[1][1], A3[0][2], A3[1][2], A3[2][2]);
    split_t<TERMS>(c[1][2], c[1][3], A3[0][3], A3[1][3], A3[2][3]);
    const __nv_bfloat16* wr = s.W3 + gq * kW2S + 16 * t + 2 * q;
    const uint32_t b0 = ld_b32(wr), b1 = ld_b32(wr + 8);
#pragma unroll
    for (int p = 0; p < TERMS; ++p) mma_bf16(y, A3[p], b0, b1);
  }

  // outputs 2q, 2q+1 of points ra (y[0], y[1]) and rb (y[2], y[3])
  if (q < 3) {
    const int o = 2 * q;
    if (ra < n) {
      tau[ra + o * ld] = TO(y[0] * s.sout[o]);
      tau[ra + (o + 1) * ld] = TO(y[1] * s.sout[o + 1]);
    }
    if (rb < n) {
      tau[rb + o * ld] = TO(y[2] * s.sout[o]);
      tau[rb + (o + 1) * ld] = TO(y[3] * s.sout[o + 1]);
    }
  }
}

// Grid-stride loop of warps over tiles of 16 points.
template <int TERMS, typename TI, typename TO>
__device__ __forceinline__ void mma_eval_all(const MMAShared& s, const TI* __restrict__ g,
                                             TO* __restrict__ tau, int64_t ld, int64_t n) {
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t w0 = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  for (int64_t t = w0; t * 16 < n; t += warps) mma_eval16<TERMS, TI, TO>(s, g, tau, ld, t * 16, n);
}

}  // namespace gbs
