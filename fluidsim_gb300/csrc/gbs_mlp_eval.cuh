// Pointwise evaluation of the closure network 9 -> 64 -> 64 -> 6 (tanh) for
// the inference kernels (the in-solver closure and gbs_mlp_forward).
//
// The BF16 weights are staged once per CTA in shared memory as float, laid
// out so that every weight read is a 16-byte broadcast load (all threads of
// a warp read the same address):
//   W1 rows padded from 9 to 12 inputs (3 float4 per hidden unit),
//   W2 row-major 64 x 64 (16 float4 per hidden unit),
//   W3 transposed to [hidden][8] (outputs 6 and 7 are zero; 2 float4).
// Arithmetic and accumulation are FP32, in the same order as the training
// kernel's forward pass (sum over inputs in increasing index).
#pragma once

#include <cuda_bf16.h>

#include "gbs_turb.h"

namespace gbs {

constexpr int kInPad = 12, kOutPad = 8;

struct MLPShared {
  float4 W1[kH * kInPad / 4];
  float4 W2[kH * kH / 4];
  float4 W3t[kH * kOutPad / 4];
  float b1[kH], b2[kH], b3[kOut], sin[kIn], sout[kOut];
};

// Every thread of the CTA calls it; a __syncthreads() must follow.
__device__ __forceinline__ void mlp_stage(MLPShared& s, const MLPWeights& w) {
  float* W1 = reinterpret_cast<float*>(s.W1);
  float* W2 = reinterpret_cast<float*>(s.W2);
  float* W3t = reinterpret_cast<float*>(s.W3t);
  for (int i = threadIdx.x; i < kH * kH; i += blockDim.x) W2[i] = __bfloat162float(w.W2[i]);
  for (int i = threadIdx.x; i < kH * kInPad; i += blockDim.x) {
    const int j = i / kInPad, c = i % kInPad;
    W1[i] = c < kIn ? __bfloat162float(w.W1[j * kIn + c]) : 0.f;
  }
  for (int i = threadIdx.x; i < kH * kOutPad; i += blockDim.x) {
    const int j = i / kOutPad, o = i % kOutPad;
    W3t[i] = o < kOut ? __bfloat162float(w.W3[o * kH + j]) : 0.f;
  }
  for (int i = threadIdx.x; i < kH; i += blockDim.x) {
    s.b1[i] = w.b1[i];
    s.b2[i] = w.b2[i];
  }
  if (threadIdx.x < kOut) {
    s.b3[threadIdx.x] = w.b3[threadIdx.x];
    s.sout[threadIdx.x] = w.out_scale[threadIdx.x];
  }
  if (threadIdx.x < kIn) s.sin[threadIdx.x] = w.in_scale[threadIdx.x];
}

__device__ __forceinline__ float4 fma4(float a, float4 w, float4 acc) {
  acc.x = fmaf(w.x, a, acc.x);
  acc.y = fmaf(w.y, a, acc.y);
  acc.z = fmaf(w.z, a, acc.z);
  acc.w = fmaf(w.w, a, acc.w);
  return acc;
}

// An offset of 0 that the compiler cannot see through.  Weight reads are
// indexed with it inside per-point loops: otherwise the compiler hoists the
// loop-invariant shared-memory reads out of the grid-stride loop into
// registers, which then spill (kilobytes of local memory per thread).
__device__ __forceinline__ int opaque_zero() {
  int o = 0;
  asm volatile("" : "+r"(o));
  return o;
}

// g: the 9 physical gradients of one point; tau: the 6 stresses.
__device__ __forceinline__ void mlp_eval(const MLPShared& s, const float (&g)[kIn],
                                         float (&tau)[kOut]) {
  const int o = opaque_zero();
  float x[kInPad];
#pragma unroll
  for (int c = 0; c < kIn; ++c) x[c] = g[c] * s.sin[c];
#pragma unroll
  for (int c = kIn; c < kInPad; ++c) x[c] = 0.f;
  float h1[kH];
#pragma unroll
  for (int j = 0; j < kH; ++j) {
    float z = s.b1[j + o];
#pragma unroll
    for (int q = 0; q < kInPad / 4; ++q) {
      const float4 w = s.W1[j * (kInPad / 4) + q + o];
      z = fmaf(w.x, x[4 * q], z);
      z = fmaf(w.y, x[4 * q + 1], z);
      z = fmaf(w.z, x[4 * q + 2], z);
      z = fmaf(w.w, x[4 * q + 3], z);
    }
    h1[j] = tanhf(z);
  }
  float4 ya = make_float4(s.b3[0], s.b3[1], s.b3[2], s.b3[3]);
  float4 yb = make_float4(s.b3[4], s.b3[5], 0.f, 0.f);
#pragma unroll 2
  for (int j = 0; j < kH; ++j) {
    float z = s.b2[j + o];
#pragma unroll
    for (int q = 0; q < kH / 4; ++q) {
      const float4 w = s.W2[j * (kH / 4) + q + o];
      z = fmaf(w.x, h1[4 * q], z);
      z = fmaf(w.y, h1[4 * q + 1], z);
      z = fmaf(w.z, h1[4 * q + 2], z);
      z = fmaf(w.w, h1[4 * q + 3], z);
    }
    const float h2 = tanhf(z);
    ya = fma4(h2, s.W3t[2 * j + o], ya);
    yb = fma4(h2, s.W3t[2 * j + 1 + o], yb);
  }
  tau[0] = ya.x * s.sout[0];
  tau[1] = ya.y * s.sout[1];
  tau[2] = ya.z * s.sout[2];
  tau[3] = ya.w * s.sout[3];
  tau[4] = yb.x * s.sout[4];
  tau[5] = yb.y * s.sout[5];
}

}  // namespace gbs
