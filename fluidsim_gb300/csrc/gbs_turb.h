// Turbulence-model forcing (gbs_turb.cu) used by the ns3d solver.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/gbspec.h"

namespace gbs {

constexpr int kIn = 9, kH = 64, kOut = 6;
constexpr int kTurbNone = 0, kTurbSmagorinsky = 1, kTurbMLP = 2, kTurbMLPBF16 = 3;

// Device pointers of the closure network (row-major W[out][in]).
struct MLPWeights {
  const __nv_bfloat16* W1;  // 64 x 9
  const __nv_bfloat16* W2;  // 64 x 64
  const __nv_bfloat16* W3;  // 6 x 64
  const float* b1;
  const float* b2;
  const float* b3;
  const float* in_scale;   // 9
  const float* out_scale;  // 6
};

struct TurbCtx {
  int type;
  int nx, ny, nz;
  double dkx, dky, dkz;
  double C_nu_T;         // smagorinsky: C Delta^2 sqrt(2)
  MLPWeights w;          // learned closure
  gbs_fft_plan* plan9;   // batched C2R of the 9 gradients
  gbs_fft_plan* plan6;   // batched R2C of the 6 stresses
  void* Gk;              // 9 spectral fields
  void* Gx;              // 9 physical fields
  void* Tx;              // 6 physical fields
  void* Tk;              // 6 spectral fields
};

// out = turbulence-model forcing of S (+ extra when not null)
template <typename T>
int turb_forcing(const TurbCtx& t, const void* S, void* out, const void* extra,
                 cudaStream_t st);

}  // namespace gbs
