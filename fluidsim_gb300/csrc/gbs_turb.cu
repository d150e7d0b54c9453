// Turbulence-model forcing added to the ns3d tendencies before projection
// and dealiasing (fluidsim/solvers/ns3d/solver.py:246-252, TurbModel.get_forcing
// fluidsim/base/turb_model/base.py:87-88).
//
// Pipeline per tendency evaluation (input: the stage state v_hat):
//   1. g_hat_{3i+j} = i k_j v_hat_i                   (9 spectral fields)
//   2. batched C2R -> physical gradients d_j u_i       (9 real fields)
//   3. pointwise model -> 6 symmetric stress fields    (xx, yy, zz, xy, xz, yz)
//        smagorinsky (turb_model/smagorinsky.py:56-110): 2 nu_T S_ij with
//          nu_T = C Delta^2 sqrt(2 S_ij S_ij);
//        learned closure: tau = MLP(g), 9 -> 64 -> 64 -> 6, tanh, BF16
//          weights, FP32 accumulation;
//   4. batched R2C                                     (6 spectral fields)
//   5. f_i = coef * i k_j t_hat_ij (coef 2 for smagorinsky as in the
//      reference's `2j * (...)`, -1 for the closure: -d_j tau_ij)
// The forcing (3 spectral fields) is read by the last pass of the step.
#include <cuda_bf16.h>

#include "gbs_internal.cuh"
#include "gbs_turb.h"
#include "gbs_mlp_mma.cuh"

namespace gbs {

// tau_ij -> component index of (xx, yy, zz, xy, xz, yz)
__constant__ int c_tau_index[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};

struct KGeo {
  int nx, ny, nz, nkx;
  double dkx, dky, dkz;
};

template <typename T>
__global__ void k_grad9(const cplx<T>* __restrict__ S, cplx<T>* __restrict__ G, KGeo g) {
  using C = cplx<T>;
  const int64_t nK = (int64_t)g.nz * g.ny * g.nkx;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nK;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int ix = (int)(i % g.nkx);
    const int64_t r = i / g.nkx;
    const int iy = (int)(r % g.ny), iz = (int)(r / g.ny);
    const T k[3] = {T(g.dkx * ix), T(g.dky * kadim(iy, g.ny)), T(g.dkz * kadim(iz, g.nz))};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const C v = S[i + c * nK];
#pragma unroll
      for (int j = 0; j < 3; ++j)  // 1j * K_j * v
        G[i + (3 * c + j) * nK] = mk<C>(-k[j] * v.y, k[j] * v.x);
    }
  }
}

// Smagorinsky stress 2 nu_T S_ij (stress_tensor.py:28-43, smagorinsky.py:63-88)
template <typename T>
__global__ void k_smagorinsky(const T* __restrict__ g, T* __restrict__ tau, int64_t n,
                              T C_nu_T) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    T d[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) d[c] = g[i + c * n];
    // d[3*i + j] = d_j u_i
    const T Sxx = d[0], Syy = d[4], Szz = d[8];
    const T Syx = T(0.5) * (d[1] + d[3]);
    const T Szx = T(0.5) * (d[2] + d[6]);
    const T Szy = T(0.5) * (d[5] + d[7]);
    const T norm = sqrt(Sxx * Sxx + Syy * Syy + Szz * Szz +
                        T(2) * (Syx * Syx + Szx * Szx + Szy * Szy));
    const T nu2 = T(2) * C_nu_T * norm;
    tau[i] = nu2 * Sxx;
    tau[i + n] = nu2 * Syy;
    tau[i + 2 * n] = nu2 * Szz;
    tau[i + 3 * n] = nu2 * Syx;
    tau[i + 4 * n] = nu2 * Szx;
    tau[i + 5 * n] = nu2 * Szy;
  }
}

// Pointwise MLP 9 -> 64 -> 64 -> 6 (tanh), BF16 weights, FP32 accumulation,
// on the tensor cores: each warp evaluates tiles of 16 points with
// mma.sync m16n8k16 (gbs_mlp_mma.cuh); activations as three BF16 terms
// (TERMS = 3) or one (TERMS = 1, the BF16 form).
template <typename T, int TERMS>
__global__ void __launch_bounds__(256, mlp_minb<TERMS>())
k_mlp_closure(const T* __restrict__ g, T* __restrict__ tau, int64_t n, MLPWeights w) {
  __shared__ MMAShared sm;
  mma_stage(sm, w);
  __syncthreads();
  mma_eval_all<TERMS, T, T>(sm, g, tau, n, n);
}

// f_i = coef * 1j * sum_j K_j t_hat_{ij}
template <typename T>
__global__ void k_div_stress(const cplx<T>* __restrict__ Tk, cplx<T>* __restrict__ F, KGeo g,
                             T coef, const cplx<T>* __restrict__ extra) {
  using C = cplx<T>;
  const int64_t nK = (int64_t)g.nz * g.ny * g.nkx;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nK;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int ix = (int)(i % g.nkx);
    const int64_t r = i / g.nkx;
    const int iy = (int)(r % g.ny), iz = (int)(r / g.ny);
    const T k[3] = {T(g.dkx * ix), T(g.dky * kadim(iy, g.ny)), T(g.dkz * kadim(iz, g.nz))};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      C acc = mk<C>(0, 0);
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const C t = Tk[i + c_tau_index[c][j] * nK];
        acc.x += k[j] * t.x;
        acc.y += k[j] * t.y;
      }
      C f = mk<C>(-coef * acc.y, coef * acc.x);
      if (extra) f = cadd(f, extra[i + c * nK]);
      F[i + c * nK] = f;
    }
  }
}

static int grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b < 152 * 16 ? b : 152 * 16);
}

template <typename T>
int turb_forcing(const TurbCtx& t, const void* S, void* out, const void* extra,
                 cudaStream_t st) {
  using C = cplx<T>;
  KGeo g{t.nx, t.ny, t.nz, t.nx / 2 + 1, t.dkx, t.dky, t.dkz};
  const int64_t nK = (int64_t)t.nz * t.ny * (t.nx / 2 + 1);
  const int64_t nX = (int64_t)t.nz * t.ny * t.nx;
  k_grad9<T><<<grid_for(nK), 256, 0, st>>>(static_cast<const C*>(S), static_cast<C*>(t.Gk), g);
  GBS_CHECK_LAUNCH();
  int rc = gbs_fft_c2r(t.plan9, t.Gk, t.Gx, 1, st);
  if (rc) return rc;
  if (t.type == kTurbSmagorinsky) {
    k_smagorinsky<T><<<grid_for(nX), 256, 0, st>>>(static_cast<const T*>(t.Gx),
                                                   static_cast<T*>(t.Tx), nX, T(t.C_nu_T));
  } else {
    int64_t nb = (nX + 127) / 128;  // 8 warps of 16 points
    if (nb > 152 * 8) nb = 152 * 8;
    if (t.type == kTurbMLPBF16)
      k_mlp_closure<T, 1><<<(int)nb, 256, 0, st>>>(static_cast<const T*>(t.Gx),
                                                  static_cast<T*>(t.Tx), nX, t.w);
    else
      k_mlp_closure<T, 3><<<(int)nb, 256, 0, st>>>(static_cast<const T*>(t.Gx),
                                                  static_cast<T*>(t.Tx), nX, t.w);
  }
  GBS_CHECK_LAUNCH();
  rc = gbs_fft_r2c(t.plan6, t.Tx, t.Tk, st);
  if (rc) return rc;
  const T coef = t.type == kTurbSmagorinsky ? T(2) : T(-1);
  k_div_stress<T><<<grid_for(nK), 256, 0, st>>>(static_cast<const C*>(t.Tk),
                                                static_cast<C*>(out), g, coef,
                                                static_cast<const C*>(extra));
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

template int turb_forcing<float>(const TurbCtx&, const void*, void*, const void*,
                                 cudaStream_t);
template int turb_forcing<double>(const TurbCtx&, const void*, void*, const void*,
                                  cudaStream_t);

}  // namespace gbs
