// Data preparation of the learned LES closure: spectral resampling with a
// box filter (filtered DNS -> LES grid), the six velocity products and the
// nine velocity-gradient fields.
#include "gbs_internal.cuh"

namespace gbs {

__device__ __forceinline__ double sinc(double x) { return x == 0.0 ? 1.0 : sin(x) / x; }

// out[f](kz, ky, kx) on (mz, my, mx/2+1) = G(k) in[f](same k on (nz, ny, nx/2+1))
// for |k_a| < m_a / 2 and k within the input grid, 0 otherwise.
// G(k) = prod_a sinc(k_a delta / 2) when delta > 0 (top-hat of width delta).
template <typename T>
__global__ void k_resample(const cplx<T>* __restrict__ in, cplx<T>* __restrict__ out, int nz,
                           int ny, int nx, int mz, int my, int mx, int nfields, double dkx,
                           double dky, double dkz, double delta) {
  using C = cplx<T>;
  const int nkx = nx / 2 + 1, mkx = mx / 2 + 1;
  const int64_t nKi = (int64_t)nz * ny * nkx, nKo = (int64_t)mz * my * mkx;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < nKo;
       o += (int64_t)gridDim.x * blockDim.x) {
    const int ix = (int)(o % mkx);
    const int64_t r = o / mkx;
    const int iy = (int)(r % my), iz = (int)(r / my);
    const int kx = ix, ky = kadim(iy, my), kz = kadim(iz, mz);
    bool ok = 2 * kx < mx && 2 * iabs(ky) < my && 2 * iabs(kz) < mz &&
              kx < nkx && 2 * iabs(ky) < ny && 2 * iabs(kz) < nz;
    if (ny == 1) ok = ok && ky == 0;
    if (nz == 1) ok = ok && kz == 0;
    T gain = T(0);
    int64_t i = 0;
    if (ok) {
      const int jy = ky >= 0 ? ky : ny + ky, jz = kz >= 0 ? kz : nz + kz;
      i = ((int64_t)jz * ny + jy) * nkx + kx;
      double gd = 1.0;
      if (delta > 0)
        gd = sinc(0.5 * delta * dkx * kx) * sinc(0.5 * delta * dky * ky) *
             sinc(0.5 * delta * dkz * kz);
      gain = T(gd);
    }
    for (int f = 0; f < nfields; ++f)
      out[o + f * nKo] = ok ? cscale(in[i + f * nKi], gain) : mk<C>(0, 0);
  }
}

// out = u_i u_j (xx, yy, zz, xy, xz, yz), or sub - u_i u_j when sub != null
template <typename T>
__global__ void k_products6(const T* __restrict__ u, T* __restrict__ out, int64_t n,
                            const T* __restrict__ sub) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T a = u[i], b = u[i + n], c = u[i + 2 * n];
    T p[6] = {a * a, b * b, c * c, a * b, a * c, b * c};
#pragma unroll
    for (int k = 0; k < 6; ++k) out[i + k * n] = sub ? sub[i + k * n] - p[k] : p[k];
  }
}

// G[3 i + j] = 1j K_j S_i, zero where the truncation |k_a| >= kc_a removes
template <typename T>
__global__ void k_gradients(const cplx<T>* __restrict__ S, cplx<T>* __restrict__ G, int nz,
                            int ny, int nx, double dkx, double dky, double dkz, int kcx,
                            int kcy, int kcz) {
  using C = cplx<T>;
  const int nkx = nx / 2 + 1;
  const int64_t nK = (int64_t)nz * ny * nkx;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nK;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int ix = (int)(i % nkx);
    const int64_t r = i / nkx;
    const int iy = (int)(r % ny), iz = (int)(r / ny);
    const int ky = kadim(iy, ny), kz = kadim(iz, nz);
    const bool rm = ix >= kcx || iabs(ky) >= kcy || iabs(kz) >= kcz;
    const T k[3] = {T(dkx * ix), T(dky * ky), T(dkz * kz)};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const C v = rm ? mk<C>(0, 0) : S[i + c * nK];
#pragma unroll
      for (int j = 0; j < 3; ++j) G[i + (3 * c + j) * nK] = mk<C>(-k[j] * v.y, k[j] * v.x);
    }
  }
}

static int nblocks(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b < 152 * 16 ? b : 152 * 16);
}

}  // namespace gbs

extern "C" {

int gbs_spectral_resample(const int64_t* shape_in, const int64_t* shape_out, int nfields,
                          const double* L, double delta, int dtype, const void* in, void* out,
                          void* stream) {
  gbs::clear_error();
  if (!shape_in || !shape_out || !L || !in || !out || nfields < 1 ||
      (dtype != GBS_F32 && dtype != GBS_F64) || shape_in[2] % 2 || shape_out[2] % 2) {
    gbs::set_error("gbs_spectral_resample: invalid argument");
    return GBS_EINVAL;
  }
  const double pi2 = 6.283185307179586;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int64_t nKo = shape_out[0] * shape_out[1] * (shape_out[2] / 2 + 1);
  const int nz = (int)shape_in[0], ny = (int)shape_in[1], nx = (int)shape_in[2];
  const int mz = (int)shape_out[0], my = (int)shape_out[1], mx = (int)shape_out[2];
  if (dtype == GBS_F64)
    gbs::k_resample<double><<<gbs::nblocks(nKo), 256, 0, st>>>(
        static_cast<const double2*>(in), static_cast<double2*>(out), nz, ny, nx, mz, my, mx,
        nfields, pi2 / L[2], pi2 / L[1], pi2 / L[0], delta);
  else
    gbs::k_resample<float><<<gbs::nblocks(nKo), 256, 0, st>>>(
        static_cast<const float2*>(in), static_cast<float2*>(out), nz, ny, nx, mz, my, mx,
        nfields, pi2 / L[2], pi2 / L[1], pi2 / L[0], delta);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

int gbs_products6(const void* u, void* out, int64_t n, const void* sub, int dtype,
                  void* stream) {
  gbs::clear_error();
  if (!u || !out || n < 1 || (dtype != GBS_F32 && dtype != GBS_F64)) {
    gbs::set_error("gbs_products6: invalid argument");
    return GBS_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == GBS_F64)
    gbs::k_products6<double><<<gbs::nblocks(n), 256, 0, st>>>(
        static_cast<const double*>(u), static_cast<double*>(out), n,
        static_cast<const double*>(sub));
  else
    gbs::k_products6<float><<<gbs::nblocks(n), 256, 0, st>>>(
        static_cast<const float*>(u), static_cast<float*>(out), n,
        static_cast<const float*>(sub));
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

int gbs_velocity_gradients(const int64_t* shape, const double* L, const int64_t* kcut,
                           int dtype, const void* S, void* G, void* stream) {
  gbs::clear_error();
  if (!shape || !L || !kcut || !S || !G || shape[2] % 2 ||
      (dtype != GBS_F32 && dtype != GBS_F64)) {
    gbs::set_error("gbs_velocity_gradients: invalid argument");
    return GBS_EINVAL;
  }
  const double pi2 = 6.283185307179586;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nz = (int)shape[0], ny = (int)shape[1], nx = (int)shape[2];
  const int64_t nK = (int64_t)nz * ny * (nx / 2 + 1);
  if (dtype == GBS_F64)
    gbs::k_gradients<double><<<gbs::nblocks(nK), 256, 0, st>>>(
        static_cast<const double2*>(S), static_cast<double2*>(G), nz, ny, nx, pi2 / L[2],
        pi2 / L[1], pi2 / L[0], (int)kcut[2], (int)kcut[1], (int)kcut[0]);
  else
    gbs::k_gradients<float><<<gbs::nblocks(nK), 256, 0, st>>>(
        static_cast<const float2*>(S), static_cast<float2*>(G), nz, ny, nx, pi2 / L[2],
        pi2 / L[1], pi2 / L[0], (int)kcut[2], (int)kcut[1], (int)kcut[0]);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

}  // extern "C"
