// FP64 spectra of a real spectral energy density (the operator methods
// compute_1dspectra, compute_3dspectrum / compute_2dspectrum and
// compute_spectrum_kzkh that fluidsim's spectra outputs call,
// fluidsim/solvers/ns3d/output/spectra.py:15-100 and
// fluidsim/solvers/ns2d/output/spectra.py:16-27).
//
// Input: e of spectral shape (nz, ny, nx/2+1) (2D: nz = 1), float or
// double.  Every mode enters with its Hermitian weight w (1 for kx = 0 and,
// nx even, for the Nyquist column; 2 otherwise), accumulated in FP64:
//   skx[ix]          = sum_{iz,iy} w e / dkx                 (nx/2+1 bins)
//   sky[|ky_adim|]   = sum w e / dky                          (ny/2+1 bins)
//   skz[|kz_adim|]   = sum w e / dkz                          (nz/2+1 bins)
//   shell[b]         = sum w e / dk,  b = floor(|k| / dk + 0.5),
//                      dk = min(dkx, dky[, dkz])              (kmax/dk + 1 bins)
//   kzkh[|kz|, b]    = sum w e / (dkz dkh), b = floor(kh / dkh + 0.5),
//                      kh = sqrt(kx^2 + ky^2), dkh = min(dkx, dky)
// The wavenumber products and sums are rounded one at a time (no
// contraction), as numpy evaluates K2 = Kx**2 + Ky**2 + Kz**2, so a mode
// lands in the same bin as in a float64 numpy restatement.
//
// One CTA per (kz plane, chunk of ky rows); each warp takes one row at a
// time.  The CTA accumulates its kx, shell and kh bins in shared memory and
// adds them to the output with one global atomic per nonzero bin; row sums
// (ky bins) are warp-reduced first.  When the bins do not fit in 48 KB of
// shared memory, the CTA adds straight into the output.
#include "gbs_internal.cuh"

namespace gbs {

struct SpecGeom {
  int ndim, nx, ny, nz, nkx;
  double dkx, dky, dkz, dk, dkh;
  int64_t nyb, nzb, n3, nkh;
};

static int64_t bin_of(double k2, double dk) {
  return (int64_t)floor(sqrt(k2) / dk + 0.5);
}

// a * a rounded on its own (the stores keep a host compiler from fusing the
// products into the sums that follow)
static double square_rn(double a) {
  volatile double r = a * a;
  return r;
}

static int make_geom(int ndim, const int64_t* shapeX, const double* deltak,
                     SpecGeom* g) {
  if ((ndim != 2 && ndim != 3) || !shapeX || !deltak) return GBS_EINVAL;
  const int64_t nz = ndim == 3 ? shapeX[0] : 1;
  const int64_t ny = shapeX[ndim - 2], nx = shapeX[ndim - 1];
  if (nx < 2 || ny < 1 || nz < 1 || nx > 65536 || ny > 65536 || nz > 65536)
    return GBS_EINVAL;
  g->ndim = ndim;
  g->nx = (int)nx;
  g->ny = (int)ny;
  g->nz = (int)nz;
  g->nkx = (int)(nx / 2 + 1);
  g->dkx = deltak[0];
  g->dky = deltak[1];
  g->dkz = ndim == 3 ? deltak[2] : 1.0;
  if (!(g->dkx > 0) || !(g->dky > 0) || !(g->dkz > 0)) return GBS_EINVAL;
  g->dkh = g->dkx < g->dky ? g->dkx : g->dky;
  g->dk = (ndim == 3 && g->dkz < g->dkh) ? g->dkz : g->dkh;
  g->nyb = ny / 2 + 1;
  g->nzb = ndim == 3 ? nz / 2 + 1 : 0;
  // the corner mode has the largest |k| and kh; same rounding as the kernel
  const double kx = g->dkx * (g->nkx - 1), ky = g->dky * (double)(ny / 2);
  const double kz = ndim == 3 ? g->dkz * (double)(nz / 2) : 0.0;
  volatile double kh2 = square_rn(kx) + square_rn(ky);
  g->nkh = ndim == 3 ? bin_of(kh2, g->dkh) + 1 : 0;
  g->n3 = bin_of(kh2 + square_rn(kz), g->dk) + 1;
  return GBS_OK;
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T>
__global__ void __launch_bounds__(256)
k_spectra(const T* __restrict__ e, SpecGeom g, int rows, double* __restrict__ skx,
          double* __restrict__ sky, double* __restrict__ skz,
          double* __restrict__ ssh, double* __restrict__ skh, int use_smem) {
  extern __shared__ double sh[];
  __shared__ double zpart[8];
  const int iz = blockIdx.x;
  const int kzi = g.ndim == 3 ? kadim(iz, g.nz) : 0;
  const int izb = kzi < 0 ? -kzi : kzi;
  const double kz = g.dkz * kzi;
  const double kz2 = __dmul_rn(kz, kz);
  double* bx = skx;
  double* bs = ssh;
  double* bh = skh ? skh + (int64_t)izb * g.nkh : nullptr;
  const int nsm = g.nkx + (int)g.n3 + (int)g.nkh;
  if (use_smem) {
    bx = sh;
    bs = sh + g.nkx;
    bh = bs + g.n3;
    for (int i = threadIdx.x; i < nsm; i += blockDim.x) sh[i] = 0.0;
    __syncthreads();
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  const int y0 = blockIdx.y * rows;
  const int y1 = min(y0 + rows, g.ny);
  const bool even = (g.nx & 1) == 0;
  double zacc = 0.0;
  for (int iy = y0 + warp; iy < y1; iy += nw) {
    const int kyi = kadim(iy, g.ny);
    const double ky = g.dky * kyi;
    const double ky2 = __dmul_rn(ky, ky);
    const T* row = e + ((int64_t)iz * g.ny + iy) * g.nkx;
    double racc = 0.0;
    for (int ix = lane; ix < g.nkx; ix += 32) {
      const double w = (ix == 0 || (even && ix == g.nx / 2)) ? 1.0 : 2.0;
      const double v = w * (double)row[ix];
      racc += v;
      if (v != 0.0) {
        if (skx) atomicAdd(bx + ix, v);
        const double kx = g.dkx * ix;
        const double kh2 = __dadd_rn(__dmul_rn(kx, kx), ky2);
        if (ssh) {
          int64_t b = (int64_t)floor(sqrt(__dadd_rn(kh2, kz2)) / g.dk + 0.5);
          if (b > g.n3 - 1) b = g.n3 - 1;
          atomicAdd(bs + b, v);
        }
        if (skh) {
          int64_t b = (int64_t)floor(sqrt(kh2) / g.dkh + 0.5);
          if (b > g.nkh - 1) b = g.nkh - 1;
          atomicAdd(bh + b, v);
        }
      }
    }
    racc = warp_sum(racc);
    if (lane == 0 && sky) atomicAdd(sky + (kyi < 0 ? -kyi : kyi), racc);
    zacc += racc;
  }
  if (skz) {
    if (lane == 0) zpart[warp] = zacc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int i = 0; i < nw; ++i) s += zpart[i];
      if (s != 0.0) atomicAdd(skz + izb, s);
    }
  }
  if (use_smem) {
    __syncthreads();
    for (int i = threadIdx.x; i < g.nkx; i += blockDim.x)
      if (skx && bx[i] != 0.0) atomicAdd(skx + i, bx[i]);
    for (int i = threadIdx.x; i < g.n3; i += blockDim.x)
      if (ssh && bs[i] != 0.0) atomicAdd(ssh + i, bs[i]);
    for (int i = threadIdx.x; i < g.nkh; i += blockDim.x)
      if (skh && bh[i] != 0.0) atomicAdd(skh + (int64_t)izb * g.nkh + i, bh[i]);
  }
}

// Divide each output by its bin width.
__global__ void k_spectra_scale(double* a, int64_t n, double width) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    a[i] = a[i] / width;
}

}  // namespace gbs

extern "C" {

int gbs_spectra_sizes(int ndim, const int64_t* shapeX, const double* deltak,
                      int64_t* sizes) {
  gbs::clear_error();
  gbs::SpecGeom g;
  if (!sizes || gbs::make_geom(ndim, shapeX, deltak, &g)) {
    gbs::set_error("gbs_spectra_sizes: invalid argument");
    return GBS_EINVAL;
  }
  sizes[0] = g.nkx;
  sizes[1] = g.nyb;
  sizes[2] = g.nzb;
  sizes[3] = g.n3;
  sizes[4] = g.nkh;
  return GBS_OK;
}

int gbs_spectra(int ndim, const int64_t* shapeX, const double* deltak, int dtype,
                const void* energy, double* skx, double* sky, double* skz,
                double* shell, double* kzkh, void* stream) {
  gbs::clear_error();
  gbs::SpecGeom g;
  if (!energy || (dtype != GBS_F32 && dtype != GBS_F64) ||
      gbs::make_geom(ndim, shapeX, deltak, &g) ||
      (ndim == 2 && (skz || kzkh))) {
    gbs::set_error("gbs_spectra: invalid argument");
    return GBS_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  struct Out {
    double* p;
    int64_t n;
    double width;
  } outs[5] = {{skx, g.nkx, g.dkx},
               {sky, g.nyb, g.dky},
               {skz, g.nzb, g.dkz},
               {shell, g.n3, g.dk},
               {kzkh, g.nzb * g.nkh, g.dkz * g.dkh}};
  for (const Out& o : outs)
    if (o.p) GBS_CUDA_TRY(cudaMemsetAsync(o.p, 0, o.n * sizeof(double), st));
  if (!skx && !sky && !skz && !shell && !kzkh) return GBS_OK;
  const int64_t nsm = g.nkx + g.n3 + g.nkh;
  const int use_smem = nsm * (int64_t)sizeof(double) <= 48 * 1024;
  const size_t smem = use_smem ? nsm * sizeof(double) : 0;
  int ychunks = 1024 / g.nz;
  if (ychunks < 1) ychunks = 1;
  if (ychunks > g.ny) ychunks = g.ny;
  const int rows = (g.ny + ychunks - 1) / ychunks;
  ychunks = (g.ny + rows - 1) / rows;
  dim3 grid(g.nz, ychunks);
  if (dtype == GBS_F64)
    gbs::k_spectra<double><<<grid, 256, smem, st>>>(
        static_cast<const double*>(energy), g, rows, skx, sky, skz, shell, kzkh,
        use_smem);
  else
    gbs::k_spectra<float><<<grid, 256, smem, st>>>(
        static_cast<const float*>(energy), g, rows, skx, sky, skz, shell, kzkh,
        use_smem);
  GBS_CHECK_LAUNCH();
  for (const Out& o : outs) {
    if (!o.p) continue;
    gbs::k_spectra_scale<<<gbs::ceil_div(o.n, 256) < 1024 ? gbs::ceil_div(o.n, 256) : 1024,
                           256, 0, st>>>(o.p, o.n, o.width);
    GBS_CHECK_LAUNCH();
  }
  return GBS_OK;
}

}  // extern "C"
