// Multi-dimensional R2C / C2R transforms (fluidfft fft2d / fft3d API).
//
// A d-dimensional transform is d axis passes over HBM:
//   forward  x (R2C, rows) -> y (columns) -> z (columns, scaled by 1/N)
//   inverse  z -> y (columns)  -> x (C2R, rows)
// Column passes read a tile of TX adjacent columns (one coalesced segment
// of TX complex per row), transform all of them in shared memory and write
// the tile back; the x pass turns nx reals into an nx/2-point complex FFT
// plus the R2C post-processing step.
#include <cstdarg>
#include <cstdlib>
#include <mutex>
#include <new>

#include "gbs_internal.cuh"
#include "gbs_fast.cuh"
#include "gbs_fast_api.h"

namespace gbs {

static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

void clear_error() { g_last_error.clear(); }

extern __shared__ __align__(16) unsigned char g_smem[];

// ------------------------------------------------------------------ twiddles
template <typename T>
__global__ void k_twiddle(cplx<T>* tw, int n) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double s, c;
  sincospi(2.0 * (double)k / (double)n, &s, &c);
  tw[k] = mk<cplx<T>>((T)c, (T)(-s));
}

template <typename T>
int make_twiddles(cplx<T>* tw, int n, cudaStream_t st) {
  k_twiddle<T><<<ceil_div(n, 256), 256, 0, st>>>(tw, n);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}
template int make_twiddles<float>(cplx<float>*, int, cudaStream_t);
template int make_twiddles<double>(cplx<double>*, int, cudaStream_t);

// --------------------------------------------------------- column transform
// Lines along a strided axis: element j of column c of outer block o of
// field f is at  f*fs + o*os + j*es + c.  Tile = TX columns.
struct ColGeom {
  int n, ncols, TX;
  int64_t es, os, fs;
};

template <typename T, int DIR>
__global__ void __launch_bounds__(kMaxThreads)
k_col(const cplx<T>* __restrict__ in, cplx<T>* out, ColGeom g,
      const cplx<T>* __restrict__ tw, T scale) {
  using C = cplx<T>;
  C* buf = reinterpret_cast<C*>(g_smem);
  C* buf2 = buf + (size_t)g.n * g.TX;
  const int c0 = blockIdx.x * g.TX;
  const int64_t base = blockIdx.z * g.fs + blockIdx.y * g.os + c0;
  const int tot = g.n * g.TX;
  for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
    int c = idx % g.TX, j = idx / g.TX;
    C v = mk<C>(0, 0);
    if (c0 + c < g.ncols) v = in[base + j * g.es + c];
    buf[idx] = v;
  }
  __syncthreads();
  fft_tile<DIR, kTPT>(buf, buf2, g.n, g.TX, g.TX, tw, 1);
  for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
    int c = idx % g.TX, j = idx / g.TX;
    if (c0 + c < g.ncols) out[base + j * g.es + c] = cscale(buf[idx], scale);
  }
}

// ---------------------------------------------------------------- row R2C
// rows of nx reals -> nkx = nx/2+1 complex, via an M = nx/2 complex FFT.
struct RowGeom {
  int M, nkx, L, LP;
  int64_t nrows;
};

template <typename T>
__global__ void __launch_bounds__(kMaxThreads)
k_row_r2c(const T* __restrict__ x, cplx<T>* __restrict__ out, RowGeom g,
          const cplx<T>* __restrict__ twx, T scale) {
  using C = cplx<T>;
  C* buf = reinterpret_cast<C*>(g_smem);
  C* buf2 = buf + (size_t)g.M * g.LP;
  const int64_t r0 = (int64_t)blockIdx.x * g.L;
  const C* xc = reinterpret_cast<const C*>(x);
  for (int idx = threadIdx.x; idx < g.L * g.M; idx += blockDim.x) {
    int j = idx % g.M, l = idx / g.M;
    C v = mk<C>(0, 0);
    if (r0 + l < g.nrows) v = xc[(r0 + l) * g.M + j];
    buf[j * g.LP + l] = v;
  }
  __syncthreads();
  fft_tile<-1, kTPT>(buf, buf2, g.M, g.L, g.LP, twx, 2);
  const T half = T(0.5);
  for (int idx = threadIdx.x; idx < g.L * g.nkx; idx += blockDim.x) {
    int k = idx % g.nkx, l = idx / g.nkx;
    if (r0 + l >= g.nrows) continue;
    C a = buf[(k == g.M ? 0 : k) * g.LP + l];
    C b = cconj(buf[(k == 0 ? 0 : g.M - k) * g.LP + l]);
    C s = cadd(a, b), d = csub(a, b);
    C wd = cmul(twx[k], d);  // W^k (a - b)
    // X = (s - i W^k d) / 2
    C X = mk<C>(half * (s.x + wd.y), half * (s.y - wd.x));
    out[(r0 + l) * g.nkx + k] = cscale(X, scale);
  }
}

// ---------------------------------------------------------------- row C2R
template <typename T>
__global__ void __launch_bounds__(kMaxThreads)
k_row_c2r(const cplx<T>* __restrict__ in, T* __restrict__ x, RowGeom g,
          const cplx<T>* __restrict__ twx) {
  using C = cplx<T>;
  C* buf = reinterpret_cast<C*>(g_smem);
  C* buf2 = buf + (size_t)g.M * g.LP;
  const int64_t r0 = (int64_t)blockIdx.x * g.L;
  for (int idx = threadIdx.x; idx < g.L * g.M; idx += blockDim.x) {
    int j = idx % g.M, l = idx / g.M;
    C Z = mk<C>(0, 0);
    if (r0 + l < g.nrows) {
      const C* row = in + (r0 + l) * g.nkx;
      C a = row[j];
      C b = cconj(row[g.M - j]);
      if (j == 0) { a.y = 0; b.y = 0; }
      C s = cadd(a, b), d = csub(a, b);
      C wd = cmulc(d, twx[j]);  // conj(W^j) (a - b)
      Z = mk<C>(s.x - wd.y, s.y + wd.x);  // s + i conj(W^j) d
    }
    buf[j * g.LP + l] = Z;
  }
  __syncthreads();
  fft_tile<+1, kTPT>(buf, buf2, g.M, g.L, g.LP, twx, 2);
  C* xc = reinterpret_cast<C*>(x);
  for (int idx = threadIdx.x; idx < g.L * g.M; idx += blockDim.x) {
    int j = idx % g.M, l = idx / g.M;
    if (r0 + l < g.nrows) xc[(r0 + l) * g.M + j] = buf[j * g.LP + l];
  }
}

// ------------------------------------------------------------ launch helpers
template <typename T, int DIR>
int launch_col(const cplx<T>* in, cplx<T>* out, int n, int ncols, int nouter,
               int nfields, int64_t es, int64_t os, int64_t fs,
               const cplx<T>* tw, T scale, cudaStream_t st) {
  if (n == 1 && in == out && scale == T(1)) return GBS_OK;  // nothing to do
  ColGeom g;
  g.n = n;
  g.ncols = ncols;
  g.TX = pick_tx(n, 1, sizeof(cplx<T>), sizeof(T) == 4 ? 16 : 8, ncols);
  g.es = es;
  g.os = os;
  g.fs = fs;
  size_t smem = tile_smem(n, g.TX, sizeof(cplx<T>));
  if (smem > kSmemMax) {
    set_error("axis length %d too large for one tile", n);
    return GBS_EINVAL;
  }
  int th = tile_threads(n, g.TX);
  int rc = allow_smem(k_col<T, DIR>, smem);
  if (rc) return rc;
  dim3 grid(ceil_div(ncols, g.TX), nouter, nfields);
  k_col<T, DIR><<<grid, th, smem, st>>>(in, out, g, tw, scale);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

template <typename T>
RowGeom row_geom(int nx, int64_t nrows) {
  RowGeom g;
  g.M = nx / 2;
  g.nkx = nx / 2 + 1;
  g.nrows = nrows;
  int L = sizeof(T) == 4 ? 16 : 8;
  while (L > 1 && (tile_smem(g.M, L + 1, sizeof(cplx<T>)) > kSmemBudget ||
                   !tile_fits(g.M, L) || L / 2 >= nrows))
    L /= 2;
  g.L = L;
  g.LP = L + 1;
  return g;
}

template <typename T>
int launch_r2c_rows(const T* x, cplx<T>* k, int nx, int64_t nrows,
                    const cplx<T>* twx, T scale, cudaStream_t st) {
  RowGeom g = row_geom<T>(nx, nrows);
  size_t smem = tile_smem(g.M, g.LP, sizeof(cplx<T>));
  int th = tile_threads(g.M, g.L);
  int rc = allow_smem(k_row_r2c<T>, smem);
  if (rc) return rc;
  k_row_r2c<T><<<ceil_div(nrows, g.L), th, smem, st>>>(x, k, g, twx, scale);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

template <typename T>
int launch_c2r_rows(const cplx<T>* k, T* x, int nx, int64_t nrows,
                    const cplx<T>* twx, cudaStream_t st) {
  RowGeom g = row_geom<T>(nx, nrows);
  size_t smem = tile_smem(g.M, g.LP, sizeof(cplx<T>));
  int th = tile_threads(g.M, g.L);
  int rc = allow_smem(k_row_c2r<T>, smem);
  if (rc) return rc;
  k_row_c2r<T><<<ceil_div(nrows, g.L), th, smem, st>>>(k, x, g, twx);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

template int launch_col<float, -1>(const cplx<float>*, cplx<float>*, int, int, int, int, int64_t, int64_t, int64_t, const cplx<float>*, float, cudaStream_t);
template int launch_col<float, 1>(const cplx<float>*, cplx<float>*, int, int, int, int, int64_t, int64_t, int64_t, const cplx<float>*, float, cudaStream_t);
template int launch_col<double, -1>(const cplx<double>*, cplx<double>*, int, int, int, int, int64_t, int64_t, int64_t, const cplx<double>*, double, cudaStream_t);
template int launch_col<double, 1>(const cplx<double>*, cplx<double>*, int, int, int, int, int64_t, int64_t, int64_t, const cplx<double>*, double, cudaStream_t);
template int launch_c2r_rows<float>(const cplx<float>*, float*, int, int64_t, const cplx<float>*, cudaStream_t);
template int launch_c2r_rows<double>(const cplx<double>*, double*, int, int64_t, const cplx<double>*, cudaStream_t);

// ------------------------------------------------------------------- plans
struct Plan {
  int ndim;
  int nz, ny, nx;  // nz = 1 for 2D
  int dtype;
  int batch;
  int64_t nX, nK;  // points per field (physical / spectral)
  void* tw[3];     // x (nx entries), y, z
  void* work;      // batch * nK complex
};

// Axis passes: compile-time-size kernels where the length has one, the
// generic kernels otherwise.
template <typename T, int DIR>
int axis_col(const cplx<T>* in, cplx<T>* out, int n, int ncols, int nouter, int nfields,
             int64_t es, int64_t os, int64_t fs, const cplx<T>* tw, T scale,
             cudaStream_t st) {
  if (fast::supported_axis(n)) {
    fast::ColArgs a;
    a.ncols = ncols;
    a.kc_in = n + 1;
    a.kc_out = n + 1;
    a.es = es;
    a.os = os;
    a.fs = fs;
    return fast::col<T>(n, in, out, a, nouter, nfields, tw, (double)scale, DIR, st);
  }
  return launch_col<T, DIR>(in, out, n, ncols, nouter, nfields, es, os, fs, tw, scale, st);
}

template <typename T>
int axis_r2c(const T* x, cplx<T>* k, int nx, int64_t nrows, const cplx<T>* twx, T scale,
             cudaStream_t st) {
  if (fast::supported_axis(nx / 2)) return fast::r2c_rows<T>(nx, x, k, nrows, twx, scale, st);
  return launch_r2c_rows<T>(x, k, nx, nrows, twx, scale, st);
}

template <typename T>
int axis_c2r(const cplx<T>* k, T* x, int nx, int64_t nrows, const cplx<T>* twx,
             cudaStream_t st) {
  if (fast::supported_axis(nx / 2)) return fast::c2r_rows<T>(nx, k, x, nrows, twx, st);
  return launch_c2r_rows<T>(k, x, nx, nrows, twx, st);
}

template <typename T>
int plan_r2c(Plan* p, const void* xv, void* kv, cudaStream_t st) {
  using C = cplx<T>;
  const T* x = static_cast<const T*>(xv);
  C* k = static_cast<C*>(kv);
  const C* twx = static_cast<const C*>(p->tw[0]);
  const C* twy = static_cast<const C*>(p->tw[1]);
  const C* twz = static_cast<const C*>(p->tw[2]);
  const int nkx = p->nx / 2 + 1;
  const T inv = T(1.0 / ((double)p->nx * p->ny * p->nz));
  int rc;
  const int64_t rows = (int64_t)p->batch * p->nz * p->ny;
  if (p->ndim == 2) {
    rc = axis_r2c<T>(x, k, p->nx, rows, twx, T(1), st);
    if (rc) return rc;
    return axis_col<T, -1>(k, k, p->ny, nkx, 1, p->batch, nkx, 0, p->nK,
                             twy, inv, st);
  }
  rc = axis_r2c<T>(x, k, p->nx, rows, twx, T(1), st);
  if (rc) return rc;
  rc = axis_col<T, -1>(k, k, p->ny, nkx, p->nz, p->batch, nkx,
                         (int64_t)p->ny * nkx, p->nK, twy, T(1), st);
  if (rc) return rc;
  return axis_col<T, -1>(k, k, p->nz, nkx, p->ny, p->batch,
                           (int64_t)p->ny * nkx, nkx, p->nK, twz, inv, st);
}

template <typename T>
int plan_c2r(Plan* p, void* kv, void* xv, int destroy, cudaStream_t st) {
  using C = cplx<T>;
  C* k = static_cast<C*>(kv);
  T* x = static_cast<T*>(xv);
  C* w = destroy ? k : static_cast<C*>(p->work);
  const C* twx = static_cast<const C*>(p->tw[0]);
  const C* twy = static_cast<const C*>(p->tw[1]);
  const C* twz = static_cast<const C*>(p->tw[2]);
  const int nkx = p->nx / 2 + 1;
  const int64_t rows = (int64_t)p->batch * p->nz * p->ny;
  int rc;
  if (p->ndim == 2) {
    rc = axis_col<T, 1>(k, w, p->ny, nkx, 1, p->batch, nkx, 0, p->nK, twy,
                          T(1), st);
    if (rc) return rc;
    return axis_c2r<T>(w, x, p->nx, rows, twx, st);
  }
  rc = axis_col<T, 1>(k, w, p->nz, nkx, p->ny, p->batch,
                        (int64_t)p->ny * nkx, nkx, p->nK, twz, T(1), st);
  if (rc) return rc;
  rc = axis_col<T, 1>(w, w, p->ny, nkx, p->nz, p->batch, nkx,
                        (int64_t)p->ny * nkx, p->nK, twy, T(1), st);
  if (rc) return rc;
  return axis_c2r<T>(w, x, p->nx, rows, twx, st);
}

int twiddle_alloc(void** out, int n, int dtype, cudaStream_t st) {
  size_t cs = dtype == GBS_F64 ? sizeof(double2) : sizeof(float2);
  GBS_CUDA_TRY(cudaMalloc(out, cs * (size_t)n));
  if (dtype == GBS_F64)
    return make_twiddles<double>(static_cast<double2*>(*out), n, st);
  return make_twiddles<float>(static_cast<float2*>(*out), n, st);
}

}  // namespace gbs

using gbs::Plan;

struct gbs_fft_plan {
  Plan p;
};

extern "C" {

const char* gbs_last_error(void) { return gbs::g_last_error.c_str(); }

const char* gbs_version(void) { return "gbspec 0.1 (sm_103a)"; }

int gbs_fft_plan_create(int ndim, const int64_t* shapeX, int dtype, int batch,
                        gbs_fft_plan** out) {
  gbs::clear_error();
  if (!out || !shapeX || (ndim != 2 && ndim != 3) || batch < 1 ||
      (dtype != GBS_F32 && dtype != GBS_F64)) {
    gbs::set_error("gbs_fft_plan_create: invalid argument");
    return GBS_EINVAL;
  }
  *out = nullptr;
  int64_t nz = ndim == 3 ? shapeX[0] : 1;
  int64_t ny = shapeX[ndim - 2];
  int64_t nx = shapeX[ndim - 1];
  if (nx < 2 || nx % 2 || ny < 1 || nz < 1 || nx > 65536 || ny > 65536 ||
      nz > 65536) {
    gbs::set_error("gbs_fft_plan_create: unsupported shape (nx must be even)");
    return GBS_EINVAL;
  }
  gbs_fft_plan* h = new (std::nothrow) gbs_fft_plan();
  if (!h) return GBS_ENOMEM;
  Plan& p = h->p;
  p.ndim = ndim;
  p.nz = (int)nz;
  p.ny = (int)ny;
  p.nx = (int)nx;
  p.dtype = dtype;
  p.batch = batch;
  p.nX = nz * ny * nx;
  p.nK = nz * ny * (nx / 2 + 1);
  p.tw[0] = p.tw[1] = p.tw[2] = p.work = nullptr;
  int rc = 0;
  int ns[3] = {(int)nx, (int)ny, (int)nz};
  for (int a = 0; a < 3 && !rc; ++a) rc = gbs::twiddle_alloc(&p.tw[a], ns[a], dtype, 0);
  size_t cs = dtype == GBS_F64 ? sizeof(double2) : sizeof(float2);
  if (!rc && cudaMalloc(&p.work, cs * p.nK * batch) != cudaSuccess) {
    gbs::set_error("gbs_fft_plan_create: cudaMalloc of the workspace failed");
    rc = GBS_ENOMEM;
  }
  if (!rc && cudaStreamSynchronize(0) != cudaSuccess) {
    gbs::set_error("gbs_fft_plan_create: %s", cudaGetErrorString(cudaGetLastError()));
    rc = GBS_ECUDA;
  }
  if (rc) {
    gbs_fft_plan_destroy(h);
    return rc;
  }
  *out = h;
  return GBS_OK;
}

int gbs_fft_plan_destroy(gbs_fft_plan* h) {
  if (!h) return GBS_OK;
  for (void* t : h->p.tw)
    if (t) cudaFree(t);
  if (h->p.work) cudaFree(h->p.work);
  delete h;
  return GBS_OK;
}

int gbs_fft_r2c(gbs_fft_plan* h, const void* x, void* k, void* stream) {
  gbs::clear_error();
  if (!h || !x || !k) {
    gbs::set_error("gbs_fft_r2c: null argument");
    return GBS_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (h->p.dtype == GBS_F64) return gbs::plan_r2c<double>(&h->p, x, k, st);
  return gbs::plan_r2c<float>(&h->p, x, k, st);
}

int gbs_fft_c2r(gbs_fft_plan* h, void* k, void* x, int may_destroy,
                void* stream) {
  gbs::clear_error();
  if (!h || !x || !k) {
    gbs::set_error("gbs_fft_c2r: null argument");
    return GBS_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (h->p.dtype == GBS_F64)
    return gbs::plan_c2r<double>(&h->p, k, x, may_destroy, st);
  return gbs::plan_c2r<float>(&h->p, k, x, may_destroy, st);
}

}  // extern "C"
