// Fused pseudo-spectral RK4 stages for ns2d / ns3d.
//
// One evaluation of the nonlinear tendencies plus the RK4 stage update is
// five kernels (ns3d; ns2d has the same shape with one axis less):
//   A  inverse z pass: read v_hat, form omega_hat = i k x v_hat on the fly,
//      transform the 6 fields along z                       (3 in, 6 out)
//   -  inverse y pass on the 6 fields                       (6 in, 6 out)
//   B  x pass: C2R of the 6 rows, v x omega in shared memory, R2C of the 3
//      products; no physical field is ever written to HBM   (6 in, 3 out)
//   -  forward y pass on the 3 products                     (3 in, 3 out)
//   C  forward z pass, 1/N, P_perp projection, dealiasing and the RK4
//      stage update (or the plain tendency / final state)   (3 + state)
// Reference: fluidsim/solvers/ns3d/solver.py:180-263,
// fluidsim/solvers/ns2d/solver.py:33-39,111-194,
// fluidsim/base/time_stepping/pseudo_spect.py:798-984.
#include <cmath>
#include <new>

#include "gbs_internal.cuh"
#include "gbs_ns.cuh"
#include "gbs_fast.cuh"
#include "gbs_fast_api.h"
#include "gbs_turb.h"

namespace gbs {

extern __shared__ __align__(16) unsigned char g_smem_ns[];

template <typename T> int make_twiddles(cplx<T>* tw, int n, cudaStream_t st);
template <typename T, int DIR>
int launch_col(const cplx<T>* in, cplx<T>* out, int n, int ncols, int nouter,
               int nfields, int64_t es, int64_t os, int64_t fs,
               const cplx<T>* tw, T scale, cudaStream_t st);

// Geometry and physics constants passed by value to every kernel.
struct NSK {
  int nx, ny, nz, nkx, M;
  int kcx, kcy, kcz;
  double dkx, dky, dkz;
  double nu2, nu4, nu8, num4;
  double beta, f;
  int has_f;
  double inv_n;
  double k2_hypo0;  // K2 at (iz, iy, ix) = (0, 0, 1): f_d_hypo[0,..,0] source
  int TX, L, LP;
  int phase;          // multiply the input state by exp(i phi)
  double sx, sy, sz;  // phase shift lengths (phi = sx kx + sy ky + sz kz)
  int proj, no_vz_kz0;  // ns3d projection of the tendencies and the state
};

__device__ __forceinline__ bool removed(const NSK& q, int ix, int ky, int kz) {
  return ix >= q.kcx || iabs(ky) >= q.kcy || iabs(kz) >= q.kcz;
}

__device__ __forceinline__ Phys phys(const NSK& q) {
  Phys p;
  p.nu2 = q.nu2;
  p.nu4 = q.nu4;
  p.nu8 = q.nu8;
  p.num4 = q.num4;
  p.k2_hypo0 = q.k2_hypo0;
  p.fnu2 = (float)q.nu2;
  p.fnu4 = (float)q.nu4;
  p.fnu8 = (float)q.nu8;
  p.fnum4 = (float)q.num4;
  p.fk2_hypo0 = (float)q.k2_hypo0;
  p.proj = q.proj;
  p.no_vz_kz0 = q.no_vz_kz0;
  return p;
}

// C2R pre-processing of row element j (see k_row_c2r in gbs_fft.cu).
template <typename C>
__device__ __forceinline__ C c2r_pre(const C* row, int j, int M, const C* twx) {
  C a = row[j];
  C b = cconj(row[M - j]);
  if (j == 0) { a.y = 0; b.y = 0; }
  C s = cadd(a, b), d = csub(a, b);
  C wd = cmulc(d, twx[j]);
  return mk<C>(s.x - wd.y, s.y + wd.x);
}

template <typename C, typename T>
__device__ __forceinline__ C r2c_post(const C* buf, int k, int M, int LP,
                                      int line, const C* twx) {
  C a = buf[(k == M ? 0 : k) * LP + line];
  C b = cconj(buf[(k == 0 ? 0 : M - k) * LP + line]);
  C s = cadd(a, b), d = csub(a, b);
  C wd = cmul(twx[k], d);
  const T h = T(0.5);
  return mk<C>(h * (s.x + wd.y), h * (s.y - wd.x));
}

// =====================================================================  ns3d
// A: inverse z pass with the curl.  grid (tiles of TX along x, ny).
// lines: field f (0..2 = v, 3..5 = omega) x column c -> line f*TX + c.
template <typename T>
__global__ void __launch_bounds__(kMaxThreads)
k3_inv_z_curl(const cplx<T>* __restrict__ S, cplx<T>* __restrict__ W, NSK q,
              const cplx<T>* __restrict__ twz) {
  using C = cplx<T>;
  C* buf = reinterpret_cast<C*>(g_smem_ns);
  C* buf2 = buf + (size_t)q.nz * q.LP;
  const int TX = q.TX, LP = q.LP;
  const int c0 = blockIdx.x * TX, iy = blockIdx.y;
  const int64_t nK = (int64_t)q.nz * q.ny * q.nkx;
  const int64_t plane = (int64_t)q.ny * q.nkx;
  const T ky = T(q.dky * kadim(iy, q.ny));
  for (int idx = threadIdx.x; idx < q.nz * TX; idx += blockDim.x) {
    const int c = idx % TX, iz = idx / TX, ix = c0 + c;
    C v[6];
#pragma unroll
    for (int f = 0; f < 6; ++f) v[f] = mk<C>(0, 0);
    if (ix < q.nkx) {
      const int64_t i = iz * plane + (int64_t)iy * q.nkx + ix;
      C vx = S[i], vy = S[i + nK], vz = S[i + 2 * nK];
      const T kx = T(q.dkx * ix), kz = T(q.dkz * kadim(iz, q.nz));
      if (q.phase) {
        const C e = phase_factor<C, T>(T(q.sx), T(q.sy), T(q.sz), kx, ky, kz);
        vx = cmul(vx, e);
        vy = cmul(vy, e);
        vz = cmul(vz, e);
      }
      v[0] = vx;
      v[1] = vy;
      v[2] = vz;
      // omega = i (k x v)   (fluidfft rotfft_from_vecfft)
      C a = mk<C>(ky * vz.x - kz * vy.x, ky * vz.y - kz * vy.y);
      C b = mk<C>(kz * vx.x - kx * vz.x, kz * vx.y - kx * vz.y);
      C d = mk<C>(kx * vy.x - ky * vx.x, kx * vy.y - ky * vx.y);
      v[3] = mk<C>(-a.y, a.x);
      v[4] = mk<C>(-b.y, b.x);
      v[5] = mk<C>(-d.y, d.x);
      if (q.has_f && ix == 0 && iy == 0 && iz == 0) v[5].x += T(q.f);
    }
#pragma unroll
    for (int f = 0; f < 6; ++f) buf[iz * LP + f * TX + c] = v[f];
  }
  __syncthreads();
  fft_tile<+1, kTPT>(buf, buf2, q.nz, 6 * TX, LP, twz, 1);
  for (int idx = threadIdx.x; idx < q.nz * TX; idx += blockDim.x) {
    const int c = idx % TX, iz = idx / TX, ix = c0 + c;
    if (ix >= q.nkx) continue;
    const int64_t i = iz * plane + (int64_t)iy * q.nkx + ix;
#pragma unroll
    for (int f = 0; f < 6; ++f) W[i + f * nK] = buf[iz * LP + f * TX + c];
  }
}

// B: x pass.  Rows (iz, iy); L rows per CTA; lines f*L + l (f < 6).
template <typename T>
__global__ void __launch_bounds__(kMaxThreads)
k3_x_product(const cplx<T>* __restrict__ W, cplx<T>* __restrict__ F, NSK q,
             const cplx<T>* __restrict__ twx, unsigned long long* vmax) {
  using C = cplx<T>;
  C* buf = reinterpret_cast<C*>(g_smem_ns);
  C* buf2 = buf + (size_t)q.M * q.LP;
  const int L = q.L, LP = q.LP, M = q.M, nkx = q.nkx;
  const int64_t nrows = (int64_t)q.nz * q.ny;
  const int64_t nK = nrows * nkx;
  const int64_t r0 = (int64_t)blockIdx.x * L;
  for (int idx = threadIdx.x; idx < L * M; idx += blockDim.x) {
    const int j = idx % M, l = idx / M;
    const bool ok = r0 + l < nrows;
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      C z = mk<C>(0, 0);
      if (ok) z = c2r_pre(W + f * nK + (r0 + l) * nkx, j, M, twx);
      buf[j * LP + f * L + l] = z;
    }
  }
  __syncthreads();
  fft_tile<+1, kTPT>(buf, buf2, M, 6 * L, LP, twx, 2);
  T mx = 0, my = 0, mz = 0;
  for (int idx = threadIdx.x; idx < L * M; idx += blockDim.x) {
    const int j = idx % M, l = idx / M;
    C* p = buf + j * LP + l;
    const C vx = p[0], vy = p[L], vz = p[2 * L];
    const C ox = p[3 * L], oy = p[4 * L], oz = p[5 * L];
    // fluidfft vector_product(v, omega) = v x omega, both packed reals
    p[0] = mk<C>(vy.x * oz.x - vz.x * oy.x, vy.y * oz.y - vz.y * oy.y);
    p[L] = mk<C>(vz.x * ox.x - vx.x * oz.x, vz.y * ox.y - vx.y * oz.y);
    p[2 * L] = mk<C>(vx.x * oy.x - vy.x * ox.x, vx.y * oy.y - vy.y * ox.y);
    if (vmax && r0 + l < nrows) {
      mx = fmax(mx, fmax(fabs(vx.x), fabs(vx.y)));
      my = fmax(my, fmax(fabs(vy.x), fabs(vy.y)));
      mz = fmax(mz, fmax(fabs(vz.x), fabs(vz.y)));
    }
  }
  __syncthreads();
  if (vmax) block_max3(mx, my, mz, vmax);
  fft_tile<-1, kTPT>(buf, buf2, M, 3 * L, LP, twx, 2);
  for (int idx = threadIdx.x; idx < L * nkx; idx += blockDim.x) {
    const int k = idx % nkx, l = idx / nkx;
    if (r0 + l >= nrows) continue;
#pragma unroll
    for (int f = 0; f < 3; ++f)
      F[f * nK + (r0 + l) * nkx + k] = r2c_post<C, T>(buf, k, M, LP, f * L + l, twx);
  }
}

// C: forward z pass + 1/N + projection + dealiasing + RK4 stage.
template <typename T>
__global__ void __launch_bounds__(kMaxThreads)
k3_fwd_z_rk(const cplx<T>* __restrict__ F, NSK q, const cplx<T>* __restrict__ twz,
            int mode, RKArgs a) {
  using C = cplx<T>;
  C* buf = reinterpret_cast<C*>(g_smem_ns);
  C* buf2 = buf + (size_t)q.nz * q.LP;
  const int TX = q.TX, LP = q.LP;
  const int c0 = blockIdx.x * TX, iy = blockIdx.y;
  const int64_t nK = (int64_t)q.nz * q.ny * q.nkx;
  const int64_t plane = (int64_t)q.ny * q.nkx;
  for (int idx = threadIdx.x; idx < q.nz * TX; idx += blockDim.x) {
    const int c = idx % TX, iz = idx / TX, ix = c0 + c;
    const int64_t i = iz * plane + (int64_t)iy * q.nkx + ix;
#pragma unroll
    for (int f = 0; f < 3; ++f)
      buf[iz * LP + f * TX + c] = ix < q.nkx ? F[i + f * nK] : mk<C>(0, 0);
  }
  __syncthreads();
  fft_tile<-1, kTPT>(buf, buf2, q.nz, 3 * TX, LP, twz, 1);
  const int kyi = kadim(iy, q.ny);
  const T ky = T(q.dky * kyi);
  const T inv_n = T(q.inv_n);
  for (int idx = threadIdx.x; idx < q.nz * TX; idx += blockDim.x) {
    const int c = idx % TX, iz = idx / TX, ix = c0 + c;
    if (ix >= q.nkx) continue;
    const int64_t i = iz * plane + (int64_t)iy * q.nkx + ix;
    const int kzi = kadim(iz, q.nz);
    const T kx = T(q.dkx * ix), kz = T(q.dkz * kzi);
    const T k2 = kx * kx + ky * ky + kz * kz;
    const bool k0 = (ix == 0 && kyi == 0 && kzi == 0);
    const bool rm = removed(q, ix, kyi, kzi);
    C N[3];
#pragma unroll
    for (int f = 0; f < 3; ++f) N[f] = cscale(buf[iz * LP + f * TX + c], inv_n);
    if (a.add) {
#pragma unroll
      for (int f = 0; f < 3; ++f) N[f] = cadd(N[f], static_cast<const C*>(a.add)[i + f * nK]);
    }
    stage_epilogue3<C, T>(mode, a, i, nK, N, kx, ky, kz, k2, k0, rm, phys(q));
  }
}

// =====================================================================  ns2d
// A: inverse y pass; fields ux, uy, d_x rot, d_y rot from rot_fft.
template <typename T>
__global__ void __launch_bounds__(kMaxThreads)
k2_inv_y(const cplx<T>* __restrict__ S, cplx<T>* __restrict__ W, NSK q,
         const cplx<T>* __restrict__ twy) {
  using C = cplx<T>;
  C* buf = reinterpret_cast<C*>(g_smem_ns);
  C* buf2 = buf + (size_t)q.ny * q.LP;
  const int TX = q.TX, LP = q.LP;
  const int c0 = blockIdx.x * TX;
  const int64_t nK = (int64_t)q.ny * q.nkx;
  for (int idx = threadIdx.x; idx < q.ny * TX; idx += blockDim.x) {
    const int c = idx % TX, iy = idx / TX, ix = c0 + c;
    C v[4];
#pragma unroll
    for (int f = 0; f < 4; ++f) v[f] = mk<C>(0, 0);
    if (ix < q.nkx) {
      C w = S[(int64_t)iy * q.nkx + ix];
      const T kx = T(q.dkx * ix), ky = T(q.dky * kadim(iy, q.ny));
      if (q.phase) w = cmul(w, phase_factor<C, T>(T(q.sx), T(q.sy), T(0), kx, ky, T(0)));
      const T k2 = kx * kx + ky * ky;
      const T inv = (ix == 0 && kadim(iy, q.ny) == 0) ? T(0) : T(1) / k2;
      const T cx = ky * inv, cy = -(kx * inv);
      v[0] = mk<C>(-cx * w.y, cx * w.x);  // i ky rot / k^2
      v[1] = mk<C>(-cy * w.y, cy * w.x);  // -i kx rot / k^2
      v[2] = mk<C>(-kx * w.y, kx * w.x);  // i kx rot
      v[3] = mk<C>(-ky * w.y, ky * w.x);  // i ky rot
    }
#pragma unroll
    for (int f = 0; f < 4; ++f) buf[iy * LP + f * TX + c] = v[f];
  }
  __syncthreads();
  fft_tile<+1, kTPT>(buf, buf2, q.ny, 4 * TX, LP, twy, 1);
  for (int idx = threadIdx.x; idx < q.ny * TX; idx += blockDim.x) {
    const int c = idx % TX, iy = idx / TX, ix = c0 + c;
    if (ix >= q.nkx) continue;
#pragma unroll
    for (int f = 0; f < 4; ++f)
      W[f * nK + (int64_t)iy * q.nkx + ix] = buf[iy * LP + f * TX + c];
  }
}

// B: x pass, compute_Frot = -ux d_x rot - uy (d_y rot + beta).
template <typename T>
__global__ void __launch_bounds__(kMaxThreads)
k2_x_product(const cplx<T>* __restrict__ W, cplx<T>* __restrict__ F, NSK q,
             const cplx<T>* __restrict__ twx, unsigned long long* vmax) {
  using C = cplx<T>;
  C* buf = reinterpret_cast<C*>(g_smem_ns);
  C* buf2 = buf + (size_t)q.M * q.LP;
  const int L = q.L, LP = q.LP, M = q.M, nkx = q.nkx;
  const int64_t nrows = q.ny;
  const int64_t nK = nrows * nkx;
  const int64_t r0 = (int64_t)blockIdx.x * L;
  for (int idx = threadIdx.x; idx < L * M; idx += blockDim.x) {
    const int j = idx % M, l = idx / M;
    const bool ok = r0 + l < nrows;
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      C z = mk<C>(0, 0);
      if (ok) z = c2r_pre(W + f * nK + (r0 + l) * nkx, j, M, twx);
      buf[j * LP + f * L + l] = z;
    }
  }
  __syncthreads();
  fft_tile<+1, kTPT>(buf, buf2, M, 4 * L, LP, twx, 2);
  T mx = 0, my = 0;
  const T beta = T(q.beta);
  for (int idx = threadIdx.x; idx < L * M; idx += blockDim.x) {
    const int j = idx % M, l = idx / M;
    C* p = buf + j * LP + l;
    const C ux = p[0], uy = p[L], px = p[2 * L], py = p[3 * L];
    C r;
    if (q.beta == 0) {
      r = mk<C>(-ux.x * px.x - uy.x * py.x, -ux.y * px.y - uy.y * py.y);
    } else {
      r = mk<C>(-ux.x * px.x - uy.x * (py.x + beta),
                -ux.y * px.y - uy.y * (py.y + beta));
    }
    p[0] = r;
    if (vmax && r0 + l < nrows) {
      mx = fmax(mx, fmax(fabs(ux.x), fabs(ux.y)));
      my = fmax(my, fmax(fabs(uy.x), fabs(uy.y)));
    }
  }
  __syncthreads();
  if (vmax) block_max3(mx, my, T(0), vmax);
  fft_tile<-1, kTPT>(buf, buf2, M, L, LP, twx, 2);
  for (int idx = threadIdx.x; idx < L * nkx; idx += blockDim.x) {
    const int k = idx % nkx, l = idx / nkx;
    if (r0 + l >= nrows) continue;
    F[(r0 + l) * nkx + k] = r2c_post<C, T>(buf, k, M, LP, l, twx);
  }
}

// C: forward y pass + 1/N + dealiasing + RK4 stage.
template <typename T>
__global__ void __launch_bounds__(kMaxThreads)
k2_fwd_y_rk(const cplx<T>* __restrict__ F, NSK q, const cplx<T>* __restrict__ twy,
            int mode, RKArgs a) {
  using C = cplx<T>;
  C* buf = reinterpret_cast<C*>(g_smem_ns);
  C* buf2 = buf + (size_t)q.ny * q.LP;
  const int TX = q.TX, LP = q.LP;
  const int c0 = blockIdx.x * TX;
  for (int idx = threadIdx.x; idx < q.ny * TX; idx += blockDim.x) {
    const int c = idx % TX, iy = idx / TX, ix = c0 + c;
    buf[iy * LP + c] = ix < q.nkx ? F[(int64_t)iy * q.nkx + ix] : mk<C>(0, 0);
  }
  __syncthreads();
  fft_tile<-1, kTPT>(buf, buf2, q.ny, TX, LP, twy, 1);
  const T inv_n = T(q.inv_n);
  for (int idx = threadIdx.x; idx < q.ny * TX; idx += blockDim.x) {
    const int c = idx % TX, iy = idx / TX, ix = c0 + c;
    if (ix >= q.nkx) continue;
    const int64_t i = (int64_t)iy * q.nkx + ix;
    const int kyi = kadim(iy, q.ny);
    const bool rm = removed(q, ix, kyi, 0);
    const C N = cscale(buf[iy * LP + c], inv_n);
    const T kx = T(q.dkx * ix), ky = T(q.dky * kyi);
    stage_epilogue1<C, T>(mode, a, i, N, kx, ky, ix == 0 && kyi == 0, rm, phys(q));
  }
}

// ================================================================ solver
constexpr int kKinds = 5;     // A, inverse y, B, forward y, C
constexpr int kMaxEv = 2048;  // event pairs recorded before a harvest

constexpr int kHostBuf = 16;  // doubles in the pinned host mirror
// limit of a device-side wait for a staging copy (the copies take
// microseconds; a wait this long means the copy engine failed)
constexpr unsigned long long kStageTimeoutNs = 1000000000ull;

struct Solver {
  gbs_ns_params p;
  NSK q;
  int nvar;
  int64_t nK;
  size_t csize;
  void* tw[3];
  void* W;
  void* F;
  void* tmp;
  void* tmp1;
  void* tmp2;                // RK2_phaseshift_exact only (allocated at first use)
  unsigned long long* dmax;  // 3 maxima (double bits)
  int* dflag;                // [0] NaN flag, [1] staging status of the x pass (sticky)
  int stall_test;            // test hook for the next x pass (GBS_STEP_TEST_STALL)
  double* dred;              // reduction partials
  double* hbuf;              // pinned host mirror (kHostBuf doubles)
  double* hbuf_dev;          // the same memory in the device address space
  double shift[2][3];        // phase shifts alpha, beta (grid spacings per axis)
  // per-kernel timing (CUDA events on the launching stream) + launch count
  int timing;
  int nev;                  // event pairs in use
  cudaEvent_t ev[kMaxEv][2];
  int ev_kind[kMaxEv];
  double t_ms[kKinds];
  long long t_count[kKinds];
  long long launches;
  // turbulence model (ns3d): forcing buffer and its pipeline
  TurbCtx turb;
  void* turbF;
  const void* forcing;  // caller-owned forcing (nvar spectral fields) or null
  // compile-time-size path (all axes powers of two in range)
  int use_fast;
  fast::Geo geo;
  // launch shapes of the generic path
  int txA, txC, Lb;
  int thA, thB, thC;
  size_t smA, smB, smC;
};

// Harvest recorded event pairs into the per-kind totals (synchronises on
// the last recorded event).
static int harvest(Solver* s) {
  if (s->nev == 0) return GBS_OK;
  GBS_CUDA_TRY(cudaEventSynchronize(s->ev[s->nev - 1][1]));
  for (int i = 0; i < s->nev; ++i) {
    float ms = 0.f;
    GBS_CUDA_TRY(cudaEventElapsedTime(&ms, s->ev[i][0], s->ev[i][1]));
    s->t_ms[s->ev_kind[i]] += ms;
    s->t_count[s->ev_kind[i]] += 1;
  }
  s->nev = 0;
  return GBS_OK;
}

struct LaunchScope {
  Solver* s;
  int slot;
  cudaStream_t st;
  LaunchScope(Solver* s_, int kind, cudaStream_t st_) : s(s_), slot(-1), st(st_) {
    s->launches += 1;
    if (!s->timing) return;
    if (s->nev == kMaxEv) harvest(s);
    slot = s->nev++;
    s->ev_kind[slot] = kind;
    cudaEventRecord(s->ev[slot][0], st);
  }
  ~LaunchScope() {
    if (slot >= 0) cudaEventRecord(s->ev[slot][1], st);
  }
};

template <typename T>
static int setup_shapes(Solver* s) {
  const size_t cs = sizeof(cplx<T>);
  NSK& q = s->q;
  const int txmax = sizeof(T) == 4 ? 16 : 8;
  if (s->p.ndim == 3) {
    s->txA = pick_tx(q.nz, 6, cs, txmax, q.nkx);
    s->txC = pick_tx(q.nz, 3, cs, txmax, q.nkx);
    s->smA = tile_smem(q.nz, 6 * s->txA, cs);
    s->smC = tile_smem(q.nz, 3 * s->txC, cs);
    s->thA = tile_threads(q.nz, 6 * s->txA);
    s->thC = tile_threads(q.nz, 3 * s->txC);
    int L = sizeof(T) == 4 ? 8 : 4;
    const int64_t nrows = (int64_t)q.nz * q.ny;
    while (L > 1 && (tile_smem(q.M, 6 * L + 1, cs) > kSmemBudget ||
                     !tile_fits(q.M, 6 * L) || L / 2 >= nrows))
      L /= 2;
    s->Lb = L;
    s->smB = tile_smem(q.M, 6 * L + 1, cs);
    s->thB = tile_threads(q.M, 6 * L);
    int rc = allow_smem(k3_inv_z_curl<T>, s->smA);
    if (!rc) rc = allow_smem(k3_x_product<T>, s->smB);
    if (!rc) rc = allow_smem(k3_fwd_z_rk<T>, s->smC);
    if (rc) return rc;
    if (s->smA > kSmemMax - 1024 || s->smB > kSmemMax - 1024 || s->smC > kSmemMax - 1024 ||
        !tile_fits(q.nz, 6 * s->txA) || !tile_fits(q.nz, 3 * s->txC) ||
        !tile_fits(q.M, 6 * L)) {
      set_error("grid too large for the fused kernels");
      return GBS_EINVAL;
    }
  } else {
    s->txA = pick_tx(q.ny, 4, cs, txmax, q.nkx);
    s->txC = pick_tx(q.ny, 1, cs, txmax, q.nkx);
    s->smA = tile_smem(q.ny, 4 * s->txA, cs);
    s->smC = tile_smem(q.ny, s->txC, cs);
    s->thA = tile_threads(q.ny, 4 * s->txA);
    s->thC = tile_threads(q.ny, s->txC);
    int L = sizeof(T) == 4 ? 8 : 4;
    while (L > 1 && (tile_smem(q.M, 4 * L + 1, cs) > kSmemBudget ||
                     !tile_fits(q.M, 4 * L) || L / 2 >= q.ny))
      L /= 2;
    s->Lb = L;
    s->smB = tile_smem(q.M, 4 * L + 1, cs);
    s->thB = tile_threads(q.M, 4 * L);
    int rc = allow_smem(k2_inv_y<T>, s->smA);
    if (!rc) rc = allow_smem(k2_x_product<T>, s->smB);
    if (!rc) rc = allow_smem(k2_fwd_y_rk<T>, s->smC);
    if (rc) return rc;
    if (s->smA > kSmemMax - 1024 || s->smB > kSmemMax - 1024 || s->smC > kSmemMax - 1024 ||
        !tile_fits(q.ny, 4 * s->txA) || !tile_fits(q.ny, s->txC) ||
        !tile_fits(q.M, 4 * L)) {
      set_error("grid too large for the fused kernels");
      return GBS_EINVAL;
    }
  }
  return GBS_OK;
}

// One tendency evaluation from `in`; kernel C runs `mode`.
// phase shift lengths of shift `phase` (1: alpha, 2: beta) in units of the
// grid spacing times s->shift
static void shift_lengths(const Solver* s, int phase, double* sx, double* sy, double* sz) {
  const double* c = s->shift[phase == 2 ? 1 : 0];
  *sx = c[0] * (s->p.Lx / s->p.nx);
  *sy = c[1] * (s->p.Ly / s->p.ny);
  *sz = s->p.ndim == 3 ? c[2] * (s->p.Lz / s->p.nz) : 0.0;
}

static fast::Geo geo_for(const Solver* s, bool pruned, int phase = 0) {
  fast::Geo g = s->geo;
  g.pr = pruned ? 1 : 0;
  g.phase = phase ? 1 : 0;
  shift_lengths(s, phase, &g.sx, &g.sy, &g.sz);
  g.ncx = pruned ? (g.kcx < g.nkx ? g.kcx : g.nkx) : g.nkx;
  const int nkeep = 2 * g.kcy - 1;
  g.nky_keep = (pruned && nkeep < g.ny) ? nkeep : g.ny;
  return g;
}

// compile-time-size path: same passes as the generic one, optionally pruned
template <typename T>
static int eval_fast(Solver* s, const void* in, bool pruned, bool want_max, int phase,
                     cudaStream_t st) {
  const fast::Geo g = geo_for(s, pruned, phase);
  unsigned long long* vmax = want_max ? s->dmax : nullptr;
  int rc;
  const int kcy_in = pruned ? g.kcy : g.ny + 1;
  if (s->p.ndim == 3) {
    {
      LaunchScope ls(s, 0, st);
      rc = fast::A3<T>(g, in, s->W, s->tw[2], st);
    }
    if (rc) return rc;
    fast::ColArgs ca;
    ca.ncols = g.ncx;
    ca.kc_in = kcy_in;
    ca.kc_out = g.ny + 1;
    ca.es = g.nkx;
    ca.os = (int64_t)g.ny * g.nkx;
    ca.fs = s->nK;
    const int nW = g.strat ? 7 : 6, nF = g.strat ? 6 : 3;
    {
      LaunchScope ls(s, 1, st);
      rc = fast::col<T>(g.ny, s->W, s->W, ca, g.nz, nW, s->tw[1], 1.0, +1, st);
    }
    if (rc) return rc;
    {
      LaunchScope ls(s, 2, st);
      fast::XStage xs{s->dflag + 1, s->stall_test ? 1000000ull : kStageTimeoutNs,
                      s->stall_test};
      s->stall_test = 0;
      rc = fast::B3<T>(g, s->W, s->F, s->tw[0], vmax, xs, st);
    }
    if (rc) return rc;
    ca.kc_in = g.ny + 1;
    ca.kc_out = kcy_in;
    {
      LaunchScope ls(s, 3, st);
      rc = fast::col<T>(g.ny, s->F, s->F, ca, g.nz, nF, s->tw[1], 1.0, -1, st);
    }
    return rc;
  }
  {
    LaunchScope ls(s, 0, st);
    rc = fast::A2<T>(g, in, s->W, s->tw[1], st);
  }
  if (rc) return rc;
  LaunchScope ls(s, 2, st);
  return fast::B2<T>(g, s->W, s->F, s->tw[0], vmax, st);
}

template <typename T>
static int finish_fast(Solver* s, int mode, const RKArgs& a, bool pruned, cudaStream_t st) {
  const fast::Geo g = geo_for(s, pruned);
  LaunchScope ls(s, 4, st);
  if (s->p.ndim == 3) return fast::C3<T>(g, s->F, s->tw[2], mode, a, st);
  return fast::C2<T>(g, s->F, s->tw[1], mode, a, st);
}

template <typename T>
static int eval(Solver* s, const void* in, int mode, const RKArgs& a,
                bool want_max, cudaStream_t st, bool pruned = false, int phase = 0) {
  if (s->use_fast) return eval_fast<T>(s, in, pruned, want_max, phase, st);
  using C = cplx<T>;
  NSK q = s->q;
  q.phase = phase ? 1 : 0;
  shift_lengths(s, phase, &q.sx, &q.sy, &q.sz);
  const C* twx = static_cast<const C*>(s->tw[0]);
  const C* twy = static_cast<const C*>(s->tw[1]);
  const C* twz = static_cast<const C*>(s->tw[2]);
  C* W = static_cast<C*>(s->W);
  C* F = static_cast<C*>(s->F);
  unsigned long long* vmax = want_max ? s->dmax : nullptr;
  int rc;
  if (s->p.ndim == 3) {
    q.TX = s->txA;
    q.LP = 6 * q.TX;
    {
      LaunchScope ls(s, 0, st);
      k3_inv_z_curl<T><<<dim3(ceil_div(q.nkx, q.TX), q.ny), s->thA, s->smA, st>>>(
          static_cast<const C*>(in), W, q, twz);
    }
    GBS_CHECK_LAUNCH();
    {
      LaunchScope ls(s, 1, st);
      rc = launch_col<T, 1>(W, W, q.ny, q.nkx, q.nz, 6, q.nkx,
                            (int64_t)q.ny * q.nkx, s->nK, twy, T(1), st);
    }
    if (rc) return rc;
    q.L = s->Lb;
    q.LP = 6 * q.L + 1;
    {
      LaunchScope ls(s, 2, st);
      k3_x_product<T><<<ceil_div((int64_t)q.nz * q.ny, q.L), s->thB, s->smB, st>>>(
          W, F, q, twx, vmax);
    }
    GBS_CHECK_LAUNCH();
    {
      LaunchScope ls(s, 3, st);
      rc = launch_col<T, -1>(F, F, q.ny, q.nkx, q.nz, 3, q.nkx,
                             (int64_t)q.ny * q.nkx, s->nK, twy, T(1), st);
    }
    if (rc) return rc;
    return GBS_OK;
  }
  q.TX = s->txA;
  q.LP = 4 * q.TX;
  {
    LaunchScope ls(s, 0, st);
    k2_inv_y<T><<<ceil_div(q.nkx, q.TX), s->thA, s->smA, st>>>(
        static_cast<const C*>(in), W, q, twy);
  }
  GBS_CHECK_LAUNCH();
  q.L = s->Lb;
  q.LP = 4 * q.L + 1;
  {
    LaunchScope ls(s, 2, st);
    k2_x_product<T><<<ceil_div(q.ny, q.L), s->thB, s->smB, st>>>(W, F, q, twx, vmax);
  }
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

template <typename T>
static int finish(Solver* s, int mode, const RKArgs& a, cudaStream_t st,
                  bool pruned = false) {
  if (s->use_fast) return finish_fast<T>(s, mode, a, pruned, st);
  using C = cplx<T>;
  NSK q = s->q;
  const C* F = static_cast<const C*>(s->F);
  LaunchScope ls(s, 4, st);
  if (s->p.ndim == 3) {
    q.TX = s->txC;
    q.LP = 3 * q.TX;
    k3_fwd_z_rk<T><<<dim3(ceil_div(q.nkx, q.TX), q.ny), s->thC, s->smC, st>>>(
        F, q, static_cast<const C*>(s->tw[2]), mode, a);
  } else {
    q.TX = s->txC;
    q.LP = q.TX;
    k2_fwd_y_rk<T><<<ceil_div(q.nkx, q.TX), s->thC, s->smC, st>>>(
        F, q, static_cast<const C*>(s->tw[1]), mode, a);
  }
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

// turbulence-model forcing of the stage input `in` (null when disabled)
template <typename T>
static int turb_stage(Solver* s, const void* in, RKArgs& a, cudaStream_t st) {
  a.add = s->forcing;
  if (s->turb.type == kTurbNone) return GBS_OK;
  int rc = turb_forcing<T>(s->turb, in, s->turbF, s->forcing, st);
  if (rc) return rc;
  a.add = s->turbF;
  return GBS_OK;
}

template <typename T>
static int tendencies(Solver* s, const void* S, void* tend, cudaStream_t st) {
  RKArgs a{};
  a.tend = tend;
  a.in = S;
  int rc = eval<T>(s, S, kTend, a, false, st);
  if (rc) return rc;
  rc = turb_stage<T>(s, S, a, st);
  if (rc) return rc;
  return finish<T>(s, kTend, a, st);
}

// Small results (maxima, flags, means) reach the host through the pinned
// mirror, written by a kernel in the device address space of that host
// memory rather than copied: a copy would wait behind the bulk transfers
// that other streams may have queued on the copy engines.
__global__ void k_publish(const unsigned* __restrict__ src, unsigned* dst, int nwords) {
  if (threadIdx.x < nwords) dst[threadIdx.x] = src[threadIdx.x];
}

// bytes (a multiple of 4, at most 128) from device memory to hbuf[slot...];
// waits for the stream
static int publish(Solver* s, const void* src, int slot, size_t bytes, cudaStream_t st) {
  k_publish<<<1, 32, 0, st>>>(static_cast<const unsigned*>(src),
                              reinterpret_cast<unsigned*>(s->hbuf_dev + slot),
                              (int)(bytes / sizeof(unsigned)));
  GBS_CHECK_LAUNCH();
  ++s->launches;
  GBS_CUDA_TRY(cudaStreamSynchronize(st));
  return GBS_OK;
}

double cfl_rule(double dt, double tmp, double cfl, double dtmax) {
  // fluidsim/base/time_stepping/base.py:334-354
  double deltat_CFL = tmp > 0 ? cfl / tmp : dtmax;
  double maybe_new_dt = deltat_CFL < dtmax ? deltat_CFL : dtmax;
  double normalize_diff = fabs(dt - maybe_new_dt) / maybe_new_dt;
  if (normalize_diff > 0.02) dt = maybe_new_dt;
  return dt;
}

static double cfl_tmp(const Solver* s, const double* m) {
  // max_ux / deltax + max_uy / deltay (+ max_uz / deltaz), base.py:330-334
  double t = m[0] / (s->p.Lx / s->p.nx) + m[1] / (s->p.Ly / s->p.ny);
  if (s->p.ndim == 3) t += m[2] / (s->p.Lz / s->p.nz);
  return t;
}

// The stages of one time step of each scheme: the evaluation input (S or
// the intermediate state written by the previous stage) and the epilogue
// mode.  pseudo_spect.py: RK4 798-984, Euler 245-280, RK2 469-517,
// RK2_trapezoid 519-569.
// The phase-shift schemes evaluate some tendencies on exp(i phi) X and
// divide them by exp(i phi) (Euler_phaseshift 374-419, RK2_phaseshift
// 571-639, RK2_phaseshift_exact 712-796).
struct Stage {
  int input;  // 0: S, 1: tmp, 2: tmp1
  int mode;
  int phase;  // shifted evaluation: 0 none, 1 shift alpha, 2 shift beta
};
static int scheme_stages(int scheme, Stage* st) {
  switch (scheme) {
    case GBS_SCHEME_RK4:
      st[0] = {0, kRK0, 0}; st[1] = {2, kRK1, 0}; st[2] = {2, kRK2, 0}; st[3] = {2, kRK3, 0};
      return 4;
    case GBS_SCHEME_EULER:
      st[0] = {0, kEuler, 0};
      return 1;
    case GBS_SCHEME_RK2:
      st[0] = {0, kR2a, 0}; st[1] = {1, kR2b, 0};
      return 2;
    case GBS_SCHEME_RK2_TRAPEZOID:
      st[0] = {0, kHeunA, 0}; st[1] = {1, kHeunB, 0};
      return 2;
    case GBS_SCHEME_EULER_PHASESHIFT:
      st[0] = {0, kStoreTmp, 0}; st[1] = {0, kEulerPS, 1};
      return 2;
    case GBS_SCHEME_RK2_PHASESHIFT:
      st[0] = {0, kPS2a, 0}; st[1] = {1, kPS2b, 1};
      return 2;
    case GBS_SCHEME_RK2_PHASESHIFT_EXACT:
      st[0] = {0, kStoreTmp1, 0}; st[1] = {0, kPSXb, 1};
      st[2] = {1, kStoreTmp2, 0}; st[3] = {1, kPSXd, 1};
      return 4;
    // pseudo_spect.py:421-467: N_d = (N(alpha S)/alpha + N(beta S)/beta) / 2
    case GBS_SCHEME_EULER_PHASESHIFT_RANDOM:
      st[0] = {0, kStoreTmp, 1}; st[1] = {0, kEulerPS, 2};
      return 2;
    // pseudo_spect.py:641-710: N_0 = N(alpha S)/alpha, S_1 = (S + dt N_0) E,
    // N_d = (N_0 + N(beta S_1)/beta) / 2
    case GBS_SCHEME_RK2_PHASESHIFT_RANDOM:
      st[0] = {0, kPS2a, 1}; st[1] = {1, kPS2b, 2};
      return 2;
    default:
      return 0;
  }
}

template <typename T>
static int step(Solver* s, int scheme, void* S, double* dt, const double* cfl, int flags,
                cudaStream_t st) {
  const int check_nan = flags & GBS_STEP_CHECK_NAN;
  const bool pr = (flags & GBS_STEP_DEALIASED) != 0;
  s->stall_test = (flags & GBS_STEP_TEST_STALL) ? 1 : 0;
  Stage stages[4];
  const int nst = scheme_stages(scheme, stages);
  if (nst == 0) {
    set_error("unknown time scheme");
    return GBS_EINVAL;
  }
  bool shifted = false;
  for (int k = 0; k < nst; ++k) shifted = shifted || stages[k].phase;
  if (shifted && s->turb.type != 0) {
    set_error("phase-shift schemes with a turbulence model are not implemented");
    return GBS_EINVAL;
  }
  if (scheme == GBS_SCHEME_RK2_PHASESHIFT_EXACT && !s->tmp2) {
    // the one scheme with a third intermediate state: allocated at its first step
    GBS_CUDA_TRY(cudaStreamSynchronize(st));
    if (cudaMalloc(&s->tmp2, s->csize * s->nvar * s->nK) != cudaSuccess) {
      s->tmp2 = nullptr;
      set_error("out of device memory");
      return GBS_ENOMEM;
    }
    GBS_CUDA_TRY(cudaMemsetAsync(s->tmp2, 0, s->csize * s->nvar * s->nK, st));
  }
  RKArgs a{};
  a.S = S;
  a.Sout = S;
  a.tmp = s->tmp;
  a.tmp1 = s->tmp1;
  a.tmp2 = s->tmp2;
  a.nan_flag = s->dflag;
  int rc;
  if (cfl) GBS_CUDA_TRY(cudaMemsetAsync(s->dmax, 0, 3 * sizeof(unsigned long long), st));
  if (check_nan) GBS_CUDA_TRY(cudaMemsetAsync(s->dflag, 0, sizeof(int), st));
  // the CFL maxima are those of the physical state (base.py:320-339); a
  // scheme whose first evaluation is shifted (RK2_phaseshift_random) gets
  // them from an unshifted evaluation of its own
  const bool cfl_apart = cfl && stages[0].phase != 0;
  if (cfl_apart) {
    a.in = S;
    rc = eval<T>(s, S, kTend, a, true, st, pr, 0);
    if (rc) return rc;
    rc = publish(s, s->dmax, 0, 3 * sizeof(double), st);
    if (rc) return rc;
    *dt = cfl_rule(*dt, cfl_tmp(s, s->hbuf), cfl[0], cfl[1]);
  }
  for (int k = 0; k < nst; ++k) {
    const void* in = stages[k].input == 0 ? S : (stages[k].input == 1 ? s->tmp : s->tmp1);
    const int m = stages[k].mode;
    a.phase = stages[k].phase;
    shift_lengths(s, stages[k].phase, &a.sx, &a.sy, &a.sz);
    a.in = in;
    if (s->p.strat && stages[k].phase) {
      set_error("phase-shift schemes are not implemented for the strat solvers");
      return GBS_EINVAL;
    }
    rc = eval<T>(s, in, m, a, k == 0 && cfl && !cfl_apart, st, pr, stages[k].phase);
    if (rc) return rc;
    if (k == 0 && cfl && !cfl_apart) {
      rc = publish(s, s->dmax, 0, 3 * sizeof(double), st);
      if (rc) return rc;
      *dt = cfl_rule(*dt, cfl_tmp(s, s->hbuf), cfl[0], cfl[1]);
    }
    a.dt = *dt;
    a.fdt = (float)*dt;
    rc = turb_stage<T>(s, in, a, st);
    if (rc) return rc;
    rc = finish<T>(s, m, a, st, pr);
    if (rc) return rc;
  }
  if (check_nan) {
    rc = publish(s, s->dflag, 4, 2 * sizeof(int), st);
    if (rc) return rc;
    int flag[2];
    memcpy(flag, s->hbuf + 4, sizeof(flag));
    if (flag[1]) {  // reported once, then cleared
      GBS_CUDA_TRY(cudaMemsetAsync(s->dflag + 1, 0, sizeof(int), st));
      set_error("x pass: a staging copy did not arrive within the time limit "
                "(the step's result is not valid)");
      return GBS_ETIMEDOUT;
    }
    if (flag[0]) {
      set_error("nan in state_spect[0] after the time step");
      return GBS_ENAN;
    }
  }
  return GBS_OK;
}

template <typename T>
static int max_velocity(Solver* s, const void* S, double* out, cudaStream_t st) {
  RKArgs a{};
  GBS_CUDA_TRY(cudaMemsetAsync(s->dmax, 0, 3 * sizeof(unsigned long long), st));
  int rc = eval<T>(s, S, kTend, a, true, st);
  if (rc) return rc;
  rc = publish(s, s->dmax, 0, 3 * sizeof(double), st);
  if (rc) return rc;
  for (int i = 0; i < s->p.ndim; ++i) out[i] = s->hbuf[i];
  return GBS_OK;
}

// --------------------------------------------------- FP64 reductions
// Spatial means: per-mode quantities with Hermitian weights, block partial
// sums reduced in a fixed order (deterministic for a given launch shape).
constexpr int kRedBlocks = 304;
constexpr int kRedThreads = 256;
constexpr int kNQ = 9;
static_assert(kNQ <= kHostBuf, "the spatial means are read back through hbuf");

template <typename T>
__global__ void __launch_bounds__(kRedThreads)
k_means(const cplx<T>* __restrict__ S, NSK q, int ndim, int strat, double inv_N2,
        double* partial) {
  using C = cplx<T>;
  const int64_t nK = (int64_t)q.nz * q.ny * q.nkx;
  double acc[kNQ] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nK;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int ix = (int)(i % q.nkx);
    const int64_t r = i / q.nkx;
    const int iy = (int)(r % q.ny), iz = (int)(r / q.ny);
    const double w = (ix == 0 || (q.nx % 2 == 0 && ix == q.nx / 2)) ? 1.0 : 2.0;
    const double kx = q.dkx * ix, ky = q.dky * kadim(iy, q.ny);
    const double kz = ndim == 3 ? q.dkz * kadim(iz, q.nz) : 0.0;
    const double k2 = ndim == 3 ? kx * kx + ky * ky + kz * kz : kx * kx + ky * ky;
    const bool k0 = ix == 0 && kadim(iy, q.ny) == 0 && (ndim == 2 || kadim(iz, q.nz) == 0);
    double fd = q.nu2 > 0 ? q.nu2 * k2 : 0.0;
    if (q.nu4 > 0) fd += q.nu4 * (k2 * k2);
    if (q.nu8 > 0) fd += q.nu8 * ((k2 * k2) * (k2 * k2));
    double fh = 0.0;
    if (q.num4 != 0) {
      double kk = k0 ? q.k2_hypo0 : k2;
      fh = q.num4 / (kk * kk);
    }
    if (ndim == 3) {
      const C a = S[i], b = S[i + nK], c = S[i + 2 * nK];
      const double ex = 0.5 * ((double)a.x * a.x + (double)a.y * a.y);
      const double ey = 0.5 * ((double)b.x * b.x + (double)b.y * b.y);
      const double ez = 0.5 * ((double)c.x * c.x + (double)c.y * c.y);
      const double e = ex + ey + ez;
      acc[0] += w * e;
      acc[1] += w * ex;
      acc[2] += w * ey;
      acc[3] += w * ez;
      acc[4] += w * fd * 2 * e;
      acc[5] += w * fh * 2 * e;
      if (strat) {  // ns3d/strat/output/spatial_means.py:27-61
        const C bb = S[i + 3 * nK];
        const double ea = 0.5 * inv_N2 * ((double)bb.x * bb.x + (double)bb.y * bb.y);
        acc[6] += w * ea;
        acc[7] += w * fd * 2 * ea;
        acc[8] += w * fh * 2 * ea;
      }
    } else {
      const C rt = S[i];
      const double z = 0.5 * ((double)rt.x * rt.x + (double)rt.y * rt.y);
      const double e = k0 ? 0.0 : z / k2;  // |u|^2/2 = |rot|^2 / (2 k^2)
      acc[0] += w * e;
      acc[1] += w * z;
      acc[2] += w * fd * 2 * e;
      acc[3] += w * fh * 2 * e;
      acc[4] += w * fd * 2 * z;
      acc[5] += w * fh * 2 * z;
      if (strat) {  // ns2d/strat/output/__init__.py:85-109: EA = (|b| / N)^2 / 2
        const C bb = S[i + nK];
        const double ea = 0.5 * inv_N2 * ((double)bb.x * bb.x + (double)bb.y * bb.y);
        acc[6] += w * ea;
        acc[7] += w * fd * 2 * ea;
        acc[8] += w * fh * 2 * ea;
      }
    }
  }
  __shared__ double red[kNQ][kRedThreads];
#pragma unroll
  for (int k = 0; k < kNQ; ++k) red[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int s = kRedThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
#pragma unroll
      for (int k = 0; k < kNQ; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < kNQ) partial[threadIdx.x * kRedBlocks + blockIdx.x] = red[threadIdx.x][0];
}

__global__ void k_sum_partials(const double* partial, int nb, double* out) {
  const int k = threadIdx.x;
  if (k >= kNQ) return;
  double s = 0;
  for (int b = 0; b < nb; ++b) s += partial[k * kRedBlocks + b];
  out[k] = s;
}

template <typename T>
static int spatial_means(Solver* s, const void* S, double* out, cudaStream_t st) {
  const double inv_N2 = (s->p.strat && s->p.N != 0) ? 1.0 / (s->p.N * s->p.N) : 0.0;
  k_means<T><<<kRedBlocks, kRedThreads, 0, st>>>(static_cast<const cplx<T>*>(S),
                                                  s->q, s->p.ndim, s->p.strat, inv_N2,
                                                  s->dred);
  GBS_CHECK_LAUNCH();
  k_sum_partials<<<1, 32, 0, st>>>(s->dred, kRedBlocks, s->dred + kNQ * kRedBlocks);
  GBS_CHECK_LAUNCH();
  const int rc = publish(s, s->dred + kNQ * kRedBlocks, 0, kNQ * sizeof(double), st);
  if (rc) return rc;
  for (int k = 0; k < kNQ; ++k) out[k] = s->hbuf[k];
  return GBS_OK;
}

static int64_t spectrum_bins(const Solver* s) {
  const NSK& q = s->q;
  double dk = q.dkx < q.dky ? q.dkx : q.dky;
  if (s->p.ndim == 3 && q.dkz < dk) dk = q.dkz;
  double kx = q.dkx * (q.nkx - 1), ky = q.dky * (q.ny / 2), kz = q.dkz * (q.nz / 2);
  double kmax = sqrt(kx * kx + ky * ky + (s->p.ndim == 3 ? kz * kz : 0.0));
  return (int64_t)floor(kmax / dk + 0.5) + 1;
}

// flag = 1 if a removed mode of any field is not +0 (bitwise).  One CTA per
// kx row (iy, iz): a row whose ky or kz is cut is removed whole, the others
// from kx = kcut_x on; no index division.
template <typename T>
__global__ void k_removed_nonzero(const cplx<T>* __restrict__ S, NSK q, int nvar,
                                  int* __restrict__ flag) {
  const int iz = blockIdx.x, iy = blockIdx.y;  // nz on x: it may exceed 65535
  const int64_t nK = (int64_t)q.nz * q.ny * q.nkx;
  const int kz = q.nz > 1 ? kadim(iz, q.nz) : 0;
  const int ix0 = removed(q, 0, kadim(iy, q.ny), kz) ? 0 : q.kcx;
  const cplx<T>* row = S + ((int64_t)iz * q.ny + iy) * q.nkx;
  bool nz = false;
  for (int ix = ix0 + threadIdx.x; ix < q.nkx; ix += blockDim.x) {
    for (int f = 0; f < nvar; ++f) {
      const cplx<T> v = row[ix + f * nK];
      nz = nz || v.x != T(0) || v.y != T(0) || signbit(v.x) || signbit(v.y);
    }
  }
  if (__syncthreads_or(nz) && threadIdx.x == 0) *flag = 1;
}

template <typename T>
__global__ void k_spectrum(const cplx<T>* __restrict__ S, NSK q, int ndim,
                           double dk, int64_t nbins, double* spec) {
  using C = cplx<T>;
  const int64_t nK = (int64_t)q.nz * q.ny * q.nkx;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nK;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int ix = (int)(i % q.nkx);
    const int64_t r = i / q.nkx;
    const int iy = (int)(r % q.ny), iz = (int)(r / q.ny);
    const double w = (ix == 0 || (q.nx % 2 == 0 && ix == q.nx / 2)) ? 1.0 : 2.0;
    const double kx = q.dkx * ix, ky = q.dky * kadim(iy, q.ny);
    const double kz = ndim == 3 ? q.dkz * kadim(iz, q.nz) : 0.0;
    const double k2 = kx * kx + ky * ky + kz * kz;
    double e;
    if (ndim == 3) {
      const C a = S[i], b = S[i + nK], c = S[i + 2 * nK];
      e = 0.5 * ((double)a.x * a.x + (double)a.y * a.y + (double)b.x * b.x +
                 (double)b.y * b.y + (double)c.x * c.x + (double)c.y * c.y);
    } else {
      const C rt = S[i];
      e = k2 > 0 ? 0.5 * ((double)rt.x * rt.x + (double)rt.y * rt.y) / k2 : 0.0;
    }
    int64_t b = (int64_t)floor(sqrt(k2) / dk + 0.5);
    if (b >= nbins) b = nbins - 1;
    atomicAdd(spec + b, w * e / dk);
  }
}

}  // namespace gbs

using gbs::Solver;

struct gbs_ns {
  Solver s;
};

static void free_turb(Solver* s) {
  gbs::TurbCtx& t = s->turb;
  if (t.plan9) gbs_fft_plan_destroy(t.plan9);
  if (t.plan6) gbs_fft_plan_destroy(t.plan6);
  void* ptrs[] = {t.Gk, t.Gx, t.Tx, t.Tk, s->turbF};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  memset(&t, 0, sizeof(t));
  s->turbF = nullptr;
}

static void free_solver(Solver* s) {
  free_turb(s);
  if (s->timing >= 0 && s->ev[0][0]) {
    for (int i = 0; i < gbs::kMaxEv; ++i) {
      cudaEventDestroy(s->ev[i][0]);
      cudaEventDestroy(s->ev[i][1]);
    }
  }
  for (void* t : s->tw)
    if (t) cudaFree(t);
  void* ptrs[] = {s->W, s->F, s->tmp, s->tmp1, s->tmp2, s->dmax, s->dflag, s->dred};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (s->hbuf) cudaFreeHost(s->hbuf);
}

namespace gbs {
int twiddle_alloc(void** out, int n, int dtype, cudaStream_t st);
}

extern "C" {

double gbs_cfl_update(double dt, double tmp, double cfl_coef,
                      double deltat_max) {
  return gbs::cfl_rule(dt, tmp, cfl_coef, deltat_max);
}

int gbs_ns_create(const gbs_ns_params* prm, gbs_ns** out) {
  gbs::clear_error();
  if (!prm || !out) {
    gbs::set_error("gbs_ns_create: null argument");
    return GBS_EINVAL;
  }
  *out = nullptr;
  const gbs_ns_params& p = *prm;
  if ((p.ndim != 2 && p.ndim != 3) || (p.dtype != GBS_F32 && p.dtype != GBS_F64) ||
      p.nx < 2 || p.nx % 2 || p.ny < 1 || p.nz < 1 || (p.ndim == 2 && p.nz != 1) ||
      p.nx > 65536 || p.ny > 65535 || p.nz > 65536 || !(p.Lx > 0) || !(p.Ly > 0) ||
      (p.ndim == 3 && !(p.Lz > 0))) {
    gbs::set_error("gbs_ns_create: invalid parameters (nx must be even)");
    return GBS_EINVAL;
  }
  if (p.strat && !gbs::fast::supported(p.ndim, (int)p.nx, (int)p.ny, (int)p.nz)) {
    gbs::set_error("gbs_ns_create: ns2d.strat / ns3d.strat run on power-of-two grids "
                   "(32..1024 per axis, nx/2 >= 32)");
    return GBS_EINVAL;
  }
  gbs_ns* h = new (std::nothrow) gbs_ns();
  if (!h) return GBS_ENOMEM;
  Solver* s = &h->s;
  memset(s, 0, sizeof(*s));
  s->p = p;
  s->nvar = p.ndim == 3 ? (p.strat ? 4 : 3) : (p.strat ? 2 : 1);
  gbs::NSK& q = s->q;
  q.nx = (int)p.nx;
  q.ny = (int)p.ny;
  q.nz = (int)p.nz;
  q.nkx = q.nx / 2 + 1;
  q.M = q.nx / 2;
  q.kcx = (int)(p.kcut_x < p.nx ? p.kcut_x : p.nx + 1);
  q.kcy = (int)(p.kcut_y < p.ny ? p.kcut_y : p.ny + 1);
  q.kcz = p.ndim == 3 ? (int)(p.kcut_z < p.nz ? p.kcut_z : p.nz + 1) : 1 << 30;
  const double pi2 = 6.283185307179586;
  q.dkx = pi2 / p.Lx;
  q.dky = pi2 / p.Ly;
  q.dkz = p.ndim == 3 ? pi2 / p.Lz : 0.0;
  q.nu2 = p.nu_2;
  q.nu4 = p.nu_4;
  q.nu8 = p.nu_8;
  q.num4 = p.nu_m4;
  q.beta = p.beta;
  q.f = p.f;
  q.has_f = p.ndim == 3 && p.has_f;
  q.inv_n = 1.0 / ((double)p.nx * p.ny * p.nz);
  q.k2_hypo0 = q.dkx * q.dkx;
  s->nK = (int64_t)q.nz * q.ny * q.nkx;
  s->csize = p.dtype == GBS_F64 ? sizeof(double2) : sizeof(float2);
  int rc = 0;
  int ns[3] = {q.nx, q.ny, q.nz};
  for (int a = 0; a < 3 && !rc; ++a) rc = gbs::twiddle_alloc(&s->tw[a], ns[a], p.dtype, 0);
  const size_t fb = s->csize * s->nK;
  // inverse-transformed fields (v, omega (+ b)) and products (v x omega (+ v b))
  const int nW = p.ndim == 3 ? (p.strat ? 7 : 6) : (p.strat ? 6 : 4);
  const int nF = p.ndim == 3 ? (p.strat ? 6 : 3) : (p.strat ? 2 : 1);
  if (!rc) {
    if (cudaMalloc(&s->W, fb * nW) != cudaSuccess ||
        cudaMalloc(&s->F, fb * nF) != cudaSuccess ||
        cudaMalloc(&s->tmp, fb * s->nvar) != cudaSuccess ||
        cudaMalloc(&s->tmp1, fb * s->nvar) != cudaSuccess ||
        cudaMalloc(&s->dmax, 4 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&s->dflag, 2 * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&s->dred, sizeof(double) * (gbs::kNQ * gbs::kRedBlocks + 16)) != cudaSuccess ||
        cudaHostAlloc(&s->hbuf, gbs::kHostBuf * sizeof(double), cudaHostAllocMapped) !=
            cudaSuccess ||
        cudaHostGetDevicePointer(&s->hbuf_dev, s->hbuf, 0) != cudaSuccess) {
      gbs::set_error("gbs_ns_create: device allocation failed (%zu MB requested)",
                     (size_t)(fb * (nW + nF + 2 * s->nvar) >> 20));
      rc = GBS_ENOMEM;
    }
  }
  if (!rc && cudaMemset(s->dflag, 0, 2 * sizeof(int)) != cudaSuccess) {
    gbs::set_error("gbs_ns_create: %s", cudaGetErrorString(cudaGetLastError()));
    rc = GBS_ECUDA;
  }
  if (!rc) rc = p.dtype == GBS_F64 ? gbs::setup_shapes<double>(s) : gbs::setup_shapes<float>(s);
  if (!rc) {
    s->use_fast = gbs::fast::supported(p.ndim, q.nx, q.ny, q.nz) ? 1 : 0;
    for (int k = 0; k < 2; ++k)
      for (int d = 0; d < 3; ++d) s->shift[k][d] = 0.5;
    gbs::fast::Geo& g = s->geo;
    g.nx = q.nx;
    g.ny = q.ny;
    g.nz = q.nz;
    g.nkx = q.nkx;
    g.M = q.M;
    g.kcx = q.kcx;
    g.kcy = q.kcy;
    g.kcz = q.kcz;
    g.ncx = q.nkx;
    g.nky_keep = q.ny;
    g.pr = 0;
    g.dkx = q.dkx;
    g.dky = q.dky;
    g.dkz = q.dkz;
    g.nu2 = q.nu2;
    g.nu4 = q.nu4;
    g.nu8 = q.nu8;
    g.num4 = q.num4;
    g.beta = q.beta;
    g.f = q.f;
    g.inv_n = q.inv_n;
    g.k2_hypo0 = q.k2_hypo0;
    g.has_f = q.has_f;
    g.strat = p.strat ? 1 : 0;
    g.N2 = p.bouss ? 0.0 : p.N * p.N;
    gbs::fast::geo_f32(g);
  }
  if (!rc) {
    // tmp / tmp1 start at zero so that modes never written stay zero
    if (cudaMemset(s->tmp, 0, fb * s->nvar) != cudaSuccess ||
        cudaMemset(s->tmp1, 0, fb * s->nvar) != cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess) {
      gbs::set_error("gbs_ns_create: %s", cudaGetErrorString(cudaGetLastError()));
      rc = GBS_ECUDA;
    }
  }
  if (rc) {
    free_solver(s);
    delete h;
    return rc;
  }
  *out = h;
  return GBS_OK;
}

int gbs_ns_destroy(gbs_ns* h) {
  if (!h) return GBS_OK;
  free_solver(&h->s);
  delete h;
  return GBS_OK;
}

int gbs_ns_tendencies(gbs_ns* h, const void* S, void* tend, void* stream) {
  gbs::clear_error();
  if (!h || !S || !tend) {
    gbs::set_error("gbs_ns_tendencies: null argument");
    return GBS_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (h->s.p.dtype == GBS_F64) return gbs::tendencies<double>(&h->s, S, tend, st);
  return gbs::tendencies<float>(&h->s, S, tend, st);
}

int gbs_ns_step(gbs_ns* h, int scheme, void* S, double* dt, const double* cfl, int flags,
                void* stream) {
  gbs::clear_error();
  if (!h || !S || !dt || !(*dt > 0) || scheme < GBS_SCHEME_RK4 ||
      scheme > GBS_SCHEME_RK2_PHASESHIFT_RANDOM) {
    gbs::set_error("gbs_ns_step: invalid argument");
    return GBS_EINVAL;
  }
  if (cfl && (!(cfl[0] > 0) || !(cfl[1] > 0))) {
    gbs::set_error("gbs_ns_step: invalid CFL parameters");
    return GBS_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (h->s.p.dtype == GBS_F64) return gbs::step<double>(&h->s, scheme, S, dt, cfl, flags, st);
  return gbs::step<float>(&h->s, scheme, S, dt, cfl, flags, st);
}

int gbs_ns_step_rk4(gbs_ns* h, void* S, double* dt, const double* cfl,
                    int flags, void* stream) {
  return gbs_ns_step(h, GBS_SCHEME_RK4, S, dt, cfl, flags, stream);
}

int gbs_ns_max_velocity(gbs_ns* h, const void* S, double* out, void* stream) {
  gbs::clear_error();
  if (!h || !S || !out) {
    gbs::set_error("gbs_ns_max_velocity: null argument");
    return GBS_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (h->s.p.dtype == GBS_F64) return gbs::max_velocity<double>(&h->s, S, out, st);
  return gbs::max_velocity<float>(&h->s, S, out, st);
}

int gbs_ns_spatial_means(gbs_ns* h, const void* S, double* out, void* stream) {
  gbs::clear_error();
  if (!h || !S || !out) {
    gbs::set_error("gbs_ns_spatial_means: null argument");
    return GBS_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (h->s.p.dtype == GBS_F64) return gbs::spatial_means<double>(&h->s, S, out, st);
  return gbs::spatial_means<float>(&h->s, S, out, st);
}

int gbs_ns_set_turb_model(gbs_ns* h, int type, double C,
                          const gbs_mlp_weights* w) {
  gbs::clear_error();
  if (!h || type < 0 || type > 3 || (type >= 2 && !w)) {
    gbs::set_error("gbs_ns_set_turb_model: invalid argument");
    return GBS_EINVAL;
  }
  Solver* s = &h->s;
  if (s->p.ndim != 3 && type != 0) {
    gbs::set_error("gbs_ns_set_turb_model: turbulence models are for ns3d");
    return GBS_EINVAL;
  }
  GBS_CUDA_TRY(cudaDeviceSynchronize());
  free_turb(s);
  if (type == 0) return GBS_OK;
  gbs::TurbCtx& t = s->turb;
  t.type = type;
  t.nx = s->q.nx;
  t.ny = s->q.ny;
  t.nz = s->q.nz;
  t.dkx = s->q.dkx;
  t.dky = s->q.dky;
  t.dkz = s->q.dkz;
  t.C_nu_T = C * (s->p.Lx / s->p.nx) * (s->p.Lx / s->p.nx) * sqrt(2.0);
  if (type >= 2) {
    t.w.W1 = static_cast<const __nv_bfloat16*>(w->W1);
    t.w.W2 = static_cast<const __nv_bfloat16*>(w->W2);
    t.w.W3 = static_cast<const __nv_bfloat16*>(w->W3);
    t.w.b1 = w->b1;
    t.w.b2 = w->b2;
    t.w.b3 = w->b3;
    t.w.in_scale = w->in_scale;
    t.w.out_scale = w->out_scale;
  }
  const int64_t shape[3] = {s->p.nz, s->p.ny, s->p.nx};
  int rc = gbs_fft_plan_create(3, shape, s->p.dtype, 9, &t.plan9);
  if (!rc) rc = gbs_fft_plan_create(3, shape, s->p.dtype, 6, &t.plan6);
  const size_t rs = s->p.dtype == GBS_F64 ? sizeof(double) : sizeof(float);
  const size_t nX = (size_t)s->p.nx * s->p.ny * s->p.nz;
  if (!rc && (cudaMalloc(&t.Gk, s->csize * s->nK * 9) != cudaSuccess ||
              cudaMalloc(&t.Gx, rs * nX * 9) != cudaSuccess ||
              cudaMalloc(&t.Tx, rs * nX * 6) != cudaSuccess ||
              cudaMalloc(&t.Tk, s->csize * s->nK * 6) != cudaSuccess ||
              cudaMalloc(&s->turbF, s->csize * s->nK * 3) != cudaSuccess)) {
    gbs::set_error("gbs_ns_set_turb_model: device allocation failed");
    rc = GBS_ENOMEM;
  }
  if (rc) {
    free_turb(s);
    return rc;
  }
  return GBS_OK;
}

int gbs_ns_set_forcing(gbs_ns* h, const void* forcing) {
  gbs::clear_error();
  if (!h) {
    gbs::set_error("gbs_ns_set_forcing: null solver");
    return GBS_EINVAL;
  }
  h->s.forcing = forcing;
  return GBS_OK;
}

int gbs_ns_timing(gbs_ns* h, int enable) {
  gbs::clear_error();
  if (!h) {
    gbs::set_error("gbs_ns_timing: null solver");
    return GBS_EINVAL;
  }
  Solver* s = &h->s;
  if (enable && !s->ev[0][0]) {
    for (int i = 0; i < gbs::kMaxEv; ++i) {
      GBS_CUDA_TRY(cudaEventCreate(&s->ev[i][0]));
      GBS_CUDA_TRY(cudaEventCreate(&s->ev[i][1]));
    }
  }
  if (enable) {
    s->nev = 0;
    for (int k = 0; k < gbs::kKinds; ++k) {
      s->t_ms[k] = 0;
      s->t_count[k] = 0;
    }
  }
  s->timing = enable ? 1 : 0;
  return GBS_OK;
}

int gbs_ns_timing_report(gbs_ns* h, double* ms, int64_t* count, int nkinds,
                         int64_t* launches) {
  gbs::clear_error();
  if (!h || nkinds < 0) {
    gbs::set_error("gbs_ns_timing_report: invalid argument");
    return GBS_EINVAL;
  }
  Solver* s = &h->s;
  int rc = gbs::harvest(s);
  if (rc) return rc;
  for (int k = 0; k < nkinds && k < gbs::kKinds; ++k) {
    if (ms) ms[k] = s->t_ms[k];
    if (count) count[k] = s->t_count[k];
  }
  if (launches) *launches = s->launches;
  return GBS_OK;
}

int gbs_ns_set_projection(gbs_ns* h, int projection, int no_vz_kz0) {
  gbs::clear_error();
  if (!h || projection < GBS_PROJ_PERPK || projection > GBS_PROJ_POLOIDAL ||
      (h->s.p.ndim != 3 && (projection != GBS_PROJ_PERPK || no_vz_kz0))) {
    gbs::set_error("gbs_ns_set_projection: invalid argument (ns3d only)");
    return GBS_EINVAL;
  }
  h->s.q.proj = h->s.geo.proj = projection;
  h->s.q.no_vz_kz0 = h->s.geo.no_vz_kz0 = no_vz_kz0 ? 1 : 0;
  return GBS_OK;
}

int gbs_ns_set_phase_shifts(gbs_ns* h, const double* alpha, const double* beta) {
  gbs::clear_error();
  if (!h || !alpha || !beta) {
    gbs::set_error("gbs_ns_set_phase_shifts: null argument");
    return GBS_EINVAL;
  }
  for (int d = 0; d < 3; ++d) {
    if (!std::isfinite(alpha[d]) || !std::isfinite(beta[d])) {
      gbs::set_error("gbs_ns_set_phase_shifts: non-finite shift");
      return GBS_EINVAL;
    }
    h->s.shift[0][d] = alpha[d];
    h->s.shift[1][d] = beta[d];
  }
  return GBS_OK;
}

int gbs_ns_is_dealiased(gbs_ns* h, const void* S, int* out, void* stream) {
  gbs::clear_error();
  if (!h || !S || !out) {
    gbs::set_error("gbs_ns_is_dealiased: null argument");
    return GBS_EINVAL;
  }
  gbs::Solver* s = &h->s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  GBS_CUDA_TRY(cudaMemsetAsync(s->dflag, 0, sizeof(int), st));
  if (s->p.dtype == GBS_F64)
    gbs::k_removed_nonzero<double><<<dim3(s->q.nz, s->q.ny), 128, 0, st>>>(
        static_cast<const double2*>(S), s->q, s->nvar, s->dflag);
  else
    gbs::k_removed_nonzero<float><<<dim3(s->q.nz, s->q.ny), 128, 0, st>>>(
        static_cast<const float2*>(S), s->q, s->nvar, s->dflag);
  GBS_CHECK_LAUNCH();
  ++s->launches;
  const int rc = gbs::publish(s, s->dflag, 5, sizeof(int), st);
  if (rc) return rc;
  int flag;
  memcpy(&flag, s->hbuf + 5, sizeof(int));
  *out = flag ? 0 : 1;
  return GBS_OK;
}

int gbs_ns_spectrum_size(gbs_ns* h, int64_t* nk) {
  gbs::clear_error();
  if (!h || !nk) {
    gbs::set_error("gbs_ns_spectrum_size: null argument");
    return GBS_EINVAL;
  }
  *nk = gbs::spectrum_bins(&h->s);
  return GBS_OK;
}

int gbs_ns_spectrum(gbs_ns* h, const void* S, double* spec, void* stream) {
  gbs::clear_error();
  if (!h || !S || !spec) {
    gbs::set_error("gbs_ns_spectrum: null argument");
    return GBS_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  Solver* s = &h->s;
  const int64_t nb = gbs::spectrum_bins(s);
  double dk = s->q.dkx < s->q.dky ? s->q.dkx : s->q.dky;
  if (s->p.ndim == 3 && s->q.dkz < dk) dk = s->q.dkz;
  GBS_CUDA_TRY(cudaMemsetAsync(spec, 0, nb * sizeof(double), st));
  if (s->p.dtype == GBS_F64)
    gbs::k_spectrum<double><<<gbs::kRedBlocks, gbs::kRedThreads, 0, st>>>(
        static_cast<const double2*>(S), s->q, s->p.ndim, dk, nb, spec);
  else
    gbs::k_spectrum<float><<<gbs::kRedBlocks, gbs::kRedThreads, 0, st>>>(
        static_cast<const float2*>(S), s->q, s->p.ndim, dk, nb, spec);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

}  // extern "C"
