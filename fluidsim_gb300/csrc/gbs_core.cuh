// Core FFT building blocks shared by every kernel of libgbspec.
//
// Data layout inside a CTA ("interleaved tile"): a tile holds `nlines`
// independent lines of length `n`; element j of line l sits at
// buf[j * LP + l] (LP >= nlines is the line pitch).  Consecutive threads
// work on consecutive lines, so shared-memory accesses of a warp are
// contiguous, and column tiles of a row-major array arrive in this layout
// straight from coalesced global loads.
//
// Power-of-two lines use a Stockham autosort FFT (radix-8 stages plus one
// radix-4 or radix-2 stage): each thread keeps 8 complex values per task in
// registers, the tile is exchanged through shared memory between stages.
// Twiddles come from a per-axis table W[k] = exp(-2 pi i k / N) generated in
// float64 (sincospi) and rounded to the working precision.
// Other lengths use a direct DFT on the tile (O(n^2) per line, exact
// twiddles from the same table); they only occur for small test grids.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#ifdef __CUDACC__
#define GBS_HD __host__ __device__ __forceinline__
#else
#define GBS_HD inline
#endif

namespace gbs {

template <typename T> struct cvec;
template <> struct cvec<float> { using type = float2; };
template <> struct cvec<double> { using type = double2; };
template <typename T> using cplx = typename cvec<T>::type;

template <typename C> GBS_HD C mk(decltype(C::x) a, decltype(C::x) b) { C r; r.x = a; r.y = b; return r; }

// FP32 complex add / subtract as one packed instruction on the paired
// registers (add.rn.f32x2 / sub.rn.f32x2, sm_100 and later): each component
// is rounded exactly as by the scalar instruction, so results are unchanged
// and the butterflies issue half the FP32 adds.  -DGBS_NO_F32X2 turns it off.
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 1000) && !defined(GBS_NO_F32X2)
#define GBS_F32X2 1
__device__ __forceinline__ float2 f32x2_add(float2 a, float2 b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;"
      : "=l"(d)
      : "l"(*reinterpret_cast<const unsigned long long*>(&a)),
        "l"(*reinterpret_cast<const unsigned long long*>(&b)));
  return *reinterpret_cast<const float2*>(&d);
}
__device__ __forceinline__ float2 f32x2_sub(float2 a, float2 b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;"
      : "=l"(d)
      : "l"(*reinterpret_cast<const unsigned long long*>(&a)),
        "l"(*reinterpret_cast<const unsigned long long*>(&b)));
  return *reinterpret_cast<const float2*>(&d);
}
#endif

template <typename C> GBS_HD C cadd(C a, C b) {
#ifdef GBS_F32X2
  if constexpr (sizeof(C) == 8) return f32x2_add(a, b);
#endif
  return mk<C>(a.x + b.x, a.y + b.y);
}
template <typename C> GBS_HD C csub(C a, C b) {
#ifdef GBS_F32X2
  if constexpr (sizeof(C) == 8) return f32x2_sub(a, b);
#endif
  return mk<C>(a.x - b.x, a.y - b.y);
}
template <typename C> GBS_HD C cmul(C a, C b) {
  return mk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename C> GBS_HD C cmulc(C a, C b) {
  return mk<C>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename C> GBS_HD C cconj(C a) { return mk<C>(a.x, -a.y); }
template <typename C, typename R> GBS_HD C cscale(C a, R s) { return mk<C>(a.x * s, a.y * s); }
// a * (s i), s = +1 or -1
template <int S, typename C> GBS_HD C mul_si(C a) {
  return S > 0 ? mk<C>(-a.y, a.x) : mk<C>(a.y, -a.x);
}

#ifdef __CUDACC__
// 1 / x correctly rounded (the IEEE quotient 1 / x): the reciprocal
// intrinsic in FP32, plain division in FP64.
__device__ __forceinline__ float crcp(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double crcp(double x) { return 1.0 / x; }
#endif

GBS_HD bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
GBS_HD int ilog2(int n) { int l = 0; while ((1 << l) < n) ++l; return l; }

// ---------------------------------------------------------------- butterflies
// DIR = -1: forward (exp(-2 pi i jk/R)); DIR = +1: inverse (unnormalised).
template <int DIR, typename C> GBS_HD void dft2(C* v) {
  C a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <int DIR, typename C> GBS_HD void dft4(C* v) {
  C s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
  C s13 = cadd(v[1], v[3]), d13 = mul_si<DIR>(csub(v[1], v[3]));
  v[0] = cadd(s02, s13);
  v[2] = csub(s02, s13);
  v[1] = cadd(d02, d13);
  v[3] = csub(d02, d13);
}

template <int DIR, typename C> GBS_HD void dft8(C* v) {
  using R = decltype(C::x);
  const R h = R(0.70710678118654752440084436210484903928);
  C e[4] = {v[0], v[2], v[4], v[6]};
  C o[4] = {v[1], v[3], v[5], v[7]};
  dft4<DIR>(e);
  dft4<DIR>(o);
  // W8 = exp(DIR 2 pi i / 8) = h (1 + DIR i)
  C o1 = mk<C>(h * (o[1].x - DIR * o[1].y), h * (o[1].y + DIR * o[1].x));
  C o2 = mul_si<DIR>(o[2]);
  C o3 = mk<C>(h * (-o[3].x - DIR * o[3].y), h * (-o[3].y + DIR * o[3].x));
  v[0] = cadd(e[0], o[0]);
  v[4] = csub(e[0], o[0]);
  v[1] = cadd(e[1], o1);
  v[5] = csub(e[1], o1);
  v[2] = cadd(e[2], o2);
  v[6] = csub(e[2], o2);
  v[3] = cadd(e[3], o3);
  v[7] = csub(e[3], o3);
}

template <int R, int DIR, typename C> GBS_HD void dftR(C* v) {
  if (R == 2) dft2<DIR>(v);
  else if (R == 4) dft4<DIR>(v);
  else dft8<DIR>(v);
}

// twiddle W^k (DIR=-1) or conj(W^k) (DIR=+1) from the forward table
template <int DIR, typename C> GBS_HD C twid(const C* tw, int k) {
  C w = tw[k];
  if (DIR > 0) w.y = -w.y;
  return w;
}

// ------------------------------------------------ power-of-two Stockham stage
// One stage of radix R on all lines of the tile.  A task is (line, jt) with
// jt in [0, n/8); it owns 8 elements: 8/R butterflies b = jt + q n/8.
// TPT tasks per thread.  Phase 0 loads + twiddles + butterflies into `v`,
// phase 1 stores; the caller separates the phases with a barrier.
template <int R, int DIR, int TPT, typename C>
GBS_HD void stockham_load(const C* buf, C (*v)[8], int n, int log2n, int Ns,
                          int log2Ns, int nlines, int LP, const C* tw,
                          int tw_stride, int tid, int nthreads) {
  const int ntasks = nlines * (n >> 3);
  const int nR = n / R;
  const int logR = (R == 2) ? 1 : (R == 4 ? 2 : 3);
  const int twmul = (1 << (log2n - log2Ns - logR)) * tw_stride;
#pragma unroll
  for (int q = 0; q < TPT; ++q) {
    int task = tid + q * nthreads;
    if (task >= ntasks) break;
    int l = task % nlines;
    int jt = task / nlines;
#pragma unroll
    for (int g = 0; g < 8 / R; ++g) {
      int b = jt + g * (n >> 3);
      int bm = b & (Ns - 1);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        C x = buf[(b + r * nR) * LP + l];
        if (Ns > 1 && r > 0) x = cmul(x, twid<DIR>(tw, r * bm * twmul));
        v[q][g * R + r] = x;
      }
      dftR<R, DIR>(&v[q][g * R]);
    }
  }
}

template <int R, int TPT, typename C>
GBS_HD void stockham_store(C* buf, C (*v)[8], int n, int Ns, int log2Ns,
                           int nlines, int LP, int tid, int nthreads) {
  const int ntasks = nlines * (n >> 3);
#pragma unroll
  for (int q = 0; q < TPT; ++q) {
    int task = tid + q * nthreads;
    if (task >= ntasks) break;
    int l = task % nlines;
    int jt = task / nlines;
#pragma unroll
    for (int g = 0; g < 8 / R; ++g) {
      int b = jt + g * (n >> 3);
      int d = ((b >> log2Ns) << log2Ns) * R + (b & (Ns - 1));
#pragma unroll
      for (int r = 0; r < R; ++r) buf[(d + r * Ns) * LP + l] = v[q][g * R + r];
    }
  }
}

// --------------------------------------------------------- generic direct DFT
// out[k] = sum_j in[j] W^(jk mod n); result written to buf2.
template <int DIR, typename C>
GBS_HD void dft_direct_part(const C* buf, C* buf2, int n, int nlines, int LP,
                            const C* tw, int tw_stride, int tid, int nthreads) {
  using Rl = decltype(C::x);
  const int total = nlines * n;
  for (int idx = tid; idx < total; idx += nthreads) {
    int l = idx % nlines;
    int k = idx / nlines;
    Rl ax = 0, ay = 0;
    int w = 0;
    for (int j = 0; j < n; ++j) {
      C x = buf[j * LP + l];
      C t = twid<DIR>(tw, w * tw_stride);
      ax += x.x * t.x - x.y * t.y;
      ay += x.x * t.y + x.y * t.x;
      w += k;
      if (w >= n) w -= n;
    }
    buf2[k * LP + l] = mk<C>(ax, ay);
  }
}

template <typename C>
GBS_HD void copy_part(const C* src, C* dst, int n, int nlines, int LP, int tid,
                      int nthreads) {
  const int total = nlines * n;
  for (int idx = tid; idx < total; idx += nthreads) {
    int l = idx % nlines;
    int k = idx / nlines;
    dst[k * LP + l] = src[k * LP + l];
  }
}

#ifdef __CUDACC__
// Whole-tile FFT of `nlines` lines of length n, in place in `buf` (natural
// order out).  `buf2` is scratch of the same size, used for non power-of-two
// n only.  Must be called by every thread of the CTA.
template <int DIR, int TPT, typename C>
__device__ __forceinline__ void fft_tile(C* buf, C* buf2, int n, int nlines,
                                         int LP, const C* tw, int tw_stride) {
  const int tid = threadIdx.x;
  const int nthreads = blockDim.x;
  if (is_pow2(n) && n >= 8) {
    const int log2n = ilog2(n);
    const int s8 = log2n / 3;
    const int rem = log2n % 3;
    int Ns = 1, log2Ns = 0;
    C v[TPT][8];
    for (int s = 0; s < s8; ++s) {
      stockham_load<8, DIR, TPT>(buf, v, n, log2n, Ns, log2Ns, nlines, LP, tw,
                                 tw_stride, tid, nthreads);
      __syncthreads();
      stockham_store<8, TPT>(buf, v, n, Ns, log2Ns, nlines, LP, tid, nthreads);
      __syncthreads();
      Ns <<= 3;
      log2Ns += 3;
    }
    if (rem == 1) {
      stockham_load<2, DIR, TPT>(buf, v, n, log2n, Ns, log2Ns, nlines, LP, tw,
                                 tw_stride, tid, nthreads);
      __syncthreads();
      stockham_store<2, TPT>(buf, v, n, Ns, log2Ns, nlines, LP, tid, nthreads);
      __syncthreads();
    } else if (rem == 2) {
      stockham_load<4, DIR, TPT>(buf, v, n, log2n, Ns, log2Ns, nlines, LP, tw,
                                 tw_stride, tid, nthreads);
      __syncthreads();
      stockham_store<4, TPT>(buf, v, n, Ns, log2Ns, nlines, LP, tid, nthreads);
      __syncthreads();
    }
  } else if (n > 1) {
    dft_direct_part<DIR>(buf, buf2, n, nlines, LP, tw, tw_stride, tid, nthreads);
    __syncthreads();
    copy_part(buf2, buf, n, nlines, LP, tid, nthreads);
    __syncthreads();
  }
}
#endif

// index -> adimensional wavenumber (ik <= n/2 -> ik, else ik - n)
GBS_HD int kadim(int ik, int n) { return ik <= n / 2 ? ik : ik - n; }
GBS_HD int iabs(int a) { return a < 0 ? -a : a; }

}  // namespace gbs
