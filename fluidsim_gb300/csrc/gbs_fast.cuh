// Compile-time-size kernels for power-of-two grids (the production path).
//
// Every line of length N = 2^LOGN is transformed by N/8 threads holding 8
// complex values each: the first Stockham stage runs on values loaded
// straight from global memory, the last one leaves its outputs in registers
// at the positions that were loaded, and the stages in between exchange
// through shared memory (two exchanges for N = 256 or 512).  All index
// arithmetic is shifts and masks.
//
// Pruning (`pr`): when the input state is known to be dealiased (true after
// every completed step), the passes skip what the 2/3 rule makes zero:
// columns with kx >= kcut_x, inverse-transform inputs with |k| >= kcut,
// forward-transform outputs that the dealiasing would zero.  Kept modes get
// exactly the same arithmetic as without pruning.
#pragma once

#include "gbs_internal.cuh"
#include "gbs_ns.cuh"
#include "gbs_fast_api.h"

namespace gbs {
namespace fast {

extern __shared__ __align__(16) unsigned char g_smem_fast[];

// Pointer qualifier of the ns2d pass bodies' field arguments.  A translation
// unit that runs the bodies inside one persistent launch, where the fields
// are written and read again by other CTAs during the launch, defines it
// empty so that no load goes through the non-coherent read-only path.
#ifndef GBS_NS2D_RESTRICT
#define GBS_NS2D_RESTRICT __restrict__
#endif

// min blocks per SM so that GBS_OCC_THREADS threads can be resident
// (1536: <= 42 registers per thread; 1024: <= 64)
#ifndef GBS_OCC_THREADS
#define GBS_OCC_THREADS 1536
#endif
constexpr int min_blocks(int th) {
  return th >= GBS_OCC_THREADS ? 1 : GBS_OCC_THREADS / th;
}
// for kernels that would spill at the tighter bound (<= 64 registers)
constexpr int min_blocks_lo(int th) { return th >= 1024 ? 1 : 1024 / th; }

template <int LOGN>
struct Line {
  static constexpr int N = 1 << LOGN;
  static constexpr int N8 = N >> 3;
  static constexpr int S8 = LOGN / 3;
  static constexpr int REM = LOGN % 3;
  static constexpr int NST = S8 + (REM ? 1 : 0);
  static constexpr int RL = REM == 0 ? 8 : (1 << REM);
  // register idx -> output position jt + outm(idx) * N8 after the last stage
  static __host__ __device__ __forceinline__ constexpr int outm(int idx) {
    return REM == 0 ? idx : (idx / RL) + (idx % RL) * (8 / RL);
  }
};

// Shared-memory swizzle: XOR the element index inside each 128-byte bank
// sweep (E = 128 / sizeof(C) elements) with x ^ (x << 1), x the index of
// the sweep, so the strided Stockham writes, the unit-stride reads and the
// column-tile accesses spread over the 32 banks.  A permutation inside
// every E-aligned group, so any E-aligned slot keeps its extent.  XOR-ing
// with x alone (-DGBS_SWZ_XOR1) leaves two 8-byte writes of a half-warp on
// one bank in the first-stage writes of the 8-column tiles and the
// second-stage writes of the rows: 2.8x the bank conflicts of x ^ (x << 1)
// in the x pass at 512^2 x 64 (7.3 M against 2.6 M), 2.3 % slower.
template <typename C>
__host__ __device__ __forceinline__ int swz(int q) {
  constexpr int E = 128 / sizeof(C);
  constexpr int LG = E == 16 ? 4 : 3;
#ifdef GBS_SWZ_XOR1
  return q ^ ((q >> LG) & (E - 1));
#else
  // linear over GF(2) (an XOR of shifts), so swz_join below applies
  const int x = q >> LG;
  return q ^ ((x ^ (x << 1)) & (E - 1));
#endif
}

// swz(b | K) from sb = swz(b), for b and K with no bit in common (b per
// thread, K a compile-time constant of an unrolled loop): the swizzle is an
// XOR with the bits of q above LG, so it splits over disjoint operands,
// swz(b | K) = sb ^ swz(K), and the bits of swz(K) at or above E meet no bit
// of sb (b and K are disjoint there, the XOR only reaches bits below E): one
// XOR with a constant below E plus an immediate offset, instead of forming q
// and its swizzle again for every access.
template <typename C>
__host__ __device__ __forceinline__ int swz_join(int sb, int K) {
  constexpr int E = 128 / sizeof(C);
  const int sK = swz<C>(K);
  return (sb ^ (sK & (E - 1))) + (sK & ~(E - 1));
}

// Shared-memory view of the line(s) one thread works on: position p of its
// line at buf[swz(p * TX + c)] (a tile of TX columns; rows: TX = 1, c = 0,
// buf the row's slot, whose offset is a multiple of E).  base(b) / at(sb, K)
// address position b | K (b and K disjoint) through swz_join.
template <typename C, int TX>
struct SwzView {
  C* buf;
  int c;
  __device__ __forceinline__ C& operator()(int p) const { return buf[swz<C>(p * TX + c)]; }
  __device__ __forceinline__ int base(int b) const { return swz<C>(b * TX + c); }
  __device__ __forceinline__ C& at(int sb, int K) const { return buf[swz_join<C>(sb, K * TX)]; }
};

__device__ __forceinline__ bool kept(int p, int n, int kc) {
  return p < kc || p > n - kc;
}

// Fetch the line holding p into L2 (writes no register).
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// Fetch bytes [p, p + n) into L2 (p 16-byte aligned, n a multiple of 16).
__device__ __forceinline__ void prefetch_l2_bulk(const void* p, unsigned n) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(n) : "memory");
}

// mbarrier and bulk-copy primitives (one CTA, no cluster).
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* m, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count)
               : "memory");
}
// makes initialised mbarriers visible to the asynchronous proxy
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// orders this thread's earlier shared-memory accesses before later
// asynchronous-proxy (bulk copy) accesses
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// one arrival that also expects `bytes` of transactions on the phase
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* m, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)),
               "r"(bytes)
               : "memory");
}
// bytes [src, src + n) of global memory to shared memory at dst; completes
// n bytes of transactions on mbarrier m (src, dst 16-byte aligned, n a
// multiple of 16)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned n, uint64_t* m) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
      "[%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(n), "r"(smem_u32(m))
      : "memory");
}
__device__ __forceinline__ bool mbar_test_parity(uint64_t* m, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; "
      "selp.u32 %0, 1, 0, p; }"
      : "=r"(ok)
      : "r"(smem_u32(m)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Wait until the phase of parity `parity` of m has completed, for at most
// timeout_ns; false when the time ran out.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* m, unsigned parity,
                                                  unsigned long long timeout_ns) {
  if (mbar_test_parity(m, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
    if (mbar_test_parity(m, parity)) return true;
    if (global_ns() - t0 > timeout_ns) return false;
  }
}

// Asynchronous copy of one complex value into shared memory (zeros when
// !on; src must then still be a valid address).  Completion: cp_async_wait().
template <typename C>
__device__ __forceinline__ void cp_async_or_zero(C* dst, const C* src, bool on) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if constexpr (sizeof(C) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(src),
                 "r"(on ? 8 : 0));
  else
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src),
                 "r"(on ? 16 : 0));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;"); }
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// Block coordinates of the CTA dy grid rows (dy * gridDim.x CTAs) after this
// one in launch order (x fastest); false for dy <= 0 or past the end of the
// grid.  CTAs start about in this order, so with dy * gridDim.x about the
// number of CTAs resident on the GPU the CTA named starts about when this
// one ends: fetching its inputs into L2 now overlaps their DRAM latency with
// this CTA's transforms.  (Whole rows: no division by the grid size.)
__device__ __forceinline__ bool cta_ahead(int dy, int& bx, int& by, int& bz) {
  if (dy <= 0) return false;
  bx = blockIdx.x;
  by = blockIdx.y + dy;
  bz = blockIdx.z;
  if (by >= (int)gridDim.y) {  // dy < gridDim.y is checked on the host
    by -= gridDim.y;
    ++bz;
  }
  return bz < (int)gridDim.z;
}

// exp(-2 pi i r / 16), r = 0..8: the x-pass pre/post-processing twiddle of
// position jt + r M/8 of a 2M-point real line is tw[jt] times this factor.
template <typename C>
__device__ __forceinline__ C w16(int r) {
  using R = decltype(C::x);
  constexpr double c1 = 0.92387953251128675613, s1 = 0.38268343236508977173;
  constexpr double h = 0.70710678118654752440;
  switch (r) {
    case 0: return mk<C>(R(1), R(0));
    case 1: return mk<C>(R(c1), R(-s1));
    case 2: return mk<C>(R(h), R(-h));
    case 3: return mk<C>(R(s1), R(-c1));
    case 4: return mk<C>(R(0), R(-1));
    case 5: return mk<C>(R(-s1), R(-c1));
    case 6: return mk<C>(R(-h), R(-h));
    case 7: return mk<C>(R(-c1), R(-s1));
    default: return mk<C>(R(-1), R(0));
  }
}

// Twiddle of position jt + r M/8 of the 2M-point table twx: FP32 derives it
// from twx[jt] (one table read per line instead of eight; one rounding more),
// FP64 reads the table.
template <typename C>
__device__ __forceinline__ C twx_at(const C* __restrict__ twx, C t0, int jt, int r, int M8) {
  if constexpr (sizeof(C) == 8) return r == 0 ? t0 : cmul(t0, w16<C>(r));
  else return twx[jt + r * M8];
}

// Stage twiddles w[r] = W^(r k) (conjugated for DIR = +1), r = 1..R-1.  FP32
// forms the powers of w = W^k by products (one table read instead of R-1,
// at most three roundings deep), which keeps the twiddle reads from taking
// the L1 bandwidth the shared-memory exchanges need; FP64 reads the table.
template <int DIR, int R, typename C>
__device__ __forceinline__ void stage_twiddles(const C* __restrict__ tw, int k, C (&w)[8]) {
  if constexpr (sizeof(C) == 8) {
    const C w1 = twid<DIR>(tw, k);
    w[1] = w1;
    if (R > 2) {
      w[2] = cmul(w1, w1);
      w[3] = cmul(w[2], w1);
    }
    if (R > 4) {
      w[4] = cmul(w[2], w[2]);
      w[5] = cmul(w[4], w1);
      w[6] = cmul(w[4], w[2]);
      w[7] = cmul(w[4], w[3]);
    }
  } else {
#pragma unroll
    for (int r = 1; r < R; ++r) w[r] = twid<DIR>(tw, r * k);
  }
}

// Barrier over the threads that share a line's slot: the warp (WARP: lines
// inside one warp), the named barrier `bar` > 0 of the line's NT threads
// (whole, contiguous warps: lines do not wait for each other), or the CTA.
template <bool WARP, int NT>
__device__ __forceinline__ void line_sync(int bar) {
  if (WARP) __syncwarp();
  else if (bar > 0) asm volatile("bar.sync %0, %1;" ::"r"(bar), "n"(NT) : "memory");
  else __syncthreads();
}

// Stockham FFT of one line whose stage-0 inputs v[r] = x[jt + r N/8] are in
// registers; `acc(p)` addresses position p of this line in shared memory.
// Every thread that shares its barriers must call it; `active` threads
// compute, the others only take part in the barriers.  Barriers: the CTA's
// (bar = 0), or per line (WARP: every line lies inside one warp, rows with
// N/8 <= 32 threads and the line index above jt; bar > 0: the named barrier
// of the line's N/8 threads), and then only the line's threads call it.
// ALT > 0: the exchanges alternate between the slot and the one ALT
// elements after it, so an exchange needs one barrier (between its writes
// and its reads; the next exchange writes the other slot, and the one
// after it comes after the next barrier); the caller must then not reuse
// either slot before a barrier of its own.
template <int DIR, int LOGN, bool WARP = false, int ALT = 0, typename C, typename Acc>
__device__ __forceinline__ void run(C (&v)[8], int jt, bool active, const Acc& acc_a,
                                    const C* __restrict__ tw, int tws, int bar = 0) {
  using P = Line<LOGN>;
  constexpr int N = P::N, N8 = P::N8;
  Acc acc_b = acc_a;
  acc_b.buf += ALT;
  if (active) dft8<DIR>(v);
  // every exchange position below is (per-thread part) | (constant part)
  const int sj = acc_a.base(jt);
#pragma unroll
  for (int s = 1; s < P::NST; ++s) {
    const Acc& acc = (ALT > 0 && (s & 1) == 0) ? acc_b : acc_a;
    const int Ns = 1 << (3 * (s - 1));  // radix-8 stage s-1 wrote with this Ns
    if (active) {
      const int sd = acc.base(((jt / Ns) * Ns << 3) + (jt % Ns));
#pragma unroll
      for (int r = 0; r < 8; ++r) acc.at(sd, r * Ns) = v[r];
    }
    line_sync<WARP, N8>(bar);
    const int Nsn = Ns << 3;
    if (active) {
      if (s < P::S8) {
        const int bm = jt & (Nsn - 1);
        const int tm = (N / (Nsn * 8)) * tws;
        C w[8];
        stage_twiddles<DIR, 8>(tw, bm * tm, w);
#pragma unroll
        for (int r = 0; r < 8; ++r) {
          C x = acc.at(sj, r * N8);
          if (r) x = cmul(x, w[r]);
          v[r] = x;
        }
        dft8<DIR>(v);
      } else {
        constexpr int RL = P::RL;
        const int tm = (N / (Nsn * RL)) * tws;
#pragma unroll
        for (int g = 0; g < 8 / RL; ++g) {
          const int b = jt + g * N8;
          const int bm = b & (Nsn - 1);
          C w[8];
          stage_twiddles<DIR, RL>(tw, bm * tm, w);
#pragma unroll
          for (int r = 0; r < RL; ++r) {
            C x = acc.at(sj, g * N8 + r * (N / RL));
            if (r) x = cmul(x, w[r]);
            v[g * RL + r] = x;
          }
          dftR<RL, DIR>(&v[g * RL]);
        }
      }
    }
    if (ALT == 0) line_sync<WARP, N8>(bar);
  }
}

// ------------------------------------------------------- plain column pass
// Lines along a strided axis (element p of column col of outer block o of
// field z at z*fs + o*os + p*es + col).  Rows with |k| >= kc_in are read as
// zero; rows with |k| >= kc_out are not stored.
struct ColArgs {
  int ncols;
  int kc_in, kc_out;
  int64_t es, os, fs;
  int pf;  // L2 prefetch distance in grid rows (0: none); set by the launcher
};

// SLOT1: one exchange slot (a barrier after each exchange's reads as well)
// and two CTAs of TX N/8 threads per SM: wide tiles at half the shared
// memory of two slots.
template <int TH, bool SLOT1>
constexpr int col_minb() { return SLOT1 ? (2048 / TH > 0 ? 2048 / TH : 1) : min_blocks(TH); }
template <typename T, int LOGN, int TX, int DIR, bool SLOT1 = false>
__global__ void __launch_bounds__(TX * (1 << LOGN) / 8,
                                  col_minb<TX * (1 << LOGN) / 8, SLOT1>())
kf_col(const cplx<T>* in, cplx<T>* out, ColArgs a, const cplx<T>* __restrict__ tw,
       T scale) {
  using C = cplx<T>;
  using P = Line<LOGN>;
  C* buf = reinterpret_cast<C*>(g_smem_fast);
  const int c = threadIdx.x % TX, jt = threadIdx.x / TX;
  const int col = blockIdx.x * TX + c;
  const bool valid = col < a.ncols;
  const int64_t base = blockIdx.z * a.fs + blockIdx.y * a.os + col;
  int bx, by, bz;
  if (cta_ahead(a.pf, bx, by, bz)) {
    // the TX lanes of each jt share its 8 rows: lane c fetches rows c, c + TX,
    // .., both ends of the row's segment of the tile (a segment may straddle
    // two 128-byte lines); the first column of a CTA in the grid is valid
    const int64_t bp = bz * a.fs + by * a.os + bx * TX;
    const int last = (a.ncols - bx * TX < TX ? a.ncols - bx * TX : TX) - 1;
#pragma unroll
    for (int r = c; r < 8; r += TX) {
      const int p = jt + r * P::N8;
      if (kept(p, P::N, a.kc_in)) {
        const cplx<T>* q = in + bp + p * a.es;
        prefetch_l2(q);
        prefetch_l2(q + last);
      }
    }
  }
  C v[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int p = jt + r * P::N8;
    v[r] = (valid && kept(p, P::N, a.kc_in)) ? in[base + p * a.es] : mk<C>(0, 0);
  }
  const SwzView<C, TX> acc{buf, c};
  run<DIR, LOGN, false, SLOT1 ? 0 : P::N * TX>(v, jt, true, acc, tw, 1);  // exchange slots
  if (!valid) return;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int p = jt + P::outm(i) * P::N8;
    if (kept(p, P::N, a.kc_out)) out[base + p * a.es] = cscale(v[i], scale);
  }
}

// Row slots in shared memory hold M complex, addressed through swz().
template <int LOGM, typename C>
__device__ __forceinline__ int padp(int p) { return swz<C>(p); }

// ------------------------------------------------------- plain row passes
// nrows rows of nx = 2M reals <-> nx/2+1 complex.  L rows per CTA, M/8
// threads per row (consecutive threads on consecutive elements of a row).
template <typename T, int LOGM, int L>
__global__ void __launch_bounds__(L * (1 << LOGM) / 8, 2)
kf_row_r2c(const T* __restrict__ x, cplx<T>* __restrict__ out, int64_t nrows,
           const cplx<T>* __restrict__ twx, T scale) {
  using C = cplx<T>;
  using P = Line<LOGM>;
  constexpr int M = P::N, M8 = P::N8, LS = M, NKX = M + 1;
  C* buf = reinterpret_cast<C*>(g_smem_fast);
  const int jt = threadIdx.x % M8, l = threadIdx.x / M8;
  const int64_t row = (int64_t)blockIdx.x * L + l;
  const bool valid = row < nrows;
  const C* xc = reinterpret_cast<const C*>(x) + row * M;
  C v[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) v[r] = valid ? xc[jt + r * M8] : mk<C>(0, 0);
  C* slot = buf + l * LS;
  const SwzView<C, 1> acc{slot, 0};
  constexpr bool WARP = Line<LOGM>::N8 <= 32;
  run<-1, LOGM, WARP>(v, jt, true, acc, twx, 2);
#pragma unroll
  for (int i = 0; i < 8; ++i) acc.at(acc.base(jt), P::outm(i) * M8) = v[i];
  if (WARP) __syncwarp(); else __syncthreads();
  if (!valid) return;
  // X[k] and X[M - k] -> spectrum k = jt + r M/8 (and k = M for jt = 0),
  // the twiddle derived from tw[jt] as in the x pass
  const C t0 = twx[jt];
  const T h = T(0.5);
  C* o = out + row * NKX;
#pragma unroll
  for (int r = 0; r <= 8; ++r) {
    if (r == 8 && jt != 0) continue;
    const int k = r < 8 ? jt + r * M8 : M;
    const C a = acc(k == M ? 0 : k);
    const C b = cconj(acc(k == 0 ? 0 : M - k));
    const C s = cadd(a, b), d = csub(a, b);
    const C wd = cmul(r < 8 ? twx_at(twx, t0, jt, r, M8) : twx[M], d);
    o[k] = cscale(mk<C>(h * (s.x + wd.y), h * (s.y - wd.x)), scale);
  }
}

template <typename T, int LOGM, int L>
__global__ void __launch_bounds__(L * (1 << LOGM) / 8, 2)
kf_row_c2r(const cplx<T>* __restrict__ in, T* __restrict__ x, int64_t nrows,
           const cplx<T>* __restrict__ twx) {
  using C = cplx<T>;
  using P = Line<LOGM>;
  constexpr int M = P::N, M8 = P::N8, LS = M, NKX = M + 1;
  C* buf = reinterpret_cast<C*>(g_smem_fast);
  const int jt = threadIdx.x % M8, l = threadIdx.x / M8;
  const int64_t row = (int64_t)blockIdx.x * L + l;
  const bool valid = row < nrows;
  const C* rowp = in + row * NKX;
  const C t0 = twx[jt];
  C v[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int j = jt + r * M8;
    C Z = mk<C>(0, 0);
    if (valid) {
      C a = rowp[j];
      C b = cconj(rowp[M - j]);
      if (j == 0) { a.y = 0; b.y = 0; }
      const C s = cadd(a, b), d = csub(a, b);
      const C wd = cmulc(d, twx_at(twx, t0, jt, r, M8));
      Z = mk<C>(s.x - wd.y, s.y + wd.x);
    }
    v[r] = Z;
  }
  C* slot = buf + l * LS;
  const SwzView<C, 1> acc{slot, 0};
  run<+1, LOGM, (Line<LOGM>::N8 <= 32)>(v, jt, true, acc, twx, 2);
  if (!valid) return;
  C* xc = reinterpret_cast<C*>(x) + row * M;
#pragma unroll
  for (int i = 0; i < 8; ++i) xc[jt + P::outm(i) * M8] = v[i];
}

// ----------------------------------------------------- ns3d geometry
struct Geo {
  int nx, ny, nz, nkx, M;
  int kcx, kcy, kcz;
  int ncx;        // columns along x that are processed
  int nky_keep;   // rows along y that are processed (A, C)
  int pr;         // input dealiased: prune
  double dkx, dky, dkz;
  double nu2, nu4, nu8, num4, beta, f, inv_n, k2_hypo0;
  int has_f;
  int phase;             // multiply the input state by exp(i phi)
  double sx, sy, sz;     // phase shift lengths (phi = sx kx + sy ky + sz kz)
  int proj, no_vz_kz0;   // ns3d projection of the tendencies and the state
  double N2;             // ns3d.strat: Brunt-Vaisala frequency squared
  int strat;             // ns3d.strat: 4 state fields (vx, vy, vz, b)
  // float copies for the FP32 kernels (geo_f32)
  float fdkx, fdky, fdkz, fnu2, fnu4, fnu8, fnum4, fk2_hypo0, fbeta, fN2, ff;
};

// Fill the float copies of a Geo's double parameters (host, after setting
// them; the per-run overrides of an ensemble set their own on the device).
inline void geo_f32(Geo& g) {
  g.fdkx = (float)g.dkx;
  g.fdky = (float)g.dky;
  g.fdkz = (float)g.dkz;
  g.fnu2 = (float)g.nu2;
  g.fnu4 = (float)g.nu4;
  g.fnu8 = (float)g.nu8;
  g.fnum4 = (float)g.num4;
  g.fk2_hypo0 = (float)g.k2_hypo0;
  g.fbeta = (float)g.beta;
  g.fN2 = (float)g.N2;
  g.ff = (float)g.f;
}

// Wavenumber k dk in the kernels' type: FP64 forms the product in double,
// FP32 multiplies dk rounded to float by the exact integer k (one rounding
// more, and no FP64 instruction per mode).
template <typename T>
__device__ __forceinline__ T wavenum(double dk, float fdk, int k) {
  if constexpr (sizeof(T) == 8) return dk * k;
  else return fdk * (float)k;
}
template <typename T>
__device__ __forceinline__ T par(double d, float f) {
  if constexpr (sizeof(T) == 8) return d;
  else return f;
}

// Per-run parameters of a batched ensemble (null pointers: single run).
struct PerRun {
  const double* nu2;
  const double* nu8;
  const double* dt;
};

__device__ __forceinline__ Phys phys_of(const Geo& g) {
  Phys q;
  q.nu2 = g.nu2;
  q.nu4 = g.nu4;
  q.nu8 = g.nu8;
  q.num4 = g.num4;
  q.k2_hypo0 = g.k2_hypo0;
  q.fnu2 = g.fnu2;
  q.fnu4 = g.fnu4;
  q.fnu8 = g.fnu8;
  q.fnum4 = g.fnum4;
  q.fk2_hypo0 = g.fk2_hypo0;
  q.proj = g.proj;
  q.no_vz_kz0 = g.no_vz_kz0;
  return q;
}

__device__ __forceinline__ int iy_of(const Geo& g, int b) {
  return (g.nky_keep == g.ny || b < g.kcy) ? b : b + (g.ny - g.nky_keep);
}

// A: inverse z pass with the curl: W = (vx, vy, vz, ox, oy, oz) (ST: + b).
// kx and ky are constant along a z line, so the curl needs only two more
// transforms (the inverse transform commutes with multiplying by them):
//   Tv = IFFT(v),  Dx = IFFT(i kz vx),  Dy = IFFT(i kz vy),
//   ox = i ky Tz - Dy,  oy = Dx - i kx Tz,  oz = i kx Ty - i ky Tx,
// 5 transforms instead of 6.  The transform kept for a later combination
// (Ty, then Tz) waits in shared memory, and the inputs of the next transform
// are copied asynchronously into shared memory while the current one runs;
// each thread reads back only what it wrote in both.
template <typename T, int LOGN, int TX, bool ST, bool PH>
__global__ void __launch_bounds__(TX * (1 << LOGN) / 8, min_blocks_lo(TX * (1 << LOGN) / 8))
kf3_inv_z(const cplx<T>* __restrict__ S, cplx<T>* __restrict__ W, Geo g,
          const cplx<T>* __restrict__ twz) {
  using C = cplx<T>;
  using P = Line<LOGN>;
  constexpr int TH = TX * P::N8;
  C* buf = reinterpret_cast<C*>(g_smem_fast);
  C* hold = buf + P::N * TX;
  C* stage = hold + P::N * TX;
  const int c = threadIdx.x % TX, jt = threadIdx.x / TX;
  const int ix = blockIdx.x * TX + c;
  const int iy = iy_of(g, blockIdx.y);
  const bool valid = ix < g.ncx;
  const int64_t plane = (int64_t)g.ny * g.nkx;
  const int64_t nK = plane * g.nz;
  const int64_t base = (int64_t)iy * g.nkx + ix;
  const T kx = wavenum<T>(g.dkx, g.fdkx, ix), ky = wavenum<T>(g.dky, g.fdky, kadim(iy, g.ny));
  const SwzView<C, TX> acc{buf, c};
  // job j: source field, whether it is multiplied by i kz
  //   0: Ty   1: Tx (-> vx, oz)   2: Tz   3: Dy (-> ox)   4: Dx (-> oy)   5: b
  auto src_of = [](int j) { return j == 0 || j == 3 ? 1 : (j == 1 || j == 4 ? 0 : (j == 2 ? 2 : 3)); };
  auto fetch = [&](int j) {
    const C* Sf = S + src_of(j) * nK + base;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int p = jt + r * P::N8;
      const bool on = valid && (!g.pr || kept(p, P::N, g.kcz));
      cp_async_or_zero(&stage[r * TH + threadIdx.x], on ? Sf + p * plane : S, on);
    }
    cp_async_commit();
  };
  constexpr int NJ = ST ? 6 : 5;
  fetch(0);
#pragma unroll 1
  for (int j = 0; j < NJ; ++j) {
    const bool dz = j == 3 || j == 4;
    C v[8];
    cp_async_wait();
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = stage[r * TH + threadIdx.x];
    if (j + 1 < NJ) fetch(j + 1);
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int p = jt + r * P::N8;
      C x = v[r];
      if (dz) {
        const T kz = wavenum<T>(g.dkz, g.fdkz, kadim(p, P::N));
        x = mk<C>(-kz * x.y, kz * x.x);
      }
      if (PH)
        x = cmul(x, phase_factor<C, T>(T(g.sx), T(g.sy), T(g.sz), kx, ky,
                                       wavenum<T>(g.dkz, g.fdkz, kadim(p, P::N))));
      v[r] = x;
    }
    run<+1, LOGN>(v, jt, true, acc, twz, 1);
    if (j == 0 || j == 2) {
#pragma unroll
      for (int i = 0; i < 8; ++i) hold[i * TH + threadIdx.x] = v[i];
    }
    if (!valid) continue;
    C* Wo;
    if (j <= 2 || j == 5) {
      Wo = W + (j == 0 ? 1 : (j == 1 ? 0 : (j == 2 ? 2 : 6))) * nK;
    } else {
      Wo = W + (j == 3 ? 3 : 4) * nK;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const C h = hold[i * TH + threadIdx.x];  // Tz
        v[i] = j == 3 ? mk<C>(-ky * h.y - v[i].x, ky * h.x - v[i].y)
                      : mk<C>(v[i].x + kx * h.y, v[i].y - kx * h.x);
      }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) Wo[base + (jt + P::outm(i) * P::N8) * plane] = v[i];
    if (j == 1) {  // oz = i kx Ty - i ky Tx (+ f: the k = 0 mode of the column kx = ky = 0)
      const T fz = (g.has_f && ix == 0 && iy == 0) ? par<T>(g.f, g.ff) : T(0);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const C h = hold[i * TH + threadIdx.x];  // Ty
        W[5 * nK + base + (jt + P::outm(i) * P::N8) * plane] =
            mk<C>(-kx * h.y + ky * v[i].y + fz, kx * h.x - ky * v[i].x);
      }
    }
  }
}

// B: x pass.  6 fields x L rows; C2R, v x omega, R2C of the 3 products.
// ST (ns3d.strat): 7 fields (+ b), 6 products (v x omega, v b).

// The products in physical space, in place in the field slots (slot of
// field f, row l at (f L + l) LS; each position of each row handled by one
// thread), and the CFL maxima of |v| over the CTA's rows.  Every thread of
// the CTA calls it; it ends with a barrier.
template <typename T, int L, int LS, bool ST>
__device__ __forceinline__ void x_products(cplx<T>* buf, int64_t nrows,
                                           unsigned long long* vmax) {
  using C = cplx<T>;
  T mx = 0, my = 0, mz = 0;
  for (int idx = threadIdx.x; idx < L * LS; idx += blockDim.x) {
    const int ll = idx / LS, j = idx % LS;
    C* p0 = buf + ll * LS + swz<C>(j);
    const C vx = p0[0], vy = p0[L * LS], vz = p0[2 * L * LS];
    const C ox = p0[3 * L * LS], oy = p0[4 * L * LS], oz = p0[5 * L * LS];
    p0[0] = mk<C>(vy.x * oz.x - vz.x * oy.x, vy.y * oz.y - vz.y * oy.y);
    p0[L * LS] = mk<C>(vz.x * ox.x - vx.x * oz.x, vz.y * ox.y - vx.y * oz.y);
    p0[2 * L * LS] = mk<C>(vx.x * oy.x - vy.x * ox.x, vx.y * oy.y - vy.y * ox.y);
    if (ST) {  // v b for the divergence of the buoyancy flux
      const C b = p0[6 * L * LS];
      p0[3 * L * LS] = mk<C>(vx.x * b.x, vx.y * b.y);
      p0[4 * L * LS] = mk<C>(vy.x * b.x, vy.y * b.y);
      p0[5 * L * LS] = mk<C>(vz.x * b.x, vz.y * b.y);
    }
    if (vmax && (int64_t)blockIdx.x * L + ll < nrows) {
      mx = fmax(mx, fmax(fabs(vx.x), fabs(vx.y)));
      my = fmax(my, fmax(fabs(vy.x), fabs(vy.y)));
      mz = fmax(mz, fmax(fabs(vz.x), fabs(vz.y)));
    }
  }
  __syncthreads();
  if (vmax) block_max3(mx, my, mz, vmax);
}

template <typename T, int LOGM, int L, bool ST>
__global__ void __launch_bounds__((ST ? 7 : 6) * L * (1 << LOGM) / 8,
                                  min_blocks((ST ? 7 : 6) * L * (1 << LOGM) / 8))
kf3_x(const cplx<T>* __restrict__ W, cplx<T>* __restrict__ F, Geo g,
      const cplx<T>* __restrict__ twx, unsigned long long* vmax) {
  using C = cplx<T>;
  using P = Line<LOGM>;
  constexpr int M = P::N, M8 = P::N8, LS = M;
  C* buf = reinterpret_cast<C*>(g_smem_fast);
  const int jt = threadIdx.x % M8;
  const int l = (threadIdx.x / M8) % L;
  const int f = threadIdx.x / (M8 * L);
  const int64_t nrows = (int64_t)g.nz * g.ny;
  const int64_t nK = nrows * g.nkx;
  const int64_t row = (int64_t)blockIdx.x * L + l;
  const bool valid = row < nrows;
  C* slot = buf + (f * L + l) * LS;
  const SwzView<C, 1> acc{slot, 0};
  const int kcx = g.pr ? g.kcx : g.nkx + 1;
  C v[8];
  const C t0 = twx[jt];
  {
    const C* rowp = W + f * nK + row * g.nkx;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int j = jt + r * M8;
      C Z = mk<C>(0, 0);
      if (valid) {
        C a = j < kcx ? rowp[j] : mk<C>(0, 0);
        C b = (M - j) < kcx ? cconj(rowp[M - j]) : mk<C>(0, 0);
        if (j == 0) { a.y = 0; b.y = 0; }
        const C s = cadd(a, b), d = csub(a, b);
        const C wd = cmulc(d, twx_at(twx, t0, jt, r, M8));
        Z = mk<C>(s.x - wd.y, s.y + wd.x);
      }
      v[r] = Z;
    }
  }
  run<+1, LOGM, (Line<LOGM>::N8 <= 32)>(v, jt, true, acc, twx, 2);
#pragma unroll
  for (int i = 0; i < 8; ++i) acc.at(acc.base(jt), P::outm(i) * M8) = v[i];
  __syncthreads();
  x_products<T, L, M, ST>(buf, nrows, vmax);
  const bool act = f < (ST ? 6 : 3);
#pragma unroll
  for (int r = 0; r < 8; ++r) v[r] = act ? acc.at(acc.base(jt), r * M8) : mk<C>(0, 0);
  // the line's first exchange overwrites positions other threads still read
  if (Line<LOGM>::N8 <= 32) __syncwarp(); else __syncthreads();
  run<-1, LOGM, (Line<LOGM>::N8 <= 32)>(v, jt, act, acc, twx, 2);
  if (act) {
#pragma unroll
    for (int i = 0; i < 8; ++i) acc.at(acc.base(jt), P::outm(i) * M8) = v[i];
  }
  __syncthreads();
  const int nout = g.pr ? (g.kcx < g.nkx ? g.kcx : g.nkx) : g.nkx;
  if (act && valid) {
    const C* sl = buf + (f * L + l) * LS;
    C* Fo = F + f * nK + row * g.nkx;
    const T h = T(0.5);
#pragma unroll
    for (int r = 0; r <= 8; ++r) {
      const int k = r < 8 ? jt + r * M8 : M;
      if ((r == 8 && jt != 0) || k >= nout) continue;
      C a = sl[padp<LOGM, C>(k == M ? 0 : k)];
      C b = cconj(sl[padp<LOGM, C>(k == 0 ? 0 : M - k)]);
      const C s = cadd(a, b), d = csub(a, b);
      const C wd = cmul(r < 8 ? twx_at(twx, t0, jt, r, M8) : twx[M], d);
      Fo[k] = mk<C>(h * (s.x + wd.y), h * (s.y - wd.x));
    }
  }
}

// Paired x passes with three-stage lines (N = 128 .. 512) give each line a
// second exchange slot (after all first slots).
template <int LOGN>
__host__ __device__ constexpr bool xp_alt() { return Line<LOGN>::NST == 3; }

// B, rows in pairs: rows 2 q and 2 q + 1 of a field travel as the real and
// imaginary parts of one complex line of N = nx points.  With A0, A1 their
// spectra extended by Hermitian symmetry (imaginary parts of k = 0 and
// k = N/2 dropped, as a C2R transform does), Z = A0 + i A1 transforms back to
// z = a0 + i a1; x_products works componentwise, so it forms the products of
// both rows at once; and the forward transform Z of p0 + i p1 splits into
//   P0[k] = (Z[k] + conj Z[N-k]) / 2,   P1[k] = (Z[k] - conj Z[N-k]) / 2i.
// No pre- or post-processing twiddles (the half-length real transforms of
// kf3_x spend about as many instructions on those as on a radix-8 stage).
// LP row pairs per CTA; N/8 threads per line.
// (FP64: one CTA per SM, so that the lines fit in registers)
template <typename T, int LOGN, int LP, bool ST>
__global__ void __launch_bounds__((ST ? 7 : 6) * LP * (1 << LOGN) / 8,
                                  sizeof(T) == 8 ? 1
                                                 : min_blocks((ST ? 7 : 6) * LP * (1 << LOGN) / 8))
kf3_xp(const cplx<T>* __restrict__ W, cplx<T>* __restrict__ F, Geo g,
       const cplx<T>* __restrict__ twx, unsigned long long* vmax) {
  using C = cplx<T>;
  using P = Line<LOGN>;
  constexpr int N = P::N, N8 = P::N8, H = N / 2;
  constexpr bool WARP = N8 <= 32;
  C* buf = reinterpret_cast<C*>(g_smem_fast);
  const int jt = threadIdx.x % N8;
  const int lp = (threadIdx.x / N8) % LP;
  const int f = threadIdx.x / (N8 * LP);
  const int64_t nrows = (int64_t)g.nz * g.ny;
  const int64_t nK = nrows * g.nkx;
  const int64_t row0 = ((int64_t)blockIdx.x * LP + lp) * 2;
  const bool v0 = row0 < nrows, v1 = row0 + 1 < nrows;
  const SwzView<C, 1> acc{buf + (f * LP + lp) * N, 0};
  const int kcx = g.pr ? g.kcx : g.nkx + 1;
  C v[8];
  {
    const C* r0 = W + f * nK + row0 * g.nkx;
    const C* r1 = r0 + g.nkx;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      // k = jt + r N/8: k < N/2 for r < 4 (stored), else N - k (mirrored)
      const int idx = r < 4 ? jt + r * N8 : (8 - r) * N8 - jt;
      const bool in = idx < kcx;
      C a0 = (v0 && in) ? r0[idx] : mk<C>(0, 0);
      C a1 = (v1 && in) ? r1[idx] : mk<C>(0, 0);
      if ((r == 0 || r == 4) && jt == 0) { a0.y = 0; a1.y = 0; }
      v[r] = r < 4 ? mk<C>(a0.x - a1.y, a0.y + a1.x) : mk<C>(a0.x + a1.y, a1.x - a0.y);
    }
  }
  // lines of two or more warps synchronise on their own named barrier; with
  // three stages the two exchanges use the line's slot and a second one
  // (ALT), and the last one (in the second slot) leaves the first free
  const int bar = WARP ? 0 : 1 + f * LP + lp;
  constexpr int ALT = xp_alt<LOGN>() ? (ST ? 7 : 6) * LP * N : 0;
  run<+1, LOGN, WARP, ALT>(v, jt, true, acc, twx, 1, bar);
  const int sj = acc.base(jt);
#pragma unroll
  for (int i = 0; i < 8; ++i) acc.at(sj, P::outm(i) * N8) = v[i];
  __syncthreads();
  x_products<T, LP, N, ST>(buf, (nrows + 1) / 2, vmax);
  // from here on each product line is read and written by its own threads;
  // idle lines leave unless they share a warp's barriers with a product line
  const bool act = f < (ST ? 6 : 3);
  if (!act && !WARP) return;
#pragma unroll
  for (int r = 0; r < 8; ++r) v[r] = act ? acc.at(sj, r * N8) : mk<C>(0, 0);
  // the line's first exchange overwrites positions other threads still read
  line_sync<WARP, N8>(bar);
  run<-1, LOGN, WARP, ALT>(v, jt, act, acc, twx, 1, bar);
  if (act) {
#pragma unroll
    for (int i = 0; i < 8; ++i) acc.at(sj, P::outm(i) * N8) = v[i];
  }
  line_sync<WARP, N8>(bar);
  if (!act) return;
  const int nout = g.pr ? (g.kcx < g.nkx ? g.kcx : g.nkx) : g.nkx;
  C* F0 = F + f * nK + row0 * g.nkx;
  C* F1 = F0 + g.nkx;
  const T h = T(0.5);
#pragma unroll
  for (int r = 0; r <= 4; ++r) {
    const int k = r < 4 ? jt + r * N8 : H;
    if ((r == 4 && jt != 0) || k >= nout) continue;
    // Z[k]: this thread's own register when the last stage is radix 8
    const C z = (P::REM == 0 && r < 4) ? v[r] : acc(k);
    const C m = acc((N - k) & (N - 1));
    if (v0) F0[k] = mk<C>(h * (z.x + m.x), h * (z.y - m.y));
    if (v1) F1[k] = mk<C>(h * (z.y + m.y), h * (m.x - z.x));
  }
}

// p, opaque to the compiler from here on: loads through the result are
// neither merged with loads through earlier copies nor moved above the
// volatile asm statements (barriers) that precede this one.  Keeps the
// stage twiddles of kf3_xr from being computed once and held in registers
// across all nine transforms.
template <typename X>
__device__ __forceinline__ const X* opaque(const X* p) {
  const X* r;
  asm volatile("mov.b64 %0, %1;" : "=l"(r) : "l"(p));
  return r;
}

// Shared memory of one row pair of kf3_xr, in complex elements: exchange
// slot(s), partner half-line, stash, two staging buffers of two rows
// (N/2 + 1 modes each); a multiple of 16 elements, so that every pair's
// exchange slot starts a 128-byte bank sweep.
template <int LOGN>
__host__ __device__ constexpr int xr_slot() {
  constexpr int N = 1 << LOGN, H = N / 2, E = 16;
  constexpr int n = N + (xp_alt<LOGN>() ? N : 0) + (H > E ? H : E) + N + 2 * (N + 2);
  return (n + E - 1) / E * E;
}

// Register index holding stage-0 position jt + r N/8 in the output order of
// run(): the i with Line::outm(i) == r.
template <int LOGN>
__host__ __device__ __forceinline__ constexpr int inv_outm(int r) {
  int i = 0;
  while (Line<LOGN>::outm(i) != r) ++i;
  return i;
}

// kf3_xr: CTAs of GBS_XR_THREADS threads per SM (2: 128 registers; 3 fits
// 80 and spills 184-316 bytes)
#ifndef GBS_XR_MINB
#define GBS_XR_MINB 2
#endif
#ifndef GBS_XR_THREADS
#define GBS_XR_THREADS 256
#endif

// B, rows in pairs (as kf3_xp), with all six fields of a pair transformed by
// the same N/8 threads, one field after the other.  run() leaves each
// inverse transform's outputs in registers at positions jt + outm(i) N/8,
// the same positions in every field, so v x omega forms in registers, and
// each product line enters its forward transform from registers: no
// shared-memory round trip for the products (a third of kf3_xp's
// shared-memory traffic).  The products accumulate as the omega lines
// arrive (ox: p_y, p_z; oy: p_z complete, p_x; oz: p_x, p_y complete); p_z
// is transformed before oz, and vx waits in shared memory (each thread
// reads back only its own values), so at most four lines are held in
// registers besides the line being transformed.  The split of each product
// line into the two rows' spectra reads Z[N - k] from a half-line region
// that holds positions N/2 .. N-1.  Barriers: the pair's two exchange slots
// alternate (three-stage lines), so consecutive transforms need no barrier
// of their own (a slot is written again only after a barrier that every
// reader of its previous contents has passed).  Not for ns3d.strat
// (kf3_xp).
//
// Inputs: the kept modes of the two rows of field f arrive by two bulk
// copies (cp.async.bulk) into one of two staging buffers of the pair,
// issued two fields ahead by thread 0 of the pair and awaited on the
// buffer's mbarrier.  Rows have nx/2 + 1 modes and row0 is even, so row0
// starts 16-byte aligned and row0 + 1 8 bytes past a 16-byte boundary: its
// copy starts at the last mode of row0 (the Nyquist mode, which a pruned
// pass does not read); the wait is bounded by
// xs.timeout_ns, after which *xs.status is set and the pass goes on (the
// step then returns GBS_ETIMEDOUT).  Fields 2..5 are also prefetched into
// L2 at the start.  The grid must cover whole pairs (nz ny even).
template <typename T, int LOGN, int LP>
__global__ void __launch_bounds__(LP * (1 << LOGN) / 8, GBS_XR_MINB)
kf3_xr(const cplx<T>* __restrict__ W, cplx<T>* __restrict__ F, Geo g,
       const cplx<T>* __restrict__ twx, unsigned long long* vmax, XStage xs) {
  using C = cplx<T>;
  using P = Line<LOGN>;
  constexpr int N = P::N, N8 = P::N8, H = N / 2;
  constexpr bool WARP = N8 <= 32;
  constexpr int E = 128 / sizeof(C);
  constexpr int ALT = xp_alt<LOGN>() ? N : 0;
  constexpr int PART = H > E ? H : E;
  constexpr int RB = N + 2;  // staging buffer: two rows of N/2 + 1 modes
  constexpr int SLOT = xr_slot<LOGN>();
  static_assert(P::NST >= 2, "a line needs at least one exchange");
  static_assert((N + ALT + PART + N) % 2 == 0 && RB % 2 == 0, "16-byte aligned buffers");
  __shared__ uint64_t mbar[LP][2];
  C* buf = reinterpret_cast<C*>(g_smem_fast);
  const int jt = threadIdx.x % N8;
  const int lp = threadIdx.x / N8;
  const int64_t nrows = (int64_t)g.nz * g.ny;
  const int64_t nK = nrows * g.nkx;
  const int64_t row0 = ((int64_t)blockIdx.x * LP + lp) * 2;
  const bool v0 = row0 < nrows;  // the pair (row0 + 1 < nrows with it)
  const SwzView<C, 1> acc{buf + lp * SLOT, 0};
  const SwzView<C, 1> part{buf + lp * SLOT + N + ALT, 0};
  C* stash = buf + lp * SLOT + N + ALT + PART;
  C* stage = stash + N;  // stage + b * RB: staging buffer b
  const int bar = WARP ? 0 : 1 + lp;
  const int kcx = g.pr ? g.kcx : g.nkx + 1;
  const int nk = kcx < g.nkx ? kcx : g.nkx;  // kept modes of a row
  const int nout = nk;
  const C* r0base = W + row0 * g.nkx;
  // copy of row0: modes 0 .. nk - 1 rounded up to 16 bytes, at most up to
  // mode nkx - 2 (the row's last mode comes with the copy of row0 + 1);
  // copy of row0 + 1: from mode nkx - 1 of row0 to mode nk - 1 of row0 + 1,
  // rounded up to 16 bytes (at most to its last mode), into buffer slots
  // nkx - 1 .. (row0 + 1 at nkx .. 2 nkx - 1)
  const unsigned c0bytes = (unsigned)min((nk * sizeof(C) + 15) & ~size_t(15),
                                         (size_t)(g.nkx - 1) * sizeof(C));
  const unsigned c1bytes = (unsigned)(((nk + 1) * sizeof(C) + 15) & ~size_t(15));
  if (jt == 0) {
    mbar_init(&mbar[lp][0], 1);
    mbar_init(&mbar[lp][1], 1);
    mbar_init_fence();
  }
  if (jt < 8 && v0) {  // fields 2..5 into L2
    const C* a = r0base + (2 + (jt >> 1)) * nK;
    if (jt & 1) prefetch_l2_bulk(a + g.nkx - 1, c1bytes);
    else prefetch_l2_bulk(a, c0bytes);
  }
  line_sync<WARP, N8>(bar);  // the barriers are initialised

  // field f into staging buffer b (thread 0 of the pair)
  auto issue = [&](int f, int b) {
    if (jt != 0 || !v0) return;
    if (xs.stall && f == 5 && blockIdx.x == 0 && lp == 0) return;  // test hook
    fence_proxy_async();  // the buffer's earlier reads come first
    mbar_arrive_expect_tx(&mbar[lp][b], c0bytes + c1bytes);
    const C* src = r0base + f * nK;
    bulk_g2s(stage + b * RB, src, c0bytes, &mbar[lp][b]);
    bulk_g2s(stage + b * RB + g.nkx - 1, src + g.nkx - 1, c1bytes, &mbar[lp][b]);
  };
  // inverse transform of field f (staging buffer f % 2) into v (output
  // order of run())
  auto inverse = [&](int f, C(&v)[8]) {
    const int b = f & 1;
    if (v0 && !mbar_wait_bounded(&mbar[lp][b], (f >> 1) & 1, xs.timeout_ns))
      atomicOr(xs.status, 1);
    const C* r0 = stage + b * RB;
    const C* r1 = r0 + g.nkx;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int idx = r < 4 ? jt + r * N8 : (8 - r) * N8 - jt;
      const bool in = v0 && idx < kcx;
      C a0 = in ? r0[idx] : mk<C>(0, 0);
      C a1 = in ? r1[idx] : mk<C>(0, 0);
      if ((r == 0 || r == 4) && jt == 0) {
        a0.y = 0;
        a1.y = 0;
      }
      v[r] = r < 4 ? mk<C>(a0.x - a1.y, a0.y + a1.x) : mk<C>(a0.x + a1.y, a1.x - a0.y);
    }
    run<+1, LOGN, WARP, ALT>(v, jt, true, acc, opaque(twx), 1, bar);
    // every thread of the pair has read the buffer (run's barriers)
    if (f + 2 <= 5) issue(f + 2, b);
  };
  // forward transform of product line p (output order of run()) into field f
  auto forward = [&](int f, const C(&p)[8]) {
    C v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = p[inv_outm<LOGN>(r)];
    run<-1, LOGN, WARP, ALT>(v, jt, true, acc, opaque(twx), 1, bar);
#pragma unroll
    for (int i = 0; i < 8; ++i)
      if (P::outm(i) >= 4) part(jt + (P::outm(i) - 4) * N8) = v[i];
    line_sync<WARP, N8>(bar);
    C* F0 = F + f * nK + row0 * g.nkx;
    C* F1 = F0 + g.nkx;
    const T h = T(0.5);
#pragma unroll
    for (int r = 0; r <= 4; ++r) {
      const int k = r < 4 ? jt + r * N8 : H;
      if ((r == 4 && jt != 0) || k >= nout || !v0) continue;
      const C z = v[inv_outm<LOGN>(r)];
      const C m = (k == 0 || k == H) ? z : part(N - k - H);
      F0[k] = mk<C>(h * (z.x + m.x), h * (z.y - m.y));
      F1[k] = mk<C>(h * (z.y + m.y), h * (m.x - z.x));
    }
  };

  issue(0, 0);
  issue(1, 1);
  T mx = 0, my = 0, mz = 0;
  auto vmax_of = [](const C(&v)[8], T& m) {
#pragma unroll
    for (int i = 0; i < 8; ++i) m = fmax(m, fmax(fabs(v[i].x), fabs(v[i].y)));
  };
  {
    C v[8];
    inverse(0, v);  // vx waits in this thread's own stash slots
    vmax_of(v, mx);
#pragma unroll
    for (int i = 0; i < 8; ++i) stash[i * N8 + jt] = v[i];
  }
  C vy[8], vz[8], px[8], py[8], pz[8];
  inverse(1, vy);
  vmax_of(vy, my);
  inverse(2, vz);
  vmax_of(vz, mz);
  {
    C o[8];
    inverse(3, o);  // ox
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      py[i] = mk<C>(vz[i].x * o[i].x, vz[i].y * o[i].y);
      pz[i] = mk<C>(-(vy[i].x * o[i].x), -(vy[i].y * o[i].y));
    }
  }
  {
    C o[8];
    inverse(4, o);  // oy
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const C vx = stash[i * N8 + jt];
      pz[i] = mk<C>(fma(vx.x, o[i].x, pz[i].x), fma(vx.y, o[i].y, pz[i].y));
      px[i] = mk<C>(-(vz[i].x * o[i].x), -(vz[i].y * o[i].y));
    }
  }
  forward(2, pz);
  {
    C o[8];
    inverse(5, o);  // oz
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const C vx = stash[i * N8 + jt];
      px[i] = mk<C>(fma(vy[i].x, o[i].x, px[i].x), fma(vy[i].y, o[i].y, px[i].y));
      py[i] = mk<C>(fma(-vx.x, o[i].x, py[i].x), fma(-vx.y, o[i].y, py[i].y));
    }
  }
  forward(0, px);
  forward(1, py);
  if (vmax) block_max3(mx, my, mz, vmax);
}

#ifndef GBS_FWDZ_BATCH
#define GBS_FWDZ_BATCH 2
#endif
// C: forward z pass + 1/N + projection + dealiasing + RK4 stage.
// ST (ns3d.strat, strat/solver.py:194-216): 6 product fields; the last three
// (v b) are combined after their transforms into the divergence
// i k . (v b)^ (kept in registers, then in a 4th slot), fz += b and
// fb = -div - N^2 vz from the state the tendency is evaluated on.
// (its field slots limit it to ~1024 resident threads per SM, so it is
// compiled for that occupancy: <= 64 registers)
template <typename T, int LOGN, int TX, bool ST, bool EXT>
__global__ void __launch_bounds__(TX * (1 << LOGN) / 8, min_blocks_lo(TX * (1 << LOGN) / 8))
kf3_fwd_z(const cplx<T>* __restrict__ F, Geo g, const cplx<T>* __restrict__ twz,
          int mode, RKArgs a) {
  using C = cplx<T>;
  using P = Line<LOGN>;
  constexpr int N = P::N, N8 = P::N8;
  C* buf = reinterpret_cast<C*>(g_smem_fast);
  const int c = threadIdx.x % TX, jt = threadIdx.x / TX;
  const int ix = blockIdx.x * TX + c;
  const int iy = iy_of(g, blockIdx.y);
  const bool valid = ix < g.ncx;
  const int64_t plane = (int64_t)g.ny * g.nkx;
  const int64_t nK = plane * g.nz;
  const int64_t base = (int64_t)iy * g.nkx + ix;
  C dv[8];  // ST: i k . (v b)^ at the positions jt + outm(i) N/8
  // !ST: the inputs of field f + 1 are copied asynchronously into its (still
  // unused) slot while field f is transformed
  constexpr int TH = TX * N8;
  auto fetch = [&](int f) {
    C* st = buf + f * N * TX;
    const C* Ff = F + f * nK + base;
#pragma unroll
    for (int r = 0; r < 8; ++r)
      cp_async_or_zero(&st[r * TH + threadIdx.x], valid ? Ff + (jt + r * N8) * plane : F, valid);
    cp_async_commit();
  };
  if (!ST) fetch(0);
#pragma unroll 1
  for (int f = 0; f < (ST ? 6 : 3); ++f) {
    C v[8];
    if (ST) {
#pragma unroll
      for (int r = 0; r < 8; ++r)
        v[r] = valid ? F[f * nK + base + (jt + r * N8) * plane] : mk<C>(0, 0);
    } else {
      cp_async_wait();
      const C* st = buf + f * N * TX;
#pragma unroll
      for (int r = 0; r < 8; ++r) v[r] = st[r * TH + threadIdx.x];
      if (f < 2) fetch(f + 1);
      __syncthreads();  // the slot becomes the exchange buffer
    }
    C* slot = buf + (ST && f > 3 ? 3 : f) * N * TX;
    const SwzView<C, TX> acc{slot, c};
    run<-1, LOGN>(v, jt, true, acc, twz, 1);
    if (!ST || f < 3) {
#pragma unroll
      for (int i = 0; i < 8; ++i) acc.at(acc.base(jt), P::outm(i) * N8) = v[i];
    } else {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const T kj = f == 3 ? wavenum<T>(g.dkx, g.fdkx, ix)
                            : (f == 4 ? wavenum<T>(g.dky, g.fdky, kadim(iy, g.ny))
                                      : wavenum<T>(g.dkz, g.fdkz, kadim(jt + P::outm(i) * N8, N)));
        const C t = mk<C>(-kj * v[i].y, kj * v[i].x);
        dv[i] = f == 3 ? t : cadd(dv[i], t);
      }
      if (f == 5) {
#pragma unroll
        for (int i = 0; i < 8; ++i) acc.at(acc.base(jt), P::outm(i) * N8) = dv[i];
      }
    }
  }
  __syncthreads();
  if (!valid) return;
  const int kyi = kadim(iy, g.ny);
  const T kx = wavenum<T>(g.dkx, g.fdkx, ix), ky = wavenum<T>(g.dky, g.fdky, kyi);
  const T inv_n = T(g.inv_n);
  const Phys q = phys_of(g);
  if constexpr (!ST && !EXT) {
    // RK4 / tendency epilogue, two positions per round in FP32: the S_0 and
    // tmp values of both are loaded before either stores (a store of one
    // position may alias the next one's loads as far as the compiler knows,
    // so it would not hoist them).  512^3: 0.93 -> 0.89 ms (4 per round:
    // 0.96, 8: 1.11).
    const bool needS = mode >= kRK0 && mode <= kRK2;
    const bool needT = mode >= kRK1 && mode <= kRK3;
    const C* S0p = static_cast<const C*>(a.S);
    const C* T0p = static_cast<const C*>(a.tmp);
    constexpr int B = sizeof(T) == 4 ? GBS_FWDZ_BATCH : 1;  // positions per round
#pragma unroll 1
    for (int r0 = 0; r0 < 8; r0 += B) {
      C S0[B][3], T0[B][3];
#pragma unroll
      for (int u = 0; u < B; ++u) {
        const int iz = jt + (r0 + u) * N8;
        const bool rm = (ix >= g.kcx) || (iabs(kyi) >= g.kcy) || (iabs(kadim(iz, N)) >= g.kcz);
        const bool ld = !(g.pr && rm);
        const int64_t i = base + iz * plane;
#pragma unroll
        for (int f = 0; f < 3; ++f) {
          S0[u][f] = (ld && needS) ? S0p[i + f * nK] : mk<C>(0, 0);
          T0[u][f] = (ld && needT) ? T0p[i + f * nK] : mk<C>(0, 0);
        }
      }
#pragma unroll
      for (int u = 0; u < B; ++u) {
        const int iz = jt + (r0 + u) * N8;
        const int kzi = kadim(iz, N);
        const bool rm = (ix >= g.kcx) || (iabs(kyi) >= g.kcy) || (iabs(kzi) >= g.kcz);
        if (g.pr && rm) continue;  // stays zero in S, tmp and tmp1
        const int64_t i = base + iz * plane;
        const T kz = wavenum<T>(g.dkz, g.fdkz, kzi);
        C N3[3];
#pragma unroll
        for (int ff = 0; ff < 3; ++ff) N3[ff] = cscale(buf[ff * N * TX + swz<C>(iz * TX + c)], inv_n);
        if (a.add) {
#pragma unroll
          for (int ff = 0; ff < 3; ++ff)
            N3[ff] = cadd(N3[ff], static_cast<const C*>(a.add)[i + ff * nK]);
        }
        const T k2 = kx * kx + ky * ky + kz * kz;
        const bool k0 = (ix == 0 && kyi == 0 && kzi == 0);
        stage_epilogue_rk4<C, T, 3>(mode, a, i, nK, N3, S0[u], T0[u], kx, ky, kz, k2, k0, rm, q);
      }
    }
    return;
  }
#pragma unroll 1
  for (int r = 0; r < 8; ++r) {
    const int iz = jt + r * N8;
    const int kzi = kadim(iz, N);
    const bool rm = (ix >= g.kcx) || (iabs(kyi) >= g.kcy) || (iabs(kzi) >= g.kcz);
    if (g.pr && rm) continue;  // stays zero in S, tmp and tmp1
    const int64_t i = base + iz * plane;
    const T kz = wavenum<T>(g.dkz, g.fdkz, kzi);
    constexpr int NV = ST ? 4 : 3;
    C N3[NV];
#pragma unroll
    for (int ff = 0; ff < NV; ++ff) N3[ff] = cscale(buf[ff * N * TX + swz<C>(iz * TX + c)], inv_n);
    if (ST) {
      const C* in = static_cast<const C*>(a.in);
      const C vz = in[i + 2 * nK], b = in[i + 3 * nK];
      N3[2] = cadd(N3[2], b);
      const T n2 = par<T>(g.N2, g.fN2);
      N3[NV - 1] = mk<C>(-N3[NV - 1].x - n2 * vz.x, -N3[NV - 1].y - n2 * vz.y);
    }
    if (a.add) {
#pragma unroll
      for (int ff = 0; ff < NV; ++ff)
        N3[ff] = cadd(N3[ff], static_cast<const C*>(a.add)[i + ff * nK]);
    }
    const T k2 = kx * kx + ky * ky + kz * kz;
    const bool k0 = (ix == 0 && kyi == 0 && kzi == 0);
    stage_epilogue3<C, T, NV, EXT>(mode, a, i, nK, N3, kx, ky, kz, k2, k0, rm, q);
  }
}

// ----------------------------------------------------- ns2d kernels
// The ns2d passes are device functions of a block index `bid` (the CTA's
// own blockIdx, or the one a multi-size ensemble launch assigns it).

// A: inverse y pass; fields ux, uy, d_x rot, d_y rot.  bid = (column tile,
// -, run).
template <typename T, int LOGN, int TX, bool PH>
__device__ __forceinline__ void kf2_inv_y_body(const cplx<T>* GBS_NS2D_RESTRICT S,
                                               cplx<T>* GBS_NS2D_RESTRICT W, const Geo& g,
                                               const cplx<T>* GBS_NS2D_RESTRICT twy, uint3 bid) {
  using C = cplx<T>;
  using P = Line<LOGN>;
  C* buf = reinterpret_cast<C*>(g_smem_fast);
  const int c = threadIdx.x % TX, jt = threadIdx.x / TX;
  const int ix = bid.x * TX + c;
  const bool valid = ix < g.ncx;
  const int64_t nK = (int64_t)g.ny * g.nkx;
  S += bid.z * nK;  // run of a batched ensemble
  W += bid.z * 4 * nK;
  const T kx = wavenum<T>(g.dkx, g.fdkx, ix);
  const SwzView<C, TX> acc{buf, c};
  // ns2d.strat: two more fields, d_x b and d_y b (b: the second state field)
#pragma unroll 1
  for (int f = 0; f < (g.strat ? 6 : 4); ++f) {
    const C* Sf = f < 4 ? S : S + nK;
    C v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int p = jt + r * P::N8;
      C x = mk<C>(0, 0);
      if (valid && (!g.pr || kept(p, P::N, g.kcy))) {
        C w = Sf[(int64_t)p * g.nkx + ix];
        const int kyi = kadim(p, P::N);
        const T ky = wavenum<T>(g.dky, g.fdky, kyi);
        if (PH) w = cmul(w, phase_factor<C, T>(T(g.sx), T(g.sy), T(0), kx, ky, T(0)));
        T cc;
        if (f == 0 || f == 1) {
          const T k2 = kx * kx + ky * ky;
          const T inv = (ix == 0 && kyi == 0) ? T(0) : crcp(k2);
          cc = f == 0 ? ky * inv : -(kx * inv);
        } else {
          cc = (f == 2 || f == 4) ? kx : ky;
        }
        x = mk<C>(-cc * w.y, cc * w.x);
      }
      v[r] = x;
    }
    run<+1, LOGN>(v, jt, true, acc, twy, 1);
    if (valid) {
#pragma unroll
      for (int i = 0; i < 8; ++i)
        W[f * nK + (int64_t)(jt + P::outm(i) * P::N8) * g.nkx + ix] = v[i];
    }
  }
}

template <typename T, int LOGN, int TX, bool PH>
__global__ void __launch_bounds__(TX * (1 << LOGN) / 8, min_blocks(TX * (1 << LOGN) / 8))
kf2_inv_y(const cplx<T>* __restrict__ S, cplx<T>* __restrict__ W, Geo g,
          const cplx<T>* __restrict__ twy) {
  kf2_inv_y_body<T, LOGN, TX, PH>(S, W, g, twy, blockIdx);
}

// B: x pass, compute_Frot = -ux d_x rot - uy (d_y rot + beta).  bid = (row
// tile, run, -).  ST (ns2d.strat, strat/solver.py:27-32): 6 fields, products
// f_rot = -ux d_x rot - uy d_y rot and f_b = -ux d_x b - uy d_y b - N^2 uy.
template <typename T, int LOGM, int L, bool ST = false>
__device__ __forceinline__ void kf2_x_body(const cplx<T>* GBS_NS2D_RESTRICT W,
                                           cplx<T>* GBS_NS2D_RESTRICT F, const Geo& g,
                                           const cplx<T>* GBS_NS2D_RESTRICT twx,
                                           unsigned long long* vmax, uint3 bid) {
  constexpr int NF = ST ? 6 : 4, NFO = ST ? 2 : 1;
  using C = cplx<T>;
  using P = Line<LOGM>;
  constexpr int M = P::N, M8 = P::N8, LS = M;
  C* buf = reinterpret_cast<C*>(g_smem_fast);
  const int jt = threadIdx.x % M8;
  const int l = (threadIdx.x / M8) % L;
  const int f = threadIdx.x / (M8 * L);
  const int64_t nrows = g.ny;
  const int64_t nK = nrows * g.nkx;
  const int64_t row = (int64_t)bid.x * L + l;
  const bool valid = row < nrows;
  W += bid.y * 4 * nK;  // run of a batched ensemble
  F += bid.y * nK;
  C* slot = buf + (f * L + l) * LS;
  const SwzView<C, 1> acc{slot, 0};
  const int kcx = g.pr ? g.kcx : g.nkx + 1;
  C v[8];
  const C t0 = twx[jt];
  {
    const C* rowp = W + f * nK + row * g.nkx;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int j = jt + r * M8;
      C Z = mk<C>(0, 0);
      if (valid) {
        C a = j < kcx ? rowp[j] : mk<C>(0, 0);
        C b = (M - j) < kcx ? cconj(rowp[M - j]) : mk<C>(0, 0);
        if (j == 0) { a.y = 0; b.y = 0; }
        const C s = cadd(a, b), d = csub(a, b);
        const C wd = cmulc(d, twx_at(twx, t0, jt, r, M8));
        Z = mk<C>(s.x - wd.y, s.y + wd.x);
      }
      v[r] = Z;
    }
  }
  run<+1, LOGM, (Line<LOGM>::N8 <= 32)>(v, jt, true, acc, twx, 2);
#pragma unroll
  for (int i = 0; i < 8; ++i) acc.at(acc.base(jt), P::outm(i) * M8) = v[i];
  __syncthreads();
  T mx = 0, my = 0;
  const T beta = par<T>(g.beta, g.fbeta);
  for (int idx = threadIdx.x; idx < L * M; idx += blockDim.x) {
    const int ll = idx / M, j = idx % M;
    C* p0 = buf + ll * LS + padp<LOGM, C>(j);
    const C ux = p0[0], uy = p0[L * LS], px = p0[2 * L * LS], py = p0[3 * L * LS];
    C res;
    if (ST || g.beta == 0)  // (ns2d.strat has no beta term)
      res = mk<C>(-ux.x * px.x - uy.x * py.x, -ux.y * px.y - uy.y * py.y);
    else
      res = mk<C>(-ux.x * px.x - uy.x * (py.x + beta), -ux.y * px.y - uy.y * (py.y + beta));
    p0[0] = res;
    if (ST) {
      const C pxb = p0[4 * L * LS], pyb = p0[5 * L * LS];
      const T n2 = par<T>(g.N2, g.fN2);
      p0[L * LS] = mk<C>(-ux.x * pxb.x - uy.x * pyb.x - n2 * uy.x,
                         -ux.y * pxb.y - uy.y * pyb.y - n2 * uy.y);
    }
    if (vmax && (int64_t)bid.x * L + ll < nrows) {
      mx = fmax(mx, fmax(fabs(ux.x), fabs(ux.y)));
      my = fmax(my, fmax(fabs(uy.x), fabs(uy.y)));
    }
  }
  __syncthreads();
  if (vmax) block_max3(mx, my, T(0), vmax);
  const bool act = f < NFO;
#pragma unroll
  for (int r = 0; r < 8; ++r) v[r] = act ? acc.at(acc.base(jt), r * M8) : mk<C>(0, 0);
  // the line's first exchange overwrites positions other threads still read
  if (Line<LOGM>::N8 <= 32) __syncwarp(); else __syncthreads();
  run<-1, LOGM, (Line<LOGM>::N8 <= 32)>(v, jt, act, acc, twx, 2);
  if (act) {
#pragma unroll
    for (int i = 0; i < 8; ++i) acc.at(acc.base(jt), P::outm(i) * M8) = v[i];
  }
  __syncthreads();
  const int nout = g.pr ? (g.kcx < g.nkx ? g.kcx : g.nkx) : g.nkx;
  for (int idx = threadIdx.x; idx < NFO * L * nout; idx += blockDim.x) {
    const int k = idx % nout, ll = (idx / nout) % L, fo = idx / (nout * L);
    const int64_t rr = (int64_t)bid.x * L + ll;
    if (rr >= nrows) continue;
    const C* sl = buf + (fo * L + ll) * LS;
    C a = sl[padp<LOGM, C>(k == M ? 0 : k)];
    C b = cconj(sl[padp<LOGM, C>(k == 0 ? 0 : M - k)]);
    const C s = cadd(a, b), d = csub(a, b);
    const C wd = cmul(twx[k], d);
    const T h = T(0.5);
    F[fo * nK + rr * g.nkx + k] = mk<C>(h * (s.x + wd.y), h * (s.y - wd.x));
  }
}

// B with rows in pairs (as kf3_xp): rows 2 q, 2 q + 1 of a field are the
// real and imaginary parts of one N = nx point complex line; LP pairs per
// CTA, N/8 threads per line, the same threads and shared memory as
// kf2_x_body with L = 2 LP rows.
template <typename T, int LOGN, int LP, bool ST = false>
__device__ __forceinline__ void kf2_xp_body(const cplx<T>* GBS_NS2D_RESTRICT W,
                                            cplx<T>* GBS_NS2D_RESTRICT F, const Geo& g,
                                            const cplx<T>* GBS_NS2D_RESTRICT twx,
                                            unsigned long long* vmax, uint3 bid) {
  constexpr int NF = ST ? 6 : 4, NFO = ST ? 2 : 1;
  using C = cplx<T>;
  using P = Line<LOGN>;
  constexpr int N = P::N, N8 = P::N8, H = N / 2;
  constexpr bool WARP = N8 <= 32;
  C* buf = reinterpret_cast<C*>(g_smem_fast);
  const int jt = threadIdx.x % N8;
  const int lp = (threadIdx.x / N8) % LP;
  const int f = threadIdx.x / (N8 * LP);
  const int64_t nrows = g.ny;
  const int64_t nK = nrows * g.nkx;
  const int64_t row0 = ((int64_t)bid.x * LP + lp) * 2;
  const bool v0 = row0 < nrows, v1 = row0 + 1 < nrows;
  W += bid.y * 4 * nK;  // run of a batched ensemble
  F += bid.y * nK;
  const SwzView<C, 1> acc{buf + (f * LP + lp) * N, 0};
  const int kcx = g.pr ? g.kcx : g.nkx + 1;
  C v[8];
  {
    const C* r0 = W + f * nK + row0 * g.nkx;
    const C* r1 = r0 + g.nkx;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int idx = r < 4 ? jt + r * N8 : (8 - r) * N8 - jt;
      const bool in = idx < kcx;
      C a0 = (v0 && in) ? r0[idx] : mk<C>(0, 0);
      C a1 = (v1 && in) ? r1[idx] : mk<C>(0, 0);
      if ((r == 0 || r == 4) && jt == 0) { a0.y = 0; a1.y = 0; }
      v[r] = r < 4 ? mk<C>(a0.x - a1.y, a0.y + a1.x) : mk<C>(a0.x + a1.y, a1.x - a0.y);
    }
  }
  const int bar = WARP ? 0 : 1 + f * LP + lp;  // as in kf3_xp
  run<+1, LOGN, WARP>(v, jt, true, acc, twx, 1, bar);
  const int sj = acc.base(jt);
#pragma unroll
  for (int i = 0; i < 8; ++i) acc.at(sj, P::outm(i) * N8) = v[i];
  __syncthreads();
  T mx = 0, my = 0;
  const T beta = par<T>(g.beta, g.fbeta);
  const int64_t npairs = (nrows + 1) / 2;
  for (int idx = threadIdx.x; idx < LP * N; idx += blockDim.x) {
    const int ll = idx / N, j = idx % N;
    C* p0 = buf + ll * N + swz<C>(j);
    const C ux = p0[0], uy = p0[LP * N], px = p0[2 * LP * N], py = p0[3 * LP * N];
    C res;
    if (ST || g.beta == 0)  // (ns2d.strat has no beta term)
      res = mk<C>(-ux.x * px.x - uy.x * py.x, -ux.y * px.y - uy.y * py.y);
    else
      res = mk<C>(-ux.x * px.x - uy.x * (py.x + beta), -ux.y * px.y - uy.y * (py.y + beta));
    p0[0] = res;
    if (ST) {
      const C pxb = p0[4 * LP * N], pyb = p0[5 * LP * N];
      const T n2 = par<T>(g.N2, g.fN2);
      p0[LP * N] = mk<C>(-ux.x * pxb.x - uy.x * pyb.x - n2 * uy.x,
                         -ux.y * pxb.y - uy.y * pyb.y - n2 * uy.y);
    }
    if (vmax && (int64_t)bid.x * LP + ll < npairs) {
      mx = fmax(mx, fmax(fabs(ux.x), fabs(ux.y)));
      my = fmax(my, fmax(fabs(uy.x), fabs(uy.y)));
    }
  }
  __syncthreads();
  if (vmax) block_max3(mx, my, T(0), vmax);
  // product lines; idle lines skip this unless they share a warp's barriers
  const bool act = f < NFO;
  if (act || WARP) {
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = act ? acc.at(sj, r * N8) : mk<C>(0, 0);
    // the line's first exchange overwrites positions other threads still read
    line_sync<WARP, N8>(bar);
    run<-1, LOGN, WARP>(v, jt, act, acc, twx, 1, bar);
    if (act) {
#pragma unroll
      for (int i = 0; i < 8; ++i) acc.at(sj, P::outm(i) * N8) = v[i];
    }
  }
  __syncthreads();
  const int nout = g.pr ? (g.kcx < g.nkx ? g.kcx : g.nkx) : g.nkx;
  const T h = T(0.5);
  for (int idx = threadIdx.x; idx < NFO * LP * nout; idx += blockDim.x) {
    const int k = idx % nout, ll = (idx / nout) % LP, fo = idx / (nout * LP);
    const int64_t r0 = ((int64_t)bid.x * LP + ll) * 2;
    if (r0 >= nrows) continue;
    const C* sl = buf + (fo * LP + ll) * N;
    const C z = sl[swz<C>(k)];
    const C m = sl[swz<C>((N - k) & (N - 1))];
    C* Fo = F + fo * nK + r0 * g.nkx + k;
    Fo[0] = mk<C>(h * (z.x + m.x), h * (z.y - m.y));
    if (r0 + 1 < nrows) Fo[g.nkx] = mk<C>(h * (z.y + m.y), h * (m.x - z.x));
  }
}

// The ns2d x pass for L rows per CTA: in pairs when L is even (FP32).
template <typename T, int LOGM, int L, bool ST = false>
__device__ __forceinline__ void kf2_x_any(const cplx<T>* GBS_NS2D_RESTRICT W,
                                          cplx<T>* GBS_NS2D_RESTRICT F, const Geo& g,
                                          const cplx<T>* GBS_NS2D_RESTRICT twx,
                                          unsigned long long* vmax, uint3 bid) {
  if constexpr (sizeof(T) == 4 && L % 2 == 0)
    kf2_xp_body<T, LOGM + 1, L / 2, ST>(W, F, g, twx, vmax, bid);
  else
    kf2_x_body<T, LOGM, L, ST>(W, F, g, twx, vmax, bid);
}

template <typename T, int LOGM, int L, bool ST = false>
__global__ void __launch_bounds__((ST ? 6 : 4) * L * (1 << LOGM) / 8, 2)
kf2_x(const cplx<T>* __restrict__ W, cplx<T>* __restrict__ F, Geo g,
      const cplx<T>* __restrict__ twx, unsigned long long* vmax) {
  kf2_x_any<T, LOGM, L, ST>(W, F, g, twx, vmax, blockIdx);
}

// C: forward y pass + 1/N + dealiasing + RK4 stage (epilogue from registers).
// bid = (column tile, -, run).
template <typename T, int LOGN, int TX, bool EXT>
__device__ __forceinline__ void kf2_fwd_y_body(const cplx<T>* GBS_NS2D_RESTRICT F, Geo g,
                                               const cplx<T>* GBS_NS2D_RESTRICT twy, int mode,
                                               RKArgs a, const PerRun& pr, uint3 bid) {
  using C = cplx<T>;
  using P = Line<LOGN>;
  C* buf = reinterpret_cast<C*>(g_smem_fast);
  const int c = threadIdx.x % TX, jt = threadIdx.x / TX;
  const int ix = bid.x * TX + c;
  const bool valid = ix < g.ncx;
  // ns2d.strat: bid.y is the field (0: rot, which gets + i kx b of the state
  // the tendency is evaluated on, strat/solver.py:185; 1: b)
  const C* bin = (g.strat && bid.y == 0)
                     ? static_cast<const C*>(a.in) + (int64_t)g.ny * g.nkx : nullptr;
  {  // run of a batched ensemble (or field of ns2d.strat): its fields and parameters
    const int64_t off = ((int64_t)bid.z * (g.strat ? 2 : 1) + bid.y) * g.ny * g.nkx;
    F += off;
    if (a.S) a.S = static_cast<const C*>(a.S) + off;
    if (a.Sout) a.Sout = static_cast<C*>(a.Sout) + off;
    if (a.tmp) a.tmp = static_cast<C*>(a.tmp) + off;
    if (a.tmp1) a.tmp1 = static_cast<C*>(a.tmp1) + off;
    if (a.tend) a.tend = static_cast<C*>(a.tend) + off;
    if (a.add) a.add = static_cast<const C*>(a.add) + off;
    if (pr.dt) {
      a.dt = pr.dt[bid.z];
      g.nu2 = pr.nu2[bid.z];
      g.nu8 = pr.nu8[bid.z];
      a.fdt = (float)a.dt;
      g.fnu2 = (float)g.nu2;
      g.fnu8 = (float)g.nu8;
    }
  }
  C v[8];
#pragma unroll
  for (int r = 0; r < 8; ++r)
    v[r] = valid ? F[(int64_t)(jt + r * P::N8) * g.nkx + ix] : mk<C>(0, 0);
  const SwzView<C, TX> acc{buf, c};
  run<-1, LOGN>(v, jt, true, acc, twy, 1);
  if (!valid) return;
  const T kx = wavenum<T>(g.dkx, g.fdkx, ix);
  const T inv_n = T(g.inv_n);
  const Phys q = phys_of(g);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int iy = jt + P::outm(i) * P::N8;
    const int kyi = kadim(iy, P::N);
    const bool rm = ix >= g.kcx || iabs(kyi) >= g.kcy;
    if (g.pr && rm) continue;
    const T ky = wavenum<T>(g.dky, g.fdky, kyi);
    const int64_t idx = (int64_t)iy * g.nkx + ix;
    C Nv = cscale(v[i], inv_n);
    if (bin) {
      const C b = bin[idx];
      Nv = cadd(Nv, mk<C>(-kx * b.y, kx * b.x));
    }
    stage_epilogue1<C, T, EXT>(mode, a, idx, Nv, kx, ky, ix == 0 && kyi == 0, rm, q);
  }
}

template <typename T, int LOGN, int TX, bool EXT>
__global__ void __launch_bounds__(TX * (1 << LOGN) / 8, min_blocks(TX * (1 << LOGN) / 8))
kf2_fwd_y(const cplx<T>* __restrict__ F, Geo g, const cplx<T>* __restrict__ twy,
          int mode, RKArgs a, PerRun pr) {
  kf2_fwd_y_body<T, LOGN, TX, EXT>(F, g, twy, mode, a, pr, blockIdx);
}

}  // namespace fast
}  // namespace gbs
