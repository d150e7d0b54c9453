// Launch shapes and runtime dispatch for the compile-time-size kernels.
#pragma once

#include <cstdlib>

#include "gbs_fast.cuh"
#include "gbs_fast_api.h"

namespace gbs {
namespace fast {

// columns per CTA for the strided passes (FP64: 4, 64 B segments); FP32
// widths per pass are compile-time knobs, set by A/B at 512^3 (ms per pruned
// launch): the ns2d column passes GBS_TX_COL = 8, the plain column kernel
// below (col_launch), the fused z passes of the ns3d step 16 (128 B
// segments of lines 1 MB apart: curl + inverse z 0.779 -> 0.756, forward z
// + RK4 0.843 -> 0.758; 4: 1.146 and 1.281)
#ifndef GBS_TX_COL
#define GBS_TX_COL 8
#endif
#ifndef GBS_TX_INVZ
#define GBS_TX_INVZ 16
#endif
#ifndef GBS_TX_FWDZ
#define GBS_TX_FWDZ 16
#endif
// (capped so that a CTA has at most 1024 threads: TX * N / 8 <= 1024)
constexpr int tx_cap(int tx, int logn) { return tx * (1 << logn) / 8 <= 1024 ? tx : 8192 >> logn; }
template <typename T, int LOGN> constexpr int tx_cols() {
  return tx_cap(sizeof(T) == 4 ? GBS_TX_COL : 4, LOGN);
}
// FP64 z passes: 4 columns (8: 512^3 FP64 3.20 -> 3.17 steps/s)
#ifndef GBS_TX_Z64
#define GBS_TX_Z64 4
#endif
template <typename T, int LOGN> constexpr int tx_invz() {
  return tx_cap(sizeof(T) == 4 ? GBS_TX_INVZ : GBS_TX_Z64, LOGN);
}
template <typename T, int LOGN> constexpr int tx_fwdz() {
  return tx_cap(sizeof(T) == 4 ? GBS_TX_FWDZ : GBS_TX_Z64, LOGN);
}
// rows per CTA for the x passes
#ifndef GBS_X_THREADS
#define GBS_X_THREADS 384
#endif
template <typename T, int LOGM, int NF> constexpr int rows_x() {
  constexpr int M8 = (1 << LOGM) / 8;
  constexpr int budget = (sizeof(T) == 4 ? GBS_X_THREADS : 192) / NF;
  return budget / M8 > 0 ? budget / M8 : 1;
}

// (the opt-in is set for every size: static shared memory, e.g. of the CFL
// reduction, counts against the 48 KB default too)
template <typename K>
static int prep(K kernel, size_t smem) {
  GBS_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
  GBS_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                    cudaSharedmemCarveoutMaxShared));
  return GBS_OK;
}

// L2 prefetch distance of the plain column passes: the CTAs resident on the
// whole GPU (x GBS_PF from the environment, default 0.5; 0 turns it off).
// (Measured at 512^3 FP32: inverse y -9 %, forward y -15 %; the same
// prefetch slowed the curl / x / forward-z kernels, which do not use it.
// With the 16-column tiles, ms per pruned launch inverse / forward y:
// GBS_PF 0: 1.076 / 0.566, 0.5: 0.905 / 0.447, 1: 0.920 / 0.452, 2: 1.026 /
// 0.587.)
static double env_knob(const char* name, double dflt) {
  const char* e = getenv(name);
  return e && *e ? atof(e) : dflt;
}

template <typename K>
static int prefetch_distance(K kernel, int threads, size_t smem) {
  static const double scale = env_knob("GBS_PF", 0.5);
  int nb = 0, dev = 0, nsm = 0;
  if (scale <= 0) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, smem) != cudaSuccess ||
      cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return (int)(nb * nsm * scale);
}

#define GBS_LOG_SWITCH(logv, BODY)                    \
  switch (logv) {                                     \
    case 5: { constexpr int LG = 5; BODY; } break;    \
    case 6: { constexpr int LG = 6; BODY; } break;    \
    case 7: { constexpr int LG = 7; BODY; } break;    \
    case 8: { constexpr int LG = 8; BODY; } break;    \
    case 9: { constexpr int LG = 9; BODY; } break;    \
    case 10: { constexpr int LG = 10; BODY; } break;  \
    default:                                          \
      set_error("no compiled kernel for this size");  \
      return GBS_EINVAL;                              \
  }

// Plain column passes (FP32): GBS_TX_COLY columns for row-strided lines
// (y passes), GBS_TX_COLZ for plane-strided ones (lines >= 64 KB apart: z
// passes of the standalone FFT).  Tiles of 16 columns (128-byte row
// segments) take one exchange slot, so that two CTAs of 1024 threads (32
// registers) fit; 8 columns take two slots.  Measured at 512^3 (ms per
// pruned launch, 8 -> 16 columns): inverse y 0.942 -> 0.930, forward y
// 0.500 -> 0.452; standalone R2C + C2R 0.803 -> 0.748 ms each (16 columns
// with two slots: inverse y 1.11, one CTA per SM); steps/s +3 % at 256^3,
// +4 % at 128^3, but -1.5 % at 64^3: lines shorter than 128 points keep 8.
#ifndef GBS_TX_COLY
#define GBS_TX_COLY 16
#endif
#ifndef GBS_TX_COLZ
#define GBS_TX_COLZ 16
#endif
template <typename T, int LOGN, int DIR, bool PLANE>
static int col_launch(const void* in, void* out, const ColArgs& a, int nouter, int nfields,
                      const void* tw, double scale, cudaStream_t st) {
  using C = cplx<T>;
  constexpr int TX = sizeof(T) != 4 ? tx_cols<T, LOGN>()
                     : (LOGN < 7 ? 8 : tx_cap(PLANE ? GBS_TX_COLZ : GBS_TX_COLY, LOGN));
  // one slot when two would hold 128 KB or more (16 columns of 512, 8 of 1024)
  constexpr bool SLOT1 = sizeof(T) == 4 && (TX > 8 || TX * (1 << LOGN) >= 8192);
  constexpr int TH = TX * (1 << LOGN) / 8;
  const size_t smem = (SLOT1 ? 1 : 2) * sizeof(C) * (size_t)(1 << LOGN) * TX;
  int rc = prep(kf_col<T, LOGN, TX, DIR, SLOT1>, smem);
  if (rc) return rc;
  static const int pf = prefetch_distance(kf_col<T, LOGN, TX, DIR, SLOT1>, TH, smem);
  ColArgs ap = a;
  dim3 grid(ceil_div(a.ncols, TX), nouter, nfields);
  // in grid rows (a resident wave of CTAs, rounded up); only for
  // row-strided columns (y passes): with plane strides (z passes) the next
  // wave's tiles span every plane
  const int dy = (int)((pf + grid.x - 1) / grid.x);
  ap.pf = (!PLANE && dy < (int)grid.y) ? dy : 0;
  kf_col<T, LOGN, TX, DIR, SLOT1><<<grid, TH, smem, st>>>(static_cast<const C*>(in),
                                                        static_cast<C*>(out), ap,
                                                        static_cast<const C*>(tw), T(scale));
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

template <typename T>
int col(int n, const void* in, void* out, const ColArgs& a, int nouter, int nfields,
        const void* tw, double scale, int dir, cudaStream_t st) {
  const int lg = ilog2(n);
  const bool plane = a.es * (int64_t)sizeof(cplx<T>) > 65536;
  if (dir > 0 && plane) {
    GBS_LOG_SWITCH(lg, return (col_launch<T, LG, 1, true>(in, out, a, nouter, nfields, tw, scale, st)));
  } else if (dir > 0) {
    GBS_LOG_SWITCH(lg, return (col_launch<T, LG, 1, false>(in, out, a, nouter, nfields, tw, scale, st)));
  } else if (plane) {
    GBS_LOG_SWITCH(lg, return (col_launch<T, LG, -1, true>(in, out, a, nouter, nfields, tw, scale, st)));
  } else {
    GBS_LOG_SWITCH(lg, return (col_launch<T, LG, -1, false>(in, out, a, nouter, nfields, tw, scale, st)));
  }
  return GBS_OK;
}

template <typename T, int LOGM>
static int r2c_launch(const void* x, void* k, int64_t nrows, const void* tw, double scale,
                      cudaStream_t st) {
  using C = cplx<T>;
  constexpr int M = 1 << LOGM;
  constexpr int L = (sizeof(T) == 4 ? 256 : 128) / (M / 8) > 0 ? (sizeof(T) == 4 ? 256 : 128) / (M / 8) : 1;
  constexpr int TH = L * M / 8;
  const size_t smem = sizeof(C) * (size_t)L * M;
  int rc = prep(kf_row_r2c<T, LOGM, L>, smem);
  if (rc) return rc;
  kf_row_r2c<T, LOGM, L><<<ceil_div(nrows, L), TH, smem, st>>>(
      static_cast<const T*>(x), static_cast<C*>(k), nrows, static_cast<const C*>(tw), T(scale));
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

template <typename T>
int r2c_rows(int nx, const void* x, void* k, int64_t nrows, const void* twx, double scale,
             cudaStream_t st) {
  GBS_LOG_SWITCH(ilog2(nx / 2), return (r2c_launch<T, LG>(x, k, nrows, twx, scale, st)));
  return GBS_OK;
}

template <typename T, int LOGM>
static int c2r_launch(const void* k, void* x, int64_t nrows, const void* tw, cudaStream_t st) {
  using C = cplx<T>;
  constexpr int M = 1 << LOGM;
  constexpr int L = (sizeof(T) == 4 ? 256 : 128) / (M / 8) > 0 ? (sizeof(T) == 4 ? 256 : 128) / (M / 8) : 1;
  constexpr int TH = L * M / 8;
  const size_t smem = sizeof(C) * (size_t)L * M;
  int rc = prep(kf_row_c2r<T, LOGM, L>, smem);
  if (rc) return rc;
  kf_row_c2r<T, LOGM, L><<<ceil_div(nrows, L), TH, smem, st>>>(
      static_cast<const C*>(k), static_cast<T*>(x), nrows, static_cast<const C*>(tw));
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

template <typename T>
int c2r_rows(int nx, const void* k, void* x, int64_t nrows, const void* twx, cudaStream_t st) {
  GBS_LOG_SWITCH(ilog2(nx / 2), return (c2r_launch<T, LG>(k, x, nrows, twx, st)));
  return GBS_OK;
}

template <typename T, int LOGN, bool ST, bool PH>
static int A3_launch(const Geo& g, const void* S, void* W, const void* tw, cudaStream_t st) {
  using C = cplx<T>;
  constexpr int TX = tx_invz<T, LOGN>();
  constexpr int TH = TX * (1 << LOGN) / 8;
  const size_t smem = 3 * sizeof(C) * (size_t)(1 << LOGN) * TX;  // exchange, hold, stage
  int rc = prep(kf3_inv_z<T, LOGN, TX, ST, PH>, smem);
  if (rc) return rc;
  dim3 grid(ceil_div(g.ncx, TX), g.nky_keep);
  kf3_inv_z<T, LOGN, TX, ST, PH><<<grid, TH, smem, st>>>(static_cast<const C*>(S),
                                                    static_cast<C*>(W), g,
                                                    static_cast<const C*>(tw));
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

template <typename T>
int A3(const Geo& g, const void* S, void* W, const void* twz, cudaStream_t st) {
  if (g.strat) {
    GBS_LOG_SWITCH(ilog2(g.nz), return (A3_launch<T, LG, true, false>(g, S, W, twz, st)));
  } else if (g.phase) {
    GBS_LOG_SWITCH(ilog2(g.nz), return (A3_launch<T, LG, false, true>(g, S, W, twz, st)));
  } else {
    GBS_LOG_SWITCH(ilog2(g.nz), return (A3_launch<T, LG, false, false>(g, S, W, twz, st)));
  }
  return GBS_OK;
}

template <typename T, int LOGM, bool ST>
static int B3_launch(const Geo& g, const void* W, void* F, const void* tw,
                     unsigned long long* vmax, cudaStream_t st) {
  using C = cplx<T>;
  constexpr int NF = ST ? 7 : 6;
  constexpr int L = rows_x<T, LOGM, NF>();
  constexpr int M = 1 << LOGM;
  constexpr int TH = NF * L * M / 8;
  const size_t smem = sizeof(C) * (size_t)NF * L * M;
  int rc = prep(kf3_x<T, LOGM, L, ST>, smem);
  if (rc) return rc;
  kf3_x<T, LOGM, L, ST><<<ceil_div((int64_t)g.nz * g.ny, L), TH, smem, st>>>(
      static_cast<const C*>(W), static_cast<C*>(F), g, static_cast<const C*>(tw), vmax);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

// Rows in pairs (kf3_xp): nx <= 1024 (one CTA of <= 1024 threads holds the
// NF lines of a pair), LP pairs per CTA up to GBS_X_THREADS threads.
// (512^3 FP32: 1.81 -> 1.55 ms against kf3_x's half-length real transforms.)
template <typename T, int LOGM, bool ST>
static int B3p_launch(const Geo& g, const void* W, void* F, const void* tw,
                      unsigned long long* vmax, cudaStream_t st) {
  using C = cplx<T>;
  constexpr int LOGN = LOGM + 1, N = 1 << LOGN, N8 = N / 8;
  constexpr int NF = ST ? 7 : 6;
  constexpr int LP = GBS_X_THREADS / NF / N8 > 0 ? GBS_X_THREADS / NF / N8 : 1;
  constexpr int TH = NF * LP * N8;
  const size_t smem = sizeof(C) * (size_t)NF * LP * N * (xp_alt<LOGN>() ? 2 : 1);
  int rc = prep(kf3_xp<T, LOGN, LP, ST>, smem);
  if (rc) return rc;
  const int64_t npairs = ((int64_t)g.nz * g.ny + 1) / 2;
  kf3_xp<T, LOGN, LP, ST><<<ceil_div(npairs, LP), TH, smem, st>>>(
      static_cast<const C*>(W), static_cast<C*>(F), g, static_cast<const C*>(tw), vmax);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

// Rows in pairs with the products in registers (kf3_xr): FP32 ns3d, LP
// pairs per CTA up to GBS_XR_THREADS threads.  Used for nx = 256 .. 1024
// (ms per pruned launch against kf3_xp: nx = 256 0.150 / 0.185 at 256^3,
// 512 1.210 / 1.324 at 512^3, 1024 0.412 / 0.452 at 1024x256x128); at
// nx = 64 and 128 its 16 warps per SM lose to kf3_xp's occupancy (0.0142 /
// 0.0101 at 64^3, 0.0407 / 0.0283 at 128^3).
#ifndef GBS_XR_LOGM_MIN
#define GBS_XR_LOGM_MIN 7
#endif
#ifndef GBS_XR_LOGM_MAX
#define GBS_XR_LOGM_MAX 9
#endif
template <typename T, int LOGM>
static int B3r_launch(const Geo& g, const void* W, void* F, const void* tw,
                      unsigned long long* vmax, const XStage& xs, cudaStream_t st) {
  using C = cplx<T>;
  constexpr int LOGN = LOGM + 1, N8 = (1 << LOGN) / 8;
  constexpr int LP = GBS_XR_THREADS / N8 > 0 ? GBS_XR_THREADS / N8 : 1;
  static_assert(N8 <= 32 || LP <= 15, "one named barrier per pair (ids 1..15)");
  constexpr int TH = LP * N8;
  const size_t smem = sizeof(C) * (size_t)LP * xr_slot<LOGN>();
  int rc = prep(kf3_xr<T, LOGN, LP>, smem);
  if (rc) return rc;
  const int64_t npairs = ((int64_t)g.nz * g.ny + 1) / 2;
  kf3_xr<T, LOGN, LP><<<ceil_div(npairs, LP), TH, smem, st>>>(
      static_cast<const C*>(W), static_cast<C*>(F), g, static_cast<const C*>(tw), vmax, xs);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

template <typename T, int LOGM, bool ST>
static int B3_pick(const Geo& g, const void* W, void* F, const void* tw,
                   unsigned long long* vmax, const XStage& xs, cudaStream_t st) {
#ifndef GBS_X_NOREG
  // (whole row pairs: the pair's staging copy spans both rows)
  if constexpr (sizeof(T) == 4 && !ST && LOGM >= GBS_XR_LOGM_MIN && LOGM <= GBS_XR_LOGM_MAX)
    if (((int64_t)g.nz * g.ny) % 2 == 0) return B3r_launch<T, LOGM>(g, W, F, tw, vmax, xs, st);
#endif
  // FP64 takes the paired form too, at one CTA per SM (up to 168
  // registers): the half-length form's FP64 instantiations spill 400-1700
  // bytes at their 40 registers (512^3 FP64 3.20 -> 3.34 steps/s)
  if constexpr (LOGM <= 9) return B3p_launch<T, LOGM, ST>(g, W, F, tw, vmax, st);
  else return B3_launch<T, LOGM, ST>(g, W, F, tw, vmax, st);
}

template <typename T>
int B3(const Geo& g, const void* W, void* F, const void* twx, unsigned long long* vmax,
       const XStage& xs, cudaStream_t st) {
  if (g.strat) {
    GBS_LOG_SWITCH(ilog2(g.M), return (B3_pick<T, LG, true>(g, W, F, twx, vmax, xs, st)));
  } else {
    GBS_LOG_SWITCH(ilog2(g.M), return (B3_pick<T, LG, false>(g, W, F, twx, vmax, xs, st)));
  }
  return GBS_OK;
}

// ns3d.strat keeps 4 field slots: narrower column tiles keep them within
// ~64 KB of shared memory
template <typename T, int LOGN, bool ST>
constexpr int tx_c3() {
  constexpr int tx = tx_fwdz<T, LOGN>();
  if (!ST) return tx;
  constexpr int cap = (64 * 1024) / (4 * (1 << LOGN) * (int)sizeof(cplx<T>));
  return cap >= tx ? tx : (cap >= 4 ? 4 : (cap >= 2 ? 2 : 1));
}

template <typename T, int LOGN, bool ST, bool EXT>
static int C3_launch(const Geo& g, const void* F, const void* tw, int mode, const RKArgs& a,
                     cudaStream_t st) {
  using C = cplx<T>;
  constexpr int TX = tx_c3<T, LOGN, ST>();
  constexpr int TH = TX * (1 << LOGN) / 8;
  const size_t smem = sizeof(C) * (size_t)(ST ? 4 : 3) * (1 << LOGN) * TX;
  int rc = prep(kf3_fwd_z<T, LOGN, TX, ST, EXT>, smem);
  if (rc) return rc;
  dim3 grid(ceil_div(g.ncx, TX), g.nky_keep);
  kf3_fwd_z<T, LOGN, TX, ST, EXT><<<grid, TH, smem, st>>>(static_cast<const C*>(F), g,
                                                    static_cast<const C*>(tw), mode, a);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

template <typename T>
int C3(const Geo& g, const void* F, const void* twz, int mode, const RKArgs& a,
       cudaStream_t st) {
  // RK4 stages and plain tendencies with the default projector use the lean
  // epilogue
  const bool ext = mode > kRK3 || a.phase || g.proj != 0 || g.no_vz_kz0;
  if (g.strat && ext) {
    GBS_LOG_SWITCH(ilog2(g.nz), return (C3_launch<T, LG, true, true>(g, F, twz, mode, a, st)));
  } else if (g.strat) {
    GBS_LOG_SWITCH(ilog2(g.nz), return (C3_launch<T, LG, true, false>(g, F, twz, mode, a, st)));
  } else if (ext) {
    GBS_LOG_SWITCH(ilog2(g.nz), return (C3_launch<T, LG, false, true>(g, F, twz, mode, a, st)));
  } else {
    GBS_LOG_SWITCH(ilog2(g.nz), return (C3_launch<T, LG, false, false>(g, F, twz, mode, a, st)));
  }
  return GBS_OK;
}

template <typename T, int LOGN, bool PH>
static int A2_launch(const Geo& g, const void* S, void* W, const void* tw, cudaStream_t st) {
  using C = cplx<T>;
  constexpr int TX = tx_cols<T, LOGN>();
  constexpr int TH = TX * (1 << LOGN) / 8;
  const size_t smem = sizeof(C) * (size_t)(1 << LOGN) * TX;
  int rc = prep(kf2_inv_y<T, LOGN, TX, PH>, smem);
  if (rc) return rc;
  kf2_inv_y<T, LOGN, TX, PH><<<ceil_div(g.ncx, TX), TH, smem, st>>>(
      static_cast<const C*>(S), static_cast<C*>(W), g, static_cast<const C*>(tw));
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

template <typename T>
int A2(const Geo& g, const void* S, void* W, const void* twy, cudaStream_t st) {
  if (g.phase) {
    GBS_LOG_SWITCH(ilog2(g.ny), return (A2_launch<T, LG, true>(g, S, W, twy, st)));
  } else {
    GBS_LOG_SWITCH(ilog2(g.ny), return (A2_launch<T, LG, false>(g, S, W, twy, st)));
  }
  return GBS_OK;
}

template <typename T, int LOGM, bool ST>
static int B2_launch(const Geo& g, const void* W, void* F, const void* tw,
                     unsigned long long* vmax, cudaStream_t st) {
  using C = cplx<T>;
  constexpr int NF = ST ? 6 : 4;
  constexpr int L = rows_x<T, LOGM, NF>();
  constexpr int M = 1 << LOGM;
  constexpr int TH = NF * L * M / 8;
  const size_t smem = sizeof(C) * (size_t)NF * L * M;
  int rc = prep(kf2_x<T, LOGM, L, ST>, smem);
  if (rc) return rc;
  kf2_x<T, LOGM, L, ST><<<ceil_div(g.ny, L), TH, smem, st>>>(
      static_cast<const C*>(W), static_cast<C*>(F), g, static_cast<const C*>(tw), vmax);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

template <typename T>
int B2(const Geo& g, const void* W, void* F, const void* twx, unsigned long long* vmax,
       cudaStream_t st) {
  if (g.strat) {
    GBS_LOG_SWITCH(ilog2(g.M), return (B2_launch<T, LG, true>(g, W, F, twx, vmax, st)));
  } else {
    GBS_LOG_SWITCH(ilog2(g.M), return (B2_launch<T, LG, false>(g, W, F, twx, vmax, st)));
  }
  return GBS_OK;
}

template <typename T, int LOGN, bool PH>
static int C2_launch(const Geo& g, const void* F, const void* tw, int mode, const RKArgs& a,
                     cudaStream_t st) {
  using C = cplx<T>;
  constexpr int TX = tx_cols<T, LOGN>();
  constexpr int TH = TX * (1 << LOGN) / 8;
  const size_t smem = sizeof(C) * (size_t)(1 << LOGN) * TX;
  int rc = prep(kf2_fwd_y<T, LOGN, TX, PH>, smem);
  if (rc) return rc;
  kf2_fwd_y<T, LOGN, TX, PH><<<dim3(ceil_div(g.ncx, TX), g.strat ? 2 : 1), TH, smem, st>>>(
      static_cast<const C*>(F), g, static_cast<const C*>(tw), mode, a, PerRun{});
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

template <typename T>
int C2(const Geo& g, const void* F, const void* twy, int mode, const RKArgs& a,
       cudaStream_t st) {
  if (mode > kRK3 || a.phase) {
    GBS_LOG_SWITCH(ilog2(g.ny), return (C2_launch<T, LG, true>(g, F, twy, mode, a, st)));
  } else {
    GBS_LOG_SWITCH(ilog2(g.ny), return (C2_launch<T, LG, false>(g, F, twy, mode, a, st)));
  }
  return GBS_OK;
}

#define GBS_FAST_INSTANTIATE(T)                                                              \
  template int r2c_rows<T>(int, const void*, void*, int64_t, const void*, double,            \
                           cudaStream_t);                                                    \
  template int c2r_rows<T>(int, const void*, void*, int64_t, const void*, cudaStream_t);     \
  template int col<T>(int, const void*, void*, const ColArgs&, int, int, const void*, double, \
                      int, cudaStream_t);                                                    \
  template int A3<T>(const Geo&, const void*, void*, const void*, cudaStream_t);             \
  template int B3<T>(const Geo&, const void*, void*, const void*, unsigned long long*,       \
                     const XStage&, cudaStream_t);                                           \
  template int C3<T>(const Geo&, const void*, const void*, int, const RKArgs&, cudaStream_t); \
  template int A2<T>(const Geo&, const void*, void*, const void*, cudaStream_t);             \
  template int B2<T>(const Geo&, const void*, void*, const void*, unsigned long long*,       \
                     cudaStream_t);                                                          \
  template int C2<T>(const Geo&, const void*, const void*, int, const RKArgs&, cudaStream_t);

}  // namespace fast
}  // namespace gbs
