// Batched ns2d ensembles: many independent runs of one grid size advanced
// together, one launch per pass for the whole batch (the run index is a
// grid dimension), each run with its own viscosities and time step.  The
// column width of the y passes and the rows per CTA of the x pass are
// runtime choices among compiled variants, picked by the autotuner of
// fluidsim_gb300.ensemble.  Float32 (the ensemble configuration's
// precision); single runs and float64 go through gbs_ns.
#include <new>

// The persistent step below runs the ns2d pass bodies on fields that other
// CTAs write during the same launch: no read-only (non-coherent) loads.
#define GBS_NS2D_RESTRICT
#include "gbs_fast_launch.cuh"
#include "gbs_internal.cuh"

namespace gbs {

template <typename T> int make_twiddles(cplx<T>* tw, int n, cudaStream_t st);

namespace fast {

template <int LOGN, int TX>
static int ensA(const Geo& g, const void* S, void* W, const void* tw, int nb, cudaStream_t st) {
  using C = cplx<float>;
  constexpr int TH = TX * (1 << LOGN) / 8;
  const size_t smem = sizeof(C) * (size_t)(1 << LOGN) * TX;
  int rc = prep(kf2_inv_y<float, LOGN, TX, false>, smem);
  if (rc) return rc;
  kf2_inv_y<float, LOGN, TX, false><<<dim3(ceil_div(g.ncx, TX), 1, nb), TH, smem, st>>>(
      static_cast<const C*>(S), static_cast<C*>(W), g, static_cast<const C*>(tw));
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

template <int LOGM, int L>
static int ensB(const Geo& g, const void* W, void* F, const void* tw, int nb, cudaStream_t st) {
  using C = cplx<float>;
  constexpr int M = 1 << LOGM;
  constexpr int TH = 4 * L * M / 8;
  const size_t smem = sizeof(C) * (size_t)4 * L * M;
  int rc = prep(kf2_x<float, LOGM, L>, smem);
  if (rc) return rc;
  kf2_x<float, LOGM, L><<<dim3(ceil_div(g.ny, L), nb), TH, smem, st>>>(
      static_cast<const C*>(W), static_cast<C*>(F), g, static_cast<const C*>(tw), nullptr);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

template <int LOGN, int TX>
static int ensC(const Geo& g, const void* F, const void* tw, int mode, const RKArgs& a,
                const PerRun& pr, int nb, cudaStream_t st) {
  using C = cplx<float>;
  constexpr int TH = TX * (1 << LOGN) / 8;
  const size_t smem = sizeof(C) * (size_t)(1 << LOGN) * TX;
  int rc = prep(kf2_fwd_y<float, LOGN, TX, false>, smem);
  if (rc) return rc;
  kf2_fwd_y<float, LOGN, TX, false><<<dim3(ceil_div(g.ncx, TX), 1, nb), TH, smem, st>>>(
      static_cast<const C*>(F), g, static_cast<const C*>(tw), mode, a, pr);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

#define GBS_ENS_LOG(logv, BODY)                       \
  switch (logv) {                                     \
    case 6: { constexpr int LG = 6; BODY; } break;    \
    case 7: { constexpr int LG = 7; BODY; } break;    \
    case 8: { constexpr int LG = 8; BODY; } break;    \
    case 9: { constexpr int LG = 9; BODY; } break;    \
    default:                                          \
      set_error("ensemble: size not compiled");       \
      return GBS_EINVAL;                              \
  }

#define GBS_ENS_TX(tx, BODY)                          \
  switch (tx) {                                       \
    case 4: { constexpr int TXV = 4; BODY; } break;   \
    case 8: { constexpr int TXV = 8; BODY; } break;   \
    case 16: { constexpr int TXV = 16; BODY; } break; \
    default:                                          \
      set_error("ensemble: tile width not compiled"); \
      return GBS_EINVAL;                              \
  }

#define GBS_ENS_L(lv, BODY)                           \
  switch (lv) {                                       \
    case 1: { constexpr int LV = 1; BODY; } break;    \
    case 2: { constexpr int LV = 2; BODY; } break;    \
    case 4: { constexpr int LV = 4; BODY; } break;    \
    case 8: { constexpr int LV = 8; BODY; } break;    \
    default:                                          \
      set_error("ensemble: rows per CTA not compiled"); \
      return GBS_EINVAL;                              \
  }

// ------------------------------------------------ one launch for all sizes
// Groups of different sizes advanced by one launch per pass: every CTA finds
// its group from the launch's CTA offsets and runs that size's compiled
// body.  All CTAs of a launch have TH threads and TH * 64 bytes of shared
// memory: the column passes take TH * 8 / ny columns per CTA, the x pass
// 2 TH / (nx / 2) rows.  TH per pass is the autotuner's choice.
constexpr int kMixMax = 4;

struct MixGroup {
  Geo g;
  const void* in;  // stage input (the state or tmp1)
  void *W, *F;
  const void *twx, *twy;
  RKArgs a;
  PerRun pr;
  int logy, logm;
  int ctaA, ctaB, ctaC;  // CTAs per run of each pass
  int startA, startB, startC;
};

struct MixArgs {
  MixGroup grp[kMixMax];
  int ngroups;
  int mode;
};

__device__ __forceinline__ int mix_group(const MixArgs& m, int pass) {
  int gi = 0;
  for (int k = 1; k < m.ngroups; ++k) {
    const int st = pass == 0 ? m.grp[k].startA : (pass == 1 ? m.grp[k].startB : m.grp[k].startC);
    if ((int)blockIdx.x >= st) gi = k;
  }
  return gi;
}

// column width for ny = 2^LOGN at TH threads (>= 4 is checked on the host)
template <int TH, int LOGN> struct MixTX {
  static constexpr int v = (TH * 8 >> LOGN) < 1 ? 1 : (TH * 8 >> LOGN);
};
template <int TH, int LOGM> struct MixRows {
  static constexpr int v = (2 * TH >> LOGM) < 1 ? 1 : (2 * TH >> LOGM);
};

template <int TH>
__global__ void __launch_bounds__(TH, min_blocks(TH)) kmix_inv_y(const __grid_constant__ MixArgs m) {
  const MixGroup& G = m.grp[mix_group(m, 0)];
  const int local = blockIdx.x - G.startA;
  const uint3 b = make_uint3(local % G.ctaA, 0, local / G.ctaA);
  const float2* S = static_cast<const float2*>(G.in);
  float2* W = static_cast<float2*>(G.W);
  const float2* tw = static_cast<const float2*>(G.twy);
  switch (G.logy) {
    case 6: kf2_inv_y_body<float, 6, MixTX<TH, 6>::v, false>(S, W, G.g, tw, b); break;
    case 7: kf2_inv_y_body<float, 7, MixTX<TH, 7>::v, false>(S, W, G.g, tw, b); break;
    case 8: kf2_inv_y_body<float, 8, MixTX<TH, 8>::v, false>(S, W, G.g, tw, b); break;
    default: kf2_inv_y_body<float, 9, MixTX<TH, 9>::v, false>(S, W, G.g, tw, b); break;
  }
}

template <int TH>
__global__ void __launch_bounds__(TH, TH >= 512 ? 2 : 1024 / TH)
kmix_x(const __grid_constant__ MixArgs m) {
  const MixGroup& G = m.grp[mix_group(m, 1)];
  const int local = blockIdx.x - G.startB;
  const uint3 b = make_uint3(local % G.ctaB, local / G.ctaB, 0);
  const float2* W = static_cast<const float2*>(G.W);
  float2* F = static_cast<float2*>(G.F);
  const float2* tw = static_cast<const float2*>(G.twx);
  switch (G.logm) {
    case 5: kf2_x_any<float, 5, MixRows<TH, 5>::v>(W, F, G.g, tw, nullptr, b); break;
    case 6: kf2_x_any<float, 6, MixRows<TH, 6>::v>(W, F, G.g, tw, nullptr, b); break;
    case 7: kf2_x_any<float, 7, MixRows<TH, 7>::v>(W, F, G.g, tw, nullptr, b); break;
    case 8: kf2_x_any<float, 8, MixRows<TH, 8>::v>(W, F, G.g, tw, nullptr, b); break;
    default: kf2_x_any<float, 9, MixRows<TH, 9>::v>(W, F, G.g, tw, nullptr, b); break;
  }
}

template <int TH>
__global__ void __launch_bounds__(TH, min_blocks_lo(TH)) kmix_fwd_y(const __grid_constant__ MixArgs m) {
  const MixGroup& G = m.grp[mix_group(m, 2)];
  const int local = blockIdx.x - G.startC;
  const uint3 b = make_uint3(local % G.ctaC, 0, local / G.ctaC);
  const float2* F = static_cast<const float2*>(G.F);
  const float2* tw = static_cast<const float2*>(G.twy);
  switch (G.logy) {
    case 6: kf2_fwd_y_body<float, 6, MixTX<TH, 6>::v, false>(F, G.g, tw, m.mode, G.a, G.pr, b); break;
    case 7: kf2_fwd_y_body<float, 7, MixTX<TH, 7>::v, false>(F, G.g, tw, m.mode, G.a, G.pr, b); break;
    case 8: kf2_fwd_y_body<float, 8, MixTX<TH, 8>::v, false>(F, G.g, tw, m.mode, G.a, G.pr, b); break;
    default: kf2_fwd_y_body<float, 9, MixTX<TH, 9>::v, false>(F, G.g, tw, m.mode, G.a, G.pr, b); break;
  }
}

#define GBS_MIX_TH(th, BODY)                          \
  switch (th) {                                       \
    case 128: { constexpr int THV = 128; BODY; } break; \
    case 256: { constexpr int THV = 256; BODY; } break; \
    case 512: { constexpr int THV = 512; BODY; } break; \
    default:                                          \
      set_error("ensemble: thread count not compiled"); \
      return GBS_EINVAL;                              \
  }

template <int TH> static int mixA(const MixArgs& m, int ncta, cudaStream_t st) {
  const size_t smem = (size_t)TH * 64;
  int rc = prep(kmix_inv_y<TH>, smem);
  if (rc) return rc;
  kmix_inv_y<TH><<<ncta, TH, smem, st>>>(m);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}
template <int TH> static int mixB(const MixArgs& m, int ncta, cudaStream_t st) {
  const size_t smem = (size_t)TH * 64;
  int rc = prep(kmix_x<TH>, smem);
  if (rc) return rc;
  kmix_x<TH><<<ncta, TH, smem, st>>>(m);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}
template <int TH> static int mixC(const MixArgs& m, int ncta, cudaStream_t st) {
  const size_t smem = (size_t)TH * 64;
  int rc = prep(kmix_fwd_y<TH>, smem);
  if (rc) return rc;
  kmix_fwd_y<TH><<<ncta, TH, smem, st>>>(m);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}

// ------------------------------------------- one persistent launch per call
// Every CTA of one cooperative launch takes work items from a queue (an
// atomic ticket) in the order (RK stage, pass, group, run, tile) and runs
// the pass body of the item.  Dependencies are per run: the x pass of a run
// waits until all inverse-y tiles of that run (this stage) are done, the
// forward-y pass until all its x rows are done, and the inverse-y pass of
// the next stage until all forward-y tiles of the previous one are done (the
// next stage reads tmp1 and overwrites W, which those tiles used).  A wait
// only ever targets items earlier in the queue, all taken by resident CTAs
// (cooperative launch), so it ends; each wait is bounded by timeout_ns all
// the same, after which the CTA writes an error status word and every CTA
// leaves at its next wait or ticket.
struct PersistArgs {
  MixGroup grp[kMixMax];
  int ngroups;
  int nstages;            // 4 per RK4 step
  int runs[kMixMax];      // runs per group
  int run_base[kMixMax];  // first run of the group in the counters
  int64_t nA, nB, nC;     // items per stage of each pass (all groups)
  unsigned* ticket;       // queue position (zeroed before the launch)
  unsigned* done;         // per run: completed A, B, C items (zeroed)
  int* status;            // 0, or kPersistTimeout
  unsigned long long timeout_ns;
  int stall_test;         // test hook: one dependency needs an item too many
  int chunk;              // tickets a CTA takes at a time
  int tpi[3];             // tiles per work item of each pass (grp[].cta*: items per run)
  int tiles[kMixMax][3];  // tiles per run of each pass
};

// tiles per work item of the persistent step's passes: the x pass's tiles
// (a few rows) are small next to an item's fixed costs (ticket, decode,
// dependency check, two CTA barriers).  96-run C4 ensemble, ms per step:
// x-pass tiles per item 1: 0.787, 4: 0.731, 8: 0.728; two column tiles
// per item as well: 0.838.
#ifndef GBS_PERSIST_TPI_A
#define GBS_PERSIST_TPI_A 1
#endif
#ifndef GBS_PERSIST_TPI_B
#define GBS_PERSIST_TPI_B 8
#endif
#ifndef GBS_PERSIST_TPI_C
#define GBS_PERSIST_TPI_C 1
#endif

constexpr int kPersistTimeout = 1;

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Thread 0 of a CTA: wait until *p >= target, another CTA failed, or the
// time limit passed.  Returns false on failure (the status word is set).
__device__ bool wait_count(const unsigned* p, unsigned target, int* status,
                           unsigned long long timeout_ns) {
  const unsigned long long t0 = globaltimer_ns();
  for (;;) {
    if (ld_acquire(p) >= target) return true;
    if (*(volatile int*)status) return false;
    if (globaltimer_ns() - t0 > timeout_ns) {
      atomicCAS(status, 0, kPersistTimeout);
      return false;
    }
    __nanosleep(100);
  }
}

// Group of item `local` within a pass block (groups in order, `per` items
// per run of each group).
__device__ __forceinline__ int persist_group(const PersistArgs& p, int pass, int64_t& local) {
  for (int k = 0; k < p.ngroups; ++k) {
    const MixGroup& G = p.grp[k];
    const int per = pass == 0 ? G.ctaA : (pass == 1 ? G.ctaB : G.ctaC);
    const int64_t n = (int64_t)per * p.runs[k];
    if (local < n) return k;
    local -= n;
  }
  return p.ngroups - 1;
}

template <int TH>
__global__ void __launch_bounds__(TH, min_blocks(TH)) kpersist(const __grid_constant__ PersistArgs p) {
  __shared__ int64_t s_item;
  __shared__ int s_fail;
  const int64_t per_stage = p.nA + p.nB + p.nC;
  const int64_t total = per_stage * p.nstages;
  // thread 0's queue state (in shared memory: only thread 0 uses it): the
  // rest of its chunk of tickets, the last dependency known to be met, and
  // completions not yet published (published before any wait, when the
  // counter changes, and at the end of a chunk)
  __shared__ int64_t next, chunk_end;
  __shared__ const unsigned* known_q;
  __shared__ unsigned known_target, npend;
  __shared__ unsigned* pend;
  if (threadIdx.x == 0) {
    next = chunk_end = 0;
    known_q = nullptr;
    known_target = npend = 0;
    pend = nullptr;
  }
  auto flush = [&]() {
    if (npend) {
      __threadfence();
      atomicAdd(pend, npend);
      npend = 0;
    }
  };
  for (;;) {
    if (threadIdx.x == 0) {
      int64_t item = total;
      if (!*(volatile int*)p.status) {
        if (next == chunk_end) {
          flush();
          next = (int64_t)atomicAdd(p.ticket, (unsigned)p.chunk);
          chunk_end = next + p.chunk;
        }
        item = next < total ? next++ : total;
      }
      if (item >= total) flush();
      s_item = item;
      s_fail = 0;
    }
    __syncthreads();
    const int64_t t = s_item;
    if (t >= total) break;
    const int sigma = (int)(t / per_stage);  // stage of the launch
    int64_t r = t % per_stage;
    const int pass = r < p.nA ? 0 : (r < p.nA + p.nB ? 1 : 2);
    r -= pass == 0 ? 0 : (pass == 1 ? p.nA : p.nA + p.nB);
    const int gi = persist_group(p, pass, r);
    const MixGroup& G = p.grp[gi];
    const int per = pass == 0 ? G.ctaA : (pass == 1 ? G.ctaB : G.ctaC);
    const int run = (int)(r / per), item = (int)(r % per);
    unsigned* cnt = p.done + 3 * (int64_t)(p.run_base[gi] + run);
    if (threadIdx.x == 0) {
      unsigned target = 0;
      const unsigned* q = cnt;
      if (pass == 0) {
        q = cnt + 2;
        target = (unsigned)sigma * G.ctaC;
      } else if (pass == 1) {
        q = cnt;
        target = (unsigned)(sigma + 1) * G.ctaA;
        if (p.stall_test && sigma == 0 && gi == 0 && run == 0) target += 1;
      } else {
        q = cnt + 1;
        target = (unsigned)(sigma + 1) * G.ctaB;
      }
      if (target > 0 && !(q == known_q && target <= known_target)) {
        flush();
        if (wait_count(q, target, p.status, p.timeout_ns)) {
          known_q = q;
          known_target = target;
        } else {
          s_fail = 1;
        }
      }
    }
    __syncthreads();
    if (s_fail) break;
    const int mode = kRK0 + (sigma & 3);
    RKArgs a = G.a;
    const float2* in = static_cast<const float2*>(mode == kRK0 ? a.S : a.tmp1);
    const int tpi = p.tpi[pass], ntile = p.tiles[gi][pass];
    for (int sub = 0; sub < tpi; ++sub) {
      const int tile = item * tpi + sub;
      if (tile >= ntile) break;
      if (sub) __syncthreads();  // the previous tile's shared memory is free
      if (pass == 0) {
        const uint3 b = make_uint3(tile, 0, run);
        float2* W = static_cast<float2*>(G.W);
        const float2* tw = static_cast<const float2*>(G.twy);
        switch (G.logy) {
          case 6: kf2_inv_y_body<float, 6, MixTX<TH, 6>::v, false>(in, W, G.g, tw, b); break;
          case 7: kf2_inv_y_body<float, 7, MixTX<TH, 7>::v, false>(in, W, G.g, tw, b); break;
          case 8: kf2_inv_y_body<float, 8, MixTX<TH, 8>::v, false>(in, W, G.g, tw, b); break;
          default: kf2_inv_y_body<float, 9, MixTX<TH, 9>::v, false>(in, W, G.g, tw, b); break;
        }
      } else if (pass == 1) {
        const uint3 b = make_uint3(tile, run, 0);
        const float2* W = static_cast<const float2*>(G.W);
        float2* F = static_cast<float2*>(G.F);
        const float2* tw = static_cast<const float2*>(G.twx);
        switch (G.logm) {
          case 5: kf2_x_any<float, 5, MixRows<TH, 5>::v>(W, F, G.g, tw, nullptr, b); break;
          case 6: kf2_x_any<float, 6, MixRows<TH, 6>::v>(W, F, G.g, tw, nullptr, b); break;
          case 7: kf2_x_any<float, 7, MixRows<TH, 7>::v>(W, F, G.g, tw, nullptr, b); break;
          case 8: kf2_x_any<float, 8, MixRows<TH, 8>::v>(W, F, G.g, tw, nullptr, b); break;
          default: kf2_x_any<float, 9, MixRows<TH, 9>::v>(W, F, G.g, tw, nullptr, b); break;
        }
      } else {
        const uint3 b = make_uint3(tile, 0, run);
        const float2* F = static_cast<const float2*>(G.F);
        const float2* tw = static_cast<const float2*>(G.twy);
        switch (G.logy) {
          case 6: kf2_fwd_y_body<float, 6, MixTX<TH, 6>::v, false>(F, G.g, tw, mode, a, G.pr, b); break;
          case 7: kf2_fwd_y_body<float, 7, MixTX<TH, 7>::v, false>(F, G.g, tw, mode, a, G.pr, b); break;
          case 8: kf2_fwd_y_body<float, 8, MixTX<TH, 8>::v, false>(F, G.g, tw, mode, a, G.pr, b); break;
          default: kf2_fwd_y_body<float, 9, MixTX<TH, 9>::v, false>(F, G.g, tw, mode, a, G.pr, b); break;
        }
      }
    }
    __syncthreads();  // the item's writes are done (and its shared memory free)
    if (threadIdx.x == 0) {
      if (pend != cnt + pass) {
        flush();
        pend = cnt + pass;
      }
      ++npend;
    }
  }
}

}  // namespace fast

struct Ensemble {
  int nx, ny, nkx, nruns;
  int64_t nK;
  fast::Geo geo;
  void *twx, *twy;
  void *W, *F, *tmp, *tmp1;
  double *nu2, *nu8, *dt;  // device, per run
  int* dflag;
  int txA, Lb, txC;
};

static void ens_free(Ensemble* e) {
  void* p[] = {e->twx, e->twy, e->W, e->F, e->tmp, e->tmp1, e->nu2, e->nu8, e->dt, e->dflag};
  for (void* q : p)
    if (q) cudaFree(q);
}

}  // namespace gbs

struct gbs_ens2d {
  gbs::Ensemble e;
};

namespace gbs {

static int ens_eval(Ensemble* e, const void* in, int mode, const RKArgs& a, bool pr,
                    cudaStream_t st) {
  fast::Geo g = e->geo;
  g.pr = pr ? 1 : 0;
  g.ncx = pr ? (g.kcx < g.nkx ? g.kcx : g.nkx) : g.nkx;
  const int lgy = ilog2(e->ny), lgm = ilog2(e->nx / 2);
  const int nb = e->nruns;
  int rc = GBS_OK;
  GBS_ENS_LOG(lgy, GBS_ENS_TX(e->txA, rc = (fast::ensA<LG, TXV>(g, in, e->W, e->twy, nb, st))));
  if (rc) return rc;
  GBS_ENS_LOG(lgm, GBS_ENS_L(e->Lb, rc = (fast::ensB<LG, LV>(g, e->W, e->F, e->twx, nb, st))));
  if (rc) return rc;
  fast::PerRun prr{e->nu2, e->nu8, e->dt};
  GBS_ENS_LOG(lgy, GBS_ENS_TX(e->txC, rc = (fast::ensC<LG, TXV>(g, e->F, e->twy, mode, a, prr,
                                                               nb, st))));
  return rc;
}

// Groups stepped by one launch per pass (they are not owned).
struct EnsembleMix {
  Ensemble* e[fast::kMixMax];
  int n;
  int thA, thB, thC;  // threads per CTA of the inverse, x and forward passes
  unsigned* pbuf;     // persistent step: ticket, per-run counters, status
  int nruns_total;
  int persist_chunk;  // tickets per grab of the persistent step
};

// every group's tiles at these thread counts: columns 4..64 wide, >= 1 row
static bool mix_fits(const EnsembleMix* x, int thA, int thB, int thC) {
  for (int k = 0; k < x->n; ++k) {
    const Ensemble* e = x->e[k];
    for (int th : {thA, thC}) {
      const int tx = th * 8 / e->ny;
      if (tx < 4 || tx > 64) return false;
    }
    if (2 * thB / (e->nx / 2) < 1) return false;
  }
  return true;
}

static int mix_eval(EnsembleMix* x, void* const* states, int mode, bool pr, cudaStream_t st) {
  fast::MixArgs m;
  memset(&m, 0, sizeof(m));
  m.ngroups = x->n;
  m.mode = mode;
  int a0 = 0, b0 = 0, c0 = 0;
  for (int k = 0; k < x->n; ++k) {
    Ensemble* e = x->e[k];
    fast::MixGroup& G = m.grp[k];
    G.g = e->geo;
    G.g.pr = pr ? 1 : 0;
    G.g.ncx = pr ? (G.g.kcx < G.g.nkx ? G.g.kcx : G.g.nkx) : G.g.nkx;
    G.in = mode == kRK0 ? states[k] : e->tmp1;
    G.W = e->W;
    G.F = e->F;
    G.twx = e->twx;
    G.twy = e->twy;
    G.a.S = states[k];
    G.a.Sout = states[k];
    G.a.tmp = e->tmp;
    G.a.tmp1 = e->tmp1;
    G.a.nan_flag = e->dflag;
    G.pr = fast::PerRun{e->nu2, e->nu8, e->dt};
    G.logy = ilog2(e->ny);
    G.logm = ilog2(e->nx / 2);
    G.ctaA = ceil_div(G.g.ncx, x->thA * 8 / e->ny);
    G.ctaB = ceil_div(e->ny, 2 * x->thB / (e->nx / 2));
    G.ctaC = ceil_div(G.g.ncx, x->thC * 8 / e->ny);
    G.startA = a0;
    G.startB = b0;
    G.startC = c0;
    a0 += G.ctaA * e->nruns;
    b0 += G.ctaB * e->nruns;
    c0 += G.ctaC * e->nruns;
  }
  int rc = GBS_OK;
  GBS_MIX_TH(x->thA, rc = fast::mixA<THV>(m, a0, st));
  if (rc) return rc;
  GBS_MIX_TH(x->thB, rc = fast::mixB<THV>(m, b0, st));
  if (rc) return rc;
  GBS_MIX_TH(x->thC, rc = fast::mixC<THV>(m, c0, st));
  return rc;
}

template <int TH>
static int persist_launch(EnsembleMix* x, void* const* states, int nsteps,
                          double timeout_s, bool stall_test, int chunk, cudaStream_t st) {
  fast::PersistArgs p;
  memset(&p, 0, sizeof(p));
  p.ngroups = x->n;
  p.nstages = 4 * nsteps;
  p.tpi[0] = GBS_PERSIST_TPI_A;
  p.tpi[1] = GBS_PERSIST_TPI_B;
  p.tpi[2] = GBS_PERSIST_TPI_C;
  int rb = 0;
  for (int k = 0; k < x->n; ++k) {
    Ensemble* e = x->e[k];
    fast::MixGroup& G = p.grp[k];
    G.g = e->geo;
    G.g.pr = 1;  // every stage of the launch starts from a dealiased state
    G.g.ncx = G.g.kcx < G.g.nkx ? G.g.kcx : G.g.nkx;
    G.W = e->W;
    G.F = e->F;
    G.twx = e->twx;
    G.twy = e->twy;
    G.a.S = states[k];
    G.a.Sout = states[k];
    G.a.tmp = e->tmp;
    G.a.tmp1 = e->tmp1;
    G.a.nan_flag = e->dflag;
    G.pr = fast::PerRun{e->nu2, e->nu8, e->dt};
    G.logy = ilog2(e->ny);
    G.logm = ilog2(e->nx / 2);
    // tiles per run of each pass, then work items per run
    p.tiles[k][0] = ceil_div(G.g.ncx, TH * 8 / e->ny);
    p.tiles[k][1] = ceil_div(e->ny, 2 * TH / (e->nx / 2));
    p.tiles[k][2] = p.tiles[k][0];
    G.ctaA = ceil_div(p.tiles[k][0], p.tpi[0]);
    G.ctaB = ceil_div(p.tiles[k][1], p.tpi[1]);
    G.ctaC = ceil_div(p.tiles[k][2], p.tpi[2]);
    p.runs[k] = e->nruns;
    p.run_base[k] = rb;
    rb += e->nruns;
    p.nA += (int64_t)G.ctaA * e->nruns;
    p.nB += (int64_t)G.ctaB * e->nruns;
    p.nC += (int64_t)G.ctaC * e->nruns;
  }
  p.ticket = x->pbuf;
  p.done = x->pbuf + 1;
  p.status = reinterpret_cast<int*>(x->pbuf + 1 + 3 * (int64_t)rb);
  p.timeout_ns = (unsigned long long)(timeout_s * 1e9);
  p.stall_test = stall_test ? 1 : 0;
  p.chunk = chunk;
  const size_t smem = (size_t)TH * 64;
  int rc = fast::prep(fast::kpersist<TH>, smem);
  if (rc) return rc;
  int dev = 0, nsm = 0, per_sm = 0;
  GBS_CUDA_TRY(cudaGetDevice(&dev));
  GBS_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  GBS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fast::kpersist<TH>, TH,
                                                             smem));
  if (per_sm < 1) {
    set_error("ensemble persistent step: no CTA of %d threads fits on an SM", TH);
    return GBS_EINVAL;
  }
  // the counters are zeroed except the status word, which keeps an earlier
  // failure until gbs_ens2d_persistent_status reads it
  GBS_CUDA_TRY(cudaMemsetAsync(x->pbuf, 0, sizeof(unsigned) * (1 + 3 * (size_t)rb), st));
  void* args[] = {&p};
  GBS_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)fast::kpersist<TH>, dim3(nsm * per_sm),
                                           dim3(TH), args, smem, st));
  return GBS_OK;
}

}  // namespace gbs

struct gbs_ens2d_mixed {
  gbs::EnsembleMix x;
};

extern "C" {

int gbs_ens2d_mixed_create(gbs_ens2d* const* groups, int ngroups, gbs_ens2d_mixed** out) {
  gbs::clear_error();
  if (!out || !groups || ngroups < 1 || ngroups > gbs::fast::kMixMax) {
    gbs::set_error("gbs_ens2d_mixed_create: 1..%d groups", gbs::fast::kMixMax);
    return GBS_EINVAL;
  }
  *out = nullptr;
  gbs_ens2d_mixed* h = new (std::nothrow) gbs_ens2d_mixed();
  if (!h) return GBS_ENOMEM;
  h->x.n = ngroups;
  for (int k = 0; k < ngroups; ++k) {
    if (!groups[k]) {
      delete h;
      gbs::set_error("gbs_ens2d_mixed_create: null group");
      return GBS_EINVAL;
    }
    h->x.e[k] = &groups[k]->e;
  }
  h->x.thA = h->x.thB = h->x.thC = 512;
  h->x.persist_chunk = 4;
  if (!gbs::mix_fits(&h->x, 512, 512, 512)) {
    delete h;
    gbs::set_error("gbs_ens2d_mixed_create: a group size has no single-launch tile");
    return GBS_EINVAL;
  }
  int runs = 0;
  for (int k = 0; k < ngroups; ++k) runs += h->x.e[k]->nruns;
  h->x.nruns_total = runs;
  const size_t pb = sizeof(unsigned) * (2 + 3 * (size_t)runs);
  if (cudaMalloc(&h->x.pbuf, pb) != cudaSuccess ||
      cudaMemset(h->x.pbuf, 0, pb) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
    (void)cudaGetLastError();
    if (h->x.pbuf) cudaFree(h->x.pbuf);
    delete h;
    gbs::set_error("gbs_ens2d_mixed_create: device allocation failed");
    return GBS_ENOMEM;
  }
  *out = h;
  return GBS_OK;
}

int gbs_ens2d_mixed_set_tuning(gbs_ens2d_mixed* h, int th_inverse, int th_x, int th_forward) {
  gbs::clear_error();
  auto ok = [](int t) { return t == 128 || t == 256 || t == 512; };
  if (!h || !ok(th_inverse) || !ok(th_x) || !ok(th_forward) ||
      !gbs::mix_fits(&h->x, th_inverse, th_x, th_forward)) {
    gbs::set_error("gbs_ens2d_mixed_set_tuning: threads in {128, 256, 512} giving every "
                   "group 4..64 columns and >= 1 row per CTA");
    return GBS_EINVAL;
  }
  h->x.thA = th_inverse;
  h->x.thB = th_x;
  h->x.thC = th_forward;
  return GBS_OK;
}

int gbs_ens2d_mixed_destroy(gbs_ens2d_mixed* h) {
  if (h && h->x.pbuf) cudaFree(h->x.pbuf);
  delete h;
  return GBS_OK;
}

// nsteps RK4 steps of every run of every group in one persistent cooperative
// launch (after one ordinary step when the states are not known dealiased).
int gbs_ens2d_persistent_step(gbs_ens2d_mixed* h, void* const* states, int nsteps,
                              int threads, double timeout_s, int flags, void* stream) {
  gbs::clear_error();
  if (!h || !states || nsteps < 1 || (threads != 256 && threads != 512) ||
      !(timeout_s > 0) || !gbs::mix_fits(&h->x, threads, threads, threads)) {
    gbs::set_error("gbs_ens2d_persistent_step: invalid argument (threads 256 or 512 giving "
                   "every group 4..64 columns and >= 1 row per CTA, timeout > 0)");
    return GBS_EINVAL;
  }
  for (int k = 0; k < h->x.n; ++k) {
    if (!states[k]) {
      gbs::set_error("gbs_ens2d_persistent_step: null state");
      return GBS_EINVAL;
    }
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = GBS_OK;
  if (!(flags & GBS_STEP_DEALIASED)) {  // first step from an arbitrary state
    for (int m = gbs::kRK0; m <= gbs::kRK3 && !rc; ++m)
      rc = gbs::mix_eval(&h->x, states, m, false, st);
    if (rc || --nsteps == 0) return rc;
  }
  const bool stall = (flags & GBS_STEP_TEST_STALL) != 0;
  const int chunk = h->x.persist_chunk;
  if (threads == 256)
    return gbs::persist_launch<256>(&h->x, states, nsteps, timeout_s, stall, chunk, st);
  return gbs::persist_launch<512>(&h->x, states, nsteps, timeout_s, stall, chunk, st);
}

int gbs_ens2d_persistent_set_chunk(gbs_ens2d_mixed* h, int chunk) {
  gbs::clear_error();
  if (!h || chunk < 1 || chunk > 64) {
    gbs::set_error("gbs_ens2d_persistent_set_chunk: chunk in 1..64");
    return GBS_EINVAL;
  }
  h->x.persist_chunk = chunk;
  return GBS_OK;
}

int gbs_ens2d_persistent_status(gbs_ens2d_mixed* h, int* status) {
  gbs::clear_error();
  if (!h || !status) {
    gbs::set_error("gbs_ens2d_persistent_status: null argument");
    return GBS_EINVAL;
  }
  int* d = reinterpret_cast<int*>(h->x.pbuf + 1 + 3 * (size_t)h->x.nruns_total);
  GBS_CUDA_TRY(cudaMemcpy(status, d, sizeof(int), cudaMemcpyDeviceToHost));
  GBS_CUDA_TRY(cudaMemset(d, 0, sizeof(int)));
  return *status ? GBS_ETIMEDOUT : GBS_OK;
}

// nsteps RK4 steps of every run of every group; states[k]: the state of group
// k.  Three launches per RK4 stage for all the groups together.
int gbs_ens2d_mixed_step(gbs_ens2d_mixed* h, void* const* states, int nsteps, int flags,
                         void* stream) {
  gbs::clear_error();
  if (!h || !states || nsteps < 1) {
    gbs::set_error("gbs_ens2d_mixed_step: invalid argument");
    return GBS_EINVAL;
  }
  for (int k = 0; k < h->x.n; ++k) {
    if (!states[k]) {
      gbs::set_error("gbs_ens2d_mixed_step: null state");
      return GBS_EINVAL;
    }
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool pr = (flags & GBS_STEP_DEALIASED) != 0;
  for (int it = 0; it < nsteps; ++it) {
    const bool p = pr || it > 0;
    for (int m = gbs::kRK0; m <= gbs::kRK3; ++m) {
      const int rc = gbs::mix_eval(&h->x, states, m, p, st);
      if (rc) return rc;
    }
  }
  return GBS_OK;
}


int gbs_ens2d_create(int64_t nx, int64_t ny, double Lx, double Ly, int64_t nruns,
                     int64_t kcut_x, int64_t kcut_y, double beta, gbs_ens2d** out) {
  gbs::clear_error();
  if (!out || nruns < 1 || nruns > 65535 || nx % 2 || !gbs::is_pow2((int)ny) ||
      !gbs::is_pow2((int)(nx / 2)) || ny < 64 || ny > 512 || nx / 2 < 64 || nx / 2 > 512 ||
      !(Lx > 0) || !(Ly > 0)) {
    gbs::set_error("gbs_ens2d_create: invalid argument (power-of-two 128..1024 x 64..512)");
    return GBS_EINVAL;
  }
  *out = nullptr;
  gbs_ens2d* h = new (std::nothrow) gbs_ens2d();
  if (!h) return GBS_ENOMEM;
  gbs::Ensemble* e = &h->e;
  memset(e, 0, sizeof(*e));
  e->nx = (int)nx;
  e->ny = (int)ny;
  e->nkx = (int)(nx / 2 + 1);
  e->nruns = (int)nruns;
  e->nK = (int64_t)ny * e->nkx;
  gbs::fast::Geo& g = e->geo;
  g.nx = e->nx;
  g.ny = e->ny;
  g.nz = 1;
  g.nkx = e->nkx;
  g.M = e->nx / 2;
  g.kcx = (int)(kcut_x < nx ? kcut_x : nx + 1);
  g.kcy = (int)(kcut_y < ny ? kcut_y : ny + 1);
  g.kcz = 1 << 30;
  g.ncx = e->nkx;
  g.nky_keep = e->ny;
  const double pi2 = 6.283185307179586;
  g.dkx = pi2 / Lx;
  g.dky = pi2 / Ly;
  g.beta = beta;
  g.inv_n = 1.0 / ((double)nx * ny);
  g.k2_hypo0 = g.dkx * g.dkx;
  gbs::fast::geo_f32(g);
  e->txA = 8;
  e->Lb = 2;
  e->txC = 8;
  const size_t fb = sizeof(float2) * e->nK * nruns;
  int rc = 0;
  if (cudaMalloc(&e->twx, sizeof(float2) * nx) != cudaSuccess ||
      cudaMalloc(&e->twy, sizeof(float2) * ny) != cudaSuccess ||
      cudaMalloc(&e->W, fb * 4) != cudaSuccess || cudaMalloc(&e->F, fb) != cudaSuccess ||
      cudaMalloc(&e->tmp, fb) != cudaSuccess || cudaMalloc(&e->tmp1, fb) != cudaSuccess ||
      cudaMalloc(&e->nu2, sizeof(double) * nruns) != cudaSuccess ||
      cudaMalloc(&e->nu8, sizeof(double) * nruns) != cudaSuccess ||
      cudaMalloc(&e->dt, sizeof(double) * nruns) != cudaSuccess ||
      cudaMalloc(&e->dflag, sizeof(int)) != cudaSuccess) {
    gbs::set_error("gbs_ens2d_create: device allocation failed");
    rc = GBS_ENOMEM;
  }
  if (!rc) rc = gbs::make_twiddles<float>(static_cast<float2*>(e->twx), e->nx, 0);
  if (!rc) rc = gbs::make_twiddles<float>(static_cast<float2*>(e->twy), e->ny, 0);
  if (!rc && (cudaMemset(e->tmp, 0, fb) != cudaSuccess ||
              cudaMemset(e->tmp1, 0, fb) != cudaSuccess ||
              cudaMemset(e->dflag, 0, sizeof(int)) != cudaSuccess ||
              cudaDeviceSynchronize() != cudaSuccess)) {
    gbs::set_error("gbs_ens2d_create: %s", cudaGetErrorString(cudaGetLastError()));
    rc = GBS_ECUDA;
  }
  if (rc) {
    gbs::ens_free(e);
    delete h;
    return rc;
  }
  *out = h;
  return GBS_OK;
}

int gbs_ens2d_destroy(gbs_ens2d* h) {
  if (!h) return GBS_OK;
  gbs::ens_free(&h->e);
  delete h;
  return GBS_OK;
}

int gbs_ens2d_set_params(gbs_ens2d* h, const double* nu2, const double* nu8, const double* dt) {
  gbs::clear_error();
  if (!h || !nu2 || !nu8 || !dt) {
    gbs::set_error("gbs_ens2d_set_params: null argument");
    return GBS_EINVAL;
  }
  gbs::Ensemble* e = &h->e;
  const size_t b = sizeof(double) * e->nruns;
  GBS_CUDA_TRY(cudaMemcpy(e->nu2, nu2, b, cudaMemcpyHostToDevice));
  GBS_CUDA_TRY(cudaMemcpy(e->nu8, nu8, b, cudaMemcpyHostToDevice));
  GBS_CUDA_TRY(cudaMemcpy(e->dt, dt, b, cudaMemcpyHostToDevice));
  return GBS_OK;
}

int gbs_ens2d_set_tuning(gbs_ens2d* h, int tx_inverse, int rows_x, int tx_forward) {
  gbs::clear_error();
  auto okt = [](int t) { return t == 4 || t == 8 || t == 16; };
  auto okl = [](int l) { return l == 1 || l == 2 || l == 4 || l == 8; };
  if (!h || !okt(tx_inverse) || !okt(tx_forward) || !okl(rows_x)) {
    gbs::set_error("gbs_ens2d_set_tuning: tile width in {4, 8, 16}, rows in {1, 2, 4, 8}");
    return GBS_EINVAL;
  }
  h->e.txA = tx_inverse;
  h->e.Lb = rows_x;
  h->e.txC = tx_forward;
  return GBS_OK;
}

// nsteps RK4 steps of every run (state: nruns x (ny, nx/2+1) complex64).
// Enqueue only (no host synchronisation): the calls can be captured into a
// CUDA graph.  Dealiasing of the state is followed by the NaN flag.
int gbs_ens2d_step(gbs_ens2d* h, void* S, int nsteps, int flags, void* stream) {
  gbs::clear_error();
  if (!h || !S || nsteps < 1) {
    gbs::set_error("gbs_ens2d_step: invalid argument");
    return GBS_EINVAL;
  }
  gbs::Ensemble* e = &h->e;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool pr = (flags & GBS_STEP_DEALIASED) != 0;
  gbs::RKArgs a{};
  a.S = S;
  a.Sout = S;
  a.tmp = e->tmp;
  a.tmp1 = e->tmp1;
  a.nan_flag = e->dflag;
  a.dt = 0.0;  // per run
  for (int it = 0; it < nsteps; ++it) {
    // a step that starts from an arbitrary state runs unpruned; the next ones
    // start from the dealiased output of the previous step
    const bool p = pr || it > 0;
    int rc = gbs::ens_eval(e, S, gbs::kRK0, a, p, st);
    if (rc) return rc;
    for (int m = gbs::kRK1; m <= gbs::kRK3; ++m) {
      rc = gbs::ens_eval(e, e->tmp1, m, a, p, st);
      if (rc) return rc;
    }
  }
  return GBS_OK;
}

int gbs_ens2d_nan_flag(gbs_ens2d* h, int* flag) {
  gbs::clear_error();
  if (!h || !flag) {
    gbs::set_error("gbs_ens2d_nan_flag: null argument");
    return GBS_EINVAL;
  }
  GBS_CUDA_TRY(cudaMemcpy(flag, h->e.dflag, sizeof(int), cudaMemcpyDeviceToHost));
  GBS_CUDA_TRY(cudaMemset(h->e.dflag, 0, sizeof(int)));
  return GBS_OK;
}

}  // extern "C"
