// Host check of the shared-memory address arithmetic of the compile-time-size
// kernels (gbs_fast.cuh), built by nvcc and run on the CPU:
//   - swz<C> maps every 128-byte group of E elements onto itself (a
//     permutation inside each group);
//   - swz_join(swz(b), K) == swz(b | K) for every b, K with no common bit
//     (the exchange addressing of run() relies on it);
//   - Line<LOGN>::outm is a permutation of 0..7 and inv_outm inverts it;
//   - the per-pair shared memory of kf3_xr (xr_slot) is a multiple of 16
//     elements, and its stash and staging buffers start 16-byte aligned.
// Prints "ok" and returns 0, or prints the first failure and returns 1.
#include <cstdio>
#include <vector>

#include "../../fluidsim_gb300/csrc/gbs_fast.cuh"

using namespace gbs;
using namespace gbs::fast;

template <typename C>
static int check_swz(int span) {
  constexpr int E = 128 / sizeof(C);
  std::vector<int> seen(span, 0);
  for (int q = 0; q < span; ++q) {
    const int s = swz<C>(q);
    if (s / E != q / E || s < 0 || s >= span) {
      printf("swz<%zu>(%d) = %d leaves its group\n", sizeof(C), q, s);
      return 1;
    }
    if (seen[s]++) {
      printf("swz<%zu> maps two positions to %d\n", sizeof(C), s);
      return 1;
    }
  }
  for (int b = 0; b < span; ++b)
    for (int K = 0; K < span; ++K) {
      if (b & K) continue;
      if (swz_join<C>(swz<C>(b), K) != swz<C>(b | K)) {
        printf("swz_join<%zu>(swz(%d), %d) != swz(%d)\n", sizeof(C), b, K, b | K);
        return 1;
      }
    }
  return 0;
}

template <int LOGN>
static int check_line() {
  int seen = 0;
  for (int i = 0; i < 8; ++i) {
    const int r = Line<LOGN>::outm(i);
    if (r < 0 || r >= 8 || (seen >> r) & 1) {
      printf("Line<%d>::outm is not a permutation\n", LOGN);
      return 1;
    }
    seen |= 1 << r;
    if (inv_outm<LOGN>(r) != i) {
      printf("inv_outm<%d>(%d) != %d\n", LOGN, r, i);
      return 1;
    }
  }
  return 0;
}

template <int LOGN>
static int check_xr() {
  constexpr int N = 1 << LOGN, H = N / 2, E = 16;
  constexpr int ALT = xp_alt<LOGN>() ? N : 0;
  constexpr int PART = H > E ? H : E;
  constexpr int stash = N + ALT + PART, stage = stash + N;
  if (xr_slot<LOGN>() % 16 || stash % 2 || stage % 2 || (N + 2) % 2 ||
      xr_slot<LOGN>() < stage + 2 * (N + 2)) {
    printf("kf3_xr shared-memory layout of LOGN = %d misaligned or short\n", LOGN);
    return 1;
  }
  return 0;
}

int main() {
  int bad = check_swz<float2>(4096) + check_swz<double2>(4096);
  bad += check_line<4>() + check_line<5>() + check_line<6>() + check_line<7>() +
         check_line<8>() + check_line<9>() + check_line<10>();
  bad += check_xr<4>() + check_xr<5>() + check_xr<6>() + check_xr<7>() + check_xr<8>() +
         check_xr<9>() + check_xr<10>();
  if (bad) return 1;
  printf("ok\n");
  return 0;
}
