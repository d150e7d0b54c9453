// Host-side helpers shared by the libgbspec translation units.
#pragma once

#include <cstdio>
#include <cstring>
#include <string>
#include <cuda_runtime.h>

#include "../../include/gbspec.h"
#include "gbs_core.cuh"

namespace gbs {

void set_error(const char* fmt, ...);
void clear_error();

// On failure the runtime's last-error state is consumed as well, so that a
// non-sticky error (an invalid argument) is not reported again by the next
// launch check of an unrelated call.
#define GBS_CUDA_TRY(expr)                                                  \
  do {                                                                      \
    cudaError_t _e = (expr);                                                \
    if (_e != cudaSuccess) {                                                \
      (void)cudaGetLastError();                                             \
      ::gbs::set_error("%s:%d: %s: %s", __FILE__, __LINE__, #expr,          \
                       cudaGetErrorString(_e));                             \
      return GBS_ECUDA;                                                     \
    }                                                                       \
  } while (0)

#define GBS_CHECK_LAUNCH() GBS_CUDA_TRY(cudaGetLastError())

inline int round_up(int a, int b) { return (a + b - 1) / b * b; }
inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// Threads for a tile of `lines` lines of length n processed with TPT tasks
// per thread (power of two) or by the direct DFT (other n).
constexpr int kTPT = 2;
constexpr int kMaxThreads = 512;

inline int tile_threads(int n, int lines) {
  if (is_pow2(n) && n >= 8) {
    int tasks = lines * (n / 8);
    int t = round_up((tasks + kTPT - 1) / kTPT, 32);
    if (t < 64) t = 64;
    if (t > kMaxThreads) t = kMaxThreads;
    return t;
  }
  int t = round_up(lines * n, 32);
  if (t < 64) t = 64;
  if (t > 256) t = 256;
  return t;
}

inline bool tile_fits(int n, int lines) {
  if (is_pow2(n) && n >= 8) return lines * (n / 8) <= kTPT * kMaxThreads;
  return true;
}

inline size_t tile_smem(int n, int LP, size_t csize) {
  size_t s = (size_t)n * LP * csize;
  if (!(is_pow2(n) && n >= 8)) s *= 2;  // direct DFT needs a second tile
  return s;
}

constexpr size_t kSmemBudget = 100 * 1024;
constexpr size_t kSmemMax = 227 * 1024;

// Largest power-of-two tile width (<= txmax) whose tile fits the budget.
inline int pick_tx(int n, int fields, size_t csize, int txmax, int ncols) {
  int tx = txmax;
  while (tx > 1 && (tile_smem(n, fields * tx, csize) > kSmemBudget ||
                    !tile_fits(n, fields * tx) || tx / 2 >= ncols))
    tx /= 2;
  return tx;
}

template <typename K>
int allow_smem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) {
    GBS_CUDA_TRY(cudaFuncSetAttribute(
        kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  }
  return GBS_OK;
}

}  // namespace gbs
