// Host entry points of the compile-time-size kernels (gbs_fast.cuh),
// instantiated for float in gbs_fast_f32.cu and double in gbs_fast_f64.cu.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "gbs_ns.cuh"

namespace gbs {
namespace fast {

struct ColArgs;
struct Geo;

// Staging of the x pass's inputs (kf3_xr): bulk copies into shared memory
// whose completion is awaited on mbarriers with a bounded wait.
struct XStage {
  int* status;                    // device word: set to 1 when a wait ran out
  unsigned long long timeout_ns;  // limit of each wait
  int stall;                      // test hook: one copy of the launch is never issued
};

// Axis lengths with compiled kernels: 2^kMinLog .. 2^kMaxLog.
constexpr int kMinLog = 5;
constexpr int kMaxLog = 10;

bool supported(int ndim, int nx, int ny, int nz);
bool supported_axis(int n);

template <typename T>
int col(int n, const void* in, void* out, const ColArgs& a, int nouter, int nfields,
        const void* tw, double scale, int dir, cudaStream_t st);
template <typename T>
int r2c_rows(int nx, const void* x, void* k, int64_t nrows, const void* twx, double scale,
             cudaStream_t st);
template <typename T>
int c2r_rows(int nx, const void* k, void* x, int64_t nrows, const void* twx, cudaStream_t st);
template <typename T>
int A3(const Geo& g, const void* S, void* W, const void* twz, cudaStream_t st);
template <typename T>
int B3(const Geo& g, const void* W, void* F, const void* twx, unsigned long long* vmax,
       const XStage& xs, cudaStream_t st);
template <typename T>
int C3(const Geo& g, const void* F, const void* twz, int mode, const RKArgs& a,
       cudaStream_t st);
template <typename T>
int A2(const Geo& g, const void* S, void* W, const void* twy, cudaStream_t st);
template <typename T>
int B2(const Geo& g, const void* W, void* F, const void* twx, unsigned long long* vmax,
       cudaStream_t st);
template <typename T>
int C2(const Geo& g, const void* F, const void* twy, int mode, const RKArgs& a,
       cudaStream_t st);

}  // namespace fast
}  // namespace gbs
