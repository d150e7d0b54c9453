// Inverse transform (C2R) that allocates no device memory.
//
// gbs_fft_c2r (through a plan) needs device memory that the plan allocates
// with cudaMalloc: the twiddle tables and a workspace for the intermediate
// spectral field.  Some callers cannot allocate device memory at all, for
// example an application whose device memory is reserved up front by its
// own pool allocator and which forbids other libraries from calling
// cudaMalloc, or a host process whose device memory budget is fixed before
// this library is loaded.  gbs_fft_c2r_noalloc serves them: it computes the
// same transform as gbs_fft_c2r(may_destroy = 0) but keeps its twiddles and
// workspace in one file-scope device array of kScratchBytes (32 MiB), which
// every GPU that loads the library holds until the process exits.
//
// The device address of that array is looked up with cudaGetSymbolAddress
// (the array's name in host code is only a host-side stand-in, not a device
// address) once per device and CUDA context: the first call on a device does
// this set-up, so that first call should come before any stream capture.
// The cache is keyed on the context's unique id, so a call made after
// cudaDeviceReset (which rebuilds the primary context and the array) looks
// the address up again instead of reusing a stale one.
//
// Under lazy module loading (CUDA_MODULE_LOADING=LAZY, the CUDA default)
// the array itself is only allocated by that first look-up.  A caller whose
// pool will later take all device memory must therefore make one call (any
// small transform) on each device before the pool reserves its memory, or
// run with CUDA_MODULE_LOADING=EAGER; after that, no call needs device
// memory beyond what it was given.
//
// All calls share the array and it keeps the contents of the last call, so
// calls whose GPU work overlaps (two streams, or two threads) race on it.
// Nothing in the array has to start at zero: every call regenerates the
// twiddles and the first pass writes the whole workspace before the next
// pass reads it.
#include <cuda.h>

#include <mutex>

#include "gbs_internal.cuh"

namespace gbs {

template <typename T> int make_twiddles(cplx<T>* tw, int n, cudaStream_t st);
template <typename T, int DIR>
int launch_col(const cplx<T>* in, cplx<T>* out, int n, int ncols, int nouter,
               int nfields, int64_t es, int64_t os, int64_t fs,
               const cplx<T>* tw, T scale, cudaStream_t st);
template <typename T>
int launch_c2r_rows(const cplx<T>* k, T* x, int nx, int64_t nrows,
                    const cplx<T>* twx, cudaStream_t st);

constexpr size_t kScratchBytes = size_t(32) << 20;  // 32 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

static std::mutex g_scratch_mu;
static unsigned char* g_scratch_ptr[kMaxDevices];
static unsigned long long g_scratch_ctx[kMaxDevices];  // context id of the entry

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Unique id of the calling thread's current CUDA context (0 if none is
// current yet), through driver entry points obtained from the runtime.
static int current_context_id(unsigned long long* id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  if (!get_current || !get_id) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    GBS_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000,
                                                  cudaEnableDefault, &q1));
    GBS_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000,
                                                  cudaEnableDefault, &q2));
    if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess ||
        !f1 || !f2) {
      set_error("gbs_fft_c2r_noalloc: driver entry points cuCtxGetCurrent / "
                "cuCtxGetId unavailable");
      return GBS_ECUDA;
    }
    get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    get_id = reinterpret_cast<CtxGetIdFn>(f2);
  }
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS) {
    set_error("gbs_fft_c2r_noalloc: cuCtxGetCurrent failed");
    return GBS_ECUDA;
  }
  *id = 0;
  if (ctx && get_id(ctx, id) != CUDA_SUCCESS) {
    set_error("gbs_fft_c2r_noalloc: cuCtxGetId failed");
    return GBS_ECUDA;
  }
  return GBS_OK;
}

// Device address of the scratch array on the current device (set-up on the
// first call per device and context).
static int scratch_address(unsigned char** out) {
  int dev = 0;
  GBS_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("gbs_fft_c2r_noalloc: device ordinal %d out of range", dev);
    return GBS_EINVAL;
  }
  unsigned long long ctx = 0;
  int rc = current_context_id(&ctx);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev] || ctx == 0 || g_scratch_ctx[dev] != ctx) {
    void* p = nullptr;
    // initialises the device's primary context if this thread has none yet
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_error("gbs_fft_c2r_noalloc: cudaGetSymbolAddress failed: %s",
                cudaGetErrorString(e));
      return GBS_ECUDA;
    }
    if (ctx == 0) {
      rc = current_context_id(&ctx);
      if (rc) return rc;
    }
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    g_scratch_ctx[dev] = ctx;
  }
  *out = g_scratch_ptr[dev];
  return GBS_OK;
}

static size_t align256(size_t b) { return (b + 255) / 256 * 256; }

template <typename T>
static int c2r_noalloc(int ndim, int nz, int ny, int nx, int batch,
                       const void* kv, void* xv, unsigned char* scratch,
                       cudaStream_t st) {
  using C = cplx<T>;
  const int nkx = nx / 2 + 1;
  const int64_t nK = (int64_t)nz * ny * nkx;
  C* twx = reinterpret_cast<C*>(scratch);
  C* twy = reinterpret_cast<C*>(scratch + align256(sizeof(C) * nx));
  C* twz = reinterpret_cast<C*>(reinterpret_cast<unsigned char*>(twy) +
                                align256(sizeof(C) * ny));
  C* w = reinterpret_cast<C*>(reinterpret_cast<unsigned char*>(twz) +
                              align256(sizeof(C) * nz));
  int rc = make_twiddles<T>(twx, nx, st);
  if (!rc) rc = make_twiddles<T>(twy, ny, st);
  if (!rc) rc = make_twiddles<T>(twz, nz, st);
  if (rc) return rc;
  const C* k = static_cast<const C*>(kv);
  T* x = static_cast<T*>(xv);
  const int64_t rows = (int64_t)batch * nz * ny;
  if (ndim == 2) {
    rc = launch_col<T, 1>(k, w, ny, nkx, 1, batch, nkx, 0, nK, twy, T(1), st);
    if (rc) return rc;
    return launch_c2r_rows<T>(w, x, nx, rows, twx, st);
  }
  rc = launch_col<T, 1>(k, w, nz, nkx, ny, batch, (int64_t)ny * nkx, nkx, nK,
                        twz, T(1), st);
  if (rc) return rc;
  rc = launch_col<T, 1>(w, w, ny, nkx, nz, batch, nkx, (int64_t)ny * nkx, nK,
                        twy, T(1), st);
  if (rc) return rc;
  return launch_c2r_rows<T>(w, x, nx, rows, twx, st);
}

}  // namespace gbs

extern "C" int gbs_fft_c2r_noalloc(int ndim, const int64_t* shapeX, int dtype,
                                   int batch, const void* k, void* x,
                                   void* stream) {
  gbs::clear_error();
  if (!shapeX || !k || !x || (ndim != 2 && ndim != 3) || batch < 1 ||
      (dtype != GBS_F32 && dtype != GBS_F64)) {
    gbs::set_error("gbs_fft_c2r_noalloc: invalid argument");
    return GBS_EINVAL;
  }
  const int64_t nz = ndim == 3 ? shapeX[0] : 1;
  const int64_t ny = shapeX[ndim - 2];
  const int64_t nx = shapeX[ndim - 1];
  if (nx < 2 || nx % 2 || ny < 1 || nz < 1 || nx > 65536 || ny > 65536 ||
      nz > 65536) {
    gbs::set_error("gbs_fft_c2r_noalloc: unsupported shape (nx must be even)");
    return GBS_EINVAL;
  }
  const size_t cs = dtype == GBS_F64 ? sizeof(double2) : sizeof(float2);
  const size_t need = gbs::align256(cs * nx) + gbs::align256(cs * ny) +
                      gbs::align256(cs * nz) +
                      cs * (size_t)batch * nz * ny * (nx / 2 + 1);
  if (need > gbs::kScratchBytes) {
    gbs::set_error(
        "gbs_fft_c2r_noalloc: this transform needs %zu bytes of scratch, more "
        "than the static maximum of %zu bytes (32 MiB); use a plan "
        "(gbs_fft_plan_create + gbs_fft_c2r) instead",
        need, gbs::kScratchBytes);
    return GBS_EINVAL;
  }
  unsigned char* scratch = nullptr;
  int rc = gbs::scratch_address(&scratch);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == GBS_F64)
    return gbs::c2r_noalloc<double>(ndim, (int)nz, (int)ny, (int)nx, batch, k, x,
                                    scratch, st);
  return gbs::c2r_noalloc<float>(ndim, (int)nz, (int)ny, (int)nx, batch, k, x,
                                 scratch, st);
}
