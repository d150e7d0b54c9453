// float instantiation of the compile-time-size kernels.
#include "gbs_fast_launch.cuh"

namespace gbs {
namespace fast {

bool supported_axis(int n) {
  return is_pow2(n) && n >= (1 << kMinLog) && n <= (1 << kMaxLog);
}

bool supported(int ndim, int nx, int ny, int nz) {
  auto ok = [](int n) { return supported_axis(n); };
  if (nx % 2 || !ok(nx / 2) || !ok(ny)) return false;
  return ndim == 2 ? nz == 1 : ok(nz);
}

GBS_FAST_INSTANTIATE(float)

}  // namespace fast
}  // namespace gbs
