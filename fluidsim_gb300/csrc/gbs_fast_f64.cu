// double instantiation of the compile-time-size kernels.
#include "gbs_fast_launch.cuh"

namespace gbs {
namespace fast {

GBS_FAST_INSTANTIATE(double)

}  // namespace fast
}  // namespace gbs
