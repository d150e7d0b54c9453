// Host emulation of gbs::fft_tile: runs the per-thread Stockham / direct-DFT
// phases of the CUDA core sequentially for every thread id, with a barrier
// between phases, so the index arithmetic can be checked without a GPU.
#include <vector>
#include "../../fluidsim_gb300/csrc/gbs_core.cuh"

using namespace gbs;
constexpr int TPT = 2;

template <int R, int DIR>
static void stage(double2* buf, int n, int log2n, int Ns, int log2Ns,
                  int nlines, int LP, const double2* tw, int tw_stride,
                  int nthreads) {
  std::vector<double2> regs((size_t)nthreads * TPT * 8);
  for (int t = 0; t < nthreads; ++t)
    stockham_load<R, DIR, TPT>(buf, reinterpret_cast<double2(*)[8]>(&regs[(size_t)t * TPT * 8]),
                               n, log2n, Ns, log2Ns, nlines, LP, tw, tw_stride, t, nthreads);
  for (int t = 0; t < nthreads; ++t)
    stockham_store<R, TPT>(buf, reinterpret_cast<double2(*)[8]>(&regs[(size_t)t * TPT * 8]),
                           n, Ns, log2Ns, nlines, LP, t, nthreads);
}

template <int DIR>
static void run(double2* buf, int n, int nlines, int LP, const double2* tw,
                int tw_stride, int nthreads) {
  if (is_pow2(n) && n >= 8) {
    int log2n = ilog2(n), s8 = log2n / 3, rem = log2n % 3, Ns = 1, l2 = 0;
    for (int s = 0; s < s8; ++s, Ns <<= 3, l2 += 3)
      stage<8, DIR>(buf, n, log2n, Ns, l2, nlines, LP, tw, tw_stride, nthreads);
    if (rem == 1) stage<2, DIR>(buf, n, log2n, Ns, l2, nlines, LP, tw, tw_stride, nthreads);
    if (rem == 2) stage<4, DIR>(buf, n, log2n, Ns, l2, nlines, LP, tw, tw_stride, nthreads);
  } else if (n > 1) {
    std::vector<double2> b2((size_t)n * LP);
    for (int t = 0; t < nthreads; ++t)
      dft_direct_part<DIR>(buf, b2.data(), n, nlines, LP, tw, tw_stride, t, nthreads);
    for (int t = 0; t < nthreads; ++t)
      copy_part(b2.data(), buf, n, nlines, LP, t, nthreads);
  }
}

extern "C" int emulate_fft_tile(int n, int nlines, int LP, int dir, int nthreads,
                                double* data, const double* tw, int tw_stride) {
  double2* buf = reinterpret_cast<double2*>(data);
  const double2* w = reinterpret_cast<const double2*>(tw);
  if (is_pow2(n) && n >= 8 && nlines * (n / 8) > TPT * nthreads) return -1;
  if (dir < 0) run<-1>(buf, n, nlines, LP, w, tw_stride, nthreads);
  else run<1>(buf, n, nlines, LP, w, tw_stride, nthreads);
  return 0;
}
