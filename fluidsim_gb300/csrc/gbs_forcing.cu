// Coarse normalized forcing, one device step (fluidsim's "tcrandom",
// "random" and "proportional" forcings,
// fluidsim/base/forcing/specific.py:137-346 (coarse grid, index maps),
// 346-425 (proportional), 428-727 (2nd_degree_eq normalization) and
// 729-868 (random and time-correlated random draws)).
//
// The forcing lives on a coarse grid of nc points per axis (coarse spectral
// shape (nc, nc, nc/2+1), 2D (nc, nc/2+1)).  Coarse mode (izc, iyc, ixc)
// maps to the full-grid mode (iz, iy, ixc), with i = ic if ic <= nc/2 else
// ic - nc + n along y and z (_ik_from_ikc, operators3d.py:1183-1193).
//
// For each forced state variable, in one CTA:
//   normalized:   fr = f1 - mix (f1 - f0)  (mix = (cos((t - t_last) pi / T)
//                 + 1) / 2 from the host; f0 = f1 for "random");
//                 a = dt/2 sum w |fr|^2, b = sum w Re(conj(v) fr), c = -P,
//                 R = the root of a R^2 + b R + c = 0 picked by which_root;
//   proportional: fr = v on the forced modes (0 elsewhere),
//                 Z = sum w |fr|^2 / 2, R = (sqrt(1 + dt P / Z) - 1) / dt;
// then forcing[var] = R fr on every coarse mode (the other modes of the
// dense forcing array are never written and stay zero).  Sums use the
// Hermitian weights of the coarse grid (w = 1 at kx = 0 and the coarse
// Nyquist column, else 2) and accumulate in FP64; v is read at the mapped
// full-grid mode in the state's precision.
#include "gbs_internal.cuh"

namespace gbs {

struct ForcingGeom {
  int ndim, nvar, type, which_root, nkeys;
  int keys[8];
  int64_t nx, ny, nz, nc, nkxc, ncz;
  double P;
};

__device__ __forceinline__ int64_t fine_index(int64_t ic, int64_t nc, int64_t n) {
  return ic <= nc / 2 ? ic : ic - nc + n;
}

__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
  return s;
}

// The 2nd-degree root fluidsim's coef_normalization_from_abc picks.
__device__ double pick_root(double a, double b, double c, int which) {
  if (!(a != 0.0)) return 0.0;  // np.roots drops the leading zero: 0 returned
  const double disc = b * b - 4.0 * a * c;
  const double s = sqrt(disc > 0.0 ? disc : 0.0);
  double lo, hi;  // the two real roots
  if (b == 0.0) {
    lo = -s / (2.0 * a);
    hi = s / (2.0 * a);
  } else {
    const double q = -0.5 * (b + copysign(s, b));
    lo = q / a;
    hi = c / q;
  }
  if (which == 1) return lo > hi ? lo : hi;  // "positive": the positive root
  // "minabs"; with b == 0 both have the same magnitude and np.roots lists
  // the negative one first, which the reference then keeps
  if (b == 0.0) return lo;
  return fabs(hi) < fabs(lo) ? hi : lo;
}

template <typename T>
__global__ void __launch_bounds__(256)
k_forcing_coarse(ForcingGeom g, const cplx<T>* __restrict__ S,
                 const double2* __restrict__ f0, const double2* __restrict__ f1,
                 const unsigned char* __restrict__ no_f, double mix, double dt,
                 cplx<T>* __restrict__ F, double* __restrict__ coef) {
  __shared__ double red[8];
  __shared__ double R;
  const int64_t nyc = g.nc, nzc = g.ndim == 3 ? g.nc : 1;
  const int64_t ncK = nzc * nyc * g.nkxc;
  const int64_t nK = g.nz * g.ny * (g.nx / 2 + 1);
  const int64_t nkx = g.nx / 2 + 1;
  for (int k = 0; k < g.nkeys; ++k) {
    const int var = g.keys[k];
    double sa = 0.0, sb = 0.0;
    for (int64_t i = threadIdx.x; i < ncK; i += blockDim.x) {
      const int64_t ixc = i % g.nkxc, r = i / g.nkxc;
      const int64_t iyc = r % nyc, izc = r / nyc;
      const int64_t iy = fine_index(iyc, nyc, g.ny);
      const int64_t iz = g.ndim == 3 ? fine_index(izc, nzc, g.nz) : 0;
      const cplx<T> v = S[var * nK + (iz * g.ny + iy) * nkx + ixc];
      const double vr = (double)v.x, vi = (double)v.y;
      double fr, fi;
      if (g.type == 0) {
        fr = __dsub_rn(f1[i].x, __dmul_rn(mix, __dsub_rn(f1[i].x, f0[i].x)));
        fi = __dsub_rn(f1[i].y, __dmul_rn(mix, __dsub_rn(f1[i].y, f0[i].y)));
      } else {
        fr = no_f[i] ? 0.0 : vr;
        fi = no_f[i] ? 0.0 : vi;
      }
      const double w = (ixc == 0 || ixc == g.nkxc - 1) ? 1.0 : 2.0;
      sa += w * (fr * fr + fi * fi);
      sb += w * (vr * fr + vi * fi);
    }
    sa = block_sum(sa, red);
    sb = block_sum(sb, red);
    if (threadIdx.x == 0) {
      double c;
      if (g.type == 0) {
        c = pick_root(dt / 2.0 * sa, sb, -g.P, g.which_root);
      } else {
        const double Z = sa / 2.0;
        c = Z > 0.0 ? (sqrt(1.0 + dt * g.P / Z) - 1.0) / dt : 0.0;
      }
      R = c;
      if (coef) coef[k] = c;
    }
    __syncthreads();
    const double c = R;
    for (int64_t i = threadIdx.x; i < ncK; i += blockDim.x) {
      const int64_t ixc = i % g.nkxc, r = i / g.nkxc;
      const int64_t iyc = r % nyc, izc = r / nyc;
      const int64_t iy = fine_index(iyc, nyc, g.ny);
      const int64_t iz = g.ndim == 3 ? fine_index(izc, nzc, g.nz) : 0;
      const int64_t at = var * nK + (iz * g.ny + iy) * nkx + ixc;
      double fr, fi;
      if (g.type == 0) {
        fr = __dsub_rn(f1[i].x, __dmul_rn(mix, __dsub_rn(f1[i].x, f0[i].x)));
        fi = __dsub_rn(f1[i].y, __dmul_rn(mix, __dsub_rn(f1[i].y, f0[i].y)));
      } else {
        const cplx<T> v = S[at];
        fr = no_f[i] ? 0.0 : (double)v.x;
        fi = no_f[i] ? 0.0 : (double)v.y;
      }
      cplx<T> out;
      out.x = (T)(c * fr);
      out.y = (T)(c * fi);
      F[at] = out;
    }
    __syncthreads();
  }
}

}  // namespace gbs

extern "C" int gbs_forcing_coarse(const gbs_forcing_params* p, const void* state_spect,
                                  const void* f0, const void* f1,
                                  const unsigned char* no_forcing, double mix,
                                  double dt, void* forcing, double* coef,
                                  void* stream) {
  gbs::clear_error();
  if (!p || !state_spect || !forcing || (p->ndim != 2 && p->ndim != 3) ||
      p->nkeys < 1 || p->nkeys > 8 || p->nc < 2 || p->nc % 2 ||
      (p->dtype != GBS_F32 && p->dtype != GBS_F64) || (p->type != 0 && p->type != 1) ||
      (p->which_root != 0 && p->which_root != 1) ||
      (p->type == 0 && (!f0 || !f1)) || (p->type == 1 && !no_forcing)) {
    gbs::set_error("gbs_forcing_coarse: invalid argument");
    return GBS_EINVAL;
  }
  const int64_t nz = p->ndim == 3 ? p->nz : 1;
  if (p->nc > p->nx || p->nc > p->ny || (p->ndim == 3 && p->nc > p->nz)) {
    gbs::set_error("gbs_forcing_coarse: coarse grid larger than the grid");
    return GBS_EINVAL;
  }
  gbs::ForcingGeom g;
  g.ndim = p->ndim;
  g.nvar = p->nvar;
  g.type = p->type;
  g.which_root = p->which_root;
  g.nkeys = p->nkeys;
  for (int k = 0; k < 8; ++k) g.keys[k] = k < p->nkeys ? p->keys[k] : 0;
  for (int k = 0; k < p->nkeys; ++k) {
    if (p->keys[k] < 0 || p->keys[k] >= p->nvar) {
      gbs::set_error("gbs_forcing_coarse: forced variable %d out of range", p->keys[k]);
      return GBS_EINVAL;
    }
  }
  g.nx = p->nx;
  g.ny = p->ny;
  g.nz = nz;
  g.nc = p->nc;
  g.nkxc = p->nc / 2 + 1;
  g.ncz = p->ndim == 3 ? p->nc : 1;
  g.P = p->forcing_rate;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const double2* a = static_cast<const double2*>(f0);
  const double2* b = static_cast<const double2*>(f1);
  if (p->dtype == GBS_F64)
    gbs::k_forcing_coarse<double><<<1, 256, 0, st>>>(
        g, static_cast<const double2*>(state_spect), a, b, no_forcing, mix, dt,
        static_cast<double2*>(forcing), coef);
  else
    gbs::k_forcing_coarse<float><<<1, 256, 0, st>>>(
        g, static_cast<const float2*>(state_spect), a, b, no_forcing, mix, dt,
        static_cast<float2*>(forcing), coef);
  GBS_CHECK_LAUNCH();
  return GBS_OK;
}
